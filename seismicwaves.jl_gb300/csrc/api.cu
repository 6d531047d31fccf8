// C-ABI edge of libswgb300: contexts, status codes, profiling and the
// acoustic entry points declared in include/swgb300.h.  Every call catches
// the library's internal errors and turns them into a status code plus a
// message retrievable with sw_ctx_last_error().
#include <cstdio>
#include <cstring>
#include <new>
#include <string>


#include "internal.h"

namespace swgb {

void wavesim_init(sw_wavesim* ws, sw_ctx* ctx, const sw_acoustic_params* p, int gradient, const sw_grad_params* gp);
void wavesim_set_vp(sw_wavesim* ws, const float* vp, bool on_device);
void acoustic_forward(sw_wavesim* ws, int nshots, const sw_acoustic_shot* shots, bool on_device);
void acoustic_gradient(sw_wavesim* ws, int nshots, const sw_acoustic_shot* shots, bool on_device, double* grad,
                       double* misfit);
void wavesim_set_tuning(sw_wavesim* ws, int tz, int variant);
void wavesim_set_band_heights(sw_wavesim* ws, int tz_forward, int tz_recompute, int tz_adjoint);
void wavesim_set_wait_test(sw_wavesim* ws, long long wait_cycles, int withhold);
void wavesim_set_precision(sw_wavesim* ws, int mode);
void wavesim_set_vp64(sw_wavesim* ws, const double* vp, bool on_device);
void wavesim_use_graphs(sw_wavesim* ws, bool on);
void acoustic_forward_snapshots(sw_wavesim* ws, int nshots, const sw_acoustic_shot* shots, bool on_device,
                                int snapevery, float* const* snapshots);
sw_ctx* wavesim_ctx(sw_wavesim* ws);
sw_wavesim* wavesim_new();
void wavesim_delete(sw_wavesim* ws);
void elastic_init(sw_elastic* es, sw_ctx* ctx, const sw_elastic_params* p, int gradient, const sw_grad_params* gp);
void elastic_set_material(sw_elastic* es, const float* lam, const float* mu, const float* rho);
void elastic_forward(sw_elastic* es, int nshots, const sw_elastic_shot* shots, bool on_device);
void elastic_gradient(sw_elastic* es, int nshots, const sw_elastic_shot* shots, bool on_device, double* g_rho,
                      double* g_lam, double* g_mu, double* misfit);
void elastic_set_tuning(sw_elastic* es, int tz);
void elastic_forward_snapshots(sw_elastic* es, int nshots, const sw_elastic_shot* shots, bool on_device,
                               int snapevery, float* const* snapshots);
sw_ctx* elastic_ctx(sw_elastic* es);
sw_elastic* elastic_new();
void elastic_delete(sw_elastic* es);
void vd_init(sw_acoustic_vd* vd, sw_ctx* ctx, const sw_acoustic_params* p, int interp, int gradient,
             const sw_grad_params* gp);
void vd_set_material(sw_acoustic_vd* vd, const float* vp, const float* rho);
void vd_forward(sw_acoustic_vd* vd, int nshots, const sw_acoustic_shot* shots, bool on_device);
void vd_forward_snapshots(sw_acoustic_vd* vd, int nshots, const sw_acoustic_shot* shots, bool on_device, int snapevery,
                          float* const* snapshots);
void vd_gradient(sw_acoustic_vd* vd, int nshots, const sw_acoustic_shot* shots, bool on_device, double* g_vp,
                 double* g_rho, double* misfit);
void vd_set_tuning(sw_acoustic_vd* vd, int tz);
void vd_set_precision(sw_acoustic_vd* vd, int mode);
void vd_set_material64(sw_acoustic_vd* vd, const double* vp, const double* rho);
sw_ctx* vd_ctx(sw_acoustic_vd* vd);
sw_acoustic_vd* vd_new();
void vd_delete(sw_acoustic_vd* vd);

[[noreturn]] void fail(int code, const std::string& msg) { throw SwError{code, msg}; }

void check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  const int code = (e == cudaErrorMemoryAllocation) ? SW_ERR_OOM : SW_ERR_CUDA;
  fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}

void dev_alloc(DevMem& m, size_t bytes, const char* what, cudaStream_t st) {
  m.release();
  if (bytes == 0) bytes = 16;
  void* p = nullptr;
  const cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free allocation error
    char buf[160];
    std::snprintf(buf, sizeof(buf), "device allocation of %.3f GB for %s failed", bytes / 1e9, what);
    fail(SW_ERR_OOM, buf);
  }
  m.p = p;
  m.bytes = bytes;
  check_cuda(cudaMemsetAsync(p, 0, bytes, st), what);
}

cudaEvent_t Profiler::get() {
  if (!pool.empty()) {
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  check_cuda(cudaEventCreate(&e), "cudaEventCreate");
  return e;
}

void Profiler::begin(cudaStream_t s, int kind, double b, cudaEvent_t* a_out) {
  *a_out = nullptr;
  if (!on) return;
  cudaEvent_t a = get();
  check_cuda(cudaEventRecord(a, s), "cudaEventRecord");
  bytes[kind] += b;
  *a_out = a;
}

void Profiler::end(cudaStream_t s, int kind, cudaEvent_t a, int nk) {
  if (!on || !a) return;
  cudaEvent_t b = get();
  check_cuda(cudaEventRecord(b, s), "cudaEventRecord");
  pending.push_back(Pending{a, b, kind, nk});
  if (pending.size() > 8192) resolve();
}

void Profiler::resolve() {
  if (pending.empty()) return;
  check_cuda(cudaEventSynchronize(pending.back().b), "cudaEventSynchronize");
  for (const Pending& p : pending) {
    float ms = 0.f;
    check_cuda(cudaEventElapsedTime(&ms, p.a, p.b), "cudaEventElapsedTime");
    total_ms[p.kind] += ms;
    launches[p.kind] += 1;
    kernels[p.kind] += p.nk;
    pool.push_back(p.a);
    pool.push_back(p.b);
  }
  pending.clear();
}

Profiler::~Profiler() {
  for (const Pending& p : pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (cudaEvent_t e : pool) cudaEventDestroy(e);
}

}  // namespace swgb

using swgb::SwError;

namespace {

template <typename F>
int guarded(sw_ctx* ctx, F&& f) {
  try {
    f();
    if (ctx) ctx->last_error.clear();
    return SW_OK;
  } catch (const SwError& e) {
    if (ctx) ctx->last_error = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->last_error = "host allocation failed";
    return SW_ERR_OOM;
  } catch (...) {
    if (ctx) ctx->last_error = "unexpected internal error";
    return SW_ERR_CUDA;
  }
}

}  // namespace

extern "C" {

int sw_version(void) { return 100; }

int sw_ctx_create(int device, void* stream, sw_ctx** out) {
  if (!out) return SW_ERR_ARG;
  *out = nullptr;
  sw_ctx* ctx = new (std::nothrow) sw_ctx();
  if (!ctx) return SW_ERR_OOM;
  int dcount = 0;
  cudaError_t e = cudaGetDeviceCount(&dcount);
  if (e != cudaSuccess || dcount == 0) {
    cudaGetLastError();
    delete ctx;
    return SW_ERR_CUDA;
  }
  if (device < 0 || device >= dcount) {
    delete ctx;
    return SW_ERR_ARG;
  }
  const int rc = guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(device), "cudaSetDevice");
    ctx->device = device;
    swgb::check_cuda(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device), "SM count");
    if (stream) {
      ctx->stream = static_cast<cudaStream_t>(stream);
      ctx->own_stream = false;
    } else {
      swgb::check_cuda(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "cudaStreamCreate");
      ctx->own_stream = true;
    }
  });
  if (rc != SW_OK) {
    delete ctx;
    return rc;
  }
  *out = ctx;
  return SW_OK;
}

int sw_ctx_destroy(sw_ctx* ctx) {
  if (!ctx) return SW_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return SW_OK;
}

const char* sw_ctx_last_error(const sw_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

void* sw_ctx_stream(const sw_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

int sw_cpml_coefficients(double vel_max, double dt, int32_t halo, double rcoef, double h, double f0,
                         int32_t freetop_axis, float* a, float* a_h, float* b, float* b_h) {
  if (halo < 0 || !(dt > 0) || !(h > 0) || !a || !b || (halo > 0 && (!a_h || !b_h))) return SW_ERR_ARG;
  const int na = 2 * (halo + 1), nh = 2 * halo;
  double* tmp = new (std::nothrow) double[2 * na + 2 * nh + 4];
  if (!tmp) return SW_ERR_OOM;
  swgb::cpml_axis_coefficients(vel_max, dt, halo, rcoef, h, f0, freetop_axis != 0, tmp, tmp + na, tmp + na + nh,
                               tmp + 2 * na + nh);
  for (int k = 0; k < na; ++k) { a[k] = (float)tmp[k]; b[k] = (float)tmp[na + nh + k]; }
  for (int k = 0; k < nh; ++k) { a_h[k] = (float)tmp[na + k]; b_h[k] = (float)tmp[2 * na + nh + k]; }
  delete[] tmp;
  return SW_OK;
}

int sw_cpml_coefficients64(double vel_max, double dt, int32_t halo, double rcoef, double h, double f0,
                           int32_t freetop_axis, double* a, double* a_h, double* b, double* b_h) {
  if (halo < 0 || !(dt > 0) || !(h > 0) || !a || !b || (halo > 0 && (!a_h || !b_h))) return SW_ERR_ARG;
  const int na = 2 * (halo + 1), nh = 2 * halo;
  double* tmp = new (std::nothrow) double[2 * na + 2 * nh + 4];
  if (!tmp) return SW_ERR_OOM;
  swgb::cpml_axis_coefficients(vel_max, dt, halo, rcoef, h, f0, freetop_axis != 0, tmp, tmp + na, tmp + na + nh,
                               tmp + 2 * na + nh);
  for (int k = 0; k < na; ++k) { a[k] = tmp[k]; b[k] = tmp[na + nh + k]; }
  for (int k = 0; k < nh; ++k) { a_h[k] = tmp[na + k]; b_h[k] = tmp[2 * na + nh + k]; }
  delete[] tmp;
  return SW_OK;
}

int sw_wavesim_create(sw_ctx* ctx, const sw_acoustic_params* params, int32_t gradient, const sw_grad_params* gparams,
                      sw_wavesim** out) {
  if (!ctx || !out) return SW_ERR_ARG;
  *out = nullptr;
  sw_wavesim* ws = nullptr;
  const int rc = guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    ws = swgb::wavesim_new();
    swgb::wavesim_init(ws, ctx, params, gradient, gparams);
  });
  if (rc != SW_OK) {
    if (ws) swgb::wavesim_delete(ws);
    return rc;
  }
  *out = ws;
  return SW_OK;
}

int sw_wavesim_destroy(sw_wavesim* ws) {
  if (!ws) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::wavesim_ctx(ws);
  if (ctx) {
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
  }
  swgb::wavesim_delete(ws);
  return SW_OK;
}

int sw_wavesim_set_vp(sw_wavesim* ws, const float* vp, int32_t on_device) {
  if (!ws) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::wavesim_ctx(ws);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::wavesim_set_vp(ws, vp, on_device != 0);
  });
}

int sw_wavesim_set_vp64(sw_wavesim* ws, const double* vp, int32_t on_device) {
  if (!ws) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::wavesim_ctx(ws);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::wavesim_set_vp64(ws, vp, on_device != 0);
  });
}

int sw_acoustic_forward(sw_wavesim* ws, int32_t nshots, const sw_acoustic_shot* shots, int32_t on_device) {
  if (!ws) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::wavesim_ctx(ws);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::acoustic_forward(ws, nshots, shots, on_device != 0);
  });
}

int sw_acoustic_gradient(sw_wavesim* ws, int32_t nshots, const sw_acoustic_shot* shots, int32_t on_device,
                         double* grad, double* misfit) {
  if (!ws) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::wavesim_ctx(ws);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::acoustic_gradient(ws, nshots, shots, on_device != 0, grad, misfit);
  });
}

int sw_profile_enable(sw_ctx* ctx, int32_t on) {
  if (!ctx) return SW_ERR_ARG;
  return guarded(ctx, [&] {
    ctx->prof.resolve();
    ctx->prof.on = on != 0;
    if (on) {
      for (int k = 0; k < swgb::KK_COUNT; ++k) {
        ctx->prof.total_ms[k] = 0;
        ctx->prof.launches[k] = 0;
        ctx->prof.kernels[k] = 0;
        ctx->prof.bytes[k] = 0;
      }
    }
  });
}

int sw_profile_read(sw_ctx* ctx, int32_t kind, double* total_ms, int64_t* launches, double* bytes) {
  if (!ctx || kind < 0 || kind >= swgb::KK_COUNT) return SW_ERR_ARG;
  return guarded(ctx, [&] {
    ctx->prof.resolve();
    if (total_ms) *total_ms = ctx->prof.total_ms[kind];
    if (launches) *launches = ctx->prof.launches[kind];
    if (bytes) *bytes = ctx->prof.bytes[kind];
  });
}

int sw_profile_read_kernels(sw_ctx* ctx, int32_t kind, int64_t* kernels) {
  if (!ctx || !kernels || kind < 0 || kind >= swgb::KK_COUNT) return SW_ERR_ARG;
  return guarded(ctx, [&] {
    ctx->prof.resolve();
    *kernels = ctx->prof.kernels[kind];
  });
}

int sw_wavesim_set_tuning(sw_wavesim* ws, int32_t tz, int32_t variant) {
  if (!ws || tz < 0 || variant < 0 || variant >= (1 << 19)) return SW_ERR_ARG;
  swgb::wavesim_set_tuning(ws, tz, variant);
  return SW_OK;
}

int sw_wavesim_set_precision(sw_wavesim* ws, int32_t mode) {
  if (!ws || mode < 0 || mode > 1) return SW_ERR_ARG;
  return guarded(swgb::wavesim_ctx(ws), [&] { swgb::wavesim_set_precision(ws, mode); });
}

int sw_wavesim_set_wait_test(sw_wavesim* ws, int64_t wait_cycles, int32_t withhold_stage) {
  if (!ws || wait_cycles < 1000 || wait_cycles > 100000000000LL || withhold_stage < -1) return SW_ERR_ARG;
  swgb::wavesim_set_wait_test(ws, wait_cycles, withhold_stage);
  return SW_OK;
}

int sw_wavesim_set_band_heights(sw_wavesim* ws, int32_t tz_forward, int32_t tz_recompute, int32_t tz_adjoint) {
  if (!ws || tz_forward < 0 || tz_recompute < 0 || tz_adjoint < 0 || tz_forward > 4096 || tz_recompute > 4096 ||
      tz_adjoint > 4096)
    return SW_ERR_ARG;
  swgb::wavesim_set_band_heights(ws, tz_forward, tz_recompute, tz_adjoint);
  return SW_OK;
}

int sw_elastic_create(sw_ctx* ctx, const sw_elastic_params* params, int32_t gradient, const sw_grad_params* gparams,
                      sw_elastic** out) {
  if (!ctx || !out) return SW_ERR_ARG;
  *out = nullptr;
  sw_elastic* es = nullptr;
  const int rc = guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    es = swgb::elastic_new();
    swgb::elastic_init(es, ctx, params, gradient, gparams);
  });
  if (rc != SW_OK) {
    if (es) swgb::elastic_delete(es);
    return rc;
  }
  *out = es;
  return SW_OK;
}

int sw_elastic_destroy(sw_elastic* es) {
  if (!es) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::elastic_ctx(es);
  if (ctx) {
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
  }
  swgb::elastic_delete(es);
  return SW_OK;
}

int sw_elastic_set_material(sw_elastic* es, const float* lambda, const float* mu, const float* rho) {
  if (!es) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::elastic_ctx(es);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::elastic_set_material(es, lambda, mu, rho);
  });
}

int sw_elastic_forward(sw_elastic* es, int32_t nshots, const sw_elastic_shot* shots, int32_t on_device) {
  if (!es) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::elastic_ctx(es);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::elastic_forward(es, nshots, shots, on_device != 0);
  });
}

int sw_elastic_gradient(sw_elastic* es, int32_t nshots, const sw_elastic_shot* shots, int32_t on_device,
                        double* grad_rho, double* grad_lambda, double* grad_mu, double* misfit) {
  if (!es) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::elastic_ctx(es);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::elastic_gradient(es, nshots, shots, on_device != 0, grad_rho, grad_lambda, grad_mu, misfit);
  });
}

int sw_elastic_set_tuning(sw_elastic* es, int32_t tz) {
  if (!es) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::elastic_ctx(es);
  return guarded(ctx, [&] { swgb::elastic_set_tuning(es, tz); });
}

int sw_wavesim_use_graphs(sw_wavesim* ws, int32_t on) {
  if (!ws) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::wavesim_ctx(ws);
  return guarded(ctx, [&] { swgb::wavesim_use_graphs(ws, on != 0); });
}

int sw_acoustic_forward_snapshots(sw_wavesim* ws, int32_t nshots, const sw_acoustic_shot* shots, int32_t on_device,
                                  int32_t snapevery, float* const* snapshots) {
  if (!ws) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::wavesim_ctx(ws);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::acoustic_forward_snapshots(ws, nshots, shots, on_device != 0, snapevery, snapshots);
  });
}

int sw_elastic_forward_snapshots(sw_elastic* es, int32_t nshots, const sw_elastic_shot* shots, int32_t on_device,
                                 int32_t snapevery, float* const* snapshots) {
  if (!es) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::elastic_ctx(es);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::elastic_forward_snapshots(es, nshots, shots, on_device != 0, snapevery, snapshots);
  });
}

int sw_acoustic_vd_create(sw_ctx* ctx, const sw_acoustic_params* params, int32_t interp_rho, int32_t gradient,
                          const sw_grad_params* gparams, sw_acoustic_vd** out) {
  if (!ctx || !out) return SW_ERR_ARG;
  *out = nullptr;
  sw_acoustic_vd* vd = nullptr;
  const int rc = guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    vd = swgb::vd_new();
    swgb::vd_init(vd, ctx, params, interp_rho, gradient, gparams);
  });
  if (rc != SW_OK) {
    if (vd) swgb::vd_delete(vd);
    return rc;
  }
  *out = vd;
  return SW_OK;
}

int sw_acoustic_vd_destroy(sw_acoustic_vd* vd) {
  if (!vd) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::vd_ctx(vd);
  if (ctx) {
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
  }
  swgb::vd_delete(vd);
  return SW_OK;
}

int sw_acoustic_vd_set_material(sw_acoustic_vd* vd, const float* vp, const float* rho) {
  if (!vd) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::vd_ctx(vd);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::vd_set_material(vd, vp, rho);
  });
}

int sw_acoustic_vd_forward(sw_acoustic_vd* vd, int32_t nshots, const sw_acoustic_shot* shots, int32_t on_device) {
  if (!vd) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::vd_ctx(vd);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::vd_forward(vd, nshots, shots, on_device != 0);
  });
}

int sw_acoustic_vd_forward_snapshots(sw_acoustic_vd* vd, int32_t nshots, const sw_acoustic_shot* shots,
                                     int32_t on_device, int32_t snapevery, float* const* snapshots) {
  if (!vd) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::vd_ctx(vd);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::vd_forward_snapshots(vd, nshots, shots, on_device != 0, snapevery, snapshots);
  });
}

int sw_acoustic_vd_gradient(sw_acoustic_vd* vd, int32_t nshots, const sw_acoustic_shot* shots, int32_t on_device,
                            double* grad_vp, double* grad_rho, double* misfit) {
  if (!vd) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::vd_ctx(vd);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::vd_gradient(vd, nshots, shots, on_device != 0, grad_vp, grad_rho, misfit);
  });
}

int sw_acoustic_vd_set_precision(sw_acoustic_vd* vd, int32_t mode) {
  if (!vd || mode < 0 || mode > 1) return SW_ERR_ARG;
  return guarded(swgb::vd_ctx(vd), [&] { swgb::vd_set_precision(vd, mode); });
}

int sw_acoustic_vd_set_material64(sw_acoustic_vd* vd, const double* vp, const double* rho) {
  if (!vd) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::vd_ctx(vd);
  return guarded(ctx, [&] {
    swgb::check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    swgb::vd_set_material64(vd, vp, rho);
  });
}

int sw_acoustic_vd_set_tuning(sw_acoustic_vd* vd, int32_t tz) {
  if (!vd) return SW_ERR_ARG;
  sw_ctx* ctx = swgb::vd_ctx(vd);
  return guarded(ctx, [&] { swgb::vd_set_tuning(vd, tz); });
}

}  // extern "C"
