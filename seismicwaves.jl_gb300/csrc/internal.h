// Internal declarations of libswgb300 (not part of the public C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "swgb300.h"

namespace swgb {

// A per-shot field: element (shot, i) lives at p[shot * s + i].
struct FieldArg {
  float* p;
  long long s;
};

// Device buffer owned by the host code (freed on destruction).
struct DevMem {
  void* p = nullptr;
  size_t bytes = 0;
  DevMem() = default;
  DevMem(const DevMem&) = delete;
  DevMem& operator=(const DevMem&) = delete;
  ~DevMem() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T>
  T* as() const { return static_cast<T*>(p); }
};

// Error raised inside the library and turned into a status at the ABI edge.
struct SwError {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg);
void check_cuda(cudaError_t e, const char* what);
// Allocates and zero-fills on `st` (so later work on that stream sees the zeros).
void dev_alloc(DevMem& m, size_t bytes, const char* what, cudaStream_t st);

// Per-kernel-kind event timing (sw_profile_*).
enum KernelKind {
  KK_STENCIL = 0, KK_ADJOINT = 1, KK_SRCREC = 2, KK_OTHER = 3, KK_RECOMPUTE = 4, KK_CORR = 5, KK_COUNT = 6
};

struct Profiler {
  bool on = false;
  double total_ms[KK_COUNT] = {};
  long long launches[KK_COUNT] = {};  // timed brackets (one step of a kind, one kernel call)
  long long kernels[KK_COUNT] = {};   // kernel launches inside them
  double bytes[KK_COUNT] = {};
  struct Pending {
    cudaEvent_t a, b;
    int kind, nk;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t get();
  void begin(cudaStream_t s, int kind, double bytes_, cudaEvent_t* a_out);
  void end(cudaStream_t s, int kind, cudaEvent_t a, int nk = 1);  // nk: kernels launched since begin
  void resolve();  // synchronises on the pending events, accumulates, recycles
  ~Profiler();
};

}  // namespace swgb

struct sw_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 0;
  std::string last_error;
  swgb::Profiler prof;
  swgb::DevMem err;  // int flag raised by kernels whose bounded waits gave up
};

namespace swgb {

// CR = C * R on the context's stream (the library's own tiled FP32 GEMM,
// dense.cu): C is a dense (nt, nt) inverse covariance, R the (nt, ncols)
// residuals of one shot.
void dense_invcov(sw_ctx* ctx, int nt, int ncols, const float* C, const float* R, float* CR);

// Host-side C-PML coefficients (double precision), one axis.
void cpml_axis_coefficients(double vel_max, double dt, int halo, double rcoef, double h, double f0,
                            bool freetop_axis, double* a, double* a_h, double* b, double* b_h);

}  // namespace swgb
