// sw_acoustic2d_forward_noalloc: the 2D acoustic forward of one shot with all
// of its working memory in a fixed, statically allocated device array.
//
// Some callers cannot let a library call cudaMalloc: code that runs inside
// another runtime's device memory pool (CUDA.jl, PyTorch's caching allocator)
// that must account for every byte on the device, deployments with a fixed
// device-memory budget, and pipelines that keep other streams busy and cannot
// afford the device-wide synchronisation cudaMalloc / cudaFree may impose.
// This entry point allocates nothing: its wavefields, C-PML memory variables
// and shot tables live in g_scratch below, a file-scope __device__ array of
// kScratchBytes that every GPU which loads the library holds until the
// process exits.  The caller still owns the inputs (vp, source time
// functions) and the output (traces), all in device memory.
//
// The array is shared by every call and keeps the last call's contents, so
// each call clears what must start at zero.  Calls whose GPU work overlaps
// (for example on two streams at once) race on the array; serialise them.
// The first call on a device looks the array's device address up
// (cudaGetSymbolAddress, with that device current) and caches it; make that
// first call before any stream capture.  The cache is keyed by device ordinal
// and assumes the device's primary context for the life of the process: a
// caller that resets the device (cudaDeviceReset) or runs the call under
// another context of the same device must not use this entry point after
// that.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "acoustic_kernels.cuh"
#include "internal.h"

namespace {

constexpr size_t kScratchBytes = size_t(64) << 20;  // 64 MiB per device
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Host code may not use g_scratch directly (its host-side name is a stand-in,
// not a device address): look the device address up once per device.
int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return SW_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return SW_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return SW_OK;
}

struct NaTables {
  int nt, nrec, nsp;
  const float* tf;   // caller's (nt, nsrc) scaled source time functions
  float* tr;         // caller's (nt, nrec) traces
  long long* pts;    // unique source points (padded linear index)
  int* ptr;          // CSR into ids
  int* ids;          // source ids
  int* bslot;        // ring slot of boundary points, -1 otherwise
  long long* rec;    // receiver points
  float* ring;       // 3 floats per boundary source point
};

// One shot: inject every unique source point (boundary points through their
// 3-value ring, as in the batched path), then record every receiver.
__global__ void k_noalloc_inject_record(NaTables T, float* pnew, float* dnew, int it) {
  for (int u = threadIdx.x; u < T.nsp; u += blockDim.x) {
    const long long lin = T.pts[u];
    float add = 0.f;
    if (T.bslot[u] >= 0) {
      for (int k = T.ptr[u]; k < T.ptr[u + 1]; ++k) add += T.tf[(long long)(it - 1) + (long long)T.ids[k] * T.nt];
      float* r = T.ring + 3 * T.bslot[u];
      const float v = r[it % 3] + add;
      r[it % 3] = v;
      pnew[lin] = v;
    } else {
      float acc = pnew[lin];
      for (int k = T.ptr[u]; k < T.ptr[u + 1]; ++k) {
        const float v = T.tf[(long long)(it - 1) + (long long)T.ids[k] * T.nt];
        acc += v;
        add += v;
      }
      pnew[lin] = acc;
      dnew[lin] += add;
    }
  }
  __syncthreads();
  for (int r = threadIdx.x; r < T.nrec; r += blockDim.x)
    T.tr[(long long)(it - 1) + (long long)r * T.nt] = pnew[T.rec[r]];
}

__global__ void k_noalloc_fact(const float* __restrict__ vp, int n0, long long npts, int P, double dt2,
                               float* __restrict__ fact) {
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < npts;
       c += (long long)gridDim.x * blockDim.x) {
    const long long rowi = c / n0;
    const double v = (double)vp[c];
    fact[rowi * P + (c - rowi * n0)] = (float)(dt2 * v * v);
  }
}

// Bump allocator over the scratch array (256-byte aligned pieces).
struct Carve {
  unsigned char* base;
  size_t used = 0;
  bool over = false;
  template <typename T>
  T* take(size_t count) {
    const size_t off = (used + 255) & ~size_t(255);
    const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    if (off + bytes > kScratchBytes) {
      over = true;
      return nullptr;
    }
    used = off + bytes;
    return reinterpret_cast<T*>(base + off);
  }
};

int run(const sw_acoustic_params* p, const float* vp, const sw_acoustic_shot* s, cudaStream_t st) {
  using namespace swgb;
  if (!p || !vp || !s || p->ndim != 2) return SW_ERR_ARG;
  const int nx = p->n[0], nz = p->n[1], H = p->halo;
  if (nx < 3 || nz < 3 || H < 0 || !(p->dt > 0) || !(p->h[0] > 0) || !(p->h[1] > 0)) return SW_ERR_ARG;
  if (nx < 2 * H + 3 || nz < 2 * H + 3) return SW_ERR_ARG;
  if (s->nt < 1 || s->nsrc < 1 || s->nrec < 1 || !s->src_idx || !s->rec_idx || !s->srctf || !s->traces || !s->cpml)
    return SW_ERR_ARG;
  for (int q = 0; q < s->nsrc; ++q)
    for (int d = 0; d < 2; ++d) {
      const int v = s->src_idx[q + (long long)d * s->nsrc];
      if (v < 1 || v > p->n[d]) return SW_ERR_ARG;
    }
  for (int q = 0; q < s->nrec; ++q)
    for (int d = 0; d < 2; ++d) {
      const int v = s->rec_idx[q + (long long)d * s->nrec];
      if (v < 1 || v > p->n[d]) return SW_ERR_ARG;
    }

  // host-side shot tables (unique source points in order of appearance)
  const int P = (nx + 31) / 32 * 32;
  const long long F = (long long)P * nz;
  std::vector<long long> pts;
  std::vector<int> ptr, ids, bslot;
  std::vector<std::vector<int>> members;
  for (int q = 0; q < s->nsrc; ++q) {
    const int i = s->src_idx[q], j = s->src_idx[q + s->nsrc];
    const long long lin = (long long)(j - 1) * P + (i - 1);
    auto it = std::find(pts.begin(), pts.end(), lin);
    if (it == pts.end()) {
      pts.push_back(lin);
      members.push_back({q});
      bslot.push_back((i == 1 || i == nx || j == 1 || j == nz) ? 1 : -1);
    } else {
      members[it - pts.begin()].push_back(q);
    }
  }
  int nring = 0;
  for (auto& b : bslot)
    if (b >= 0) b = nring++;
  for (auto& m : members) {
    ptr.push_back((int)ids.size());
    ids.insert(ids.end(), m.begin(), m.end());
  }
  ptr.push_back((int)ids.size());
  std::vector<long long> rec(s->nrec);
  for (int q = 0; q < s->nrec; ++q)
    rec[q] = (long long)(s->rec_idx[q + s->nrec] - 1) * P + (s->rec_idx[q] - 1);

  // scratch layout
  void* base = nullptr;
  int rc = scratch_address(&base);
  if (rc != SW_OK) return rc;
  Carve c{static_cast<unsigned char*>(base)};
  const long long psz0 = (long long)2 * H * nz, psz1 = (long long)2 * H * P;
  const long long xsz0 = (long long)(2 * H + 2) * nz, xsz1 = (long long)(2 * H + 2) * P;
  const int L = 2 * (2 * H + 2) + 2 * (2 * H);
  float* fact = c.take<float>(F);
  float* pb[2] = {c.take<float>(F), c.take<float>(F)};
  float* db = c.take<float>(F);
  float* psi[2][2] = {{c.take<float>(psz0), c.take<float>(psz1)}, {c.take<float>(psz0), c.take<float>(psz1)}};
  float* xi[2] = {c.take<float>(xsz0), c.take<float>(xsz1)};
  float* cpml = c.take<float>(2 * L);
  NaTables T;
  T.nt = s->nt;
  T.nrec = s->nrec;
  T.nsp = (int)pts.size();
  T.tf = s->srctf;
  T.tr = s->traces;
  T.pts = c.take<long long>(pts.size());
  T.ptr = c.take<int>(ptr.size());
  T.ids = c.take<int>(ids.size());
  T.bslot = c.take<int>(bslot.size());
  T.rec = c.take<long long>(rec.size());
  T.ring = c.take<float>(3 * std::max(nring, 1));
  if (c.over) return SW_ERR_CAPACITY;

  auto ok = [](cudaError_t e) { return e == cudaSuccess; };
  bool good = true;
  // everything that must start at zero (the array keeps the previous call's contents)
  for (float* f : {pb[0], pb[1], db}) good = good && ok(cudaMemsetAsync(f, 0, F * sizeof(float), st));
  for (int k = 0; k < 2; ++k) {
    good = good && ok(cudaMemsetAsync(psi[k][0], 0, std::max<long long>(psz0, 1) * sizeof(float), st));
    good = good && ok(cudaMemsetAsync(psi[k][1], 0, std::max<long long>(psz1, 1) * sizeof(float), st));
  }
  good = good && ok(cudaMemsetAsync(xi[0], 0, xsz0 * sizeof(float), st));
  good = good && ok(cudaMemsetAsync(xi[1], 0, xsz1 * sizeof(float), st));
  good = good && ok(cudaMemsetAsync(T.ring, 0, 3 * std::max(nring, 1) * sizeof(float), st));
  good = good && ok(cudaMemcpyAsync(cpml, s->cpml, 2 * L * sizeof(float), cudaMemcpyHostToDevice, st));
  good = good && ok(cudaMemcpyAsync(T.pts, pts.data(), pts.size() * sizeof(long long), cudaMemcpyHostToDevice, st));
  good = good && ok(cudaMemcpyAsync(T.ptr, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  good = good && ok(cudaMemcpyAsync(T.ids, ids.data(), ids.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  good = good && ok(cudaMemcpyAsync(T.bslot, bslot.data(), bslot.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  good = good && ok(cudaMemcpyAsync(T.rec, rec.data(), rec.size() * sizeof(long long), cudaMemcpyHostToDevice, st));
  if (!good) {
    cudaGetLastError();
    return SW_ERR_CUDA;
  }
  const long long npts = (long long)nx * nz;
  k_noalloc_fact<<<(unsigned)std::min<long long>((npts + 255) / 256, 4096), 256, 0, st>>>(vp, nx, npts, P,
                                                                                       p->dt * p->dt, fact);

  int sms = 148;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tiles_x = (P + 511) / 512;
  // the batched path's rule for the register-pipelined stencil: 8-row bands,
  // 4-row bands when 8-row ones would leave the GPU under-filled
  const int TZ = (long long)tiles_x * ((nz - 2 + 7) / 8) < 4LL * sms ? 4 : 8;
  const int tiles_z = (nz - 2 + TZ - 1) / TZ;

  StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n0 = nx;
  a.n1 = nz;
  a.n2 = 1;
  a.P = P;
  a.halo = H;
  for (int d = 0; d < 2; ++d) {
    const double ih = 1.0 / p->h[d];
    a.ih[d] = (float)ih;
    a.ih2[d] = (float)(ih * ih);
  }
  a.fact = fact;
  a.cpml = cpml;
  a.cpml_stride = 2 * L;
  a.nshots = 1;
  a.tiles_x = tiles_x;
  a.tiles_y = 1;
  a.tiles_z = tiles_z;
  a.TZ = TZ;
  a.withhold = -1;
  int pc = 0, pk = 0;
  for (int it = 1; it <= s->nt; ++it) {
    a.pcur = FieldArg{pb[pc], F};
    a.pnew = FieldArg{pb[1 - pc], F};
    a.din = FieldArg{db, F};
    a.dout = a.din;
    for (int d = 0; d < 2; ++d) {
      a.psi_in[d] = FieldArg{psi[pk][d], 0};
      a.psi_out[d] = FieldArg{psi[1 - pk][d], 0};
      a.xi_in[d] = FieldArg{xi[d], 0};
      a.xi_out[d] = a.xi_in[d];
    }
    k_ac2d_step<MODE_FWD, 4><<<(unsigned)(tiles_x * tiles_z), 128, 0, st>>>(a);
    k_noalloc_inject_record<<<1, 128, 0, st>>>(T, pb[1 - pc], db, it);
    pc = 1 - pc;
    pk = 1 - pk;
  }
  if (cudaGetLastError() != cudaSuccess) return SW_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return SW_ERR_CUDA;
  }
  return SW_OK;
}

}  // namespace

extern "C" int sw_acoustic2d_forward_noalloc(const sw_acoustic_params* params, const float* vp,
                                             const sw_acoustic_shot* shot, void* stream) {
  return run(params, vp, shot, static_cast<cudaStream_t>(stream));
}
