// Cross-correlation time-shift misfit (CCTSMisfit, src/inversion/misfits/CCTSMisfit.jl:17-80)
// on the device, shared by the acoustic paths (constant and variable density,
// one trace per receiver) and the elastic one (one trace per receiver and
// component: the (nt, 2, nrec) records are 2 nrec traces of nt samples).
//
// Per trace (observed u, synthetic v, nt samples):
//   xcorr(u, v) = conv(u, reverse(v)) (DSP.jl), 2 nt - 1 values; at 1-based
//   index k it is sum_i u[i] v[i - (k - nt)];
//   dtau = (first k of max |xcorr| - (nt - 1)) * dt, misfit += dtau^2 / 2;
//   dchi/du = dtau / N * ds/dt, ds/dt central differences (first sample
//   (v[2] - 0) / 2dt, last sample 0), N = trapezoidal integral of (ds/dt)^2
//   over the times dt .. nt dt.
// The adjoint source is -dchi/du times the receiver's prescale factor (1
// without a prescale field); amax (if given) takes the running maximum of
// its magnitude as float bits (the elastic path scales its adjoint sources by
// a power of two chosen from it).
//
// One block per trace.  u and a zero-padded copy of v (3 nt - 2 values) sit
// in shared memory; lane l of warp w evaluates the 8 lags
// L0 + 256 w' + l + 32 q (q = 0..7) of its pass, so the 32 lanes of a warp
// read 32 consecutive words of v for every u[i] they share (no bank
// conflicts).  The lag sums are FP32 (their argmax is what matters), N and the
// misfit FP64.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <sstream>
#include <vector>

#include "internal.h"

namespace swgb {
namespace {

struct CctsShot {
  int nt, nrec, kind;      // kind 1: CCTS (other shots are skipped)
  double dt;               // CCTSMisfit.dt
  const float* tr;         // synthetic (nt, nrec)
  const float* obs;        // observed (nt, nrec)
  float* adj;              // adjoint source (nt, nrec)
  const long long* rec_lin;  // receiver -> index into the prescale field
};

constexpr int CCTS_THREADS = 256;

inline size_t ccts_smem_bytes(int nt) { return (size_t)(4 * nt) * sizeof(float); }

// gridDim = (max receivers, shots); partial[shot * gridDim.x + r] = dtau^2 (0 when unused)
__global__ void __launch_bounds__(CCTS_THREADS) k_ccts(const CctsShot* __restrict__ shots,
                                                       const float* __restrict__ prescale,
                                                       double* __restrict__ partial,
                                                       unsigned int* __restrict__ amax = nullptr) {
  extern __shared__ float sm[];
  const int r = blockIdx.x, s = blockIdx.y;
  const CctsShot S = shots[s];
  double* part = partial + (long long)s * gridDim.x + r;
  if (S.kind != 1 || r >= S.nrec) {  // block uniform
    if (threadIdx.x == 0) *part = 0.0;
    return;
  }
  const int nt = S.nt;
  const float* u = S.obs + (long long)r * nt;
  const float* v = S.tr + (long long)r * nt;
  float* su = sm;           // nt
  float* sv = sm + nt;      // 3 nt - 2: sv[nt - 1 + j] = v[j]
  for (int j = threadIdx.x; j < 3 * nt - 2; j += blockDim.x) {
    const int q = j - (nt - 1);
    sv[j] = (q >= 0 && q < nt) ? v[q] : 0.0f;
  }
  for (int j = threadIdx.x; j < nt; j += blockDim.x) su[j] = u[j];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int nlag = 2 * nt - 1;
  float best = -1.0f;
  int kbest = 0x7fffffff;
  // lags L = -(nt - 1) + g, g = 0 .. nlag - 1; a warp covers 256 consecutive g per pass
  for (int g0 = warp * 256; g0 < nlag; g0 += nwarp * 256) {
    float acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0f;
    // sv index for lag L at sample i: nt - 1 + i - L = 2 (nt - 1) + i - g
    const int base = 2 * (nt - 1) - (g0 + lane);
    for (int i = 0; i < nt; ++i) {
      const float x = su[i];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int idx = base + i - 32 * q;
        acc[q] = fmaf(x, (idx >= 0 && idx < 3 * nt - 2) ? sv[idx] : 0.0f, acc[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int g = g0 + lane + 32 * q;
      if (g < nlag) {
        const float a = fabsf(acc[q]);
        const int k = g + 1;  // 1-based index into xcorr
        if (a > best || (a == best && k < kbest)) { best = a; kbest = k; }
      }
    }
  }
  // block argmax: largest |xcorr|, first index among equals
  __shared__ float rb[CCTS_THREADS];
  __shared__ int rk[CCTS_THREADS];
  __shared__ double rn[CCTS_THREADS];
  rb[threadIdx.x] = best;
  rk[threadIdx.x] = kbest;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const float b2 = rb[threadIdx.x + o];
      const int k2 = rk[threadIdx.x + o];
      if (b2 > rb[threadIdx.x] || (b2 == rb[threadIdx.x] && k2 < rk[threadIdx.x])) {
        rb[threadIdx.x] = b2;
        rk[threadIdx.x] = k2;
      }
    }
    __syncthreads();
  }
  const double dtau = (double)(rk[0] - (nt - 1)) * S.dt;
  // ds/dt and the trapezoidal norm
  const double i2dt = 1.0 / (2.0 * S.dt);
  auto dsdt = [&](int t) -> double {  // 0-based sample t
    if (t == 0) return nt >= 2 ? ((double)sv[nt] - 0.0) * i2dt : 0.0;
    if (t >= nt - 1) return 0.0;
    return ((double)sv[nt - 1 + t + 1] - (double)sv[nt - 1 + t - 1]) * i2dt;
  };
  double nacc = 0.0;
  for (int t = threadIdx.x; t < nt - 1; t += blockDim.x) {
    const double a = dsdt(t), b = dsdt(t + 1);
    nacc += S.dt * (a * a + b * b) * 0.5;
  }
  rn[threadIdx.x] = nacc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) rn[threadIdx.x] += rn[threadIdx.x + o];
    __syncthreads();
  }
  const double f = dtau / rn[0];
  const float pre = prescale ? prescale[S.rec_lin[r]] : 1.0f;
  float* adj = S.adj + (long long)r * nt;
  float mx = 0.0f;
  for (int t = threadIdx.x; t < nt; t += blockDim.x) {
    adj[t] = (-(float)(f * dsdt(t))) * pre;
    mx = fmaxf(mx, fabsf(adj[t]));
  }
  if (amax) {
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(amax, __float_as_uint(mx));  // non-negative floats order like their bits
  }
  if (threadIdx.x == 0) *part = dtau * dtau;  // the sum kernels apply the 1/2
}

// misfit_kind 0 (L2Misfit) or 1 (CCTSMisfit, whose device kernel keeps a trace
// and a padded copy of it in shared memory: 16 nt bytes)
inline void validate_misfit_kind(const sw_acoustic_shot& s, int k) {
  std::ostringstream os;
  if (s.misfit_kind != 0 && s.misfit_kind != 1) {
    os << "shot " << k << ": misfit_kind must be 0 (L2) or 1 (CCTS)";
    fail(SW_ERR_ARG, os.str());
  }
  if (s.misfit_kind == 1) {
    if (!(s.misfit_dt > 0)) fail(SW_ERR_ARG, "Timestep size must be positive!");
    if (s.nt > 13000) {
      os << "shot " << k << ": the device CCTS misfit takes records of at most 13000 samples";
      fail(SW_ERR_UNSUPPORTED, os.str());
    }
  }
}

// CCTS descriptors of a batch into dst (room for kind.size() entries), uploaded
// before any graph capture; returns the largest receiver count of the CCTS
// shots (0: none, nothing uploaded)
inline int upload_ccts(sw_ctx* ctx, CctsShot* dst, const std::vector<int>& kind, const std::vector<double>& mdt,
                const std::vector<int>& nt, const std::vector<int>& nrec, const std::vector<const float*>& tr,
                const std::vector<const float*>& obs, const std::vector<float*>& adj,
                const std::vector<const long long*>& rec_lin, size_t* smem) {
  bool any = false;
  int maxrec = 0, maxnt = 0;
  std::vector<CctsShot> v(kind.size());
  for (size_t k = 0; k < kind.size(); ++k) {
    v[k] = CctsShot{nt[k], nrec[k], kind[k], mdt[k], tr[k], obs[k], adj[k], rec_lin[k]};
    if (kind[k] == 1) {
      any = true;
      maxrec = std::max(maxrec, nrec[k]);
      maxnt = std::max(maxnt, nt[k]);
    }
  }
  if (!any) return 0;
  check_cuda(cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(CctsShot), cudaMemcpyHostToDevice, ctx->stream),
             "CCTS table upload");
  check_cuda(cudaStreamSynchronize(ctx->stream), "CCTS table upload");
  *smem = ccts_smem_bytes(maxnt);
  check_cuda(cudaFuncSetAttribute(k_ccts, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem), "CCTS smem");
  return maxrec;
}

}  // namespace
}  // namespace swgb
