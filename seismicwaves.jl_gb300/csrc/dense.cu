// Dense inverse-covariance products on the device: the L2 misfit with a full
// invcov (src/inversion/misfits/L2Misfit.jl:24-95) needs, per shot,
// CR = C R with C the (nt, nt) inverse covariance and R the (nt, ncols)
// masked residuals, both column-major (ncols = receivers, or receivers x 2
// components on the elastic path).  FP32 arithmetic with FMA accumulation in
// k order (no TF32: the misfit is held to 1e-6 against FP64).
//
// Shared-memory tiled GEMM: a block of 256 threads computes a 64 x 64 tile
// of CR, 4 x 4 outputs per thread, staging 64 x 16 panels of C and 16 x 64
// panels of R per step of k (each thread loads 4 values of each panel, the
// loads of C coalesced along its columns, those of R along k).  The product
// runs once per gradient call, between the forward and the adjoint; it is
// not on the time-stepping path.
#include "internal.h"

namespace swgb {
namespace {

constexpr int GT = 64;  // output tile edge
constexpr int GK = 16;  // k panel depth

__global__ void __launch_bounds__(256) k_gemm_nn(int m, int n, const float* __restrict__ A,
                                                 const float* __restrict__ B, float* __restrict__ C) {
  __shared__ float As[GK][GT + 4];  // As[k][i] = A(m0 + i, k0 + k)
  __shared__ float Bs[GK][GT + 4];  // Bs[k][j] = B(k0 + k, n0 + j)
  const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;  // outputs: rows m0 + 4 ty + r, columns n0 + 4 tx + c
  float acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = 0.f;
  const int ai = tid % GT, ak = (tid / GT) * 4;  // A panel: row ai, k ak .. ak+3
  const int bk = tid % GK, bj = (tid / GK) * 4;  // B panel: k bk, columns bj .. bj+3
  for (int k0 = 0; k0 < m; k0 += GK) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = m0 + ai, k = k0 + ak + q;
      As[ak + q][ai] = (i < m && k < m) ? A[(long long)i + (long long)k * m] : 0.f;
      const int kb = k0 + bk, j = n0 + bj + q;
      Bs[bk][bj + q] = (kb < m && j < n) ? B[(long long)kb + (long long)j * m] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][4 * ty + r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[kk][4 * tx + c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = __fmaf_rn(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int j = n0 + 4 * tx + c;
    if (j >= n) continue;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int i = m0 + 4 * ty + r;
      if (i < m) C[(long long)i + (long long)j * m] = acc[r][c];
    }
  }
}

}  // namespace

void dense_invcov(sw_ctx* ctx, int nt, int ncols, const float* C, const float* R, float* CR) {
  if (nt <= 0 || ncols <= 0) return;
  const dim3 grid((unsigned)((ncols + GT - 1) / GT), (unsigned)((nt + GT - 1) / GT));
  k_gemm_nn<<<grid, 256, 0, ctx->stream>>>(nt, ncols, C, R, CR);
  check_cuda(cudaGetLastError(), "dense inverse covariance launch");
}

}  // namespace swgb
