// Isotropic elastic 2D (P-SV) C-PML path: the batched forward and the batched
// gradient with respect to rho, lambda and mu.
//
// Reference behaviour restated here (SeismicWaves.jl v0.9.0, paths relative to
// its source tree):
//   update_sigma_xx_sigma_zz!, update_sigma_xz!, update_ux!, update_uz!
//       src/models/elastic/backends/shared/elastic2D_iso_xPU.jl:1-79
//   4th-order staggered derivatives and the free-surface mirror rules
//       src/models/elastic/backends/shared/freesurface_derivatives_4th_mirror.jl:72-234
//   C-PML memory variables (the dtilde-4th operator)  src/utils/fdgenerated.jl:177-199
//   moment-tensor / external-force injection, recording  elastic2D_iso_xPU.jl:81-118
//   forward / adjoint step orchestration  elastic2D_iso_xPU.jl:120-448
//   swforward_1shot! / swgradient_1shot!  src/models/elastic/ela_forward.jl:4-159,
//                                         src/models/elastic/ela_gradient.jl:4-362
//   correlate_gradients!  src/models/elastic/backends/shared/correlate_gradient_xPU.jl:1-83
//   precomp_elaprop! + back_interp  src/models/elastic/ela_models.jl:156-173, src/utils/interpolations.jl:1-47
//   L2 misfit on (nt, 2, nrec) traces  src/inversion/misfits/L2Misfit.jl:44-95
//
// Layout.  Every field of a shot is a zero-padded (nz + 4) x P array (x
// fastest, P a multiple of 32): node (i, j) (1-based) sits at row j + 1 and
// column i + 31.  The reference's "missing point = 0" boundary rules of the
// 4th-order derivatives all read points outside their array, so the padding
// (which no kernel writes) supplies them; only the free-surface mirror rules
// are coded.  The C-PML memory variables live in compact strips: x strips
// (nz rows x W columns) and z strips ((2 halo + 3) rows x P).  The reference's
// "full" index maps send the last left cell and the first right cell to one
// array element whose coefficient a is 0 (so it stays 0); here the right strip
// is stored one cell further, which gives every point its own cell.
//
// Time stepping.  The displacement is advanced in increment form (state u and
// du = u[n] - u[n-1]; du += D; u += du with D = dt^2/rho * div sigma), which
// is the reference's 2 u - u_old + D in exact arithmetic and keeps the FP32
// rounding error of the second time difference out of the fields.  The
// gradient's rho term correlates the adjoint displacement with
// u[it] - 2 u[it-1] + u[it-2] = D(it), which the forward and recompute steps
// write directly; the lambda / mu terms need the strains of u[it-1], which the
// same steps store in a slot.  Checkpoints (u, du and the eight memory
// variables) are taken after every K-th step; the adjoint recomputes each
// window of K steps from its checkpoint, on one schedule for all shots of the
// batch (a shot takes part in step it while it <= its nt).
//
// Scaling.  Each shot's forward sources and the adjoint sources are multiplied
// by powers of two (chosen from their maxima) so that the FP32 fields and the
// products of forward and adjoint strains stay far from the FP32 underflow
// range; traces and gradients are scaled back exactly, and a shot's traces do
// not depend on the other shots of its batch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <sstream>
#include <vector>

#include "internal.h"
#include "ccts.cuh"

namespace swgb {
namespace el {

constexpr int XPAD = 32; // columns left of i = 1 (keeps each warp's 32 points on one 128-byte line)
constexpr int ZPAD = 2;  // rows above j = 1
constexpr int BX = 128;  // threads per block (x)
constexpr int CTZ = 2;   // rows per block (correlation); the stencil kernels take theirs as a template parameter

struct Geo {
  int nx, nz, P, halo, ft, W;
  long long F;  // floats per padded field
  float idx, idz;
  __host__ __device__ __forceinline__ long long lin(int i, int j) const {
    return (long long)(j + ZPAD - 1) * P + (i + XPAD - 1);
  }
};

struct Args {
  Geo g;
  // state, [shot][F]
  float* ux; float* uz; float* dux; float* duz;
  float* sxx; float* szz; float* sxz;
  // C-PML memory variables, [shot][xs] / [shot][zs]
  // x strips: 0 = dsxx/dx (half map), 1 = dsxz/dx (full), 2 = dux/dx (full), 3 = duz/dx (half)
  // z strips: 0 = dszz/dz (half), 1 = dsxz/dz (full), 2 = dux/dz (half), 3 = duz/dz (full)
  float* px[4]; float* pz[4];
  long long xs, zs;
  // material (padded, shared by the shots)
  const float* lam; const float* mu; const float* dtr_i; const float* dtr_j; const float* mu_ij;
  // C-PML coefficients of each shot: axis x then z, each [a(na), a_h(nh), b(na), b_h(nh)]
  const float* cp; int cps;
  // gradient slots (u[it-1] and D(it) of this step), [shot][F]; null when not written
  float* sUx; float* sUz; float* sDx; float* sDz;
};

__device__ __forceinline__ float d4(float f1, float f2, float f3, float f4, float inv) {
  const float c1 = 1.0f / 24.0f, c2 = 27.0f / 24.0f;
  return (c1 * f1 - c2 * f2 + c2 * f3 - c1 * f4) * inv;
}

// C-PML cell selection.  "half": the maps of fdgenerated.jl:178-195 with
// half = false on an array of n points (left pos <= halo, right pos >= n-halo,
// coefficient index k = pos - n + 2 halo + 1); "full": half = true on an array
// of n-1 points (left pos <= halo+1, right pos >= n-1-halo, k = pos - n + 2 halo + 2).
// Returns k (1-based, 0 = outside the strips) and the storage column.
__device__ __forceinline__ int cpml_half(int pos, int n, int halo, int& col) {
  if (pos <= halo) { col = pos - 1; return pos; }
  if (pos >= n - halo) { const int k = pos - n + 2 * halo + 1; col = k - 1; return k; }
  return 0;
}
__device__ __forceinline__ int cpml_full(int pos, int n, int halo, int& col) {
  if (pos <= halo + 1) { col = pos - 1; return pos; }
  if (pos >= n - 1 - halo) { const int k = pos - n + 2 * halo + 2; col = k; return k; }
  return 0;
}
// psi = b psi + a dv; returns dv + psi
__device__ __forceinline__ float cpml_upd(float* psi, float a, float b, float dv) {
  const float nv = b * (*psi) + a * dv;
  *psi = nv;
  return dv + nv;
}

// Raw 4th-order derivatives at the stress nodes (shared by the stress update
// and the gradient correlation); c = lin(i, j), P = pitch.
__device__ __forceinline__ float dux_dx(const float* __restrict__ u, long long c, float inv) {
  return d4(__ldg(u + c - 2), __ldg(u + c - 1), __ldg(u + c), __ldg(u + c + 1), inv);
}
__device__ __forceinline__ float duz_dz_raw(const float* __restrict__ u, long long c, int P, int j, int ft, float inv) {
  if (ft && j == 2) {
    const float u1 = __ldg(u + c - P);
    return d4(u1, u1, __ldg(u + c), __ldg(u + c + P), inv);
  }
  return d4(__ldg(u + c - 2 * P), __ldg(u + c - P), __ldg(u + c), __ldg(u + c + P), inv);
}
__device__ __forceinline__ float duz_dx(const float* __restrict__ u, long long c, float inv) {
  return d4(__ldg(u + c - 1), __ldg(u + c), __ldg(u + c + 1), __ldg(u + c + 2), inv);
}
__device__ __forceinline__ float dux_dz(const float* __restrict__ u, long long c, int P, int j, int ft, float inv) {
  if (ft && j == 1) {
    const float u2 = __ldg(u + c + P);
    return d4(u2, __ldg(u + c), u2, __ldg(u + c + 2 * P), inv);
  }
  return d4(__ldg(u + c - P), __ldg(u + c), __ldg(u + c + P), __ldg(u + c + 2 * P), inv);
}

__device__ __forceinline__ float ldz(const float* __restrict__ p, long long c, bool ok) {
  return ok ? __ldg(p + c) : 0.0f;
}

constexpr unsigned FULL = 0xffffffffu;

// Stress update (update_sigma_xx_sigma_zz! + update_sigma_xz!) for the shot
// blockIdx.z; nodes i <= nx-1, j <= nz-1 of the band blockIdx.y.  Each thread
// walks its column down the band with the column's z neighbours in registers;
// x neighbours come from the adjacent lanes (loaded at the warp edges).
template <int TZ>
__global__ void __launch_bounds__(BX) k_el_stress(const Args A) {
  const Geo g = A.g;
  const int s = blockIdx.z;
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j0 = blockIdx.y * TZ + 1;
  const int j1 = min(j0 + TZ - 1, g.nz - 1);
  if (j0 > j1) return;
  const bool act = i <= g.nx - 1;
  const bool ldok = i <= g.nx + 2;  // columns inside the padded row
  const long long so = (long long)s * g.F;
  const float* __restrict__ ux = A.ux + so;
  const float* __restrict__ uz = A.uz + so;
  float* __restrict__ sxx = A.sxx + so;
  float* __restrict__ szz = A.szz + so;
  float* __restrict__ sxz = A.sxz + so;
  const int na = 2 * g.halo + 2, nh = 2 * g.halo;
  const float* cx = A.cp + (long long)s * A.cps;
  const float* cz = cx + 2 * na + 2 * nh;
  float* pxE = A.px[2] + (long long)s * A.xs;
  float* pxG = A.px[3] + (long long)s * A.xs;
  float* pzH = A.pz[2] + (long long)s * A.zs;
  float* pzF = A.pz[3] + (long long)s * A.zs;
  int colE = 0, colG = 0;
  const int kE = cpml_full(i, g.nx, g.halo, colE);  // dux/dx at sigma_xx nodes (ux has nx-1 points)
  const int kG = cpml_half(i, g.nx, g.halo, colG);  // duz/dx at sigma_xz nodes (uz has nx points)
  const int jlo = g.ft ? 1 : 2;
  const int P = g.P;
  long long c = g.lin(i, j0);
  // column windows: ux rows j-1 .. j+2, uz rows j-2 .. j+1
  float xu0 = ldz(ux, c - P, ldok), xu1 = ldz(ux, c, ldok), xu2 = ldz(ux, c + P, ldok), xu3 = ldz(ux, c + 2 * P, ldok);
  float zu0 = ldz(uz, c - 2 * P, ldok), zu1 = ldz(uz, c - P, ldok), zu2 = ldz(uz, c, ldok), zu3 = ldz(uz, c + P, ldok);
  for (int j = j0; j <= j1; ++j, c += P) {
    float uxm1 = __shfl_up_sync(FULL, xu1, 1), uxm2 = __shfl_up_sync(FULL, xu1, 2);
    float uxp1 = __shfl_down_sync(FULL, xu1, 1);
    float uzm1 = __shfl_up_sync(FULL, zu2, 1), uzp1 = __shfl_down_sync(FULL, zu2, 1);
    float uzp2 = __shfl_down_sync(FULL, zu2, 2);
    if (lane < 2) uxm2 = ldz(ux, c - 2, ldok);
    if (lane == 0) {
      uxm1 = ldz(ux, c - 1, ldok);
      uzm1 = ldz(uz, c - 1, ldok);
    }
    if (lane == 31) {
      uxp1 = ldz(ux, c + 1, ldok);
      uzp1 = ldz(uz, c + 1, ldok);
    }
    if (lane >= 30) uzp2 = ldz(uz, c + 2, ldok);
    if (act) {
      if (i >= 2 && j >= jlo) {
        const float l = __ldg(A.lam + c), m = __ldg(A.mu + c);
        const float l2m = l + 2.0f * m;
        const float dux = d4(uxm2, uxm1, xu1, uxp1, g.idx);
        float duz;
        if (g.ft && j == 1) duz = (-l / l2m) * dux;
        else if (g.ft && j == 2) duz = d4(zu1, zu1, zu2, zu3, g.idz);
        else duz = d4(zu0, zu1, zu2, zu3, g.idz);
        float duxc = dux, duzc = duz;
        if (kE) duxc = cpml_upd(pxE + (long long)(j - 1) * g.W + colE, cx[kE - 1], cx[na + nh + kE - 1], dux);
        int colF = 0;
        const int kF = cpml_full(j, g.nz, g.halo, colF);  // duz/dz (uz has nz-1 points)
        if (kF) duzc = cpml_upd(pzF + (long long)colF * P + (i - 1), cz[kF - 1], cz[na + nh + kF - 1], duz);
        sxx[c] = l2m * duxc + l * duzc;
        szz[c] = (j == 1) ? 0.0f : l * duxc + l2m * duzc;
      }
      const float dzx = d4(uzm1, zu2, uzp1, uzp2, g.idx);
      const float dxz = (g.ft && j == 1) ? d4(xu2, xu1, xu2, xu3, g.idz) : d4(xu0, xu1, xu2, xu3, g.idz);
      float dzxc = dzx, dxzc = dxz;
      if (kG) dzxc = cpml_upd(pxG + (long long)(j - 1) * g.W + colG, cx[na + kG - 1], cx[2 * na + nh + kG - 1], dzx);
      int colH = 0;
      const int kH = cpml_half(j, g.nz, g.halo, colH);  // dux/dz (ux has nz points)
      if (kH) dxzc = cpml_upd(pzH + (long long)colH * P + (i - 1), cz[na + kH - 1], cz[2 * na + nh + kH - 1], dxz);
      sxz[c] = __ldg(A.mu_ij + c) * (dzxc + dxzc);
    }
    const bool more = j + 1 <= j1;
    xu0 = xu1; xu1 = xu2; xu2 = xu3; xu3 = ldz(ux, c + 3 * P, ldok && more);
    zu0 = zu1; zu1 = zu2; zu2 = zu3; zu3 = ldz(uz, c + 2 * P, ldok && more);
  }
}

// Displacement update (update_ux! + update_uz!) in increment form; nodes
// i <= nx, j <= nz of the band blockIdx.y.  With slots, also stores u[it-1]
// and D(it) for the gradient.  Same register walk as the stress update.
template <int TZ>
__global__ void __launch_bounds__(BX) k_el_disp(const Args A) {
  const Geo g = A.g;
  const int s = blockIdx.z;
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j0 = blockIdx.y * TZ + 1;
  const int j1 = min(j0 + TZ - 1, g.nz);
  if (j0 > j1) return;
  const bool ldok = i <= g.nx + 2;
  const long long so = (long long)s * g.F;
  float* __restrict__ ux = A.ux + so;
  float* __restrict__ uz = A.uz + so;
  float* __restrict__ dux = A.dux + so;
  float* __restrict__ duz = A.duz + so;
  const float* __restrict__ sxx = A.sxx + so;
  const float* __restrict__ szz = A.szz + so;
  const float* __restrict__ sxz = A.sxz + so;
  const int na = 2 * g.halo + 2, nh = 2 * g.halo;
  const float* cx = A.cp + (long long)s * A.cps;
  const float* cz = cx + 2 * na + 2 * nh;
  float* pxA = A.px[0] + (long long)s * A.xs;
  float* pxC = A.px[1] + (long long)s * A.xs;
  float* pzD = A.pz[0] + (long long)s * A.zs;
  float* pzB = A.pz[1] + (long long)s * A.zs;
  int colA = 0, colC = 0;
  const int kA = cpml_half(i, g.nx, g.halo, colA);  // dsxx/dx at ux nodes (sigma_xx has nx points)
  const int kC = cpml_full(i, g.nx, g.halo, colC);  // dsxz/dx at uz nodes (sigma_xz has nx-1 points)
  const bool slots = A.sUx != nullptr;
  const int P = g.P;
  long long c = g.lin(i, j0);
  // column windows: sigma_xz rows j-2 .. j+1, sigma_zz rows j-1 .. j+2
  float q0 = ldz(sxz, c - 2 * P, ldok), q1 = ldz(sxz, c - P, ldok), q2 = ldz(sxz, c, ldok), q3 = ldz(sxz, c + P, ldok);
  float w0 = ldz(szz, c - P, ldok), w1 = ldz(szz, c, ldok), w2 = ldz(szz, c + P, ldok), w3 = ldz(szz, c + 2 * P, ldok);
  for (int j = j0; j <= j1; ++j, c += P) {
    const float xc = ldz(sxx, c, ldok);
    float xm1 = __shfl_up_sync(FULL, xc, 1), xp1 = __shfl_down_sync(FULL, xc, 1), xp2 = __shfl_down_sync(FULL, xc, 2);
    float qm1 = __shfl_up_sync(FULL, q2, 1), qm2 = __shfl_up_sync(FULL, q2, 2), qp1 = __shfl_down_sync(FULL, q2, 1);
    if (lane == 0) {
      xm1 = ldz(sxx, c - 1, ldok);
      qm1 = ldz(sxz, c - 1, ldok);
    }
    if (lane < 2) qm2 = ldz(sxz, c - 2, ldok);
    if (lane == 31) {
      xp1 = ldz(sxx, c + 1, ldok);
      qp1 = ldz(sxz, c + 1, ldok);
    }
    if (lane >= 30) xp2 = ldz(sxx, c + 2, ldok);
    if (i <= g.nx - 1) {
      const float d1 = d4(xm1, xc, xp1, xp2, g.idx);
      float d2;
      if (g.ft && j == 1) d2 = d4(-q3, -q2, q2, q3, g.idz);
      else if (g.ft && j == 2) d2 = d4(-q1, q1, q2, q3, g.idz);
      else d2 = d4(q0, q1, q2, q3, g.idz);
      float d1c = d1, d2c = d2;
      if (kA) d1c = cpml_upd(pxA + (long long)(j - 1) * g.W + colA, cx[na + kA - 1], cx[2 * na + nh + kA - 1], d1);
      int colB = 0;
      const int kB = cpml_full(j, g.nz, g.halo, colB);  // dsxz/dz (sigma_xz has nz-1 points)
      if (kB) d2c = cpml_upd(pzB + (long long)colB * P + (i - 1), cz[kB - 1], cz[na + nh + kB - 1], d2);
      const float D = __ldg(A.dtr_i + c) * (d1c + d2c);
      const float u = ux[c];
      const float du = dux[c] + D;
      if (slots) {
        A.sUx[so + c] = u;
        A.sDx[so + c] = D;
      }
      ux[c] = u + du;
      dux[c] = du;
    }
    if (i <= g.nx && j <= g.nz - 1) {
      const float d1 = d4(qm2, qm1, q2, qp1, g.idx);
      const float d2 = (g.ft && j == 1) ? d4(-w2, w1, w2, w3, g.idz) : d4(w0, w1, w2, w3, g.idz);
      float d1c = d1, d2c = d2;
      if (kC) d1c = cpml_upd(pxC + (long long)(j - 1) * g.W + colC, cx[kC - 1], cx[na + nh + kC - 1], d1);
      int colD = 0;
      const int kD = cpml_half(j, g.nz, g.halo, colD);  // dszz/dz (sigma_zz has nz points)
      if (kD) d2c = cpml_upd(pzD + (long long)colD * P + (i - 1), cz[na + kD - 1], cz[2 * na + nh + kD - 1], d2);
      const float D = __ldg(A.dtr_j + c) * (d1c + d2c);
      const float u = uz[c];
      const float du = duz[c] + D;
      if (slots) {
        A.sUz[so + c] = u;
        A.sDz[so + c] = D;
      }
      uz[c] = u + du;
      duz[c] = du;
    }
    const bool more = j + 1 <= j1;
    q0 = q1; q1 = q2; q2 = q3; q3 = ldz(sxz, c + 2 * P, ldok && more);
    w0 = w1; w1 = w2; w2 = w3; w3 = ldz(szz, c + 3 * P, ldok && more);
  }
}

// ---------------------------------------------------------------------------
// Vector forms of the two update kernels: four consecutive x points per thread
// (one float4 per row and field), a warp covers 128 points and a block of four
// warps 512.  Same arithmetic per point as k_el_stress / k_el_disp; the z
// neighbours are float4 windows in registers, the x neighbours the adjacent
// lanes' elements (loaded at the warp edges).  Points outside a node range
// are computed but not stored.
// ---------------------------------------------------------------------------
struct F4 {
  float v[4];
};
__device__ __forceinline__ F4 ld4z(const float* __restrict__ p, long long c, bool ok) {
  F4 r;
  if (ok) {
    const float4 t = __ldg(reinterpret_cast<const float4*>(p + c));
    r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
  } else {
    r.v[0] = r.v[1] = r.v[2] = r.v[3] = 0.0f;
  }
  return r;
}
__device__ __forceinline__ F4 ld4rwz(const float* p, long long c) {
  const float4 t = *reinterpret_cast<const float4*>(p + c);
  F4 r;
  r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
  return r;
}
__device__ __forceinline__ void st4v(float* p, long long c, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p + c) = make_float4(v[0], v[1], v[2], v[3]);
}

template <int TZ>
__global__ void __launch_bounds__(BX, 6) k_el_stress4(const Args A) {
  const Geo g = A.g;
  const int s = blockIdx.z;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wx0 = (blockIdx.x * 4 + warp) * 128;
  const int j0 = blockIdx.y * TZ + 1;
  const int j1 = min(j0 + TZ - 1, g.nz - 1);
  if (j0 > j1 || wx0 >= g.nx) return;  // block / warp uniform
  const int i0 = wx0 + lane * 4 + 1;
  const bool ldok = i0 <= g.nx + 2;
  const long long so = (long long)s * g.F;
  const float* __restrict__ ux = A.ux + so;
  const float* __restrict__ uz = A.uz + so;
  float* __restrict__ sxx = A.sxx + so;
  float* __restrict__ szz = A.szz + so;
  float* __restrict__ sxz = A.sxz + so;
  const int na = 2 * g.halo + 2, nh = 2 * g.halo;
  const float* cx = A.cp + (long long)s * A.cps;
  const float* cz = cx + 2 * na + 2 * nh;
  const int jlo = g.ft ? 1 : 2;
  const int P = g.P;
  // x strips touch this thread's points only near the left and right edges
  const bool xstrip = i0 <= g.halo + 1 || i0 + 3 >= g.nx - 1 - g.halo;
  const bool xx_all = i0 >= 2 && i0 + 3 <= g.nx - 1;  // all four points are sigma_xx nodes
  const bool xz_all = i0 + 3 <= g.nx - 1;             // all four points are sigma_xz nodes
  long long c = g.lin(i0, j0);
  F4 xu0 = ld4z(ux, c - P, ldok), xu1 = ld4z(ux, c, ldok), xu2 = ld4z(ux, c + P, ldok), xu3 = ld4z(ux, c + 2 * P, ldok);
  F4 zu0 = ld4z(uz, c - 2 * P, ldok), zu1 = ld4z(uz, c - P, ldok), zu2 = ld4z(uz, c, ldok), zu3 = ld4z(uz, c + P, ldok);
  for (int j = j0; j <= j1; ++j, c += P) {
    const bool more = j + 1 <= j1;
    F4 xun = ld4z(ux, c + 3 * P, ldok && more);
    F4 zun = ld4z(uz, c + 2 * P, ldok && more);
    // ux at i0-2 .. i0+4, uz at i0-1 .. i0+5 (row j)
    float ua[7], za[7];
    ua[0] = __shfl_up_sync(FULL, xu1.v[2], 1);
    ua[1] = __shfl_up_sync(FULL, xu1.v[3], 1);
    ua[6] = __shfl_down_sync(FULL, xu1.v[0], 1);
    za[0] = __shfl_up_sync(FULL, zu2.v[3], 1);
    za[5] = __shfl_down_sync(FULL, zu2.v[0], 1);
    za[6] = __shfl_down_sync(FULL, zu2.v[1], 1);
    if (lane == 0) {
      ua[0] = ldz(ux, c - 2, ldok);
      ua[1] = ldz(ux, c - 1, ldok);
      za[0] = ldz(uz, c - 1, ldok);
    }
    if (lane == 31) {
      ua[6] = ldz(ux, c + 4, ldok);
      za[5] = ldz(uz, c + 4, ldok);
      za[6] = ldz(uz, c + 5, ldok);
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      ua[2 + e] = xu1.v[e];
      za[1 + e] = zu2.v[e];
    }
    const F4 L4 = ld4z(A.lam, c, ldok), M4 = ld4z(A.mu, c, ldok), MIJ = ld4z(A.mu_ij, c, ldok);
    int colF = 0, colH = 0;
    const int kF = cpml_full(j, g.nz, g.halo, colF);  // duz/dz at sigma_xx nodes (uz has nz-1 points)
    const int kH = cpml_half(j, g.nz, g.halo, colH);  // dux/dz at sigma_xz nodes (ux has nz points)
    float oxx[4], ozz[4], oxz[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int i = i0 + e;
      const float l = L4.v[e], m = M4.v[e];
      const float l2m = l + 2.0f * m;
      // sigma_xx, sigma_zz
      const float dux = d4(ua[e], ua[e + 1], ua[e + 2], ua[e + 3], g.idx);
      float duz;
      if (g.ft && j == 1) duz = (-l / l2m) * dux;
      else if (g.ft && j == 2) duz = d4(zu1.v[e], zu1.v[e], zu2.v[e], zu3.v[e], g.idz);
      else duz = d4(zu0.v[e], zu1.v[e], zu2.v[e], zu3.v[e], g.idz);
      const bool xx = i >= 2 && i <= g.nx - 1 && j >= jlo;
      float duxc = dux, duzc = duz;
      if (xstrip && xx) {
        int colE = 0;
        const int kE = cpml_full(i, g.nx, g.halo, colE);
        if (kE) duxc = cpml_upd(A.px[2] + (long long)s * A.xs + (long long)(j - 1) * g.W + colE, cx[kE - 1],
                                cx[na + nh + kE - 1], dux);
      }
      if (kF && xx)
        duzc = cpml_upd(A.pz[3] + (long long)s * A.zs + (long long)colF * P + (i - 1), cz[kF - 1],
                        cz[na + nh + kF - 1], duz);
      oxx[e] = l2m * duxc + l * duzc;
      ozz[e] = (j == 1) ? 0.0f : l * duxc + l2m * duzc;
      // sigma_xz
      const float dzx = d4(za[e], za[e + 1], za[e + 2], za[e + 3], g.idx);
      const float dxz = (g.ft && j == 1) ? d4(xu2.v[e], xu1.v[e], xu2.v[e], xu3.v[e], g.idz)
                                         : d4(xu0.v[e], xu1.v[e], xu2.v[e], xu3.v[e], g.idz);
      const bool xz = i <= g.nx - 1;
      float dzxc = dzx, dxzc = dxz;
      if (xstrip && xz) {
        int colG = 0;
        const int kG = cpml_half(i, g.nx, g.halo, colG);
        if (kG) dzxc = cpml_upd(A.px[3] + (long long)s * A.xs + (long long)(j - 1) * g.W + colG, cx[na + kG - 1],
                                cx[2 * na + nh + kG - 1], dzx);
      }
      if (kH && xz)
        dxzc = cpml_upd(A.pz[2] + (long long)s * A.zs + (long long)colH * P + (i - 1), cz[na + kH - 1],
                        cz[2 * na + nh + kH - 1], dxz);
      oxz[e] = MIJ.v[e] * (dzxc + dxzc);
    }
    if (ldok) {
      if (xx_all && j >= jlo) {
        st4v(sxx, c, oxx);
        st4v(szz, c, ozz);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          if (i >= 2 && i <= g.nx - 1 && j >= jlo) {
            sxx[c + e] = oxx[e];
            szz[c + e] = ozz[e];
          }
        }
      }
      if (xz_all) {
        st4v(sxz, c, oxz);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (i0 + e <= g.nx - 1) sxz[c + e] = oxz[e];
      }
    }
    xu0 = xu1; xu1 = xu2; xu2 = xu3; xu3 = xun;
    zu0 = zu1; zu1 = zu2; zu2 = zu3; zu3 = zun;
  }
}

// COMP: 2 updates ux and uz; 0 only ux, 1 only uz (two launches with fewer
// registers each: the uz half loads no sigma_xx and no sigma_xz column, the ux
// half no sigma_zz)
template <int COMP>
struct ElDispBounds {
  static constexpr int MINB = COMP == 2 ? 5 : 7;
};
template <int TZ, int COMP = 2>
__global__ void __launch_bounds__(BX, ElDispBounds<COMP>::MINB) k_el_disp4(const Args A) {
  const Geo g = A.g;
  const int s = blockIdx.z;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wx0 = (blockIdx.x * 4 + warp) * 128;
  const int j0 = blockIdx.y * TZ + 1;
  const int j1 = min(j0 + TZ - 1, g.nz);
  if (j0 > j1 || wx0 >= g.nx) return;
  const int i0 = wx0 + lane * 4 + 1;
  const bool ldok = i0 <= g.nx + 2;
  const long long so = (long long)s * g.F;
  float* __restrict__ ux = A.ux + so;
  float* __restrict__ uz = A.uz + so;
  float* __restrict__ dux = A.dux + so;
  float* __restrict__ duz = A.duz + so;
  const float* __restrict__ sxx = A.sxx + so;
  const float* __restrict__ szz = A.szz + so;
  const float* __restrict__ sxz = A.sxz + so;
  const int na = 2 * g.halo + 2, nh = 2 * g.halo;
  const float* cx = A.cp + (long long)s * A.cps;
  const float* cz = cx + 2 * na + 2 * nh;
  const bool slots = A.sUx != nullptr;
  const int P = g.P;
  const bool xstrip = i0 <= g.halo + 1 || i0 + 3 >= g.nx - 1 - g.halo;
  const bool ux_all = i0 + 3 <= g.nx - 1;  // all four points are ux nodes
  const bool uz_all = i0 + 3 <= g.nx;      // all four points are uz nodes
  constexpr bool DOX = COMP != 1, DOZ = COMP != 0;
  long long c = g.lin(i0, j0);
  F4 q0{}, q1{}, q3{}, w0{}, w1{}, w2{}, w3{}, xc{};
  if (DOX) {
    q0 = ld4z(sxz, c - 2 * P, ldok);
    q1 = ld4z(sxz, c - P, ldok);
    q3 = ld4z(sxz, c + P, ldok);
    xc = ld4z(sxx, c, ldok);
  }
  F4 q2 = ld4z(sxz, c, ldok);
  if (DOZ) {
    w0 = ld4z(szz, c - P, ldok);
    w1 = ld4z(szz, c, ldok);
    w2 = ld4z(szz, c + P, ldok);
    w3 = ld4z(szz, c + 2 * P, ldok);
  }
  for (int j = j0; j <= j1; ++j, c += P) {
    const bool more = j + 1 <= j1;
    F4 qn{}, wn{}, xcn{};
    if (DOX) {
      qn = ld4z(sxz, c + 2 * P, ldok && more);
      xcn = ld4z(sxx, c + P, ldok && more);
    } else {
      qn = ld4z(sxz, c + P, ldok && more);  // only row j+1 (next q2)
    }
    if (DOZ) wn = ld4z(szz, c + 3 * P, ldok && more);
    // sigma_xx at i0-1 .. i0+5, sigma_xz at i0-2 .. i0+4 (row j)
    float xa[7], qa[7];
    if (DOX) {
      xa[0] = __shfl_up_sync(FULL, xc.v[3], 1);
      xa[5] = __shfl_down_sync(FULL, xc.v[0], 1);
      xa[6] = __shfl_down_sync(FULL, xc.v[1], 1);
      if (lane == 0) xa[0] = ldz(sxx, c - 1, ldok);
      if (lane == 31) {
        xa[5] = ldz(sxx, c + 4, ldok);
        xa[6] = ldz(sxx, c + 5, ldok);
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) xa[1 + e] = xc.v[e];
    }
    if (DOZ) {
      qa[0] = __shfl_up_sync(FULL, q2.v[2], 1);
      qa[1] = __shfl_up_sync(FULL, q2.v[3], 1);
      qa[6] = __shfl_down_sync(FULL, q2.v[0], 1);
      if (lane == 0) {
        qa[0] = ldz(sxz, c - 2, ldok);
        qa[1] = ldz(sxz, c - 1, ldok);
      }
      if (lane == 31) qa[6] = ldz(sxz, c + 4, ldok);
#pragma unroll
      for (int e = 0; e < 4; ++e) qa[2 + e] = q2.v[e];
    }
    int colB = 0, colD = 0;
    const int kB = cpml_full(j, g.nz, g.halo, colB);  // dsxz/dz at ux nodes (sigma_xz has nz-1 points)
    const int kD = cpml_half(j, g.nz, g.halo, colD);  // dszz/dz at uz nodes (sigma_zz has nz points)
    if (ldok && DOX) {
      // ux nodes
      const F4 R = ld4z(A.dtr_i, c, true);
      F4 U = ld4rwz(ux, c), DU = ld4rwz(dux, c);
      float nu[4], ndu[4], Dv[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        const float d1 = d4(xa[e], xa[e + 1], xa[e + 2], xa[e + 3], g.idx);
        float d2;
        if (g.ft && j == 1) d2 = d4(-q3.v[e], -q2.v[e], q2.v[e], q3.v[e], g.idz);
        else if (g.ft && j == 2) d2 = d4(-q1.v[e], q1.v[e], q2.v[e], q3.v[e], g.idz);
        else d2 = d4(q0.v[e], q1.v[e], q2.v[e], q3.v[e], g.idz);
        const bool on = i <= g.nx - 1;
        float d1c = d1, d2c = d2;
        if (xstrip && on) {
          int colA = 0;
          const int kA = cpml_half(i, g.nx, g.halo, colA);
          if (kA) d1c = cpml_upd(A.px[0] + (long long)s * A.xs + (long long)(j - 1) * g.W + colA, cx[na + kA - 1],
                                 cx[2 * na + nh + kA - 1], d1);
        }
        if (kB && on)
          d2c = cpml_upd(A.pz[1] + (long long)s * A.zs + (long long)colB * P + (i - 1), cz[kB - 1],
                         cz[na + nh + kB - 1], d2);
        Dv[e] = R.v[e] * (d1c + d2c);
        ndu[e] = DU.v[e] + Dv[e];
        nu[e] = U.v[e] + ndu[e];
      }
      if (ux_all) {
        if (slots) {
          st4v(A.sUx + so, c, U.v);
          st4v(A.sDx + so, c, Dv);
        }
        st4v(ux, c, nu);
        st4v(dux, c, ndu);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (i0 + e <= g.nx - 1) {
            if (slots) {
              A.sUx[so + c + e] = U.v[e];
              A.sDx[so + c + e] = Dv[e];
            }
            ux[c + e] = nu[e];
            dux[c + e] = ndu[e];
          }
      }
    }
    if (ldok && DOZ) {
      // uz nodes
      if (j <= g.nz - 1) {
        const F4 Rj = ld4z(A.dtr_j, c, true);
        F4 V = ld4rwz(uz, c), DV = ld4rwz(duz, c);
        float nv[4], ndv[4], Dz[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          const float d1 = d4(qa[e], qa[e + 1], qa[e + 2], qa[e + 3], g.idx);
          const float d2 = (g.ft && j == 1) ? d4(-w2.v[e], w1.v[e], w2.v[e], w3.v[e], g.idz)
                                            : d4(w0.v[e], w1.v[e], w2.v[e], w3.v[e], g.idz);
          const bool on = i <= g.nx;
          float d1c = d1, d2c = d2;
          if (xstrip && on) {
            int colC = 0;
            const int kC = cpml_full(i, g.nx, g.halo, colC);
            if (kC) d1c = cpml_upd(A.px[1] + (long long)s * A.xs + (long long)(j - 1) * g.W + colC, cx[kC - 1],
                                   cx[na + nh + kC - 1], d1);
          }
          if (kD && on)
            d2c = cpml_upd(A.pz[0] + (long long)s * A.zs + (long long)colD * P + (i - 1), cz[na + kD - 1],
                           cz[2 * na + nh + kD - 1], d2);
          Dz[e] = Rj.v[e] * (d1c + d2c);
          ndv[e] = DV.v[e] + Dz[e];
          nv[e] = V.v[e] + ndv[e];
        }
        if (uz_all) {
          if (slots) {
            st4v(A.sUz + so, c, V.v);
            st4v(A.sDz + so, c, Dz);
          }
          st4v(uz, c, nv);
          st4v(duz, c, ndv);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (i0 + e <= g.nx) {
              if (slots) {
                A.sUz[so + c + e] = V.v[e];
                A.sDz[so + c + e] = Dz[e];
              }
              uz[c + e] = nv[e];
              duz[c + e] = ndv[e];
            }
        }
      }
    }
    if (DOX) {
      q0 = q1; q1 = q2; q2 = q3; q3 = qn;
      xc = xcn;
    } else {
      q2 = qn;
    }
    if (DOZ) {
      w0 = w1; w1 = w2; w2 = w3; w3 = wn;
    }
  }
}

// ---------------------------------------------------------------------------
// Sources, receivers, misfit
// ---------------------------------------------------------------------------
// Unique-point CSR of one injection table: point p (padded index lin[p]) gets
// sum over e in [ptr[p], ptr[p+1]) of coef[e] * tf(item[e]).
struct Inj {
  int np;
  const long long* lin;
  const int* ptr;
  const int* item;
  const float* coef;
};

struct ShotDesc {
  int nt, kind, nsrc, nrec;
  const float* tf;  // srctf, device: kind 0 (nt, nsrc), kind 1 (nt, 2, nsrc)
  const float* mtp; // (3, nsrc) moment tensors, device
  float sf;         // this shot's source scale (a power of two)
  Inj src[2];       // sources: kind 0 -> sigma grids, kind 1 -> ux / uz grids
  Inj adj[2];       // receivers as adjoint forces on ux / uz
  const int* rptr[2];        // recording CSR by receiver (nrec+1)
  const long long* rlin[2];
  const float* rcoef[2];
  float* tr;                 // traces (nt, 2, nrec)
  const float* obs;          // observed
  const float* ic;           // diagonal inverse covariance or null
  const float* mask;         // window mask (nt) or null
  float* adjsrc;             // adjoint source (nt, 2, nrec)
  const float* icd;          // dense inverse covariance (nt, nt) or null
  float* resid;              // dense case: masked residuals (nt, 2 nrec)
  const float* cres;         // dense case: C^-1 r (nt, 2 nrec), from the dense product (dense.cu)
  int mkind;                 // 0 L2, 1 CCTS (k_ccts writes this shot's adjoint source)
};

// sigma_xx += Mxx w tf, sigma_zz += Mzz w tf (table 0), sigma_xz += Mxz w tf (table 1)
__global__ void k_el_inject_sigma(const ShotDesc* __restrict__ desc, int it, long long F, float* sxx, float* szz,
                                  float* sxz) {
  const int s = blockIdx.y;
  const ShotDesc& D = desc[s];
  if (it > D.nt || D.kind != 0) return;
  const float scale = D.sf;
  const long long so = (long long)s * F;
  for (int t = 0; t < 2; ++t) {
    const Inj J = D.src[t];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < J.np; p += gridDim.x * blockDim.x) {
      float a = 0.0f, b = 0.0f;
      for (int e = J.ptr[p]; e < J.ptr[p + 1]; ++e) {
        const int k = J.item[e];
        const float v = J.coef[e] * (D.tf[(long long)(it - 1) + (long long)k * D.nt] * scale);
        if (t == 0) {
          a += D.mtp[3 * k] * v;
          b += D.mtp[3 * k + 1] * v;
        } else {
          a += D.mtp[3 * k + 2] * v;
        }
      }
      const long long c = so + J.lin[p];
      if (t == 0) {
        sxx[c] += a;
        szz[c] += b;
      } else {
        sxz[c] += a;
      }
    }
  }
}

// u += w tf / rho dt^2 on the ux (table 0) and uz (table 1) grids; adjoint = 1
// uses the receivers' tables and the adjoint source scaled by *adj_scale (a
// device value, set by k_el_adj_scale; the forward sources use the shot's
// own scale).  With D slots, D(it) gets the
// same increment (it is part of the second time difference).
__global__ void k_el_inject_force(const ShotDesc* __restrict__ desc, int it, int adjoint,
                                  const float* __restrict__ adj_scale, long long F,
                                  float* ux, float* uz, float* dux, float* duz, float* Dx, float* Dz,
                                  const float* __restrict__ dtr_i, const float* __restrict__ dtr_j) {
  const int s = blockIdx.y;
  const ShotDesc& D = desc[s];
  if (it > D.nt) return;
  if (!adjoint && D.kind != 1) return;
  const long long so = (long long)s * F;
  const float* tf = adjoint ? D.adjsrc : D.tf;
  const float scale = adjoint ? *adj_scale : D.sf;
  for (int t = 0; t < 2; ++t) {
    const Inj J = adjoint ? D.adj[t] : D.src[t];
    float* u = t == 0 ? ux : uz;
    float* du = t == 0 ? dux : duz;
    float* Dd = t == 0 ? Dx : Dz;
    const float* dtr = t == 0 ? dtr_i : dtr_j;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < J.np; p += gridDim.x * blockDim.x) {
      float acc = 0.0f;
      for (int e = J.ptr[p]; e < J.ptr[p + 1]; ++e) {
        const int k = J.item[e];
        acc += J.coef[e] * (tf[(long long)(it - 1) + (long long)D.nt * (t + 2LL * k)] * scale);
      }
      const long long c = J.lin[p];
      const float v = acc * dtr[c];
      u[so + c] += v;
      du[so + c] += v;
      if (Dd) Dd[so + c] += v;
    }
  }
}

// trace(it, comp, r) = sum_e w_e u(p_e), scaled back by the shot's source scale
__global__ void k_el_record(const ShotDesc* __restrict__ desc, int it, long long F, const float* __restrict__ ux,
                            const float* __restrict__ uz) {
  const int s = blockIdx.y;
  const ShotDesc& D = desc[s];
  if (it > D.nt) return;
  const float inv_scale = 1.0f / D.sf;
  const long long so = (long long)s * F;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 2 * D.nrec; q += gridDim.x * blockDim.x) {
    const int t = q & 1, r = q >> 1;
    const float* u = (t == 0 ? ux : uz) + so;
    float acc = 0.0f;
    for (int e = D.rptr[t][r]; e < D.rptr[t][r + 1]; ++e) acc += D.rcoef[t][e] * u[D.rlin[t][e]];
    D.tr[(long long)(it - 1) + (long long)D.nt * (t + 2LL * r)] = acc * inv_scale;
  }
}

// The power of two 2^e with 2^e * max|C^-1 r| close to 2^20 (1 for a zero or
// non-finite maximum), the adjoint source's scale, written to scales[1] on
// the device, so that no host round trip sits between the misfit and the
// adjoint (the gradient's time loop can run as one CUDA graph).
__global__ void k_el_adj_scale(const unsigned int* __restrict__ amax, float* __restrict__ scales) {
  const float v = __uint_as_float(*amax);
  float sc = 1.0f;
  if (v > 0.0f && isfinite(v)) {
    const int e = 20 - (int)lround(log2((double)v));
    sc = ldexpf(1.0f, max(-100, min(100, e)));
  }
  scales[1] = sc;
}

// Residuals, windows, C^-1 r, misfit partials (FP64), adjoint source -C^-1 r
// and the running maximum of |C^-1 r| (as float bits).
__global__ void k_el_misfit(const ShotDesc* __restrict__ desc, double* __restrict__ partial,
                            unsigned int* __restrict__ amax) {
  const int shot = blockIdx.y;
  const ShotDesc& D = desc[shot];
  const long long total = D.mkind == 1 ? 0 : (long long)D.nt * 2 * D.nrec;  // CCTS shots: k_ccts
  double acc = 0.0;
  float mx = 0.0f;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int t = (int)(q % D.nt);
    float res = D.tr[q] - D.obs[q];
    if (D.mask) res *= D.mask[t];
    const float cres = D.cres ? D.cres[q] : (D.ic ? D.ic[t] * res : res);
    acc += (double)res * (double)cres;
    D.adjsrc[q] = -cres;
    mx = fmaxf(mx, fabsf(cres));
  }
  __shared__ double red[256];
  __shared__ float redm[256];
  red[threadIdx.x] = acc;
  redm[threadIdx.x] = mx;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) {
      red[threadIdx.x] += red[threadIdx.x + k];
      redm[threadIdx.x] = fmaxf(redm[threadIdx.x], redm[threadIdx.x + k]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[(long long)shot * gridDim.x + blockIdx.x] = red[0];
    atomicMax(amax, __float_as_uint(redm[0]));  // non-negative floats order like their bits
  }
}

// Masked residuals of the shots with a dense inverse covariance.
__global__ void k_el_residual_dense(const ShotDesc* __restrict__ desc) {
  const ShotDesc& D = desc[blockIdx.y];
  if (!D.icd) return;
  const long long total = (long long)D.nt * 2 * D.nrec;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    float res = D.tr[q] - D.obs[q];
    if (D.mask) res *= D.mask[q % D.nt];
    D.resid[q] = res;
  }
}

__global__ void k_el_absmax(const float* __restrict__ v, long long n, unsigned int* __restrict__ out) {
  float mx = 0.0f;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    mx = fmaxf(mx, fabsf(v[q]));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(mx));
}

__global__ void k_el_misfit_sum(const double* __restrict__ partial, int n, double* out, int accumulate) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = (accumulate ? *out : 0.0) + 0.5 * red[0];
}

// ---------------------------------------------------------------------------
// Gradient correlation (correlate_gradients!) of adjoint step it, summed over
// the shots of each group and added to the group's Kahan-compensated FP32
// accumulators: acc[group][q][F], q = 0 rho_ihalf (times dt^2), 1 rho_jhalf
// (times dt^2), 2 lambda, 3 mu, 4 mu_ihalf_jhalf; compensations at q + 5.
// ---------------------------------------------------------------------------
struct CorrArgs {
  Geo g;
  int nshots, gsize;
  const float* cs;                     // per shot: common scale / own source scale (a power of two)
  const float* aux; const float* auz;  // adjoint displacement after step it
  const float* fux; const float* fuz;  // forward u[it-1] (slot)
  const float* Dx; const float* Dz;    // forward D(it) (slot)
  const float* lam; const float* mu;
  float* acc;
};

__device__ __forceinline__ void kahan_add_el(float* g, float* c, float y) {
  const float yy = __fsub_rn(y, *c);
  const float t = __fadd_rn(*g, yy);
  *c = __fsub_rn(__fsub_rn(t, *g), yy);
  *g = t;
}

// Shots outer, rows inner: each thread keeps the five sums of its CTZ rows in
// registers while it walks the shots of its group (two shots in flight).
__global__ void __launch_bounds__(BX) k_el_corr(const CorrArgs A) {
  const Geo g = A.g;
  const int grp = blockIdx.z;
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  if (i > g.nx) return;
  const int s0 = grp * A.gsize, s1 = min(s0 + A.gsize, A.nshots);
  float* acc = A.acc + (long long)grp * 10 * g.F;
  const int jlo = g.ft ? 1 : 2;
  const int j0 = blockIdx.y * CTZ + 1;
  const bool on_ux = i <= g.nx - 1;
  const bool xx_col = i >= 2 && i <= g.nx - 1;
  float v[5][CTZ];
#pragma unroll
  for (int r = 0; r < CTZ; ++r) {
#pragma unroll
    for (int q = 0; q < 5; ++q) v[q][r] = 0.0f;
  }
  float fsr = 0.0f;  // -lambda / (lambda + 2 mu) on the free surface (row j = 1)
  if (g.ft && j0 == 1 && xx_col) {
    const long long c1 = g.lin(i, 1);
    const float l = __ldg(A.lam + c1);
    fsr = -l / (l + 2.0f * __ldg(A.mu + c1));
  }
#pragma unroll 2
  for (int s = s0; s < s1; ++s) {
    const long long so = (long long)s * g.F;
    const float cs = __ldg(A.cs + s);
    const float* aux = A.aux + so;
    const float* auz = A.auz + so;
    const float* fux = A.fux + so;
    const float* fuz = A.fuz + so;
    const float* Dx = A.Dx + so;
    const float* Dz = A.Dz + so;
#pragma unroll
    for (int r = 0; r < CTZ; ++r) {
      const int j = j0 + r;
      if (j <= g.nz) {
        const long long c = g.lin(i, j);
        const bool on_uz = j <= g.nz - 1;
        if (on_ux) v[0][r] += cs * (__ldg(aux + c) * __ldg(Dx + c));
        if (on_uz) v[1][r] += cs * (__ldg(auz + c) * __ldg(Dz + c));
        if (xx_col && j >= jlo && on_uz) {
          const float exx = dux_dx(fux, c, g.idx);
          const float exa = dux_dx(aux, c, g.idx);
          float ezz, eza;
          if (g.ft && j == 1) {
            ezz = fsr * exx;
            eza = fsr * exa;
          } else {
            ezz = duz_dz_raw(fuz, c, g.P, j, g.ft, g.idz);
            eza = duz_dz_raw(auz, c, g.P, j, g.ft, g.idz);
          }
          v[2][r] += cs * ((exx + ezz) * (exa + eza));
          v[3][r] += cs * (exx * exa + ezz * eza);
        }
        if (on_ux && on_uz) {
          const float e = duz_dx(fuz, c, g.idx) + dux_dz(fux, c, g.P, j, g.ft, g.idz);
          const float ea = duz_dx(auz, c, g.idx) + dux_dz(aux, c, g.P, j, g.ft, g.idz);
          v[4][r] += cs * (e * ea);  // 2 (exz exz' + ezx ezx') with exz = e / 2
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < CTZ; ++r) {
    const int j = j0 + r;
    if (j > g.nz) break;
    const long long c = g.lin(i, j);
    const bool on_uz = j <= g.nz - 1;
    const bool half = g.ft && j == 1;
    if (on_ux) kahan_add_el(acc + c, acc + 5 * g.F + c, half ? 0.5f * v[0][r] : v[0][r]);
    if (on_uz) kahan_add_el(acc + g.F + c, acc + 6 * g.F + c, v[1][r]);
    if (xx_col && j >= jlo && on_uz) {
      kahan_add_el(acc + 2 * g.F + c, acc + 7 * g.F + c, half ? 0.5f * v[2][r] : v[2][r]);
      kahan_add_el(acc + 3 * g.F + c, acc + 8 * g.F + c, half ? v[3][r] : 2.0f * v[3][r]);
    }
    if (on_ux && on_uz) kahan_add_el(acc + 4 * g.F + c, acc + 9 * g.F + c, v[4][r]);
  }
}

// Four x points per thread, 512 per block, one row per block (blockIdx.y):
// the same sums as k_el_corr.  For every shot the thread loads float4s of the
// rows it needs (ux rows j-1 .. j+2, uz rows j-2 .. j+1, forward and adjoint,
// D of row j) and takes the x neighbours from the adjacent lanes (loaded at
// the warp edges); the z re-reads of neighbouring rows hit L1/L2.
__global__ void __launch_bounds__(BX) k_el_corr4(const CorrArgs A) {
  const Geo g = A.g;
  const int grp = blockIdx.z;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wx0 = (blockIdx.x * 4 + warp) * 128;
  const int j = blockIdx.y + 1;
  if (wx0 >= g.nx || j > g.nz) return;  // warp uniform; no block-level synchronisation
  const int i0 = wx0 + lane * 4 + 1;
  const bool ldok = i0 <= g.nx + 2;
  const int s0 = grp * A.gsize, s1 = min(s0 + A.gsize, A.nshots);
  float* acc = A.acc + (long long)grp * 10 * g.F;
  const int jlo = g.ft ? 1 : 2;
  const bool on_uz = j <= g.nz - 1;
  const bool fs1 = g.ft && j == 1, fs2 = g.ft && j == 2;
  const int P = g.P;
  const long long c = g.lin(i0, j);
  float fsr[4] = {0.f, 0.f, 0.f, 0.f};  // -lambda / (lambda + 2 mu) on the free surface (row 1)
  if (fs1 && ldok) {
    const F4 L = ld4z(A.lam, c, true), M = ld4z(A.mu, c, true);
#pragma unroll
    for (int e = 0; e < 4; ++e) fsr[e] = (L.v[e] + 2.0f * M.v[e]) != 0.0f ? -L.v[e] / (L.v[e] + 2.0f * M.v[e]) : 0.0f;
  }
  float v[5][4];
#pragma unroll
  for (int q = 0; q < 5; ++q)
#pragma unroll
    for (int e = 0; e < 4; ++e) v[q][e] = 0.0f;
  for (int s = s0; s < s1; ++s) {
    const long long so = (long long)s * g.F;
    const float cs = __ldg(A.cs + s);
    float sx[2][4], sz[2][4], exz[2][4];  // [forward, adjoint]: exx, ezz, 2 exz at the 4 points
    float rho_x[4], rho_z[4];
#pragma unroll
    for (int w = 0; w < 2; ++w) {
      const float* ux = (w == 0 ? A.fux : A.aux) + so;
      const float* uz = (w == 0 ? A.fuz : A.auz) + so;
      // ux rows j-1 .. j+2, uz rows j-2 .. j+1
      const F4 xm = ld4z(ux, c - P, ldok), x0 = ld4z(ux, c, ldok), xp = ld4z(ux, c + P, ldok),
               xpp = ld4z(ux, c + 2 * P, ldok);
      const F4 zmm = ld4z(uz, c - 2 * P, ldok), zm = ld4z(uz, c - P, ldok), z0 = ld4z(uz, c, ldok),
               zp = ld4z(uz, c + P, ldok);
      if (w == 1) {
        const F4 DX = ld4z(A.Dx + so, c, ldok), DZ = ld4z(A.Dz + so, c, ldok);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          rho_x[e] = x0.v[e] * DX.v[e];
          rho_z[e] = z0.v[e] * DZ.v[e];
        }
      }
      // ux at i0-2 .. i0+4 and uz at i0-1 .. i0+5 of row j
      float ua[7], za[7];
      ua[0] = __shfl_up_sync(FULL, x0.v[2], 1);
      ua[1] = __shfl_up_sync(FULL, x0.v[3], 1);
      ua[6] = __shfl_down_sync(FULL, x0.v[0], 1);
      za[0] = __shfl_up_sync(FULL, z0.v[3], 1);
      za[5] = __shfl_down_sync(FULL, z0.v[0], 1);
      za[6] = __shfl_down_sync(FULL, z0.v[1], 1);
      if (lane == 0) {
        ua[0] = ldz(ux, c - 2, ldok);
        ua[1] = ldz(ux, c - 1, ldok);
        za[0] = ldz(uz, c - 1, ldok);
      }
      if (lane == 31) {
        ua[6] = ldz(ux, c + 4, ldok);
        za[5] = ldz(uz, c + 4, ldok);
        za[6] = ldz(uz, c + 5, ldok);
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        ua[2 + e] = x0.v[e];
        za[1 + e] = z0.v[e];
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float exx = d4(ua[e], ua[e + 1], ua[e + 2], ua[e + 3], g.idx);
        float ezz;
        if (fs1) ezz = fsr[e] * exx;
        else if (fs2) ezz = d4(zm.v[e], zm.v[e], z0.v[e], zp.v[e], g.idz);
        else ezz = d4(zmm.v[e], zm.v[e], z0.v[e], zp.v[e], g.idz);
        const float dzx = d4(za[e], za[e + 1], za[e + 2], za[e + 3], g.idx);
        const float dxz = fs1 ? d4(xp.v[e], x0.v[e], xp.v[e], xpp.v[e], g.idz)
                              : d4(xm.v[e], x0.v[e], xp.v[e], xpp.v[e], g.idz);
        sx[w][e] = exx;
        sz[w][e] = ezz;
        exz[w][e] = dzx + dxz;
      }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      v[0][e] += cs * rho_x[e];
      v[1][e] += cs * rho_z[e];
      v[2][e] += cs * ((sx[0][e] + sz[0][e]) * (sx[1][e] + sz[1][e]));
      v[3][e] += cs * (sx[0][e] * sx[1][e] + sz[0][e] * sz[1][e]);
      v[4][e] += cs * (exz[0][e] * exz[1][e]);
    }
  }
  if (!ldok) return;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    const long long ce = c + e;
    const bool on_ux = i <= g.nx - 1;
    if (on_ux) kahan_add_el(acc + ce, acc + 5 * g.F + ce, fs1 ? 0.5f * v[0][e] : v[0][e]);
    if (on_uz && i <= g.nx) kahan_add_el(acc + g.F + ce, acc + 6 * g.F + ce, v[1][e]);
    if (i >= 2 && i <= g.nx - 1 && j >= jlo && on_uz) {
      kahan_add_el(acc + 2 * g.F + ce, acc + 7 * g.F + ce, fs1 ? 0.5f * v[2][e] : v[2][e]);
      kahan_add_el(acc + 3 * g.F + ce, acc + 8 * g.F + ce, fs1 ? v[3][e] : 2.0f * v[3][e]);
    }
    if (on_ux && on_uz) kahan_add_el(acc + 4 * g.F + ce, acc + 9 * g.F + ce, v[4][e]);
  }
}

// One snapshot block per shot (blockIdx.y): ux, uz, sxx, szz, sxz unpadded and
// scaled back from the shot's source scale, into stage + shot * B.
__global__ void k_el_snapshot(Geo g, const ShotDesc* __restrict__ desc, const float* __restrict__ ux,
                              const float* __restrict__ uz, const float* __restrict__ sxx,
                              const float* __restrict__ szz, const float* __restrict__ sxz, long long B,
                              float* __restrict__ stage) {
  const int s = blockIdx.y;
  const float inv = 1.0f / desc[s].sf;
  const long long so = (long long)s * g.F;
  const long long n0 = (long long)(g.nx - 1) * g.nz, n1 = (long long)g.nx * (g.nz - 1);
  const long long n2 = (long long)g.nx * g.nz, n4 = (long long)(g.nx - 1) * (g.nz - 1);
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < B; q += (long long)gridDim.x * blockDim.x) {
    const float* f;
    long long r = q;
    int w;
    if (r < n0) { f = ux; w = g.nx - 1; }
    else if ((r -= n0) < n1) { f = uz; w = g.nx; }
    else if ((r -= n1) < n2) { f = sxx; w = g.nx; }
    else if ((r -= n2) < n2) { f = szz; w = g.nx; }
    else { r -= n2; f = sxz; w = g.nx - 1; (void)n4; }
    const int i = (int)(r % w) + 1, j = (int)(r / w) + 1;
    stage[(long long)s * B + q] = f[so + g.lin(i, j)] * inv;
  }
}

// Mute ball of one position (mutearoundpoint!, src/utils/mute_grad.jl:13-80).
struct MuteBall {
  int lo[2], hi[2];
  double pos[2];
  double rmax;
};

__device__ __forceinline__ double acc_val(const float* acc, int q, long long F, long long c) {
  return (double)acc[q * F + c] - (double)acc[(q + 5) * F + c];
}

// Final gradients (FP64, (nx, nz) column-major), summed over the groups:
// lambda; mu + back_interp(mu_ihalf_jhalf); back_interp(rho_ihalf) +
// back_interp(rho_jhalf) (times 1/dt^2); each group's sum muted around its
// shot's positions; times 1 / (scales[0] scales[1]) (the forward and adjoint
// source scales).
__global__ void k_el_reduce(Geo g, int ngroups, const float* __restrict__ acc, const double* __restrict__ rho,
                            const double* __restrict__ mu, int irho, int imu, double inv_dt2,
                            const float* __restrict__ scales,
                            const MuteBall* __restrict__ balls, const int* __restrict__ ball_ptr,
                            double* __restrict__ grho, double* __restrict__ glam, double* __restrict__ gmu,
                            int accumulate) {
  const long long npts = (long long)g.nx * g.nz;
  const double inv_scale = 1.0 / ((double)scales[0] * (double)scales[1]);
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < npts;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q % g.nx) + 1, j = (int)(q / g.nx) + 1;
    auto M = [&](int a, int b) { return (long long)(a - 1) + (long long)(b - 1) * g.nx; };
    const double rho_c = rho[q], mu_c = mu[q];
    // back-interpolation weights of the (up to 4) half points around (i, j)
    double wri[2] = {0, 0}, wrj[2] = {0, 0}, wm[4] = {0, 0, 0, 0};
    bool vri[2], vrj[2], vm[4];
    for (int p = 0; p < 2; ++p) {
      const int ci = i - 1 + p;  // rho_ihalf cell (ci, j), ci in 1..nx-1, node = ci + (1 - p)
      vri[p] = ci >= 1 && ci <= g.nx - 1;
      if (vri[p]) {
        if (irho == 1) {
          const double h = 2.0 / (1.0 / rho[M(ci, j)] + 1.0 / rho[M(ci + 1, j)]);
          wri[p] = h * h / (rho_c * rho_c) * 0.5;
        } else wri[p] = 0.5;
      }
      const int cj = j - 1 + p;
      vrj[p] = cj >= 1 && cj <= g.nz - 1;
      if (vrj[p]) {
        if (irho == 1) {
          const double h = 2.0 / (1.0 / rho[M(i, cj)] + 1.0 / rho[M(i, cj + 1)]);
          wrj[p] = h * h / (rho_c * rho_c) * 0.5;
        } else wrj[p] = 0.5;
      }
    }
    for (int p = 0; p < 4; ++p) {
      const int ci = i - 1 + (p & 1), cj = j - 1 + (p >> 1);
      vm[p] = ci >= 1 && ci <= g.nx - 1 && cj >= 1 && cj <= g.nz - 1;
      if (vm[p]) {
        if (imu == 1) {
          const double h = 4.0 / (1.0 / mu[M(ci, cj)] + 1.0 / mu[M(ci + 1, cj)] + 1.0 / mu[M(ci, cj + 1)] +
                                  1.0 / mu[M(ci + 1, cj + 1)]);
          wm[p] = h * h / (mu_c * mu_c) * 0.25;
        } else wm[p] = 0.25;
      }
    }
    double sr = 0.0, sl = 0.0, sm = 0.0;
    for (int gi = 0; gi < ngroups; ++gi) {
      const float* a = acc + (long long)gi * 10 * g.F;
      double r = 0.0, m = 0.0;
      for (int p = 0; p < 2; ++p) {
        if (vri[p]) r += wri[p] * acc_val(a, 0, g.F, g.lin(i - 1 + p, j));
        if (vrj[p]) r += wrj[p] * acc_val(a, 1, g.F, g.lin(i, j - 1 + p));
      }
      r *= inv_dt2;
      for (int p = 0; p < 4; ++p)
        if (vm[p]) m += wm[p] * acc_val(a, 4, g.F, g.lin(i - 1 + (p & 1), j - 1 + (p >> 1)));
      const long long c = g.lin(i, j);
      double l = acc_val(a, 2, g.F, c);
      m += acc_val(a, 3, g.F, c);
      if (ball_ptr) {
        double f = 1.0;
        for (int b = ball_ptr[gi]; b < ball_ptr[gi + 1]; ++b) {
          const MuteBall B = balls[b];
          if (i < B.lo[0] || i > B.hi[0] || j < B.lo[1] || j > B.hi[1]) continue;
          const double x = (i - 1) * (double)g.idx, z = (j - 1) * (double)g.idz;  // idx/idz carry h here
          const double rr = sqrt((B.pos[0] - x) * (B.pos[0] - x) + (B.pos[1] - z) * (B.pos[1] - z));
          if (rr <= B.rmax) f *= rr / B.rmax;
        }
        r *= f;
        l *= f;
        m *= f;
      }
      sr += r;
      sl += l;
      sm += m;
    }
    sr *= inv_scale;
    sl *= inv_scale;
    sm *= inv_scale;
    grho[q] = accumulate ? grho[q] + sr : sr;
    glam[q] = accumulate ? glam[q] + sl : sl;
    gmu[q] = accumulate ? gmu[q] + sm : sm;
  }
}

}  // namespace el
}  // namespace swgb

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using namespace swgb;
using namespace swgb::el;

struct sw_elastic {
  sw_ctx* ctx = nullptr;
  sw_elastic_params prm{};
  bool gradient = false;
  sw_grad_params gp{};
  Geo g{};
  int na = 0, nh = 0, cps = 0;
  long long xs = 0, zs = 0;  // strip floats per shot (rounded to 32)
  bool has_mat = false;
  double vel_max = 0.0;
  DevMem lam, mu, dtr_i, dtr_j, mu_ij, rho_d, mu_d;
  // state
  int cap = 0;  // shots the state buffers hold
  int cap_slots = 0, cap_ck = 0, cap_groups = 0;
  DevMem st[7], ast[7];            // ux uz dux duz sxx szz sxz
  DevMem px[4], pz[4], apx[4], apz[4];
  DevMem slots;                    // [K][4][cap][F]
  DevMem ck;                       // [M][4][cap][F] then [M][8][cap][strip]
  DevMem acc;                      // [groups][10][F]
  // tables
  DevMem d_desc, d_ll, d_int, d_flt, d_tf, d_tr, d_obs, d_ic, d_mask, d_adj, d_mt, d_cp;
  DevMem d_partial, d_amax, d_balls, d_ball_ptr, d_cs;
  DevMem d_icd, d_dres;  // dense inverse covariances; residuals and C^-1 r of those shots
  DevMem d_snap;                     // snapshot stage (one block per shot)
  int snapevery = 0;                 // snapshots requested by the current forward call
  float* const* snap_out = nullptr;  // per caller shot: nt/snapevery blocks [ux, uz, sxx, szz, sxz]
  int tz = 8;  // rows per block of the stencil kernels (8, 16 or 32; 8 measured fastest)
  bool vec = true;  // four x points per thread (k_el_*4) instead of one
  bool split_disp = true;  // the displacement update as two launches, ux then uz (tz + 128: one launch)
  DevMem d_scales;        // [0] the forward sources' common scale, [1] the adjoint source's scale
  DevMem d_ccts, d_partial2;  // CCTS descriptors and per-trace misfit terms
  DevMem d_gout, d_mout;  // gradient / misfit of the host-buffer path (stable addresses for the graphs)
  // CUDA graphs of a group's whole gradient (forward, misfit, adjoint,
  // reduction), keyed by what the captured launches depend on
  long long gen = 0;  // bumped whenever a device buffer the kernels see is (re)allocated
  std::map<std::vector<long long>, cudaGraphExec_t> graphs;
  std::map<std::vector<long long>, int> graph_uses;
  void drop_graphs() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    graph_uses.clear();
  }
  ~sw_elastic() { drop_graphs(); }
};

namespace {

inline long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

void ensure(sw_elastic* es, DevMem& m, size_t bytes, const char* what) {
  if (m.bytes >= bytes && m.p) return;
  dev_alloc(m, bytes, what, es->ctx->stream);
  ++es->gen;
}

// Runs `work` (the device work of one group's gradient: launches, memsets and
// device copies, no host synchronisation, no allocation) through a CUDA
// graph: captured on the second call with `key`, replayed afterwards (at most
// 32 graphs per simulation); directly while profiling or when the caller's
// stream is itself being captured (the launches then join the caller's graph).
template <typename Work>
void el_run_graph(sw_elastic* es, std::vector<long long> key, Work&& work) {
  cudaStream_t st = es->ctx->stream;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  check_cuda(cudaStreamIsCapturing(st, &cs), "cudaStreamIsCapturing");
  if (es->ctx->prof.on || cs != cudaStreamCaptureStatusNone) {
    work();
    return;
  }
  key.push_back(es->gen);
  auto it = es->graphs.find(key);
  if (it == es->graphs.end()) {
    if (es->graph_uses.size() > 4096) es->graph_uses.clear();
    if (++es->graph_uses[key] < 2 || es->graphs.size() >= 32) {
      work();
      return;
    }
    check_cuda(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin stream capture");
    try {
      work();
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(st, &g);
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      throw;
    }
    cudaGraph_t g = nullptr;
    check_cuda(cudaStreamEndCapture(st, &g), "end stream capture");
    cudaGraphExec_t ex = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    check_cuda(e, "graph instantiate");
    it = es->graphs.emplace(key, ex).first;
  }
  check_cuda(cudaGraphLaunch(it->second, st), "graph launch");
}

template <typename T>
void upload(sw_elastic* es, DevMem& m, const std::vector<T>& v, const char* what) {
  ensure(es, m, std::max<size_t>(v.size() * sizeof(T), 16), what);
  if (!v.empty())
    check_cuda(cudaMemcpyAsync(m.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, es->ctx->stream), what);
}

struct HostShot {
  int orig;
  int nt;
};

// grid extents (1-based, inclusive) of the table grids
struct Ext {
  int ni, nj;
};
Ext grid_ext(const sw_elastic* es, int which) {
  const int nx = es->g.nx, nz = es->g.nz;
  switch (which) {
    case 0: return {nx, nz};          // sigma_xx / sigma_zz nodes
    case 1: return {nx - 1, nz - 1};  // sigma_xz
    case 2: return {nx - 1, nz};      // ux
    default: return {nx, nz - 1};     // uz
  }
}

void validate_table(const sw_elastic* es, const sw_point_table& t, int count, int which, const char* what, int k,
                    bool stress_src) {
  if (count <= 0) return;
  if (!t.offsets || !t.ij || !t.coef) {
    std::ostringstream os;
    os << "shot " << k << ": " << what << " table is NULL";
    fail(SW_ERR_ARG, os.str());
  }
  if (t.offsets[0] != 0) fail(SW_ERR_ARG, std::string(what) + " table offsets must start at 0");
  const Ext e = grid_ext(es, which);
  for (int q = 0; q < count; ++q) {
    if (t.offsets[q + 1] < t.offsets[q]) fail(SW_ERR_ARG, std::string(what) + " table offsets must not decrease");
    for (int p = t.offsets[q]; p < t.offsets[q + 1]; ++p) {
      const int i = t.ij[2 * p], j = t.ij[2 * p + 1];
      if (i < 1 || i > e.ni || j < 1 || j > e.nj) {
        std::ostringstream os;
        os << "shot " << k << ": " << what << " point (" << i << ", " << j << ") lies outside its grid";
        fail(SW_ERR_ARG, os.str());
      }
      if (stress_src && which == 0) {
        // nodes the stress update never writes would accumulate the source
        const bool top_fixed = !es->g.ft && j == 1;
        if (i == 1 || i == es->g.nx || j == es->g.nz || top_fixed) {
          std::ostringstream os;
          os << "shot " << k << ": source point (" << i << ", " << j
             << ") lies on a boundary stress node that is never updated (move the source inside)";
          fail(SW_ERR_UNSUPPORTED, os.str());
        }
      }
    }
  }
}

void validate_shot(const sw_elastic* es, const sw_elastic_shot& s, int k, bool grad) {
  std::ostringstream os;
  if (s.nt < 1) { os << "shot " << k << ": Number of timesteps must be positive!"; fail(SW_ERR_ARG, os.str()); }
  if (s.kind != 0 && s.kind != 1) { os << "shot " << k << ": unknown source kind"; fail(SW_ERR_ARG, os.str()); }
  if (s.nsrc < 1) fail(SW_ERR_ARG, "There must be at least one source!");
  if (s.nrec < 1) fail(SW_ERR_ARG, "There must be at least one receiver!");
  if (!s.srctf || !s.traces || !s.cpml) { os << "shot " << k << ": srctf, traces and cpml are required"; fail(SW_ERR_ARG, os.str()); }
  if (s.kind == 0 && !s.momtens) fail(SW_ERR_ARG, "Number of moment tensors must match number of sources!");
  validate_table(es, s.src[0], s.nsrc, s.kind == 0 ? 0 : 2, "source", k, s.kind == 0);
  validate_table(es, s.src[1], s.nsrc, s.kind == 0 ? 1 : 3, "source", k, s.kind == 0);
  validate_table(es, s.rec[0], s.nrec, 2, "receiver (ux)", k, false);
  validate_table(es, s.rec[1], s.nrec, 3, "receiver (uz)", k, false);
  if (grad) {
    if (!s.observed) { os << "shot " << k << ": observed traces are required"; fail(SW_ERR_ARG, os.str()); }
    if (es->gp.check_freq >= s.nt) fail(SW_ERR_ARG, "Checkpointing frequency must be smaller than the number of timesteps!");
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
    for (int w = 0; w < s.nwin; ++w) {
      const int a = s.windows[2 * w], b = s.windows[2 * w + 1];
      if (!(1 <= a && a <= b && b <= s.nt))
        fail(SW_ERR_ARG, "Windows indices must be between 1 and maximum number of timesteps!");
    }
  }
}

size_t per_shot_bytes(const sw_elastic* es, bool grad, int max_nt) {
  const size_t F = (size_t)es->g.F, strips = 4 * (size_t)(es->xs + es->zs);
  size_t b = (7 * F + strips) * sizeof(float);
  if (grad) {
    const int K = es->gp.check_freq;
    const int M = (max_nt + K - 1) / K;
    b += (7 * F + strips) * sizeof(float);                 // adjoint state
    b += (size_t)K * 4 * F * sizeof(float);                // slots
    b += (size_t)std::max(M - 1, 0) * (4 * F + 2 * strips) * sizeof(float);  // checkpoints
    b += (size_t)max_nt * 2 * 400 * sizeof(float) * 3;     // traces, observed, adjoint source (rough)
  }
  return b;
}

void ensure_state(sw_elastic* es, int S, bool grad, int max_nt, int ngroups) {
  const long long F = es->g.F;
  if (es->cap < S || (grad && !es->ast[0].p)) {
    for (int f = 0; f < 7; ++f) dev_alloc(es->st[f], (size_t)S * F * sizeof(float), "elastic fields", es->ctx->stream);
    for (int d = 0; d < 4; ++d) {
      dev_alloc(es->px[d], (size_t)S * es->xs * sizeof(float), "elastic memory variables", es->ctx->stream);
      dev_alloc(es->pz[d], (size_t)S * es->zs * sizeof(float), "elastic memory variables", es->ctx->stream);
    }
    if (grad) {
      for (int f = 0; f < 7; ++f)
        dev_alloc(es->ast[f], (size_t)S * F * sizeof(float), "adjoint fields", es->ctx->stream);
      for (int d = 0; d < 4; ++d) {
        dev_alloc(es->apx[d], (size_t)S * es->xs * sizeof(float), "adjoint memory variables", es->ctx->stream);
        dev_alloc(es->apz[d], (size_t)S * es->zs * sizeof(float), "adjoint memory variables", es->ctx->stream);
      }
    }
    es->cap = S;
    es->cap_slots = 0;
    es->cap_ck = 0;
    ++es->gen;
  }
  if (grad) {
    const int K = es->gp.check_freq;
    const int M = (max_nt + K - 1) / K;
    const size_t slot_b = (size_t)K * 4 * es->cap * F * sizeof(float);
    if (es->slots.bytes < slot_b) { dev_alloc(es->slots, slot_b, "gradient slots", es->ctx->stream); ++es->gen; }
    // per checkpoint: u, du (4 fields) and the 8 memory-variable strips of every shot
    const size_t ck_b = (size_t)std::max(M - 1, 1) * (4 * (size_t)es->cap * F + 4 * (size_t)es->cap * (es->xs + es->zs)) *
                        sizeof(float);
    if (es->ck.bytes < ck_b) { dev_alloc(es->ck, ck_b, "checkpoints", es->ctx->stream); ++es->gen; }
    const size_t acc_b = (size_t)ngroups * 10 * F * sizeof(float);
    if (es->acc.bytes < acc_b) { dev_alloc(es->acc, acc_b, "gradient accumulators", es->ctx->stream); ++es->gen; }
  }
}

struct InjBuild {
  std::vector<long long> lin;
  std::vector<int> ptr, item;
  std::vector<float> coef;
};

// unique-point CSR of a table (points summed over its items)
InjBuild build_inj(const sw_elastic* es, const sw_point_table& t, int count) {
  std::map<long long, std::vector<std::pair<int, float>>> pts;
  std::vector<long long> order;
  for (int k = 0; k < count; ++k)
    for (int p = t.offsets[k]; p < t.offsets[k + 1]; ++p) {
      const long long c = es->g.lin(t.ij[2 * p], t.ij[2 * p + 1]);
      auto it = pts.find(c);
      if (it == pts.end()) {
        order.push_back(c);
        pts[c] = {};
      }
      pts[c].push_back({k, t.coef[p]});
    }
  InjBuild b;
  b.ptr.push_back(0);
  for (long long c : order) {
    b.lin.push_back(c);
    for (auto& e : pts[c]) {
      b.item.push_back(e.first);
      b.coef.push_back(e.second);
    }
    b.ptr.push_back((int)b.item.size());
  }
  return b;
}

// Everything is concatenated into three typed pools; the descriptors carry
// offsets that are turned into device pointers after the upload.
struct Pools {
  std::vector<long long> ll;
  std::vector<int> in;
  std::vector<float> fl;
  template <typename T>
  static size_t put(std::vector<T>& pool, const std::vector<T>& v) {
    const size_t off = pool.size();
    pool.insert(pool.end(), v.begin(), v.end());
    while (pool.size() % 4) pool.push_back(T(0));
    return off;
  }
};

struct DescOff {
  size_t src_lin[2], src_ptr[2], src_item[2], src_coef[2];
  int src_np[2];
  size_t adj_lin[2], adj_ptr[2], adj_item[2], adj_coef[2];
  int adj_np[2];
  size_t rptr[2], rlin[2], rcoef[2];
  size_t mt, mask;
  bool has_mask;
};

void build_tables(sw_elastic* es, const sw_elastic_shot* shots, const std::vector<HostShot>& group, bool on_device,
                  bool grad, std::vector<ShotDesc>& desc) {
  cudaStream_t st = es->ctx->stream;
  const int S = (int)group.size();
  Pools P;
  std::vector<DescOff> offs(S);
  long long tf_total = 0, tr_total = 0;
  std::vector<long long> tf_off(S), tr_off(S);
  for (int k = 0; k < S; ++k) {
    const sw_elastic_shot& s = shots[group[k].orig];
    tf_off[k] = tf_total;
    tf_total += round_up((long long)s.nt * s.nsrc * (s.kind == 1 ? 2 : 1), 4);
    tr_off[k] = tr_total;
    tr_total += round_up((long long)s.nt * 2 * s.nrec, 4);
  }
  for (int k = 0; k < S; ++k) {
    const sw_elastic_shot& s = shots[group[k].orig];
    DescOff& o = offs[k];
    for (int t = 0; t < 2; ++t) {
      InjBuild b = build_inj(es, s.src[t], s.nsrc);
      o.src_np[t] = (int)b.lin.size();
      o.src_lin[t] = Pools::put(P.ll, b.lin);
      o.src_ptr[t] = Pools::put(P.in, b.ptr);
      o.src_item[t] = Pools::put(P.in, b.item);
      o.src_coef[t] = Pools::put(P.fl, b.coef);
      InjBuild a = build_inj(es, s.rec[t], s.nrec);
      o.adj_np[t] = (int)a.lin.size();
      o.adj_lin[t] = Pools::put(P.ll, a.lin);
      o.adj_ptr[t] = Pools::put(P.in, a.ptr);
      o.adj_item[t] = Pools::put(P.in, a.item);
      o.adj_coef[t] = Pools::put(P.fl, a.coef);
      std::vector<int> rp(s.rec[t].offsets, s.rec[t].offsets + s.nrec + 1);
      std::vector<long long> rl;
      std::vector<float> rc;
      for (int e = 0; e < rp[s.nrec]; ++e) {
        rl.push_back(es->g.lin(s.rec[t].ij[2 * e], s.rec[t].ij[2 * e + 1]));
        rc.push_back(s.rec[t].coef[e]);
      }
      o.rptr[t] = Pools::put(P.in, rp);
      o.rlin[t] = Pools::put(P.ll, rl);
      o.rcoef[t] = Pools::put(P.fl, rc);
    }
    std::vector<float> mt(3 * (size_t)s.nsrc, 0.0f);
    if (s.kind == 0) std::copy(s.momtens, s.momtens + 3 * s.nsrc, mt.begin());
    o.mt = Pools::put(P.fl, mt);
    o.has_mask = grad && s.nwin > 0;
    if (o.has_mask) {
      std::vector<float> mask(s.nt, 0.0f);
      for (int w = 0; w < s.nwin; ++w)
        for (int t = s.windows[2 * w] - 1; t <= s.windows[2 * w + 1] - 1; ++t) mask[t] = 1.0f;
      o.mask = Pools::put(P.fl, mask);
    }
  }
  upload(es, es->d_ll, P.ll, "elastic tables");
  upload(es, es->d_int, P.in, "elastic tables");
  upload(es, es->d_flt, P.fl, "elastic tables");
  // bulk per-shot arrays
  ensure(es, es->d_tf, (size_t)tf_total * sizeof(float), "source time functions");
  ensure(es, es->d_tr, (size_t)tr_total * sizeof(float), "traces");
  if (grad) {
    ensure(es, es->d_obs, (size_t)tr_total * sizeof(float), "observed traces");
    ensure(es, es->d_adj, (size_t)tr_total * sizeof(float), "adjoint sources");
  }
  long long icd_total = 0, dres_total = 0;
  for (int k = 0; k < S; ++k) {
    const sw_elastic_shot& s = shots[group[k].orig];
    if (grad && s.invcov) {
      icd_total += (long long)s.nt * s.nt;
      dres_total += (long long)s.nt * 2 * s.nrec;
    }
  }
  if (dres_total) {
    if (!on_device) ensure(es, es->d_icd, icd_total * sizeof(float), "dense inverse covariance");
    ensure(es, es->d_dres, 2 * dres_total * sizeof(float), "dense residuals");
  }
  long long ic_total = 0;
  std::vector<long long> ic_off(S, -1);
  for (int k = 0; k < S; ++k) {
    const sw_elastic_shot& s = shots[group[k].orig];
    if (grad && s.invcov_diag) {
      ic_off[k] = ic_total;
      ic_total += round_up(s.nt, 4);
    }
  }
  if (ic_total) ensure(es, es->d_ic, (size_t)ic_total * sizeof(float), "inverse covariance");
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  std::vector<float> cps(S * (size_t)es->cps);
  for (int k = 0; k < S; ++k) {
    const sw_elastic_shot& s = shots[group[k].orig];
    const long long ntf = (long long)s.nt * s.nsrc * (s.kind == 1 ? 2 : 1);
    check_cuda(cudaMemcpyAsync(es->d_tf.as<float>() + tf_off[k], s.srctf, ntf * sizeof(float), kind, st), "srctf upload");
    if (grad) {
      check_cuda(cudaMemcpyAsync(es->d_obs.as<float>() + tr_off[k], s.observed, (size_t)s.nt * 2 * s.nrec * sizeof(float),
                                 kind, st), "observed upload");
      if (s.invcov_diag)
        check_cuda(cudaMemcpyAsync(es->d_ic.as<float>() + ic_off[k], s.invcov_diag, s.nt * sizeof(float), kind, st),
                   "invcov upload");
    }
    std::copy(s.cpml, s.cpml + es->cps, cps.begin() + (size_t)k * es->cps);
  }
  upload(es, es->d_cp, cps, "C-PML coefficients");
  check_cuda(cudaMemsetAsync(es->d_tr.p, 0, (size_t)tr_total * sizeof(float), st), "traces clear");
  const long long* LL = es->d_ll.as<long long>();
  const int* IN = es->d_int.as<int>();
  const float* FL = es->d_flt.as<float>();
  desc.assign(S, ShotDesc{});
  for (int k = 0; k < S; ++k) {
    const sw_elastic_shot& s = shots[group[k].orig];
    const DescOff& o = offs[k];
    ShotDesc& D = desc[k];
    D.nt = s.nt;
    D.kind = s.kind;
    D.nsrc = s.nsrc;
    D.nrec = s.nrec;
    D.tf = es->d_tf.as<float>() + tf_off[k];
    D.mtp = FL + o.mt;
    for (int t = 0; t < 2; ++t) {
      D.src[t] = Inj{o.src_np[t], LL + o.src_lin[t], IN + o.src_ptr[t], IN + o.src_item[t], FL + o.src_coef[t]};
      D.adj[t] = Inj{o.adj_np[t], LL + o.adj_lin[t], IN + o.adj_ptr[t], IN + o.adj_item[t], FL + o.adj_coef[t]};
      D.rptr[t] = IN + o.rptr[t];
      D.rlin[t] = LL + o.rlin[t];
      D.rcoef[t] = FL + o.rcoef[t];
    }
    D.tr = es->d_tr.as<float>() + tr_off[k];
    D.obs = grad ? es->d_obs.as<float>() + tr_off[k] : nullptr;
    D.ic = (grad && s.invcov_diag) ? es->d_ic.as<float>() + ic_off[k] : nullptr;
    D.mask = o.has_mask ? FL + o.mask : nullptr;
    D.adjsrc = grad ? es->d_adj.as<float>() + tr_off[k] : nullptr;
    D.mkind = grad ? s.misfit_kind : 0;
  }
  long long icd_o = 0, dres_o = 0;
  for (int k = 0; k < S; ++k) {
    const sw_elastic_shot& s = shots[group[k].orig];
    if (!(grad && s.invcov)) continue;
    ShotDesc& D = desc[k];
    if (on_device) {
      D.icd = s.invcov;
    } else {
      float* cp = es->d_icd.as<float>() + icd_o;
      check_cuda(cudaMemcpyAsync(cp, s.invcov, (size_t)s.nt * s.nt * sizeof(float), cudaMemcpyHostToDevice, st),
                 "invcov upload");
      D.icd = cp;
      icd_o += (long long)s.nt * s.nt;
    }
    D.resid = es->d_dres.as<float>() + dres_o;
    D.cres = es->d_dres.as<float>() + dres_total + dres_o;
    dres_o += (long long)s.nt * 2 * s.nrec;
  }
  upload(es, es->d_desc, desc, "shot descriptors");
}

void download_traces(sw_elastic* es, const sw_elastic_shot* shots, const std::vector<HostShot>& group,
                     const std::vector<ShotDesc>& desc, bool on_device) {
  for (size_t k = 0; k < group.size(); ++k) {
    const sw_elastic_shot& s = shots[group[k].orig];
    check_cuda(cudaMemcpyAsync(s.traces, desc[k].tr, (size_t)s.nt * 2 * s.nrec * sizeof(float),
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, es->ctx->stream),
               "traces download");
  }
}

int active_count(const std::vector<HostShot>& g, int it) {
  int a = 0;
  while (a < (int)g.size() && g[a].nt >= it) ++a;
  return a;
}

// power of two 2^e with 2^e * vmax close to 2^20 (1 for vmax == 0)
float pow2_scale(float vmax) {
  if (!(vmax > 0.0f) || !std::isfinite(vmax)) return 1.0f;
  const int e = 20 - (int)std::lround(std::log2((double)vmax));
  return std::ldexp(1.0f, std::max(-100, std::min(100, e)));
}

float device_absmax(sw_elastic* es, const float* v, long long n) {
  cudaStream_t st = es->ctx->stream;
  ensure(es, es->d_amax, 16, "max reduction");
  check_cuda(cudaMemsetAsync(es->d_amax.p, 0, sizeof(unsigned), st), "max clear");
  if (n > 0) {
    const int blocks = (int)std::min<long long>((n + 255) / 256, 1024);
    k_el_absmax<<<blocks, 256, 0, st>>>(v, n, es->d_amax.as<unsigned>());
    check_cuda(cudaGetLastError(), "max launch");
  }
  unsigned bits = 0;
  check_cuda(cudaMemcpyAsync(&bits, es->d_amax.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "max download");
  check_cuda(cudaStreamSynchronize(st), "max");
  float f;
  std::memcpy(&f, &bits, sizeof(float));
  return f;
}

struct Run {
  sw_elastic* es;
  cudaStream_t st;
  const ShotDesc* ddesc;
  float sf_ref = 1.0f;  // the largest source scale of the group (the gradient's common scale)
  bool any_mt = true, any_force = true;  // source kinds present in the group (skip empty launches)
  // blocks per shot of the source / adjoint-source / recording kernels: one
  // thread per unique point (or receiver component) of the largest table
  int gx_src = 1, gx_adj = 1, gx_rec = 1;
  void size_grids(const std::vector<ShotDesc>& desc) {
    int ns = 1, na = 1, nr = 1;
    for (const auto& d : desc) {
      for (int t = 0; t < 2; ++t) {
        ns = std::max(ns, d.src[t].np);
        na = std::max(na, d.adj[t].np);
      }
      nr = std::max(nr, 2 * d.nrec);
    }
    gx_src = (ns + 127) / 128;
    gx_adj = (na + 127) / 128;
    gx_rec = (nr + 255) / 256;
  }

  Args args(bool adjoint) const {
    Args a{};
    a.g = es->g;
    DevMem* f = adjoint ? es->ast : es->st;
    a.ux = f[0].as<float>(); a.uz = f[1].as<float>(); a.dux = f[2].as<float>(); a.duz = f[3].as<float>();
    a.sxx = f[4].as<float>(); a.szz = f[5].as<float>(); a.sxz = f[6].as<float>();
    for (int d = 0; d < 4; ++d) {
      a.px[d] = (adjoint ? es->apx : es->px)[d].as<float>();
      a.pz[d] = (adjoint ? es->apz : es->pz)[d].as<float>();
    }
    a.xs = es->xs;
    a.zs = es->zs;
    a.lam = es->lam.as<float>(); a.mu = es->mu.as<float>();
    a.dtr_i = es->dtr_i.as<float>(); a.dtr_j = es->dtr_j.as<float>(); a.mu_ij = es->mu_ij.as<float>();
    a.cp = es->d_cp.as<float>();
    a.cps = es->cps;
    return a;
  }
  // algorithmic bytes of one step (stress + displacement kernels): per point and
  // shot, stress R ux uz (8) W sigma x3 (12), displacement R sigma x3 (12),
  // R/W u, du (32), slots W u[it-1], D (16); shared material 20 (lambda, mu,
  // mu_ij, dt^2/rho on both half grids)
  double step_bytes(int S, bool slots) const {
    const double pts = (double)es->g.nx * es->g.nz;
    return pts * (S * (64.0 + (slots ? 16.0 : 0.0)) + 20.0);
  }
  void inject_sigma(int S, int it) {
    if (S <= 0) return;
    DevMem* f = es->st;
    cudaEvent_t ev = nullptr;
    es->ctx->prof.begin(st, KK_SRCREC, 0.0, &ev);
    k_el_inject_sigma<<<dim3(gx_src, S), 128, 0, st>>>(ddesc, it, es->g.F, f[4].as<float>(), f[5].as<float>(),
                                                  f[6].as<float>());
    check_cuda(cudaGetLastError(), "stress injection launch");
    es->ctx->prof.end(st, KK_SRCREC, ev);
  }
  void inject_force(int S, int it, bool adjoint, const float* adj_scale, float* sD[2]) {
    if (S <= 0) return;
    DevMem* f = adjoint ? es->ast : es->st;
    cudaEvent_t ev = nullptr;
    es->ctx->prof.begin(st, KK_SRCREC, 0.0, &ev);
    k_el_inject_force<<<dim3(adjoint ? gx_adj : gx_src, S), 128, 0, st>>>(ddesc, it, adjoint ? 1 : 0, adj_scale,
                                                                         es->g.F,
                                                                         f[0].as<float>(),
                                                  f[1].as<float>(), f[2].as<float>(), f[3].as<float>(),
                                                  sD ? sD[0] : nullptr, sD ? sD[1] : nullptr, es->dtr_i.as<float>(),
                                                  es->dtr_j.as<float>());
    check_cuda(cudaGetLastError(), "force injection launch");
    es->ctx->prof.end(st, KK_SRCREC, ev);
  }
  void record(int S, int it) {
    if (S <= 0) return;
    cudaEvent_t ev = nullptr;
    es->ctx->prof.begin(st, KK_SRCREC, 0.0, &ev);
    k_el_record<<<dim3(gx_rec, S), 256, 0, st>>>(ddesc, it, es->g.F, es->st[0].as<float>(), es->st[1].as<float>());
    check_cuda(cudaGetLastError(), "record launch");
    es->ctx->prof.end(st, KK_SRCREC, ev);
  }
};

void zero_state(sw_elastic* es, int S, bool adjoint) {
  cudaStream_t st = es->ctx->stream;
  DevMem* f = adjoint ? es->ast : es->st;
  for (int k = 0; k < 7; ++k)
    check_cuda(cudaMemsetAsync(f[k].p, 0, (size_t)S * es->g.F * sizeof(float), st), "state clear");
  for (int d = 0; d < 4; ++d) {
    check_cuda(cudaMemsetAsync((adjoint ? es->apx : es->px)[d].p, 0, (size_t)S * es->xs * sizeof(float), st), "psi clear");
    check_cuda(cudaMemsetAsync((adjoint ? es->apz : es->pz)[d].p, 0, (size_t)S * es->zs * sizeof(float), st), "psi clear");
  }
}

template <int TZ>
// returns the number of kernels launched
int launch_stencil_tz(const sw_elastic* es, cudaStream_t st, const Args& a, int S, bool stress) {
  int nk = 1;
  if (es->vec) {  // four points per thread: 512 per block
    const dim3 grid((es->g.nx + 511) / 512, (es->g.nz + TZ - 1) / TZ, S);
    if (stress) {
      k_el_stress4<TZ><<<grid, BX, 0, st>>>(a);
    } else if (es->split_disp) {  // ux and uz updates as two launches
      k_el_disp4<TZ, 0><<<grid, BX, 0, st>>>(a);
      k_el_disp4<TZ, 1><<<grid, BX, 0, st>>>(a);
      nk = 2;
    } else {
      k_el_disp4<TZ><<<grid, BX, 0, st>>>(a);
    }
  } else {
    const dim3 grid((es->g.nx + BX - 1) / BX, (es->g.nz + TZ - 1) / TZ, S);
    if (stress) k_el_stress<TZ><<<grid, BX, 0, st>>>(a);
    else k_el_disp<TZ><<<grid, BX, 0, st>>>(a);
  }
  check_cuda(cudaGetLastError(), stress ? "stress launch" : "displacement launch");
  return nk;
}

int launch_stencil(const sw_elastic* es, cudaStream_t st, const Args& a, int S, bool stress) {
  if (es->tz == 16) return launch_stencil_tz<16>(es, st, a, S, stress);
  if (es->tz == 32) return launch_stencil_tz<32>(es, st, a, S, stress);
  return launch_stencil_tz<8>(es, st, a, S, stress);
}

// stress, [sigma sources], displacement, [force sources], [recording]
void full_step(Run& R, int S, int it, bool record, int kind, float* sU[2], float* sD[2]) {
  if (S <= 0) return;
  sw_elastic* es = R.es;
  Args a = R.args(false);
  if (sU) { a.sUx = sU[0]; a.sUz = sU[1]; a.sDx = sD[0]; a.sDz = sD[1]; }
  cudaEvent_t ev = nullptr;
  es->ctx->prof.begin(R.st, kind, 0.0, &ev);
  launch_stencil(es, R.st, a, S, true);
  es->ctx->prof.end(R.st, kind, ev);
  if (R.any_mt) R.inject_sigma(S, it);
  es->ctx->prof.begin(R.st, kind, R.step_bytes(S, sU != nullptr), &ev);
  const int nk = launch_stencil(es, R.st, a, S, false);
  es->ctx->prof.end(R.st, kind, ev, nk);
  if (R.any_force) R.inject_force(S, it, false, nullptr, sD);
  if (record) R.record(S, it);
}

void adjoint_step(Run& R, int S, int it) {
  if (S <= 0) return;
  sw_elastic* es = R.es;
  Args a = R.args(true);
  cudaEvent_t ev = nullptr;
  es->ctx->prof.begin(R.st, KK_ADJOINT, R.step_bytes(S, false), &ev);
  int nk = launch_stencil(es, R.st, a, S, true);
  nk += launch_stencil(es, R.st, a, S, false);
  es->ctx->prof.end(R.st, KK_ADJOINT, ev, nk);
  R.inject_force(S, it, true, es->d_scales.as<float>() + 1, nullptr);
}

// savesnapshot!("ucur" => ..., "σ" => ...) of ela_forward.jl:74-78 for the active shots:
// one block per snapshot, [ux (nx-1, nz), uz (nx, nz-1), sxx, szz (nx, nz), sxz (nx-1, nz-1)].
long long snapshot_floats(const sw_elastic* es) {
  const long long nx = es->g.nx, nz = es->g.nz;
  return (nx - 1) * nz + nx * (nz - 1) + 2 * nx * nz + (nx - 1) * (nz - 1);
}

void save_snapshots(sw_elastic* es, const std::vector<HostShot>& group, int A, int it) {
  const long long B = snapshot_floats(es);
  cudaStream_t st = es->ctx->stream;
  ensure(es, es->d_snap, (size_t)es->cap * B * sizeof(float), "snapshot stage");
  const dim3 grid((unsigned)std::min<long long>((B + 255) / 256, 1024), A);
  k_el_snapshot<<<grid, 256, 0, st>>>(es->g, es->d_desc.as<ShotDesc>(), es->st[0].as<float>(), es->st[1].as<float>(),
                                      es->st[4].as<float>(), es->st[5].as<float>(), es->st[6].as<float>(), B,
                                      es->d_snap.as<float>());
  check_cuda(cudaGetLastError(), "snapshot launch");
  for (int k = 0; k < A; ++k) {
    float* dst = es->snap_out[group[k].orig] + (long long)(it / es->snapevery - 1) * B;
    check_cuda(cudaMemcpyAsync(dst, es->d_snap.as<float>() + (long long)k * B, (size_t)B * sizeof(float),
                               cudaMemcpyDefault, st),
               "snapshot copy");
  }
}

std::vector<HostShot> sorted_order(int nshots, const sw_elastic_shot* shots) {
  std::vector<HostShot> order(nshots);
  for (int k = 0; k < nshots; ++k) order[k] = HostShot{k, shots[k].nt};
  std::stable_sort(order.begin(), order.end(), [](const HostShot& a, const HostShot& b) { return a.nt > b.nt; });
  return order;
}

std::vector<std::vector<HostShot>> plan_groups(sw_elastic* es, const std::vector<HostShot>& order, bool grad) {
  size_t free_b = 0, total_b = 0;
  check_cuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
  size_t owned = es->slots.bytes + es->ck.bytes + es->acc.bytes;
  for (int f = 0; f < 7; ++f) owned += es->st[f].bytes + es->ast[f].bytes;
  for (int d = 0; d < 4; ++d) owned += es->px[d].bytes + es->pz[d].bytes + es->apx[d].bytes + es->apz[d].bytes;
  const double budget = 0.85 * (double)(free_b + owned);
  std::vector<std::vector<HostShot>> groups;
  size_t i = 0;
  while (i < order.size()) {
    const size_t per = per_shot_bytes(es, grad, order[i].nt);
    size_t cnt = (size_t)std::max(1.0, std::floor(budget / (double)per));
    cnt = std::min(cnt, order.size() - i);
    groups.emplace_back(order.begin() + i, order.begin() + i + cnt);
    i += cnt;
  }
  return groups;
}

// Per-shot source scales from each shot's largest |tf| (times |M| for moment
// tensors): a shot's fields do not depend on the other shots of the batch.
// Returns the largest scale; the gradient correlation brings every shot to it
// (cs = largest / own, a power of two).
float set_forward_scales(sw_elastic* es, const sw_elastic_shot* shots, const std::vector<HostShot>& group,
                         std::vector<ShotDesc>& desc) {
  float ref = 0.0f;
  for (size_t k = 0; k < group.size(); ++k) {
    const sw_elastic_shot& s = shots[group[k].orig];
    const long long n = (long long)s.nt * s.nsrc * (s.kind == 1 ? 2 : 1);
    float m = device_absmax(es, desc[k].tf, n);
    if (s.kind == 0) {
      float mm = 0.0f;
      for (int q = 0; q < 3 * s.nsrc; ++q) mm = std::max(mm, std::fabs(s.momtens[q]));
      m *= mm;
    }
    desc[k].sf = pow2_scale(m);
    ref = std::max(ref, desc[k].sf);
  }
  std::vector<float> cs(group.size());
  for (size_t k = 0; k < group.size(); ++k) cs[k] = ref / desc[k].sf;
  upload(es, es->d_desc, desc, "shot descriptors");
  upload(es, es->d_cs, cs, "shot scales");
  return ref;
}

}  // namespace

// ---------------------------------------------------------------------------
// Entry points used by api.cu
// ---------------------------------------------------------------------------
namespace swgb {

void elastic_init(sw_elastic* es, sw_ctx* ctx, const sw_elastic_params* p, int gradient, const sw_grad_params* gp) {
  if (!p) fail(SW_ERR_ARG, "params is NULL");
  if (p->halo < 0) fail(SW_ERR_ARG, "CPML halo size must be non-negative!");
  if (!(p->dt > 0)) fail(SW_ERR_ARG, "Timestep size must be positive!");
  for (int d = 0; d < 2; ++d) {
    if (p->n[d] <= 0) fail(SW_ERR_ARG, "All numbers of grid points must be positive!");
    if (!(p->h[d] > 0)) fail(SW_ERR_ARG, "All grid spacings must be positive!");
  }
  for (int d = 0; d < 2; ++d) {
    const bool cpml_axis = !(p->freetop && d == 1);
    if (p->n[d] < 2 * p->halo + 3) {
      std::ostringstream os;
      if (cpml_axis) {
        os << "Number grid points in the dimensions with C-PML boundaries must be at least 2*halo+3 = "
           << 2 * p->halo + 3 << "!";
        fail(SW_ERR_ARG, os.str());
      }
      os << "the free-surface axis needs at least 2*halo+3 = " << 2 * p->halo + 3
         << " grid points in this backend (its two damping strips must not overlap)";
      fail(SW_ERR_UNSUPPORTED, os.str());
    }
    if (p->n[d] < 5) fail(SW_ERR_UNSUPPORTED, "the 4th-order elastic stencil needs at least 5 points per axis");
  }
  if (p->interp_rho < 0 || p->interp_rho > 1 || p->interp_mu < 0 || p->interp_mu > 1)
    fail(SW_ERR_ARG, "interpolation method must be 0 (arithmetic) or 1 (harmonic)");
  es->ctx = ctx;
  es->prm = *p;
  es->gradient = gradient != 0;
  if (es->gradient) {
    es->gp = gp ? *gp : sw_grad_params{1, 0, 0, 0, 0};
    if (es->gp.check_freq < 1) fail(SW_ERR_ARG, "check_freq must be positive");
    if (es->gp.mute_radius_src < 0 || es->gp.mute_radius_rec < 0)
      fail(SW_ERR_ARG, "mutearoundpoint!(): The smoothing radius must be positive.");
    if (es->gp.snapshot_bf16) fail(SW_ERR_UNSUPPORTED, "BF16 checkpoint snapshots are not available for the elastic path");
  }
  Geo& g = es->g;
  g.nx = p->n[0];
  g.nz = p->n[1];
  g.halo = p->halo;
  g.ft = p->freetop ? 1 : 0;
  g.P = (int)round_up(g.nx + XPAD + 8, 32);  // the vector kernels read up to column nx + 36
  g.F = (long long)g.P * (g.nz + 2 * ZPAD);
  g.W = (int)round_up(2 * g.halo + 3, 4);
  g.idx = (float)(1.0 / p->h[0]);
  g.idz = (float)(1.0 / p->h[1]);
  es->na = 2 * g.halo + 2;
  es->nh = 2 * g.halo;
  es->cps = 2 * (2 * es->na + 2 * es->nh);
  es->xs = round_up((long long)g.nz * g.W, 32);
  es->zs = round_up((long long)(2 * g.halo + 3) * g.P, 32);
  const size_t F = (size_t)g.F;
  for (DevMem* m : {&es->lam, &es->mu, &es->dtr_i, &es->dtr_j, &es->mu_ij})
    dev_alloc(*m, F * sizeof(float), "elastic material", ctx->stream);
  dev_alloc(es->rho_d, (size_t)g.nx * g.nz * sizeof(double), "density", ctx->stream);
  dev_alloc(es->mu_d, (size_t)g.nx * g.nz * sizeof(double), "shear modulus", ctx->stream);
}

void elastic_set_material(sw_elastic* es, const float* lam, const float* mu, const float* rho) {
  if (!lam || !mu || !rho) fail(SW_ERR_ARG, "lambda, mu and rho are required");
  const Geo& g = es->g;
  const long long np = (long long)g.nx * g.nz;
  for (long long c = 0; c < np; ++c) {
    if (!(lam[c] >= 0)) fail(SW_ERR_ARG, "Lamè coefficient λ must be positive!");
    if (!(mu[c] >= 0)) fail(SW_ERR_ARG, "Lamè coefficient μ must be positive!");
    if (!(rho[c] > 0)) fail(SW_ERR_ARG, "Density must be positive!");
  }
  auto M = [&](int i, int j) { return (size_t)(i - 1) + (size_t)(j - 1) * g.nx; };
  std::vector<float> L(g.F, 0.0f), U(g.F, 0.0f), Ri(g.F, 0.0f), Rj(g.F, 0.0f), Uij(g.F, 0.0f);
  std::vector<double> rd(np), md(np);
  const double dt2 = es->prm.dt * es->prm.dt;
  double vmax = 0.0;
  auto avg = [&](const float* m, int i, int j, int di, int dj, int method) {
    double s = 0;
    int n = 0;
    for (int b = 0; b <= dj; ++b)
      for (int a = 0; a <= di; ++a) {
        const double v = m[M(i + a, j + b)];
        s += method == 1 ? 1.0 / v : v;
        ++n;
      }
    s /= n;
    return method == 1 ? 1.0 / s : s;
  };
  for (int j = 1; j <= g.nz; ++j)
    for (int i = 1; i <= g.nx; ++i) {
      const size_t c = M(i, j);
      const long long q = g.lin(i, j);
      L[q] = lam[c];
      U[q] = mu[c];
      rd[c] = rho[c];
      md[c] = mu[c];
      vmax = std::max(vmax, std::sqrt(((double)lam[c] + 2.0 * mu[c]) / rho[c]));
      if (i <= g.nx - 1) Ri[q] = (float)(dt2 / avg(rho, i, j, 1, 0, es->prm.interp_rho));
      if (j <= g.nz - 1) Rj[q] = (float)(dt2 / avg(rho, i, j, 0, 1, es->prm.interp_rho));
      if (i <= g.nx - 1 && j <= g.nz - 1) Uij[q] = (float)avg(mu, i, j, 1, 1, es->prm.interp_mu);
    }
  cudaStream_t st = es->ctx->stream;
  auto up = [&](DevMem& m, const void* src, size_t bytes) {
    check_cuda(cudaMemcpyAsync(m.p, src, bytes, cudaMemcpyHostToDevice, st), "material upload");
  };
  up(es->lam, L.data(), L.size() * sizeof(float));
  up(es->mu, U.data(), U.size() * sizeof(float));
  up(es->dtr_i, Ri.data(), Ri.size() * sizeof(float));
  up(es->dtr_j, Rj.data(), Rj.size() * sizeof(float));
  up(es->mu_ij, Uij.data(), Uij.size() * sizeof(float));
  up(es->rho_d, rd.data(), rd.size() * sizeof(double));
  up(es->mu_d, md.data(), md.size() * sizeof(double));
  check_cuda(cudaStreamSynchronize(st), "material upload");
  es->vel_max = vmax;
  es->has_mat = true;
}

void elastic_forward(sw_elastic* es, int nshots, const sw_elastic_shot* shots, bool on_device) {
  if (!es->has_mat) fail(SW_ERR_STATE, "material properties not set (sw_elastic_set_material)");
  if (nshots < 1 || !shots) fail(SW_ERR_ARG, "no shots");
  for (int k = 0; k < nshots; ++k) validate_shot(es, shots[k], k, false);
  const std::vector<HostShot> order = sorted_order(nshots, shots);
  for (const auto& group : plan_groups(es, order, false)) {
    const int S = (int)group.size();
    ensure_state(es, S, false, group.front().nt, 1);
    std::vector<ShotDesc> desc;
    build_tables(es, shots, group, on_device, false, desc);
    const float sf_ref = set_forward_scales(es, shots, group, desc);
    Run R{es, es->ctx->stream, es->d_desc.as<ShotDesc>(), sf_ref};
    R.size_grids(desc);
    R.any_mt = R.any_force = false;
    for (const auto& h : group) (shots[h.orig].kind == 0 ? R.any_mt : R.any_force) = true;
    zero_state(es, S, false);
    for (int it = 1; it <= group.front().nt; ++it) {
      const int A = active_count(group, it);
      full_step(R, A, it, true, KK_STENCIL, nullptr, nullptr);
      if (es->snapevery > 0 && it % es->snapevery == 0) save_snapshots(es, group, A, it);
    }
    download_traces(es, shots, group, desc, on_device);
  }
  check_cuda(cudaStreamSynchronize(es->ctx->stream), "elastic forward");
  es->ctx->prof.resolve();
}

void elastic_forward_snapshots(sw_elastic* es, int nshots, const sw_elastic_shot* shots, bool on_device,
                               int snapevery, float* const* snapshots) {
  if (snapevery < 1 || !snapshots) fail(SW_ERR_ARG, "snapevery must be positive and snapshots non-NULL");
  for (int k = 0; k < nshots; ++k) {
    if (shots && snapevery >= shots[k].nt)
      fail(SW_ERR_ARG, "Checkpointing frequency must be smaller than the number of timesteps!");
    if (!snapshots[k]) fail(SW_ERR_ARG, "snapshot buffer is NULL");
  }
  es->snapevery = snapevery;
  es->snap_out = snapshots;
  try {
    elastic_forward(es, nshots, shots, on_device);
  } catch (...) {
    es->snapevery = 0;
    es->snap_out = nullptr;
    throw;
  }
  es->snapevery = 0;
  es->snap_out = nullptr;
}

void elastic_gradient(sw_elastic* es, int nshots, const sw_elastic_shot* shots, bool on_device, double* g_rho,
                      double* g_lam, double* g_mu, double* misfit) {
  if (!es->gradient) fail(SW_ERR_STATE, "The wavesim object was not built for gradient computations. (Was `gradient=true` specified?)");
  if (!es->has_mat) fail(SW_ERR_STATE, "material properties not set (sw_elastic_set_material)");
  if (nshots < 1 || !shots) fail(SW_ERR_ARG, "no shots");
  if (!g_rho || !g_lam || !g_mu) fail(SW_ERR_ARG, "gradient outputs are NULL");
  for (int k = 0; k < nshots; ++k) validate_shot(es, shots[k], k, true);
  const bool mute = es->gp.mute_radius_src > 0 || es->gp.mute_radius_rec > 0;
  if (mute)
    for (int k = 0; k < nshots; ++k) {
      const sw_elastic_shot& s = shots[k];
      if ((es->gp.mute_radius_src > 0 && !s.src_pos) || (es->gp.mute_radius_rec > 0 && !s.rec_pos))
        fail(SW_ERR_ARG, "muting needs src_pos / rec_pos");
    }
  cudaStream_t st = es->ctx->stream;
  const Geo& g = es->g;
  const long long np = (long long)g.nx * g.nz;
  const int K = es->gp.check_freq;
  double* out[3] = {g_rho, g_lam, g_mu};
  double* mout = misfit;
  if (!on_device) {
    ensure(es, es->d_gout, (size_t)3 * np * sizeof(double), "gradient output");
    for (int q = 0; q < 3; ++q) out[q] = es->d_gout.as<double>() + q * np;
  }
  if (!on_device || !mout) {
    ensure(es, es->d_mout, sizeof(double), "misfit output");
    mout = es->d_mout.as<double>();
  }
  const std::vector<HostShot> order = sorted_order(nshots, shots);
  bool first_group = true;
  for (const auto& group : plan_groups(es, order, true)) {
    const int S = (int)group.size();
    const int ntmax = group.front().nt;
    const int gsize = mute ? 1 : S;
    const int ngroups = (S + gsize - 1) / gsize;
    ensure_state(es, S, true, ntmax, ngroups);
    std::vector<ShotDesc> desc;
    build_tables(es, shots, group, on_device, true, desc);
    const float sf_ref = set_forward_scales(es, shots, group, desc);
    Run R{es, st, es->d_desc.as<ShotDesc>(), sf_ref};
    R.size_grids(desc);
    R.any_mt = R.any_force = false;
    for (const auto& h : group) (shots[h.orig].kind == 0 ? R.any_mt : R.any_force) = true;
    const long long F = g.F;
    const int cap = es->cap;
    float* slots = es->slots.as<float>();
    auto slot_ptrs = [&](int k, float* sU[2], float* sD[2]) {
      float* base = slots + (size_t)k * 4 * cap * F;
      sU[0] = base;
      sU[1] = base + (size_t)cap * F;
      sD[0] = base + (size_t)2 * cap * F;
      sD[1] = base + (size_t)3 * cap * F;
    };
    const int M = (ntmax + K - 1) / K;  // windows (m = 0 .. M-1), window m = steps mK+1 .. min((m+1)K, ntmax)
    const size_t ckF = (size_t)4 * cap * F;
    const size_t ckP = (size_t)cap * (es->xs + es->zs) * 4;
    auto ck_base = [&](int m) {  // checkpoint after step mK, m = 1 .. M-1
      return es->ck.as<float>() + (size_t)(m - 1) * (ckF + ckP);
    };
    auto save_ck = [&](int m) {
      float* b = ck_base(m);
      for (int f = 0; f < 4; ++f)
        check_cuda(cudaMemcpyAsync(b + (size_t)f * cap * F, es->st[f].p, (size_t)S * F * sizeof(float),
                                   cudaMemcpyDeviceToDevice, st), "checkpoint save");
      float* pb = b + ckF;
      for (int d = 0; d < 4; ++d) {
        check_cuda(cudaMemcpyAsync(pb + (size_t)d * cap * es->xs, es->px[d].p, (size_t)S * es->xs * sizeof(float),
                                   cudaMemcpyDeviceToDevice, st), "checkpoint save");
        check_cuda(cudaMemcpyAsync(pb + (size_t)4 * cap * es->xs + (size_t)d * cap * es->zs, es->pz[d].p,
                                   (size_t)S * es->zs * sizeof(float), cudaMemcpyDeviceToDevice, st),
                   "checkpoint save");
      }
    };
    auto load_ck = [&](int m) {
      if (m == 0) {
        zero_state(es, S, false);
        return;
      }
      float* b = ck_base(m);
      for (int f = 0; f < 4; ++f)
        check_cuda(cudaMemcpyAsync(es->st[f].p, b + (size_t)f * cap * F, (size_t)S * F * sizeof(float),
                                   cudaMemcpyDeviceToDevice, st), "checkpoint load");
      float* pb = b + ckF;
      for (int d = 0; d < 4; ++d) {
        check_cuda(cudaMemcpyAsync(es->px[d].p, pb + (size_t)d * cap * es->xs, (size_t)S * es->xs * sizeof(float),
                                   cudaMemcpyDeviceToDevice, st), "checkpoint load");
        check_cuda(cudaMemcpyAsync(es->pz[d].p, pb + (size_t)4 * cap * es->xs + (size_t)d * cap * es->zs,
                                   (size_t)S * es->zs * sizeof(float), cudaMemcpyDeviceToDevice, st),
                   "checkpoint load");
      }
    };
    // mute balls per group (= per shot when muting)
    std::vector<MuteBall> balls;
    std::vector<int> bptr(1, 0);
    if (mute) {
      const double hmax = std::max(es->prm.h[0], es->prm.h[1]);
      for (int k = 0; k < S; ++k) {
        const sw_elastic_shot& s = shots[group[k].orig];
        for (int fam = 0; fam < 2; ++fam) {
          const int radius = fam == 0 ? es->gp.mute_radius_src : es->gp.mute_radius_rec;
          if (radius <= 0) continue;
          const double* pos = fam == 0 ? s.src_pos : s.rec_pos;
          const int npos = fam == 0 ? s.nsrc : s.nrec;
          for (int p = 0; p < npos; ++p) {
            MuteBall b{};
            for (int d = 0; d < 2; ++d) {
              const double x = pos[p + (long long)d * npos], h = es->prm.h[d];
              const int ijk = (int)std::round((x - std::fmod(x, h)) / h) + 1;  // floor(Int, div(x, h)) + 1
              b.lo[d] = ijk - radius;
              b.hi[d] = ijk + radius;
              b.pos[d] = x;
            }
            b.rmax = radius * hmax;
            balls.push_back(b);
          }
        }
        bptr.push_back((int)balls.size());
      }
      upload(es, es->d_balls, balls, "mute balls");
      upload(es, es->d_ball_ptr, bptr, "mute balls");
    }
    // the group's device work -- forward, misfit (with the dense C^-1
    // products), adjoint scale, adjoint with recompute and correlation,
    // reduction -- as one CUDA graph
    const int nblk = 64;
    ensure(es, es->d_partial, (size_t)nblk * S * sizeof(double), "misfit partials");
    ensure(es, es->d_amax, 16, "max reduction");
    size_t ccts_smem = 0;
    int ccts_rec = 0;
    {  // CCTS shots: one trace per receiver component, no prescale
      std::vector<int> kind(S), nt(S), nrec(S);
      std::vector<double> mdt(S);
      std::vector<const float*> tr(S), obs(S);
      std::vector<float*> adj(S);
      std::vector<const long long*> rl(S, nullptr);
      for (int k = 0; k < S; ++k) {
        const sw_elastic_shot& s = shots[group[k].orig];
        kind[k] = s.misfit_kind;
        mdt[k] = s.misfit_dt;
        nt[k] = desc[k].nt;
        nrec[k] = 2 * desc[k].nrec;
        tr[k] = desc[k].tr;
        obs[k] = desc[k].obs;
        adj[k] = desc[k].adjsrc;
      }
      ensure(es, es->d_ccts, (size_t)S * sizeof(CctsShot), "CCTS table");
      ccts_rec = upload_ccts(es->ctx, es->d_ccts.as<CctsShot>(), kind, mdt, nt, nrec, tr, obs, adj, rl, &ccts_smem);
      if (ccts_rec) ensure(es, es->d_partial2, (size_t)ccts_rec * S * sizeof(double), "CCTS partials");
    }
    {
      const std::vector<float> sc = {sf_ref, 1.0f};
      upload(es, es->d_scales, sc, "source scales");
    }
    std::vector<long long> key = {S, ntmax, es->tz, es->vec ? 1 : 0, es->split_disp ? 1 : 0, first_group ? 1 : 0,
                                  mute ? 1 : 0,
                                  R.gx_src, R.gx_adj, R.gx_rec, (long long)(uintptr_t)out[0],
                                  (long long)(uintptr_t)out[1], (long long)(uintptr_t)out[2],
                                  (long long)(uintptr_t)mout};
    for (const auto& h : group) key.push_back(h.nt);
    for (const auto& h : group) key.push_back(shots[h.orig].kind);
    for (int k = 0; k < S; ++k)  // the dense products' operands are launch arguments
      if (desc[k].icd) key.insert(key.end(), {k, desc[k].nrec, (long long)(uintptr_t)desc[k].icd});
    auto body = [&] {
      // forward with checkpoints; the last window writes its slots directly
      zero_state(es, S, false);
      const int last_start = (M - 1) * K;
      for (int it = 1; it <= ntmax; ++it) {
        const int A = active_count(group, it);
        if (it > last_start) {
          float* sU[2];
          float* sD[2];
          slot_ptrs(it - last_start - 1, sU, sD);
          full_step(R, A, it, true, KK_STENCIL, sU, sD);
        } else {
          full_step(R, A, it, true, KK_STENCIL, nullptr, nullptr);
        }
        if (it % K == 0 && it / K <= M - 1) save_ck(it / K);
      }
      // misfit and adjoint source
      check_cuda(cudaMemsetAsync(es->d_amax.p, 0, sizeof(unsigned), st), "max clear");
      {
        cudaEvent_t ev = nullptr;
        bool any_dense = false;
        for (const auto& d : desc) any_dense = any_dense || d.icd;
        if (any_dense) {  // C^-1 r of the shots with a dense inverse covariance (dense.cu), per component
          k_el_residual_dense<<<dim3(nblk, S), 256, 0, st>>>(R.ddesc);
          check_cuda(cudaGetLastError(), "residual launch");
          for (const auto& d : desc)
            if (d.icd) dense_invcov(es->ctx, d.nt, 2 * d.nrec, d.icd, d.resid, const_cast<float*>(d.cres));
        }
        es->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
        k_el_misfit<<<dim3(nblk, S), 256, 0, st>>>(R.ddesc, es->d_partial.as<double>(), es->d_amax.as<unsigned>());
        check_cuda(cudaGetLastError(), "misfit launch");
        k_el_misfit_sum<<<1, 256, 0, st>>>(es->d_partial.as<double>(), nblk * S, mout, first_group ? 0 : 1);
        if (ccts_rec) {  // CCTS shots: misfit terms and adjoint sources per component trace
          k_ccts<<<dim3(ccts_rec, S), CCTS_THREADS, ccts_smem, st>>>(es->d_ccts.as<CctsShot>(), nullptr,
                                                                     es->d_partial2.as<double>(),
                                                                     es->d_amax.as<unsigned>());
          check_cuda(cudaGetLastError(), "CCTS misfit launch");
          k_el_misfit_sum<<<1, 256, 0, st>>>(es->d_partial2.as<double>(), ccts_rec * S, mout, 1);
          check_cuda(cudaGetLastError(), "CCTS misfit sum launch");
        }
        check_cuda(cudaGetLastError(), "misfit sum launch");
        es->ctx->prof.end(st, KK_OTHER, ev);
      }
      k_el_adj_scale<<<1, 1, 0, st>>>(es->d_amax.as<unsigned>(), es->d_scales.as<float>());
      check_cuda(cudaGetLastError(), "adjoint scale launch");
      // adjoint with recompute and correlation
      zero_state(es, S, true);
      check_cuda(cudaMemsetAsync(es->acc.p, 0, (size_t)ngroups * 10 * F * sizeof(float), st), "accumulators clear");
      Args ca = R.args(true);
      for (int m = M - 1; m >= 0; --m) {
        const int t0 = m * K + 1, t1 = std::min((m + 1) * K, ntmax);
        if (m < M - 1) {
          load_ck(m);
          for (int t = t0; t <= t1; ++t) {
            float* sU[2];
            float* sD[2];
            slot_ptrs(t - t0, sU, sD);
            full_step(R, active_count(group, t), t, false, KK_RECOMPUTE, sU, sD);
          }
        }
        for (int it = t1; it >= t0; --it) {
          const int A = active_count(group, it);
          if (A <= 0) continue;
          adjoint_step(R, A, it);
          float* sU[2];
          float* sD[2];
          slot_ptrs(it - t0, sU, sD);
          CorrArgs c{};
          c.g = g;
          c.nshots = A;
          c.gsize = gsize;
          c.cs = es->d_cs.as<float>();
          c.aux = ca.ux; c.auz = ca.uz;
          c.fux = sU[0]; c.fuz = sU[1];
          c.Dx = sD[0]; c.Dz = sD[1];
          c.lam = es->lam.as<float>(); c.mu = es->mu.as<float>();
          c.acc = es->acc.as<float>();
          const int ng = (A + gsize - 1) / gsize;
          const dim3 grid((g.nx + BX - 1) / BX, (g.nz + CTZ - 1) / CTZ, ng);
          cudaEvent_t ev = nullptr;
          const double pts = (double)g.nx * g.nz;
          es->ctx->prof.begin(st, KK_CORR, pts * (A * 24.0 + ng * 80.0), &ev);
          if (es->vec) {
            const dim3 grid4((g.nx + 511) / 512, g.nz, ng);
            k_el_corr4<<<grid4, BX, 0, st>>>(c);
          } else {
            k_el_corr<<<grid, BX, 0, st>>>(c);
          }
          check_cuda(cudaGetLastError(), "correlation launch");
          es->ctx->prof.end(st, KK_CORR, ev);
        }
      }
      {
        Geo gh = g;
        gh.idx = (float)es->prm.h[0];  // the reduction uses the spacings
        gh.idz = (float)es->prm.h[1];
        cudaEvent_t ev = nullptr;
        es->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
        const int blocks = (int)std::min<long long>((np + 255) / 256, 8192);
        k_el_reduce<<<blocks, 256, 0, st>>>(gh, ngroups, es->acc.as<float>(), es->rho_d.as<double>(), es->mu_d.as<double>(),
                                            es->prm.interp_rho, es->prm.interp_mu,
                                            1.0 / (es->prm.dt * es->prm.dt), es->d_scales.as<float>(),
                                            mute ? es->d_balls.as<MuteBall>() : nullptr,
                                            mute ? es->d_ball_ptr.as<int>() : nullptr, out[0], out[1], out[2],
                                            first_group ? 0 : 1);
        check_cuda(cudaGetLastError(), "gradient reduction launch");
        es->ctx->prof.end(st, KK_OTHER, ev);
      }
    };
    el_run_graph(es, key, body);
    download_traces(es, shots, group, desc, on_device);
    check_cuda(cudaStreamSynchronize(st), "elastic gradient group");
    first_group = false;
  }
  if (!on_device) {
    check_cuda(cudaMemcpyAsync(g_rho, out[0], np * sizeof(double), cudaMemcpyDeviceToHost, st), "gradient download");
    check_cuda(cudaMemcpyAsync(g_lam, out[1], np * sizeof(double), cudaMemcpyDeviceToHost, st), "gradient download");
    check_cuda(cudaMemcpyAsync(g_mu, out[2], np * sizeof(double), cudaMemcpyDeviceToHost, st), "gradient download");
  }
  if (misfit && (!on_device || mout != misfit))
    check_cuda(cudaMemcpyAsync(misfit, mout, sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               st), "misfit download");
  check_cuda(cudaStreamSynchronize(st), "elastic gradient");
  es->ctx->prof.resolve();
}

void elastic_set_tuning(sw_elastic* es, int tz) {
  // tz = rows per block (8, 16, 32; 0 = 8); + 64 selects the one-point-per-thread kernels;
  // + 128 runs the four-point displacement update as one launch instead of two (ux, uz)
  const int rows = tz % 64;
  if (tz < 0 || tz >= 256 || (rows != 0 && rows != 8 && rows != 16 && rows != 32))
    fail(SW_ERR_ARG, "tz must be 0, 8, 16 or 32, optionally + 64 and + 128");
  es->tz = rows == 0 ? 8 : rows;
  es->vec = (tz & 64) == 0;
  es->split_disp = (tz & 128) == 0;
}
sw_ctx* elastic_ctx(sw_elastic* es) { return es->ctx; }
sw_elastic* elastic_new() { return new sw_elastic(); }
void elastic_delete(sw_elastic* es) { delete es; }

}  // namespace swgb
