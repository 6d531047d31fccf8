// Variable-density acoustic 2D C-PML path (staggered 4th-order pressure /
// velocity scheme): the batched forward and the batched gradient with respect
// to vp and rho.
//
// Reference behaviour restated here (SeismicWaves.jl v0.9.0, paths relative to
// its source tree):
//   update_p_CPML!, update_vx_CPML!, update_vy_CPML!,
//   inject_sources!, record_receivers!  src/models/acoustic/backends/shared/acoustic2D_VD_xPU.jl:1-78
//   staggered 4th-order derivative and its boundary rules  src/utils/fdgen.jl:44-135
//   C-PML memory variables (the dtilde operator)  src/utils/fdgen.jl:137-161
//   forward / adjoint step orchestration  acoustic2D_VD_xPU.jl:80-169
//   correlate_gradient_m0!, correlate_gradient_m1!  correlate_gradient_xPU.jl:12-21,
//                                                   acoustic2D_VD_xPU.jl:171-192
//   precompute_fact! (fact_m0 = vp^2 rho dt, fact_m1 = interp(1/rho) dt)  src/models/acoustic/acou_models.jl:292-300
//   swforward_1shot! / swgradient_1shot! (VD)  src/models/acoustic/acou_forward.jl:83-125,
//                                              src/models/acoustic/acou_gradient.jl:97-202
//   back_interp  src/utils/interpolations.jl:15-47;  L2 misfit  src/inversion/misfits/L2Misfit.jl:24-77
//
// Layout.  p, vx and vz of a shot are zero-padded (nz + 4) x P arrays (x
// fastest, P a multiple of 32); node (i, j) (1-based) sits at row j + 1 and
// column i + 31, vx(i, j) (the point i + 1/2) and vz(i, j) (j + 1/2) share
// that slot.  The reference's derivative rules count a point outside its array
// as 0; the padding (and vx(nx, .), vz(., nz), which no kernel writes)
// supplies those zeros, so the stencils carry no boundary branches.  The C-PML
// memory variables live in compact strips: x strips (nz rows x W columns) and
// z strips ((2 halo + 2) rows x P), indexed by the reference's coefficient
// index.
//
// Kernels per time step: the pressure update (fused with the gradient
// correlation on the adjoint), one small injection / recording kernel, and
// the velocity update.  The pressure update reads p only at its own point, so
// it can write to a different array than it reads: the gradient keeps p of
// every step of the current checkpoint window in slots (the reference's K+1
// buffer), and the forward / recompute steps write p straight into them.
//
// Gradient.  The adjoint step correlates its new adjoint pressure with
// p[it] - p[it-1] and the adjoint velocities with the 4th-order derivatives of
// p[it] inside the pressure kernel; the adjoint injection at the receivers
// adds its share of the pressure term afterwards.  The three products are
// summed per shot in FP32 over one checkpoint window (K steps) and then added
// into FP64 totals, so no FP32 sum runs over more than K terms.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <sstream>
#include <vector>

#include "internal.h"
#include "ccts.cuh"
#include "ff.cuh"

namespace swgb {
namespace vd {

constexpr int XPAD = 32;  // columns left of i = 1
constexpr int ZPAD = 2;   // rows above j = 1
constexpr int BX = 128;   // threads per block (4 warps x 128 points)

struct Geo {
  int nx, nz, P, halo, W;
  long long F;  // floats per padded field
  float idx, idz;
  __host__ __device__ __forceinline__ long long lin(int i, int j) const {
    return (long long)(j + ZPAD - 1) * P + (i + XPAD - 1);
  }
};

struct PArgs {
  Geo g;
  const float* vx; const float* vz;  // [shot][F]
  const float* pin; float* pout;     // [shot][F]; may be the same array
  float* xi_x; float* xi_z;          // [shot][xs] / [shot][zs]
  long long xs, zs;
  const float* m0;                   // fact_m0 (padded, shared by the shots)
  const float* cp; int cps;          // per shot: axis x then z, [a(na), a_h(nh), b(na), b_h(nh)]
  // adjoint only: correlation with the forward pressure slots
  const float* pc; const float* po;  // p[it], p[it-1], [shot][F]
  float* acc;                        // [shot][3][F]: m0 term, m1 x term, m1 z term
  float idt;
};

struct VArgs {
  Geo g;
  const float* p;                    // [shot][F]
  float* vx; float* vz;
  float* psi_x; float* psi_z;
  long long xs, zs;
  const float* m1x; const float* m1z;
  const float* cp; int cps;
};

__device__ __forceinline__ float d4(float f1, float f2, float f3, float f4, float inv) {
  const float c1 = 1.0f / 24.0f, c2 = 27.0f / 24.0f;
  return (c1 * f1 - c2 * f2 + c2 * f3 - c1 * f4) * inv;
}

// Coefficient index (1-based, 0 = no memory variable) of fdgen.jl:137-161.
// Pressure update (halfgrid = false on the velocity array of n-1 points):
// pos <= halo+1 on the left, pos >= n-halo on the right, k = pos - n + 2 halo + 2.
// Velocity update (halfgrid = true on the pressure array of n points):
// pos <= halo, pos >= n-halo, k = pos - n + 2 halo + 1.
__host__ __device__ __forceinline__ int k_pres(int pos, int n, int halo) {
  if (pos <= halo + 1) return pos;
  if (pos >= n - halo) return pos - n + 2 * halo + 2;
  return 0;
}
__host__ __device__ __forceinline__ int k_vel(int pos, int n, int halo) {
  if (pos <= halo) return pos;
  if (pos >= n - halo) return pos - n + 2 * halo + 1;
  return 0;
}
// psi = b psi + a dv; returns dv + psi
__device__ __forceinline__ float cpml_upd(float* psi, float a, float b, float dv) {
  const float nv = b * (*psi) + a * dv;
  *psi = nv;
  return dv + nv;
}

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
// plain (coherent) load for arrays the kernel also writes
__device__ __forceinline__ F4 ld4p(const float* p, long long c, bool ok) {
  F4 r;
  if (ok) {
    const float4 t = *reinterpret_cast<const float4*>(p + c);
    r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
  } else {
    r.v[0] = r.v[1] = r.v[2] = r.v[3] = 0.0f;
  }
  return r;
}
__device__ __forceinline__ F4 ld4rw(const float* p, long long c) {
  const float4 t = *reinterpret_cast<const float4*>(p + c);
  F4 r;
  r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
  return r;
}
__device__ __forceinline__ void st4v(float* p, long long c, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p + c) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ float ldz(const float* __restrict__ p, long long c, bool ok) {
  return ok ? __ldg(p + c) : 0.0f;
}

constexpr unsigned FULL = 0xffffffffu;

// Pressure update (update_p_CPML! on 2:nx-1, 2:nz-1; every other node copies
// p through) for the shot blockIdx.z: four x points per thread, each warp 128
// consecutive points, a block 512 points x TZ rows.  The thread walks its
// columns down the band: vz rows j-2 .. j+1 stay in registers, the x
// neighbours of vx come from the adjacent lanes.  CORR (adjoint): also
// acc[0] += -(p_new (pc - po) / dt), acc[1] += vx dpc/dx, acc[2] += vz dpc/dz
// (pc rows j-1 .. j+2 in registers).
// Resident blocks per SM: the correlating adjoint kernel runs faster at 7
// (<= 72 registers; 5.06 against 4.92 TB/s for the adjoint step pair on 64
// shots), the forward one is left at its own register count (55) by a bound
// it already meets.
template <bool CORR>
struct VdPBounds {
  static constexpr int MINB = CORR ? 7 : 8;
};

template <int TZ, bool CORR>
__global__ void __launch_bounds__(BX, VdPBounds<CORR>::MINB) k_vd_p(const PArgs A) {
  const Geo g = A.g;
  const int s = blockIdx.z;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wx0 = (blockIdx.x * 4 + warp) * 128;
  const int j0 = blockIdx.y * TZ + 1;
  const int j1 = min(j0 + TZ - 1, g.nz);
  if (j0 > j1 || wx0 >= g.nx) return;  // warp uniform (no block-level synchronisation below)
  const int i0 = wx0 + lane * 4 + 1;
  const bool ldok = i0 <= g.nx + 2;
  const long long so = (long long)s * g.F;
  const float* __restrict__ vx = A.vx + so;
  const float* __restrict__ vz = A.vz + so;
  const float* pin = A.pin + so;
  float* pout = A.pout + so;
  const int na = 2 * g.halo + 2, nh = 2 * g.halo;
  const float* cx = A.cp + (long long)s * A.cps;
  const float* cz = cx + 2 * na + 2 * nh;
  float* xix = A.xi_x + (long long)s * A.xs;
  float* xiz = A.xi_z + (long long)s * A.zs;
  const int P = g.P;
  const bool xstrip = i0 <= g.halo + 1 || i0 + 3 >= g.nx - g.halo;
  const float* __restrict__ pc = CORR ? A.pc + so : nullptr;
  const float* __restrict__ po = CORR ? A.po + so : nullptr;
  float* acc = CORR ? A.acc + 3 * so : nullptr;
  long long c = g.lin(i0, j0);
  F4 z0 = ld4z(vz, c - 2 * P, ldok), z1 = ld4z(vz, c - P, ldok), z2 = ld4z(vz, c, ldok), z3 = ld4z(vz, c + P, ldok);
  F4 q0, q1, q2, q3;
  if (CORR) {
    q0 = ld4z(pc, c - P, ldok); q1 = ld4z(pc, c, ldok); q2 = ld4z(pc, c + P, ldok); q3 = ld4z(pc, c + 2 * P, ldok);
  }
  for (int j = j0; j <= j1; ++j, c += P) {
    const bool more = j + 1 <= j1;
    const F4 zn = ld4z(vz, c + 2 * P, ldok && more);
    F4 qn;
    if (CORR) qn = ld4z(pc, c + 3 * P, ldok && more);
    const F4 X = ld4z(vx, c, ldok);
    // vx at i0-2 .. i0+4 (row j)
    float xa[7];
    xa[0] = __shfl_up_sync(FULL, X.v[2], 1);
    xa[1] = __shfl_up_sync(FULL, X.v[3], 1);
    xa[6] = __shfl_down_sync(FULL, X.v[0], 1);
    if (lane == 0) {
      xa[0] = ldz(vx, c - 2, ldok);
      xa[1] = ldz(vx, c - 1, ldok);
    }
    if (lane == 31) xa[6] = ldz(vx, c + 4, ldok);
#pragma unroll
    for (int e = 0; e < 4; ++e) xa[2 + e] = X.v[e];
    const F4 PI = ld4p(pin, c, ldok), M0 = ld4z(A.m0, c, ldok);
    const bool jin = j >= 2 && j <= g.nz - 1;
    const int kz = jin ? k_pres(j, g.nz, g.halo) : 0;
    float out[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int i = i0 + e;
      float dvx = d4(xa[e], xa[e + 1], xa[e + 2], xa[e + 3], g.idx);  // vx[i-2 .. i+1]
      float dvz = d4(z0.v[e], z1.v[e], z2.v[e], z3.v[e], g.idz);      // vz rows j-2 .. j+1
      if (jin && i >= 2 && i <= g.nx - 1) {
        if (xstrip) {
          const int kx = k_pres(i, g.nx, g.halo);
          if (kx) dvx = cpml_upd(xix + (long long)(j - 1) * g.W + (kx - 1), cx[kx - 1], cx[na + nh + kx - 1], dvx);
        }
        if (kz) dvz = cpml_upd(xiz + (long long)(kz - 1) * P + (i - 1), cz[kz - 1], cz[na + nh + kz - 1], dvz);
        out[e] = PI.v[e] - M0.v[e] * (dvx + dvz);
      } else {
        out[e] = PI.v[e];
      }
    }
    if (ldok) {
      if (i0 + 3 <= g.nx) {
        st4v(pout, c, out);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (i0 + e <= g.nx) pout[c + e] = out[e];
      }
    }
    if (CORR) {
      // pc at i0-1 .. i0+5 (row j)
      float pa[7];
      pa[0] = __shfl_up_sync(FULL, q1.v[3], 1);
      pa[5] = __shfl_down_sync(FULL, q1.v[0], 1);
      pa[6] = __shfl_down_sync(FULL, q1.v[1], 1);
      if (lane == 0) pa[0] = ldz(pc, c - 1, ldok);
      if (lane == 31) {
        pa[5] = ldz(pc, c + 4, ldok);
        pa[6] = ldz(pc, c + 5, ldok);
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) pa[1 + e] = q1.v[e];
      if (ldok) {
        // Outside the nodes every factor below is a zero of the padding (or of
        // vx(nx, .) / vz(., nz)), so whole float4s are updated.
        const F4 PO = ld4z(po, c, true);
        F4 G0 = ld4rw(acc, c), G1 = ld4rw(acc + g.F, c), G2 = ld4rw(acc + 2 * g.F, c);
        float n0[4], n1[4], n2[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          n0[e] = G0.v[e] + (-(out[e] * (q1.v[e] - PO.v[e]) * A.idt));
          n1[e] = G1.v[e] + X.v[e] * d4(pa[e], pa[e + 1], pa[e + 2], pa[e + 3], g.idx);
          n2[e] = G2.v[e] + z2.v[e] * d4(q0.v[e], q1.v[e], q2.v[e], q3.v[e], g.idz);
        }
        st4v(acc, c, n0);
        st4v(acc + g.F, c, n1);
        st4v(acc + 2 * g.F, c, n2);
      }
      q0 = q1; q1 = q2; q2 = q3; q3 = qn;
    }
    z0 = z1; z1 = z2; z2 = z3; z3 = zn;
  }
}

// Velocity update (update_vx_CPML! on 1:nx-1 x 1:nz, update_vy_CPML! on
// 1:nx x 1:nz-1) for the shot blockIdx.z; p rows j-1 .. j+2 in registers.
template <int TZ>
__global__ void __launch_bounds__(BX) k_vd_v(const VArgs A) {
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
  const float* __restrict__ p = A.p + so;
  float* vx = A.vx + so;
  float* vz = A.vz + so;
  const int na = 2 * g.halo + 2, nh = 2 * g.halo;
  const float* cx = A.cp + (long long)s * A.cps;
  const float* cz = cx + 2 * na + 2 * nh;
  float* psx = A.psi_x + (long long)s * A.xs;
  float* psz = A.psi_z + (long long)s * A.zs;
  const int P = g.P;
  const bool xstrip = i0 <= g.halo || i0 + 3 >= g.nx - g.halo;
  long long c = g.lin(i0, j0);
  F4 w0 = ld4z(p, c - P, ldok), w1 = ld4z(p, c, ldok), w2 = ld4z(p, c + P, ldok), w3 = ld4z(p, c + 2 * P, ldok);
  for (int j = j0; j <= j1; ++j, c += P) {
    const bool more = j + 1 <= j1;
    const F4 wn = ld4z(p, c + 3 * P, ldok && more);
    // p at i0-1 .. i0+5 (row j)
    float pa[7];
    pa[0] = __shfl_up_sync(FULL, w1.v[3], 1);
    pa[5] = __shfl_down_sync(FULL, w1.v[0], 1);
    pa[6] = __shfl_down_sync(FULL, w1.v[1], 1);
    if (lane == 0) pa[0] = ldz(p, c - 1, ldok);
    if (lane == 31) {
      pa[5] = ldz(p, c + 4, ldok);
      pa[6] = ldz(p, c + 5, ldok);
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) pa[1 + e] = w1.v[e];
    if (ldok) {
      const F4 VX = ld4rw(vx, c), MX = ld4z(A.m1x, c, true);
      float nv[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        float d = d4(pa[e], pa[e + 1], pa[e + 2], pa[e + 3], g.idx);  // p[i-1 .. i+2]
        if (xstrip && i <= g.nx - 1) {
          const int kx = k_vel(i, g.nx, g.halo);
          if (kx) d = cpml_upd(psx + (long long)(j - 1) * g.W + (kx - 1), cx[na + kx - 1], cx[2 * na + nh + kx - 1], d);
        }
        nv[e] = VX.v[e] - MX.v[e] * d;
      }
      if (i0 + 3 <= g.nx - 1) {
        st4v(vx, c, nv);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (i0 + e <= g.nx - 1) vx[c + e] = nv[e];
      }
      if (j <= g.nz - 1) {
        const int kz = k_vel(j, g.nz, g.halo);
        const F4 VZ = ld4rw(vz, c), MZ = ld4z(A.m1z, c, true);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          float d = d4(w0.v[e], w1.v[e], w2.v[e], w3.v[e], g.idz);  // p rows j-1 .. j+2
          if (kz && i <= g.nx)
            d = cpml_upd(psz + (long long)(kz - 1) * P + (i - 1), cz[na + kz - 1], cz[2 * na + nh + kz - 1], d);
          nv[e] = VZ.v[e] - MZ.v[e] * d;
        }
        if (i0 + 3 <= g.nx) {
          st4v(vz, c, nv);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (i0 + e <= g.nx) vz[c + e] = nv[e];
        }
      }
    }
    w0 = w1; w1 = w2; w2 = w3; w3 = wn;
  }
}

// ---------------------------------------------------------------------------
// Compensated forward step (sw_acoustic_vd_set_precision(vd, 1)): p, vx and
// vz as double-FP32 values (high parts in the usual arrays, low parts in their
// own), fact_m0 / fact_m1 and 1/dx, 1/dz as FP32 pairs of their FP64 values,
// the staggered differences c2 (f3 - f2) + c1 (f1 - f4) and both updates in
// double-FP32 (ff.cuh), the C-PML memory variables and coefficients in FP64.
// Same update order and index rules as k_vd_p / k_vd_v; forward modes only
// (the recompute and the adjoint stay FP32, starting from FP32-rounded
// checkpoints).
// ---------------------------------------------------------------------------
struct HArgs {
  Geo g;
  const float* pin; float* pout;     // p high parts [shot][F] (pin may equal pout)
  float* plo;                        // p low parts [shot][F], updated in place
  float* vx; float* vz;              // velocity high parts
  float* vxl; float* vzl;            // velocity low parts
  double* xi_x; double* xi_z;        // pressure-update memory variables (FP64)
  double* psi_x; double* psi_z;      // velocity-update memory variables (FP64)
  long long xs, zs;
  const float* m0; const float* m0l;
  const float* m1x; const float* m1xl;
  const float* m1z; const float* m1zl;
  const double* cp; int cps;         // FP64 coefficients per shot, as cp of PArgs
  float idxl, idzl;                  // low parts of 1/dx, 1/dz (the high parts are g.idx, g.idz)
};

// c1 f1 - c2 f2 + c2 f3 - c1 f4 = c2 (f3 - f2) + c1 (f1 - f4), times 1/h
__device__ __forceinline__ ff ffd4(ff f1, ff f2, ff f3, ff f4, ff inv) {
  constexpr double C1 = 1.0 / 24.0;
  const ff c1{(float)C1, (float)(C1 - (double)(float)C1)};
  const ff c2{1.125f, 0.f};  // 27/24, exact
  return ff_mul(ff_add(ff_mul(ff_sub(f3, f2), c2), ff_mul(ff_sub(f1, f4), c1)), inv);
}
// psi = b psi + a dv; returns dv + psi (cpml_upd in FP64)
__device__ __forceinline__ ff cpml_upd64(double* psi, double a, double b, ff dv) {
  const double d = ff_to_d(dv);
  const double nv = b * (*psi) + a * d;
  *psi = nv;
  return d_to_ff(d + nv);
}

template <int TZ>
__global__ void __launch_bounds__(BX) k_vd_p_hp(const HArgs A) {
  const Geo g = A.g;
  const int s = blockIdx.z;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wx0 = (blockIdx.x * 4 + warp) * 128;
  const int j0 = blockIdx.y * TZ + 1;
  const int j1 = min(j0 + TZ - 1, g.nz);
  if (j0 > j1 || wx0 >= g.nx) return;  // warp uniform
  const int i0 = wx0 + lane * 4 + 1;
  const bool ldok = i0 <= g.nx + 2;
  const long long so = (long long)s * g.F;
  const float* vx = A.vx + so;
  const float* vz = A.vz + so;
  const float* vxl = A.vxl + so;
  const float* vzl = A.vzl + so;
  const float* pin = A.pin + so;
  float* pout = A.pout + so;
  float* plo = A.plo + so;
  const int na = 2 * g.halo + 2, nh = 2 * g.halo;
  const double* cx = A.cp + (long long)s * A.cps;
  const double* cz = cx + 2 * na + 2 * nh;
  double* xix = A.xi_x + (long long)s * A.xs;
  double* xiz = A.xi_z + (long long)s * A.zs;
  const int P = g.P;
  const bool xstrip = i0 <= g.halo + 1 || i0 + 3 >= g.nx - g.halo;
  const ff idx{g.idx, A.idxl}, idz{g.idz, A.idzl};
  long long c = g.lin(i0, j0);
  F4 z0 = ld4p(vz, c - 2 * P, ldok), z1 = ld4p(vz, c - P, ldok), z2 = ld4p(vz, c, ldok), z3 = ld4p(vz, c + P, ldok);
  F4 l0 = ld4p(vzl, c - 2 * P, ldok), l1 = ld4p(vzl, c - P, ldok), l2 = ld4p(vzl, c, ldok), l3 = ld4p(vzl, c + P, ldok);
  for (int j = j0; j <= j1; ++j, c += P) {
    const bool more = j + 1 <= j1;
    const F4 zn = ld4p(vz, c + 2 * P, ldok && more), ln = ld4p(vzl, c + 2 * P, ldok && more);
    const F4 X = ld4p(vx, c, ldok), XL = ld4p(vxl, c, ldok);
    float xa[7], xb[7];  // vx at i0-2 .. i0+4 (row j): high and low parts
    xa[0] = __shfl_up_sync(FULL, X.v[2], 1);
    xa[1] = __shfl_up_sync(FULL, X.v[3], 1);
    xa[6] = __shfl_down_sync(FULL, X.v[0], 1);
    xb[0] = __shfl_up_sync(FULL, XL.v[2], 1);
    xb[1] = __shfl_up_sync(FULL, XL.v[3], 1);
    xb[6] = __shfl_down_sync(FULL, XL.v[0], 1);
    if (lane == 0) {
      xa[0] = ldz(vx, c - 2, ldok);
      xa[1] = ldz(vx, c - 1, ldok);
      xb[0] = ldz(vxl, c - 2, ldok);
      xb[1] = ldz(vxl, c - 1, ldok);
    }
    if (lane == 31) {
      xa[6] = ldz(vx, c + 4, ldok);
      xb[6] = ldz(vxl, c + 4, ldok);
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      xa[2 + e] = X.v[e];
      xb[2 + e] = XL.v[e];
    }
    const F4 PI = ld4p(pin, c, ldok), PL = ld4p(plo, c, ldok);
    const F4 M0 = ld4z(A.m0, c, ldok), M0L = ld4z(A.m0l, c, ldok);
    const bool jin = j >= 2 && j <= g.nz - 1;
    const int kz = jin ? k_pres(j, g.nz, g.halo) : 0;
    float oh[4], ol[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int i = i0 + e;
      if (jin && i >= 2 && i <= g.nx - 1) {
        ff dvx = ffd4(ff{xa[e], xb[e]}, ff{xa[e + 1], xb[e + 1]}, ff{xa[e + 2], xb[e + 2]}, ff{xa[e + 3], xb[e + 3]},
                      idx);
        ff dvz = ffd4(ff{z0.v[e], l0.v[e]}, ff{z1.v[e], l1.v[e]}, ff{z2.v[e], l2.v[e]}, ff{z3.v[e], l3.v[e]}, idz);
        if (xstrip) {
          const int kx = k_pres(i, g.nx, g.halo);
          if (kx) dvx = cpml_upd64(xix + (long long)(j - 1) * g.W + (kx - 1), cx[kx - 1], cx[na + nh + kx - 1], dvx);
        }
        if (kz) dvz = cpml_upd64(xiz + (long long)(kz - 1) * P + (i - 1), cz[kz - 1], cz[na + nh + kz - 1], dvz);
        const ff o = ff_sub(ff{PI.v[e], PL.v[e]}, ff_mul(ff{M0.v[e], M0L.v[e]}, ff_add(dvx, dvz)));
        oh[e] = o.hi;
        ol[e] = o.lo;
      } else {
        oh[e] = PI.v[e];
        ol[e] = PL.v[e];
      }
    }
    if (ldok) {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (i0 + e <= g.nx) {
          pout[c + e] = oh[e];
          plo[c + e] = ol[e];
        }
    }
    z0 = z1; z1 = z2; z2 = z3; z3 = zn;
    l0 = l1; l1 = l2; l2 = l3; l3 = ln;
  }
}

template <int TZ>
__global__ void __launch_bounds__(BX) k_vd_v_hp(const HArgs A) {
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
  const float* p = A.pout + so;  // the pressure just updated
  const float* pl = A.plo + so;
  float* vx = A.vx + so;
  float* vz = A.vz + so;
  float* vxl = A.vxl + so;
  float* vzl = A.vzl + so;
  const int na = 2 * g.halo + 2, nh = 2 * g.halo;
  const double* cx = A.cp + (long long)s * A.cps;
  const double* cz = cx + 2 * na + 2 * nh;
  double* psx = A.psi_x + (long long)s * A.xs;
  double* psz = A.psi_z + (long long)s * A.zs;
  const int P = g.P;
  const bool xstrip = i0 <= g.halo || i0 + 3 >= g.nx - g.halo;
  const ff idx{g.idx, A.idxl}, idz{g.idz, A.idzl};
  long long c = g.lin(i0, j0);
  F4 w0 = ld4p(p, c - P, ldok), w1 = ld4p(p, c, ldok), w2 = ld4p(p, c + P, ldok), w3 = ld4p(p, c + 2 * P, ldok);
  F4 u0 = ld4p(pl, c - P, ldok), u1 = ld4p(pl, c, ldok), u2 = ld4p(pl, c + P, ldok), u3 = ld4p(pl, c + 2 * P, ldok);
  for (int j = j0; j <= j1; ++j, c += P) {
    const bool more = j + 1 <= j1;
    const F4 wn = ld4p(p, c + 3 * P, ldok && more), un = ld4p(pl, c + 3 * P, ldok && more);
    float pa[7], pb[7];  // p at i0-1 .. i0+5 (row j): high and low parts
    pa[0] = __shfl_up_sync(FULL, w1.v[3], 1);
    pa[5] = __shfl_down_sync(FULL, w1.v[0], 1);
    pa[6] = __shfl_down_sync(FULL, w1.v[1], 1);
    pb[0] = __shfl_up_sync(FULL, u1.v[3], 1);
    pb[5] = __shfl_down_sync(FULL, u1.v[0], 1);
    pb[6] = __shfl_down_sync(FULL, u1.v[1], 1);
    if (lane == 0) {
      pa[0] = ldz(p, c - 1, ldok);
      pb[0] = ldz(pl, c - 1, ldok);
    }
    if (lane == 31) {
      pa[5] = ldz(p, c + 4, ldok);
      pa[6] = ldz(p, c + 5, ldok);
      pb[5] = ldz(pl, c + 4, ldok);
      pb[6] = ldz(pl, c + 5, ldok);
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      pa[1 + e] = w1.v[e];
      pb[1 + e] = u1.v[e];
    }
    if (ldok) {
      const F4 VX = ld4rw(vx, c), VXL = ld4rw(vxl, c), MX = ld4z(A.m1x, c, true), MXL = ld4z(A.m1xl, c, true);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (i > g.nx - 1) continue;
        ff d = ffd4(ff{pa[e], pb[e]}, ff{pa[e + 1], pb[e + 1]}, ff{pa[e + 2], pb[e + 2]}, ff{pa[e + 3], pb[e + 3]}, idx);
        if (xstrip) {
          const int kx = k_vel(i, g.nx, g.halo);
          if (kx) d = cpml_upd64(psx + (long long)(j - 1) * g.W + (kx - 1), cx[na + kx - 1], cx[2 * na + nh + kx - 1], d);
        }
        const ff nv = ff_sub(ff{VX.v[e], VXL.v[e]}, ff_mul(ff{MX.v[e], MXL.v[e]}, d));
        vx[c + e] = nv.hi;
        vxl[c + e] = nv.lo;
      }
      if (j <= g.nz - 1) {
        const int kz = k_vel(j, g.nz, g.halo);
        const F4 VZ = ld4rw(vz, c), VZL = ld4rw(vzl, c), MZ = ld4z(A.m1z, c, true), MZL = ld4z(A.m1zl, c, true);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          if (i > g.nx) continue;
          ff d = ffd4(ff{w0.v[e], u0.v[e]}, ff{w1.v[e], u1.v[e]}, ff{w2.v[e], u2.v[e]}, ff{w3.v[e], u3.v[e]}, idz);
          if (kz) d = cpml_upd64(psz + (long long)(kz - 1) * P + (i - 1), cz[na + kz - 1], cz[2 * na + nh + kz - 1], d);
          const ff nv = ff_sub(ff{VZ.v[e], VZL.v[e]}, ff_mul(ff{MZ.v[e], MZL.v[e]}, d));
          vz[c + e] = nv.hi;
          vzl[c + e] = nv.lo;
        }
      }
    }
    w0 = w1; w1 = w2; w2 = w3; w3 = wn;
    u0 = u1; u1 = u2; u2 = u3; u3 = un;
  }
}

// FP64 memory variables into the FP32 checkpoint strips (compensated forward)
__global__ void k_vd_d2f(const double* __restrict__ src, float* __restrict__ dst, long long n) {
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    dst[q] = (float)src[q];
}

// ---------------------------------------------------------------------------
// Sources, receivers, misfit, reductions
// ---------------------------------------------------------------------------
struct ShotDesc {
  int nt, nsrc, nrec;
  int nsp, nrp;                 // unique source / receiver points
  const long long* sp_lin;      // unique source points (padded index)
  const int* sp_ptr;            // nsp + 1
  const int* sp_ids;            // source index of each entry
  const long long* rp_lin;
  const int* rp_ptr;
  const int* rp_ids;
  const long long* rec_lin;     // per receiver
  const float* tf;              // (nt, nsrc)
  float* tr;                    // (nt, nrec)
  const float* obs;
  const float* ic;              // diagonal inverse covariance (nt) or null
  const float* mask;            // window mask (nt) or null
  float* adj;                   // prescaled adjoint sources (nt, nrec)
  const float* icd;             // dense inverse covariance (nt, nt) or null
  float* resid;                 // dense case: masked residuals
  const float* cres;            // dense case: C^-1 r
  int mkind;                    // 0 L2, 1 CCTS (k_ccts writes this shot's adjoint source)
};

// inject_sources! then record_receivers! (the velocity update in between does
// not touch p): one block per active shot; a point that several sources share
// receives them in source order.
__global__ void k_vd_srcrec(const ShotDesc* __restrict__ desc, int it, long long F, float* p, int record,
                            float* plo) {
  const ShotDesc D = desc[blockIdx.x];
  if (it > D.nt) return;  // block uniform
  float* pp = p + (long long)blockIdx.x * F;
  float* pl = plo ? plo + (long long)blockIdx.x * F : nullptr;  // compensated forward: low parts
  for (int u = threadIdx.x; u < D.nsp; u += blockDim.x) {
    const long long c = D.sp_lin[u];
    if (pl) {
      ff v{pp[c], pl[c]};
      for (int k = D.sp_ptr[u]; k < D.sp_ptr[u + 1]; ++k)
        v = ff_add(v, ff{D.tf[(long long)(it - 1) + (long long)D.sp_ids[k] * D.nt], 0.f});
      pp[c] = v.hi;
      pl[c] = v.lo;
      continue;
    }
    float v = pp[c];
    for (int k = D.sp_ptr[u]; k < D.sp_ptr[u + 1]; ++k) v += D.tf[(long long)(it - 1) + (long long)D.sp_ids[k] * D.nt];
    pp[c] = v;
  }
  if (!record) return;
  __syncthreads();
  for (int r = threadIdx.x; r < D.nrec; r += blockDim.x) {
    const long long q = D.rec_lin[r];
    D.tr[(long long)(it - 1) + (long long)r * D.nt] = pl ? __fadd_rn(pp[q], pl[q]) : pp[q];
  }
}

// Adjoint injection at the receivers and the matching share of the pressure
// correlation term, -(added value) (pc - po) / dt, which the fused kernel took
// before the injection.
__global__ void k_vd_adjinj(const ShotDesc* __restrict__ desc, int it, long long F, float* ap, const float* pc,
                            const float* po, float* acc, float idt) {
  const ShotDesc D = desc[blockIdx.x];
  if (it > D.nt) return;
  const long long so = (long long)blockIdx.x * F;
  float* a = ap + so;
  float* g0 = acc + 3 * so;
  for (int u = threadIdx.x; u < D.nrp; u += blockDim.x) {
    const long long c = D.rp_lin[u];
    float v = a[c], add = 0.0f;
    for (int k = D.rp_ptr[u]; k < D.rp_ptr[u + 1]; ++k) {
      const float s = D.adj[(long long)(it - 1) + (long long)D.rp_ids[k] * D.nt];
      v += s;
      add += s;
    }
    a[c] = v;
    g0[c] += -(add * (pc[so + c] - po[so + c]) * idt);
  }
}

__global__ void k_vd_residual_dense(const ShotDesc* __restrict__ desc) {
  const ShotDesc& D = desc[blockIdx.y];
  if (!D.icd) return;
  const long long total = (long long)D.nt * D.nrec;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
    float r = D.tr[q] - D.obs[q];
    if (D.mask) r *= D.mask[q % D.nt];
    D.resid[q] = r;
  }
}

// Residuals, window mask, C^-1 r, misfit partial sums (FP64) and the adjoint
// source -C^-1 r * fact_m0(rec) (prescale_residuals!).  gridDim = (blocks, shots).
__global__ void k_vd_misfit(const ShotDesc* __restrict__ desc, const float* __restrict__ m0,
                            double* __restrict__ partial) {
  const int shot = blockIdx.y;
  const ShotDesc D = desc[shot];
  const long long total = D.mkind == 1 ? 0 : (long long)D.nt * D.nrec;  // CCTS shots: k_ccts
  double acc = 0.0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
    const int t = (int)(q % D.nt);
    const int r = (int)(q / D.nt);
    float res = D.tr[q] - D.obs[q];
    if (D.mask) res *= D.mask[t];
    const float cres = D.cres ? D.cres[q] : (D.ic ? D.ic[t] * res : res);
    acc += (double)res * (double)cres;
    D.adj[q] = (-cres) * m0[D.rec_lin[r]];
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(long long)shot * gridDim.x + blockIdx.x] = red[0];
}

__global__ void k_vd_misfit_sum(const double* __restrict__ partial, int n, double* out, int accumulate) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = (accumulate ? *out : 0.0) + 0.5 * red[0];
}

// End of a checkpoint window: the FP32 window sums of the first A shots are
// added into the FP64 totals of their groups (gsize consecutive shots each);
// the host clears the sums right after.  Four consecutive padded points per
// thread (the padding holds zeros); the shot loop only loads, so the loads of
// several shots are in flight together.
__global__ void k_vd_flush(Geo g, int A, int gsize, const float* __restrict__ acc, double* __restrict__ tot) {
  const long long F4 = g.F / 4;  // F is a multiple of 4
  const float4* a4 = reinterpret_cast<const float4*>(acc);
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < 3 * F4; q += (long long)gridDim.x * blockDim.x) {
    const long long f = q / F4, r = q - f * F4;  // field, float4 index in the field
    for (int s0 = 0; s0 < A; s0 += gsize) {
      double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
      const int s1 = min(s0 + gsize, A);
#pragma unroll 8
      for (int s = s0; s < s1; ++s) {
        const float4 v = __ldg(a4 + ((long long)s * 3 + f) * F4 + r);
        t0 += (double)v.x;
        t1 += (double)v.y;
        t2 += (double)v.z;
        t3 += (double)v.w;
      }
      double* T = tot + ((long long)(s0 / gsize) * 3 + f) * g.F + 4 * r;
      T[0] += t0;
      T[1] += t1;
      T[2] += t2;
      T[3] += t3;
    }
  }
}

struct MuteBall {
  int lo[2], hi[2];
  double pos[2];
  double rmax;
};

// Final gradients (FP64, (nx, nz) column-major), summed over the groups:
// g0 and g1 = back_interp of the two staggered m1 totals (weights 1/2, or the
// harmonic-mean chain rule on m1 = 1/rho), each group muted around its shot's
// positions, then vp: -2 g0 / (vp^3 rho), rho: -g0 / (vp^2 rho^2) - g1 / rho
// (acou_gradient.jl:184-201).
__global__ void k_vd_reduce(Geo g, int ngroups, const double* __restrict__ tot, const double* __restrict__ vp,
                            const double* __restrict__ rho, int interp, double hx, double hz,
                            const MuteBall* __restrict__ balls, const int* __restrict__ ball_ptr,
                            double* __restrict__ gvp, double* __restrict__ grho, int accumulate) {
  const long long npts = (long long)g.nx * g.nz;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < npts; q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q % g.nx) + 1, j = (int)(q / g.nx) + 1;
    auto M = [&](int a, int b) { return (long long)(a - 1) + (long long)(b - 1) * g.nx; };
    const double r_c = rho[q];
    double wx[2] = {0.0, 0.0}, wz[2] = {0.0, 0.0};
    bool vx[2], vz[2];
    for (int p = 0; p < 2; ++p) {
      const int ci = i - 1 + p;  // x half point (ci + 1/2, j)
      vx[p] = ci >= 1 && ci <= g.nx - 1;
      if (vx[p]) {
        if (interp == 1) {
          const double f = 2.0 / (rho[M(ci, j)] + rho[M(ci + 1, j)]);  // harmonic mean of 1/rho
          wx[p] = f * f * r_c * r_c * 0.5;
        } else {
          wx[p] = 0.5;
        }
      }
      const int cj = j - 1 + p;
      vz[p] = cj >= 1 && cj <= g.nz - 1;
      if (vz[p]) {
        if (interp == 1) {
          const double f = 2.0 / (rho[M(i, cj)] + rho[M(i, cj + 1)]);
          wz[p] = f * f * r_c * r_c * 0.5;
        } else {
          wz[p] = 0.5;
        }
      }
    }
    const long long c = g.lin(i, j);
    double s0 = 0.0, s1 = 0.0;
    for (int gi = 0; gi < ngroups; ++gi) {
      const double* T = tot + (long long)gi * 3 * g.F;
      double a0 = T[c], a1 = 0.0;
      for (int p = 0; p < 2; ++p) {
        if (vx[p]) a1 += wx[p] * T[g.F + g.lin(i - 1 + p, j)];
        if (vz[p]) a1 += wz[p] * T[2 * g.F + g.lin(i, j - 1 + p)];
      }
      if (ball_ptr) {
        double f = 1.0;
        for (int b = ball_ptr[gi]; b < ball_ptr[gi + 1]; ++b) {
          const MuteBall B = balls[b];
          if (i < B.lo[0] || i > B.hi[0] || j < B.lo[1] || j > B.hi[1]) continue;
          const double x = (i - 1) * hx, z = (j - 1) * hz;
          const double rr = sqrt((B.pos[0] - x) * (B.pos[0] - x) + (B.pos[1] - z) * (B.pos[1] - z));
          if (rr <= B.rmax) f *= rr / B.rmax;
        }
        a0 *= f;
        a1 *= f;
      }
      s0 += a0;
      s1 += a1;
    }
    const double v = vp[q];
    const double ov = -2.0 * s0 / (v * v * v * r_c);
    const double orr = -s0 / (v * v * r_c * r_c) - s1 / r_c;
    gvp[q] = accumulate ? gvp[q] + ov : ov;
    grho[q] = accumulate ? grho[q] + orr : orr;
  }
}

// savesnapshot!("pcur", "vcur") staging: one block row per shot, [p (nx, nz),
// vx (nx-1, nz), vz (nx, nz-1)] unpadded into stage + shot * B.
__global__ void k_vd_snapshot(Geo g, const float* __restrict__ p, const float* __restrict__ vx,
                              const float* __restrict__ vz, long long B, float* __restrict__ stage) {
  const int s = blockIdx.y;
  const long long so = (long long)s * g.F;
  const long long n0 = (long long)g.nx * g.nz, n1 = (long long)(g.nx - 1) * g.nz;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < B; q += (long long)gridDim.x * blockDim.x) {
    const float* f;
    long long r = q;
    int w;
    if (r < n0) { f = p; w = g.nx; }
    else if ((r -= n0) < n1) { f = vx; w = g.nx - 1; }
    else { r -= n1; f = vz; w = g.nx; }
    const int i = (int)(r % w) + 1, j = (int)(r / w) + 1;
    stage[(long long)s * B + q] = f[so + g.lin(i, j)];
  }
}

}  // namespace vd
}  // namespace swgb

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using namespace swgb;
using namespace swgb::vd;

struct sw_acoustic_vd {
  sw_ctx* ctx = nullptr;
  sw_acoustic_params prm{};
  int interp = 0;
  bool gradient = false;
  sw_grad_params gp{};
  Geo g{};
  int na = 0, nh = 0, cps = 0;
  long long xs = 0, zs = 0;
  bool has_mat = false;
  DevMem m0, m1x, m1z, vp_d, rho_d;
  int cap = 0;
  DevMem st[3], ast[3];        // p vx vz
  DevMem xi[2], psi[2], axi[2], apsi[2];  // strips: [0] x, [1] z
  DevMem slots;                // [K+1][cap][F]
  DevMem ck;                   // [M-2][p, vx, vz][cap][F] then 4 strips [cap][xs|zs]
  DevMem acc;                  // [cap][3][F]
  DevMem tot;                  // [groups][3][F] double
  DevMem d_desc, d_ll, d_int, d_flt, d_tf, d_tr, d_obs, d_ic, d_adj, d_cp, d_partial, d_balls, d_ball_ptr;
  DevMem d_icd, d_dres, d_snap, d_ccts, d_partial2;
  int snapevery = 0;
  float* const* snap_out = nullptr;
  int tz = 8;
  // compensated forward (precision 1): low parts of p, vx, vz and of the
  // material factors, FP64 memory variables and coefficients
  int precision = 0;
  int hp_cap = 0;
  DevMem plo, vxl, vzl, xi64[2], psi64[2], m0l, m1xl, m1zl, d_cp64;
  std::vector<float> m0l_h, m1xl_h, m1zl_h;
};

namespace {

inline long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

void ensure(sw_acoustic_vd* vd, DevMem& m, size_t bytes, const char* what) {
  if (m.bytes >= bytes && m.p) return;
  dev_alloc(m, bytes, what, vd->ctx->stream);
}

template <typename T>
void upload(sw_acoustic_vd* vd, DevMem& m, const std::vector<T>& v, const char* what) {
  ensure(vd, m, std::max<size_t>(v.size() * sizeof(T), 16), what);
  if (!v.empty())
    check_cuda(cudaMemcpyAsync(m.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, vd->ctx->stream), what);
}

struct HostShot {
  int orig;
  int nt;
};

void validate_shot(const sw_acoustic_vd* vd, const sw_acoustic_shot& s, int k, bool grad) {
  std::ostringstream os;
  if (s.nt < 1) { os << "shot " << k << ": Number of timesteps must be positive!"; fail(SW_ERR_ARG, os.str()); }
  if (s.nsrc < 1) fail(SW_ERR_ARG, "There must be at least one source!");
  if (s.nrec < 1) fail(SW_ERR_ARG, "There must be at least one receiver!");
  if (!s.src_idx || !s.srctf || !s.rec_idx || !s.traces || !s.cpml) {
    os << "shot " << k << ": src_idx, srctf, rec_idx, traces and cpml are required";
    fail(SW_ERR_ARG, os.str());
  }
  for (int q = 0; q < s.nsrc + s.nrec; ++q) {
    const bool src = q < s.nsrc;
    const int32_t* idx = src ? s.src_idx : s.rec_idx;
    const int n = src ? s.nsrc : s.nrec, r = src ? q : q - s.nsrc;
    const int i = idx[r], j = idx[r + n];
    if (i < 1 || i > vd->g.nx || j < 1 || j > vd->g.nz) {
      os << "shot " << k << ": " << (src ? "source" : "receiver") << " (" << i << ", " << j << ") lies outside the grid";
      fail(SW_ERR_ARG, os.str());
    }
  }
  if (grad) {
    if (!s.observed) { os << "shot " << k << ": observed traces are required"; fail(SW_ERR_ARG, os.str()); }
    if (vd->gp.check_freq >= s.nt) fail(SW_ERR_ARG, "Checkpointing frequency must be smaller than the number of timesteps!");
    for (int w = 0; w < s.nwin; ++w) {
      const int a = s.windows[2 * w], b = s.windows[2 * w + 1];
      if (!(1 <= a && a <= b && b <= s.nt))
        fail(SW_ERR_ARG, "Windows indices must be between 1 and maximum number of timesteps!");
    }
    validate_misfit_kind(s, k);
  }
}

size_t per_shot_bytes(const sw_acoustic_vd* vd, bool grad, int max_nt) {
  const size_t F = (size_t)vd->g.F, strips = 2 * (size_t)(vd->xs + vd->zs);
  size_t b = (3 * F + strips) * sizeof(float);
  if (grad) {
    const int K = vd->gp.check_freq;
    const int M = (max_nt + K - 1) / K;
    b += (3 * F + strips) * sizeof(float);                                    // adjoint state
    b += (size_t)(K + 1) * F * sizeof(float);                                 // pressure slots
    b += (size_t)std::max(M - 2, 0) * (3 * F + strips) * sizeof(float);      // checkpoints
    b += 3 * F * sizeof(float) + 3 * F * sizeof(double);                      // window sums, totals
    b += (size_t)max_nt * 400 * sizeof(float) * 3;                            // traces, observed, adjoint (rough)
  }
  return b;
}

int checkpoints_needed(const sw_acoustic_vd* vd, int max_nt) {
  const int K = vd->gp.check_freq;
  const int M = (max_nt + K - 1) / K;
  return std::max(M - 2, 0);
}

void ensure_state(sw_acoustic_vd* vd, int S, bool grad, int max_nt, int ngroups) {
  const long long F = vd->g.F;
  cudaStream_t st = vd->ctx->stream;
  if (vd->cap < S || (grad && !vd->ast[0].p)) {
    for (int f = 0; f < 3; ++f) dev_alloc(vd->st[f], (size_t)S * F * sizeof(float), "VD fields", st);
    for (int d = 0; d < 2; ++d) {
      const long long w = d == 0 ? vd->xs : vd->zs;
      dev_alloc(vd->xi[d], (size_t)S * w * sizeof(float), "VD memory variables", st);
      dev_alloc(vd->psi[d], (size_t)S * w * sizeof(float), "VD memory variables", st);
    }
    if (grad) {
      for (int f = 0; f < 3; ++f) dev_alloc(vd->ast[f], (size_t)S * F * sizeof(float), "VD adjoint fields", st);
      for (int d = 0; d < 2; ++d) {
        const long long w = d == 0 ? vd->xs : vd->zs;
        dev_alloc(vd->axi[d], (size_t)S * w * sizeof(float), "VD adjoint memory variables", st);
        dev_alloc(vd->apsi[d], (size_t)S * w * sizeof(float), "VD adjoint memory variables", st);
      }
      vd->slots.release();
      vd->ck.release();
      vd->acc.release();
    }
    vd->cap = S;
  }
  if (vd->precision == 1 && vd->hp_cap < vd->cap) {
    for (DevMem* m : {&vd->plo, &vd->vxl, &vd->vzl})
      dev_alloc(*m, (size_t)vd->cap * F * sizeof(float), "VD low parts", st);
    for (int d = 0; d < 2; ++d) {
      const long long w = d == 0 ? vd->xs : vd->zs;
      dev_alloc(vd->xi64[d], (size_t)vd->cap * w * sizeof(double), "VD memory variables (FP64)", st);
      dev_alloc(vd->psi64[d], (size_t)vd->cap * w * sizeof(double), "VD memory variables (FP64)", st);
    }
    vd->hp_cap = vd->cap;
  }
  if (grad) {
    const int K = vd->gp.check_freq;
    const size_t cap = (size_t)vd->cap;
    // the slots' padding must stay zero: allocated zeroed, and no kernel writes outside the nodes
    const size_t slot_b = (size_t)(K + 1) * cap * F * sizeof(float);
    if (vd->slots.bytes < slot_b) dev_alloc(vd->slots, slot_b, "VD pressure slots", st);
    const size_t ck_b = (size_t)std::max(checkpoints_needed(vd, max_nt), 1) *
                        (3 * cap * F + 2 * cap * (vd->xs + vd->zs)) * sizeof(float);
    if (vd->ck.bytes < ck_b) dev_alloc(vd->ck, ck_b, "VD checkpoints", st);
    const size_t acc_b = cap * 3 * F * sizeof(float);
    if (vd->acc.bytes < acc_b) dev_alloc(vd->acc, acc_b, "VD window sums", st);
    const size_t tot_b = (size_t)ngroups * 3 * F * sizeof(double);
    if (vd->tot.bytes < tot_b) dev_alloc(vd->tot, tot_b, "VD gradient totals", st);
  }
}

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

// unique points of an index table, CSR over the items that share a point (in item order)
void unique_points(const sw_acoustic_vd* vd, const int32_t* idx, int count, std::vector<long long>& lin,
                   std::vector<int>& ptr, std::vector<int>& ids) {
  std::map<long long, std::vector<int>> pts;
  std::vector<long long> order;
  for (int k = 0; k < count; ++k) {
    const long long c = vd->g.lin(idx[k], idx[k + count]);
    auto it = pts.find(c);
    if (it == pts.end()) {
      order.push_back(c);
      pts[c] = {};
    }
    pts[c].push_back(k);
  }
  lin.clear();
  ptr.assign(1, 0);
  ids.clear();
  for (long long c : order) {
    lin.push_back(c);
    for (int k : pts[c]) ids.push_back(k);
    ptr.push_back((int)ids.size());
  }
}

void build_tables(sw_acoustic_vd* vd, const sw_acoustic_shot* shots, const std::vector<HostShot>& group,
                  bool on_device, bool grad, std::vector<ShotDesc>& desc) {
  cudaStream_t st = vd->ctx->stream;
  const int S = (int)group.size();
  Pools P;
  struct Off {
    size_t sp_lin, sp_ptr, sp_ids, rp_lin, rp_ptr, rp_ids, rec_lin, mask;
    int nsp, nrp;
    bool has_mask;
  };
  std::vector<Off> offs(S);
  long long tf_total = 0, tr_total = 0;
  std::vector<long long> tf_off(S), tr_off(S);
  for (int k = 0; k < S; ++k) {
    const sw_acoustic_shot& s = shots[group[k].orig];
    tf_off[k] = tf_total;
    tf_total += round_up((long long)s.nt * s.nsrc, 4);
    tr_off[k] = tr_total;
    tr_total += round_up((long long)s.nt * s.nrec, 4);
  }
  for (int k = 0; k < S; ++k) {
    const sw_acoustic_shot& s = shots[group[k].orig];
    Off& o = offs[k];
    std::vector<long long> lin;
    std::vector<int> ptr, ids;
    unique_points(vd, s.src_idx, s.nsrc, lin, ptr, ids);
    o.nsp = (int)lin.size();
    o.sp_lin = Pools::put(P.ll, lin);
    o.sp_ptr = Pools::put(P.in, ptr);
    o.sp_ids = Pools::put(P.in, ids);
    unique_points(vd, s.rec_idx, s.nrec, lin, ptr, ids);
    o.nrp = (int)lin.size();
    o.rp_lin = Pools::put(P.ll, lin);
    o.rp_ptr = Pools::put(P.in, ptr);
    o.rp_ids = Pools::put(P.in, ids);
    std::vector<long long> rl(s.nrec);
    for (int r = 0; r < s.nrec; ++r) rl[r] = vd->g.lin(s.rec_idx[r], s.rec_idx[r + s.nrec]);
    o.rec_lin = Pools::put(P.ll, rl);
    o.has_mask = grad && s.nwin > 0;
    if (o.has_mask) {
      std::vector<float> mask(s.nt, 0.0f);
      for (int w = 0; w < s.nwin; ++w)
        for (int t = s.windows[2 * w] - 1; t <= s.windows[2 * w + 1] - 1; ++t) mask[t] = 1.0f;
      o.mask = Pools::put(P.fl, mask);
    }
  }
  upload(vd, vd->d_ll, P.ll, "VD tables");
  upload(vd, vd->d_int, P.in, "VD tables");
  upload(vd, vd->d_flt, P.fl, "VD tables");
  ensure(vd, vd->d_tf, (size_t)std::max<long long>(tf_total, 4) * sizeof(float), "source time functions");
  ensure(vd, vd->d_tr, (size_t)std::max<long long>(tr_total, 4) * sizeof(float), "traces");
  if (grad) {
    ensure(vd, vd->d_obs, (size_t)tr_total * sizeof(float), "observed traces");
    ensure(vd, vd->d_adj, (size_t)tr_total * sizeof(float), "adjoint sources");
  }
  long long icd_total = 0, dres_total = 0, ic_total = 0;
  std::vector<long long> ic_off(S, -1);
  for (int k = 0; k < S; ++k) {
    const sw_acoustic_shot& s = shots[group[k].orig];
    if (grad && s.invcov && s.misfit_kind == 0) {
      icd_total += (long long)s.nt * s.nt;
      dres_total += (long long)s.nt * s.nrec;
    } else if (grad && s.invcov_diag) {
      ic_off[k] = ic_total;
      ic_total += round_up(s.nt, 4);
    }
  }
  if (dres_total) {
    if (!on_device) ensure(vd, vd->d_icd, icd_total * sizeof(float), "dense inverse covariance");
    ensure(vd, vd->d_dres, 2 * dres_total * sizeof(float), "dense residuals");
  }
  if (ic_total) ensure(vd, vd->d_ic, (size_t)ic_total * sizeof(float), "inverse covariance");
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  std::vector<float> cps(S * (size_t)vd->cps);
  std::vector<double> cps64(vd->precision == 1 ? S * (size_t)vd->cps : 0);
  for (int k = 0; k < S; ++k) {
    const sw_acoustic_shot& s = shots[group[k].orig];
    check_cuda(cudaMemcpyAsync(vd->d_tf.as<float>() + tf_off[k], s.srctf, (size_t)s.nt * s.nsrc * sizeof(float), kind, st),
               "srctf upload");
    if (grad) {
      check_cuda(cudaMemcpyAsync(vd->d_obs.as<float>() + tr_off[k], s.observed, (size_t)s.nt * s.nrec * sizeof(float),
                                 kind, st), "observed upload");
      if (ic_off[k] >= 0)
        check_cuda(cudaMemcpyAsync(vd->d_ic.as<float>() + ic_off[k], s.invcov_diag, s.nt * sizeof(float), kind, st),
                   "invcov upload");
    }
    std::copy(s.cpml, s.cpml + vd->cps, cps.begin() + (size_t)k * vd->cps);
    if (vd->precision == 1)  // FP64 coefficients of the compensated forward (the FP32 ones widened if absent)
      for (int q = 0; q < vd->cps; ++q) cps64[(size_t)k * vd->cps + q] = s.cpml64 ? s.cpml64[q] : (double)s.cpml[q];
  }
  upload(vd, vd->d_cp, cps, "C-PML coefficients");
  if (vd->precision == 1) upload(vd, vd->d_cp64, cps64, "C-PML coefficients (FP64)");
  check_cuda(cudaMemsetAsync(vd->d_tr.p, 0, (size_t)std::max<long long>(tr_total, 4) * sizeof(float), st), "traces clear");
  const long long* LL = vd->d_ll.as<long long>();
  const int* IN = vd->d_int.as<int>();
  const float* FL = vd->d_flt.as<float>();
  desc.assign(S, ShotDesc{});
  long long icd_o = 0, dres_o = 0;
  for (int k = 0; k < S; ++k) {
    const sw_acoustic_shot& s = shots[group[k].orig];
    const Off& o = offs[k];
    ShotDesc& D = desc[k];
    D.nt = s.nt;
    D.nsrc = s.nsrc;
    D.nrec = s.nrec;
    D.nsp = o.nsp;
    D.nrp = o.nrp;
    D.sp_lin = LL + o.sp_lin;
    D.sp_ptr = IN + o.sp_ptr;
    D.sp_ids = IN + o.sp_ids;
    D.rp_lin = LL + o.rp_lin;
    D.rp_ptr = IN + o.rp_ptr;
    D.rp_ids = IN + o.rp_ids;
    D.rec_lin = LL + o.rec_lin;
    D.tf = vd->d_tf.as<float>() + tf_off[k];
    D.tr = vd->d_tr.as<float>() + tr_off[k];
    if (grad) {
      D.obs = vd->d_obs.as<float>() + tr_off[k];
      D.adj = vd->d_adj.as<float>() + tr_off[k];
      D.ic = ic_off[k] >= 0 ? vd->d_ic.as<float>() + ic_off[k] : nullptr;
      D.mask = o.has_mask ? FL + o.mask : nullptr;
      D.mkind = s.misfit_kind;
      if (s.invcov && s.misfit_kind == 0) {
        if (on_device) {
          D.icd = s.invcov;
        } else {
          float* cp = vd->d_icd.as<float>() + icd_o;
          check_cuda(cudaMemcpyAsync(cp, s.invcov, (size_t)s.nt * s.nt * sizeof(float), cudaMemcpyHostToDevice, st),
                     "invcov upload");
          D.icd = cp;
          icd_o += (long long)s.nt * s.nt;
        }
        D.resid = vd->d_dres.as<float>() + dres_o;
        D.cres = vd->d_dres.as<float>() + dres_total + dres_o;
        dres_o += (long long)s.nt * s.nrec;
      }
    }
  }
  upload(vd, vd->d_desc, desc, "shot descriptors");
}

void download_traces(sw_acoustic_vd* vd, const sw_acoustic_shot* shots, const std::vector<HostShot>& group,
                     const std::vector<ShotDesc>& desc, bool on_device) {
  for (size_t k = 0; k < group.size(); ++k) {
    const sw_acoustic_shot& s = shots[group[k].orig];
    check_cuda(cudaMemcpyAsync(s.traces, desc[k].tr, (size_t)s.nt * s.nrec * sizeof(float),
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, vd->ctx->stream),
               "traces download");
  }
}

int active_count(const std::vector<HostShot>& g, int it) {
  int a = 0;
  while (a < (int)g.size() && g[a].nt >= it) ++a;
  return a;
}

std::vector<HostShot> sorted_order(int nshots, const sw_acoustic_shot* shots) {
  std::vector<HostShot> order(nshots);
  for (int k = 0; k < nshots; ++k) order[k] = HostShot{k, shots[k].nt};
  std::stable_sort(order.begin(), order.end(), [](const HostShot& a, const HostShot& b) { return a.nt > b.nt; });
  return order;
}

std::vector<std::vector<HostShot>> plan_groups(sw_acoustic_vd* vd, const std::vector<HostShot>& order, bool grad) {
  size_t free_b = 0, total_b = 0;
  check_cuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
  size_t owned = vd->slots.bytes + vd->ck.bytes + vd->acc.bytes + vd->tot.bytes;
  for (int f = 0; f < 3; ++f) owned += vd->st[f].bytes + vd->ast[f].bytes;
  for (int d = 0; d < 2; ++d) owned += vd->xi[d].bytes + vd->psi[d].bytes + vd->axi[d].bytes + vd->apsi[d].bytes;
  const double budget = 0.85 * (double)(free_b + owned);
  std::vector<std::vector<HostShot>> groups;
  size_t i = 0;
  while (i < order.size()) {
    const size_t per = per_shot_bytes(vd, grad, order[i].nt);
    size_t cnt = (size_t)std::max(1.0, std::floor(budget / (double)per));
    cnt = std::min(cnt, order.size() - i);
    groups.emplace_back(order.begin() + i, order.begin() + i + cnt);
    i += cnt;
  }
  return groups;
}

void zero_state(sw_acoustic_vd* vd, int S, bool adjoint) {
  cudaStream_t st = vd->ctx->stream;
  DevMem* f = adjoint ? vd->ast : vd->st;
  for (int k = 0; k < 3; ++k)
    check_cuda(cudaMemsetAsync(f[k].p, 0, (size_t)S * vd->g.F * sizeof(float), st), "state clear");
  if (!adjoint && vd->precision == 1) {
    for (DevMem* m : {&vd->plo, &vd->vxl, &vd->vzl})
      check_cuda(cudaMemsetAsync(m->p, 0, (size_t)S * vd->g.F * sizeof(float), st), "low parts clear");
    for (int d = 0; d < 2; ++d) {
      const long long w = d == 0 ? vd->xs : vd->zs;
      check_cuda(cudaMemsetAsync(vd->xi64[d].p, 0, (size_t)S * w * sizeof(double), st), "xi clear");
      check_cuda(cudaMemsetAsync(vd->psi64[d].p, 0, (size_t)S * w * sizeof(double), st), "psi clear");
    }
  }
  for (int d = 0; d < 2; ++d) {
    const long long w = d == 0 ? vd->xs : vd->zs;
    check_cuda(cudaMemsetAsync((adjoint ? vd->axi : vd->xi)[d].p, 0, (size_t)S * w * sizeof(float), st), "xi clear");
    check_cuda(cudaMemsetAsync((adjoint ? vd->apsi : vd->psi)[d].p, 0, (size_t)S * w * sizeof(float), st), "psi clear");
  }
}

template <int TZ>
void launch_p_tz(const sw_acoustic_vd* vd, cudaStream_t st, const PArgs& a, int S, bool corr) {
  const dim3 grid((vd->g.nx + 511) / 512, (vd->g.nz + TZ - 1) / TZ, S);
  if (corr) k_vd_p<TZ, true><<<grid, BX, 0, st>>>(a);
  else k_vd_p<TZ, false><<<grid, BX, 0, st>>>(a);
  check_cuda(cudaGetLastError(), "pressure update launch");
}
template <int TZ>
void launch_v_tz(const sw_acoustic_vd* vd, cudaStream_t st, const VArgs& a, int S) {
  const dim3 grid((vd->g.nx + 511) / 512, (vd->g.nz + TZ - 1) / TZ, S);
  k_vd_v<TZ><<<grid, BX, 0, st>>>(a);
  check_cuda(cudaGetLastError(), "velocity update launch");
}

struct Run {
  sw_acoustic_vd* vd;
  cudaStream_t st;
  const ShotDesc* ddesc;

  PArgs pargs(bool adjoint, const float* pin, float* pout) const {
    PArgs a{};
    a.g = vd->g;
    DevMem* f = adjoint ? vd->ast : vd->st;
    a.vx = f[1].as<float>();
    a.vz = f[2].as<float>();
    a.pin = pin;
    a.pout = pout;
    a.xi_x = (adjoint ? vd->axi : vd->xi)[0].as<float>();
    a.xi_z = (adjoint ? vd->axi : vd->xi)[1].as<float>();
    a.xs = vd->xs;
    a.zs = vd->zs;
    a.m0 = vd->m0.as<float>();
    a.cp = vd->d_cp.as<float>();
    a.cps = vd->cps;
    a.idt = (float)(1.0 / vd->prm.dt);
    return a;
  }
  VArgs vargs(bool adjoint, const float* p) const {
    VArgs a{};
    a.g = vd->g;
    DevMem* f = adjoint ? vd->ast : vd->st;
    a.p = p;
    a.vx = f[1].as<float>();
    a.vz = f[2].as<float>();
    a.psi_x = (adjoint ? vd->apsi : vd->psi)[0].as<float>();
    a.psi_z = (adjoint ? vd->apsi : vd->psi)[1].as<float>();
    a.xs = vd->xs;
    a.zs = vd->zs;
    a.m1x = vd->m1x.as<float>();
    a.m1z = vd->m1z.as<float>();
    a.cp = vd->d_cp.as<float>();
    a.cps = vd->cps;
    return a;
  }
  void launch_p(const PArgs& a, int S, bool corr) const {
    if (vd->tz == 16) launch_p_tz<16>(vd, st, a, S, corr);
    else if (vd->tz == 32) launch_p_tz<32>(vd, st, a, S, corr);
    else launch_p_tz<8>(vd, st, a, S, corr);
  }
  void launch_v(const VArgs& a, int S) const {
    if (vd->tz == 16) launch_v_tz<16>(vd, st, a, S);
    else if (vd->tz == 32) launch_v_tz<32>(vd, st, a, S);
    else launch_v_tz<8>(vd, st, a, S);
  }
  // algorithmic bytes per node and shot: pressure R vx vz p, W p (16); velocity
  // R p vx vz, W vx vz (20); shared by the shots: fact_m0, fact_m1 x2 (12)
  double fwd_bytes(int S) const { return (double)vd->g.nx * vd->g.nz * (S * 36.0 + 12.0); }
  // adjoint: the same 36 plus the correlation R pc po (8) and the window sums' R/W (24)
  double adj_bytes(int S) const { return (double)vd->g.nx * vd->g.nz * (S * 68.0 + 12.0); }

  // forward_onestep_CPML!: p (pin -> pout), injection + recording, velocities
  HArgs hargs(const float* pin, float* pout) const {
    HArgs a{};
    a.g = vd->g;
    a.pin = pin;
    a.pout = pout;
    a.plo = vd->plo.as<float>();
    a.vx = vd->st[1].as<float>();
    a.vz = vd->st[2].as<float>();
    a.vxl = vd->vxl.as<float>();
    a.vzl = vd->vzl.as<float>();
    a.xi_x = vd->xi64[0].as<double>();
    a.xi_z = vd->xi64[1].as<double>();
    a.psi_x = vd->psi64[0].as<double>();
    a.psi_z = vd->psi64[1].as<double>();
    a.xs = vd->xs;
    a.zs = vd->zs;
    a.m0 = vd->m0.as<float>();
    a.m0l = vd->m0l.as<float>();
    a.m1x = vd->m1x.as<float>();
    a.m1xl = vd->m1xl.as<float>();
    a.m1z = vd->m1z.as<float>();
    a.m1zl = vd->m1zl.as<float>();
    a.cp = vd->d_cp64.as<double>();
    a.cps = vd->cps;
    const double ix = 1.0 / vd->prm.h[0], iz = 1.0 / vd->prm.h[1];
    a.idxl = (float)(ix - (double)(float)ix);
    a.idzl = (float)(iz - (double)(float)iz);
    return a;
  }
  // compensated forward_onestep_CPML! (k_vd_p_hp, injection with low parts, k_vd_v_hp)
  void forward_step_hp(int S, int it, const float* pin, float* pout, bool record, int kind) const {
    const HArgs a = hargs(pin, pout);
    const int TZ = 8;
    const dim3 grid((vd->g.nx + 511) / 512, (vd->g.nz + TZ - 1) / TZ, S);
    cudaEvent_t ev = nullptr;
    vd->ctx->prof.begin(st, kind, fwd_bytes(S) + hp_extra_bytes(S), &ev);
    k_vd_p_hp<TZ><<<grid, BX, 0, st>>>(a);
    check_cuda(cudaGetLastError(), "compensated pressure update launch");
    vd->ctx->prof.end(st, kind, ev);
    vd->ctx->prof.begin(st, KK_SRCREC, 0.0, &ev);
    k_vd_srcrec<<<S, 128, 0, st>>>(ddesc, it, vd->g.F, pout, record ? 1 : 0, vd->plo.as<float>());
    check_cuda(cudaGetLastError(), "injection launch");
    vd->ctx->prof.end(st, KK_SRCREC, ev);
    vd->ctx->prof.begin(st, kind, 0.0, &ev);
    k_vd_v_hp<TZ><<<grid, BX, 0, st>>>(a);
    check_cuda(cudaGetLastError(), "compensated velocity update launch");
    vd->ctx->prof.end(st, kind, ev);
  }
  // extra bytes of the compensated step per node and shot: R/W the low parts of p, vx, vz (24),
  // R the low parts of the factors once (12)
  double hp_extra_bytes(int S) const { return (double)vd->g.nx * vd->g.nz * (S * 24.0 + 12.0); }

  void forward_step(int S, int it, const float* pin, float* pout, bool record, int kind) const {
    if (S <= 0) return;
    if (vd->precision == 1 && kind == KK_STENCIL) {  // the forward pass (the recompute stays FP32)
      forward_step_hp(S, it, pin, pout, record, kind);
      return;
    }
    cudaEvent_t ev = nullptr;
    vd->ctx->prof.begin(st, kind, fwd_bytes(S), &ev);
    launch_p(pargs(false, pin, pout), S, false);
    vd->ctx->prof.end(st, kind, ev);
    vd->ctx->prof.begin(st, KK_SRCREC, 0.0, &ev);
    k_vd_srcrec<<<S, 128, 0, st>>>(ddesc, it, vd->g.F, pout, record ? 1 : 0, nullptr);
    check_cuda(cudaGetLastError(), "injection launch");
    vd->ctx->prof.end(st, KK_SRCREC, ev);
    vd->ctx->prof.begin(st, kind, 0.0, &ev);
    launch_v(vargs(false, pout), S);
    vd->ctx->prof.end(st, kind, ev);
  }
  // adjoint_onestep_CPML! + correlations: velocities, p with the fused
  // correlation, adjoint injection at the receivers
  void adjoint_step(int S, int it, const float* pc, const float* po) const {
    if (S <= 0) return;
    float* ap = vd->ast[0].as<float>();
    cudaEvent_t ev = nullptr;
    vd->ctx->prof.begin(st, KK_ADJOINT, adj_bytes(S), &ev);
    launch_v(vargs(true, ap), S);
    PArgs a = pargs(true, ap, ap);
    a.pc = pc;
    a.po = po;
    a.acc = vd->acc.as<float>();
    launch_p(a, S, true);
    vd->ctx->prof.end(st, KK_ADJOINT, ev, 2);
    vd->ctx->prof.begin(st, KK_SRCREC, 0.0, &ev);
    k_vd_adjinj<<<S, 128, 0, st>>>(ddesc, it, vd->g.F, ap, pc, po, vd->acc.as<float>(), a.idt);
    check_cuda(cudaGetLastError(), "adjoint injection launch");
    vd->ctx->prof.end(st, KK_SRCREC, ev);
  }
};

long long snapshot_floats(const sw_acoustic_vd* vd) {
  const long long nx = vd->g.nx, nz = vd->g.nz;
  return nx * nz + (nx - 1) * nz + nx * (nz - 1);
}

void save_snapshots(sw_acoustic_vd* vd, const std::vector<HostShot>& group, int A, int it) {
  const long long B = snapshot_floats(vd);
  cudaStream_t st = vd->ctx->stream;
  ensure(vd, vd->d_snap, (size_t)vd->cap * B * sizeof(float), "snapshot stage");
  const dim3 grid((unsigned)std::min<long long>((B + 255) / 256, 1024), A);
  k_vd_snapshot<<<grid, 256, 0, st>>>(vd->g, vd->st[0].as<float>(), vd->st[1].as<float>(), vd->st[2].as<float>(), B,
                                      vd->d_snap.as<float>());
  check_cuda(cudaGetLastError(), "snapshot launch");
  for (int k = 0; k < A; ++k) {
    float* dst = vd->snap_out[group[k].orig] + (long long)(it / vd->snapevery - 1) * B;
    check_cuda(cudaMemcpyAsync(dst, vd->d_snap.as<float>() + (long long)k * B, (size_t)B * sizeof(float),
                               cudaMemcpyDefault, st),
               "snapshot copy");
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Entry points used by api.cu
// ---------------------------------------------------------------------------
namespace swgb {

void vd_init(sw_acoustic_vd* vd, sw_ctx* ctx, const sw_acoustic_params* p, int interp, int gradient,
             const sw_grad_params* gp) {
  if (!p) fail(SW_ERR_ARG, "params is NULL");
  if (p->ndim != 2) fail(SW_ERR_UNSUPPORTED, "the variable-density path of this backend is 2D");
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
    if (p->n[d] < 4) fail(SW_ERR_UNSUPPORTED, "the 4th-order staggered stencil needs at least 4 points per axis");
  }
  if (interp < 0 || interp > 1) fail(SW_ERR_ARG, "interpolation method must be 0 (arithmetic) or 1 (harmonic)");
  vd->ctx = ctx;
  vd->prm = *p;
  vd->interp = interp;
  vd->gradient = gradient != 0;
  if (vd->gradient) {
    vd->gp = gp ? *gp : sw_grad_params{1, 0, 0, 0, 0};
    if (vd->gp.check_freq < 1) fail(SW_ERR_ARG, "check_freq must be positive");
    if (vd->gp.mute_radius_src < 0 || vd->gp.mute_radius_rec < 0)
      fail(SW_ERR_ARG, "mutearoundpoint!(): The smoothing radius must be positive.");
    if (vd->gp.snapshot_bf16)
      fail(SW_ERR_UNSUPPORTED, "BF16 checkpoint snapshots are not available for the variable-density path");
  }
  Geo& g = vd->g;
  g.nx = p->n[0];
  g.nz = p->n[1];
  g.halo = p->halo;
  g.P = (int)round_up(g.nx + XPAD + 8, 32);  // the kernels read up to column nx + 38
  g.F = (long long)g.P * (g.nz + 2 * ZPAD);
  g.W = (int)round_up(2 * g.halo + 2, 4);
  g.idx = (float)(1.0 / p->h[0]);
  g.idz = (float)(1.0 / p->h[1]);
  vd->na = 2 * g.halo + 2;
  vd->nh = 2 * g.halo;
  vd->cps = 2 * (2 * vd->na + 2 * vd->nh);
  vd->xs = round_up((long long)g.nz * g.W, 32);
  vd->zs = round_up((long long)(2 * g.halo + 2) * g.P, 32);
  const size_t F = (size_t)g.F;
  for (DevMem* m : {&vd->m0, &vd->m1x, &vd->m1z}) dev_alloc(*m, F * sizeof(float), "VD material", ctx->stream);
  dev_alloc(vd->vp_d, (size_t)g.nx * g.nz * sizeof(double), "vp", ctx->stream);
  dev_alloc(vd->rho_d, (size_t)g.nx * g.nz * sizeof(double), "rho", ctx->stream);
}

void vd_upload_low(sw_acoustic_vd* vd) {
  cudaStream_t st = vd->ctx->stream;
  const size_t F = (size_t)vd->g.F;
  for (DevMem* m : {&vd->m0l, &vd->m1xl, &vd->m1zl})
    if (!m->p) dev_alloc(*m, F * sizeof(float), "VD material low parts", st);
  check_cuda(cudaMemcpyAsync(vd->m0l.p, vd->m0l_h.data(), F * sizeof(float), cudaMemcpyHostToDevice, st), "upload");
  check_cuda(cudaMemcpyAsync(vd->m1xl.p, vd->m1xl_h.data(), F * sizeof(float), cudaMemcpyHostToDevice, st), "upload");
  check_cuda(cudaMemcpyAsync(vd->m1zl.p, vd->m1zl_h.data(), F * sizeof(float), cudaMemcpyHostToDevice, st), "upload");
  check_cuda(cudaStreamSynchronize(st), "material upload");
}

void vd_set_precision(sw_acoustic_vd* vd, int mode) {
  vd->precision = mode;
  if (mode == 1 && vd->has_mat) vd_upload_low(vd);
}

// update_matprop! + precompute_fact! (acou_models.jl:273-300); T = float or double
template <typename T>
void vd_set_material_t(sw_acoustic_vd* vd, const T* vp, const T* rho) {
  if (!vp || !rho) fail(SW_ERR_ARG, "vp and rho are required");
  const Geo& g = vd->g;
  const long long np = (long long)g.nx * g.nz;
  for (long long c = 0; c < np; ++c) {
    if (!(vp[c] > 0)) fail(SW_ERR_ARG, "Pressure velocity material property must be positive!");
    if (!(rho[c] > 0)) fail(SW_ERR_ARG, "Density material property must be positive!");
  }
  auto M = [&](int i, int j) { return (size_t)(i - 1) + (size_t)(j - 1) * g.nx; };
  std::vector<float> m0(g.F, 0.0f), mx(g.F, 0.0f), mz(g.F, 0.0f);
  vd->m0l_h.assign(g.F, 0.0f);  // low parts of the factors (compensated forward)
  vd->m1xl_h.assign(g.F, 0.0f);
  vd->m1zl_h.assign(g.F, 0.0f);
  auto split = [](double v, float& hi, float& lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
  };
  std::vector<double> vpd(np), rd(np);
  const double dt = vd->prm.dt;
  // 1/rho at a half point: arithmetic mean of 1/rho, or its harmonic mean (= 1 / mean of rho)
  auto m1 = [&](size_t a, size_t b) {
    return vd->interp == 1 ? 2.0 / ((double)rho[a] + (double)rho[b]) : 0.5 * (1.0 / rho[a] + 1.0 / rho[b]);
  };
  for (int j = 1; j <= g.nz; ++j)
    for (int i = 1; i <= g.nx; ++i) {
      const size_t c = M(i, j);
      const long long q = g.lin(i, j);
      vpd[c] = vp[c];
      rd[c] = rho[c];
      split((double)vp[c] * vp[c] * rho[c] * dt, m0[q], vd->m0l_h[q]);
      if (i <= g.nx - 1) split(m1(c, M(i + 1, j)) * dt, mx[q], vd->m1xl_h[q]);
      if (j <= g.nz - 1) split(m1(c, M(i, j + 1)) * dt, mz[q], vd->m1zl_h[q]);
    }
  cudaStream_t st = vd->ctx->stream;
  auto up = [&](DevMem& m, const void* src, size_t bytes) {
    check_cuda(cudaMemcpyAsync(m.p, src, bytes, cudaMemcpyHostToDevice, st), "material upload");
  };
  up(vd->m0, m0.data(), m0.size() * sizeof(float));
  up(vd->m1x, mx.data(), mx.size() * sizeof(float));
  up(vd->m1z, mz.data(), mz.size() * sizeof(float));
  up(vd->vp_d, vpd.data(), vpd.size() * sizeof(double));
  up(vd->rho_d, rd.data(), rd.size() * sizeof(double));
  check_cuda(cudaStreamSynchronize(st), "material upload");
  vd->has_mat = true;
  if (vd->precision == 1) vd_upload_low(vd);
}
void vd_set_material(sw_acoustic_vd* vd, const float* vp, const float* rho) { vd_set_material_t(vd, vp, rho); }
void vd_set_material64(sw_acoustic_vd* vd, const double* vp, const double* rho) { vd_set_material_t(vd, vp, rho); }

void vd_forward(sw_acoustic_vd* vd, int nshots, const sw_acoustic_shot* shots, bool on_device) {
  if (!vd->has_mat) fail(SW_ERR_STATE, "material properties not set (sw_acoustic_vd_set_material)");
  if (nshots < 1 || !shots) fail(SW_ERR_ARG, "no shots");
  for (int k = 0; k < nshots; ++k) validate_shot(vd, shots[k], k, false);
  const std::vector<HostShot> order = sorted_order(nshots, shots);
  for (const auto& group : plan_groups(vd, order, false)) {
    const int S = (int)group.size();
    ensure_state(vd, S, false, group.front().nt, 1);
    std::vector<ShotDesc> desc;
    build_tables(vd, shots, group, on_device, false, desc);
    Run R{vd, vd->ctx->stream, vd->d_desc.as<ShotDesc>()};
    zero_state(vd, S, false);
    float* p = vd->st[0].as<float>();
    for (int it = 1; it <= group.front().nt; ++it) {
      const int A = active_count(group, it);
      R.forward_step(A, it, p, p, true, KK_STENCIL);
      if (vd->snapevery > 0 && it % vd->snapevery == 0) save_snapshots(vd, group, A, it);
    }
    download_traces(vd, shots, group, desc, on_device);
  }
  check_cuda(cudaStreamSynchronize(vd->ctx->stream), "VD forward");
  vd->ctx->prof.resolve();
}

void vd_forward_snapshots(sw_acoustic_vd* vd, int nshots, const sw_acoustic_shot* shots, bool on_device, int snapevery,
                          float* const* snapshots) {
  if (snapevery < 1 || !snapshots) fail(SW_ERR_ARG, "snapevery must be positive and snapshots non-NULL");
  for (int k = 0; k < nshots; ++k) {
    if (shots && snapevery >= shots[k].nt)
      fail(SW_ERR_ARG, "Checkpointing frequency must be smaller than the number of timesteps!");
    if (!snapshots[k]) fail(SW_ERR_ARG, "snapshot buffer is NULL");
  }
  vd->snapevery = snapevery;
  vd->snap_out = snapshots;
  try {
    vd_forward(vd, nshots, shots, on_device);
  } catch (...) {
    vd->snapevery = 0;
    vd->snap_out = nullptr;
    throw;
  }
  vd->snapevery = 0;
  vd->snap_out = nullptr;
}

void vd_gradient(sw_acoustic_vd* vd, int nshots, const sw_acoustic_shot* shots, bool on_device, double* g_vp,
                 double* g_rho, double* misfit) {
  if (!vd->gradient)
    fail(SW_ERR_STATE, "The wavesim object was not built for gradient computations. (Was `gradient=true` specified?)");
  if (!vd->has_mat) fail(SW_ERR_STATE, "material properties not set (sw_acoustic_vd_set_material)");
  if (nshots < 1 || !shots) fail(SW_ERR_ARG, "no shots");
  if (!g_vp || !g_rho) fail(SW_ERR_ARG, "gradient outputs are NULL");
  for (int k = 0; k < nshots; ++k) validate_shot(vd, shots[k], k, true);
  const bool mute = vd->gp.mute_radius_src > 0 || vd->gp.mute_radius_rec > 0;
  if (mute)
    for (int k = 0; k < nshots; ++k) {
      const sw_acoustic_shot& s = shots[k];
      if ((vd->gp.mute_radius_src > 0 && !s.src_pos) || (vd->gp.mute_radius_rec > 0 && !s.rec_pos))
        fail(SW_ERR_ARG, "muting needs src_pos / rec_pos");
    }
  cudaStream_t st = vd->ctx->stream;
  const Geo& g = vd->g;
  const long long np = (long long)g.nx * g.nz;
  const long long F = g.F;
  const int K = vd->gp.check_freq;
  DevMem dout, dmis;
  double* out[2] = {g_vp, g_rho};
  double* mout = misfit;
  if (!on_device) {
    dev_alloc(dout, (size_t)2 * np * sizeof(double), "gradient output", st);
    for (int q = 0; q < 2; ++q) out[q] = dout.as<double>() + q * np;
  }
  if (!on_device || !mout) {
    dev_alloc(dmis, sizeof(double), "misfit output", st);
    mout = dmis.as<double>();
  }
  const std::vector<HostShot> order = sorted_order(nshots, shots);
  bool first_group = true;
  for (const auto& group : plan_groups(vd, order, true)) {
    const int S = (int)group.size();
    const int ntmax = group.front().nt;
    const int gsize = mute ? 1 : S;
    const int ngroups = (S + gsize - 1) / gsize;
    ensure_state(vd, S, true, ntmax, ngroups);
    std::vector<ShotDesc> desc;
    build_tables(vd, shots, group, on_device, true, desc);
    Run R{vd, st, vd->d_desc.as<ShotDesc>()};
    const int cap = vd->cap;
    auto slot = [&](int k) { return vd->slots.as<float>() + (size_t)k * cap * F; };
    const int M = (ntmax + K - 1) / K;  // windows m = 0 .. M-1: steps mK+1 .. min((m+1)K, ntmax)
    const size_t ckF = (size_t)3 * cap * F;
    const size_t ckS = (size_t)2 * cap * (vd->xs + vd->zs);
    auto ck_base = [&](int m) { return vd->ck.as<float>() + (size_t)(m - 1) * (ckF + ckS); };  // m = 1 .. M-2
    auto strip_ptrs = [&](float* b, float* ptr[4]) {
      ptr[0] = b + ckF;                                      // xi x
      ptr[1] = ptr[0] + (size_t)cap * vd->xs;                 // psi x
      ptr[2] = ptr[1] + (size_t)cap * vd->xs;                 // xi z
      ptr[3] = ptr[2] + (size_t)cap * vd->zs;                 // psi z
    };
    auto copy = [&](void* dst, const void* src, size_t bytes, const char* what) {
      check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st), what);
    };
    auto save_ck = [&](int m) {
      float* b = ck_base(m);
      for (int f = 0; f < 3; ++f) copy(b + (size_t)f * cap * F, vd->st[f].p, (size_t)S * F * sizeof(float), "checkpoint save");
      float* sp[4];
      strip_ptrs(b, sp);
      if (vd->precision == 1) {  // the compensated forward keeps FP64 memory variables
        const double* src[4] = {vd->xi64[0].as<double>(), vd->psi64[0].as<double>(), vd->xi64[1].as<double>(),
                                vd->psi64[1].as<double>()};
        for (int q = 0; q < 4; ++q) {
          const long long n = (long long)S * (q < 2 ? vd->xs : vd->zs);
          k_vd_d2f<<<(unsigned)std::min<long long>((n + 255) / 256, 1024), 256, 0, st>>>(src[q], sp[q], n);
          check_cuda(cudaGetLastError(), "checkpoint strip conversion");
        }
        return;
      }
      copy(sp[0], vd->xi[0].p, (size_t)S * vd->xs * sizeof(float), "checkpoint save");
      copy(sp[1], vd->psi[0].p, (size_t)S * vd->xs * sizeof(float), "checkpoint save");
      copy(sp[2], vd->xi[1].p, (size_t)S * vd->zs * sizeof(float), "checkpoint save");
      copy(sp[3], vd->psi[1].p, (size_t)S * vd->zs * sizeof(float), "checkpoint save");
    };
    // state after step mK: velocities and memory variables into the state, p into slot 0
    auto load_ck = [&](int m) {
      if (m == 0) {
        zero_state(vd, S, false);
        check_cuda(cudaMemsetAsync(slot(0), 0, (size_t)S * F * sizeof(float), st), "slot clear");
        return;
      }
      float* b = ck_base(m);
      copy(slot(0), b, (size_t)S * F * sizeof(float), "checkpoint load");
      for (int f = 1; f < 3; ++f) copy(vd->st[f].p, b + (size_t)f * cap * F, (size_t)S * F * sizeof(float), "checkpoint load");
      float* sp[4];
      strip_ptrs(b, sp);
      copy(vd->xi[0].p, sp[0], (size_t)S * vd->xs * sizeof(float), "checkpoint load");
      copy(vd->psi[0].p, sp[1], (size_t)S * vd->xs * sizeof(float), "checkpoint load");
      copy(vd->xi[1].p, sp[2], (size_t)S * vd->zs * sizeof(float), "checkpoint load");
      copy(vd->psi[1].p, sp[3], (size_t)S * vd->zs * sizeof(float), "checkpoint load");
    };
    // forward: in place up to the last window, then p of each step into the slots
    zero_state(vd, S, false);
    const int last_start = (M - 1) * K;
    float* p = vd->st[0].as<float>();
    for (int it = 1; it <= ntmax; ++it) {
      const int A = active_count(group, it);
      if (it < last_start) R.forward_step(A, it, p, p, true, KK_STENCIL);
      else if (it == last_start) R.forward_step(A, it, p, slot(0), true, KK_STENCIL);
      else R.forward_step(A, it, slot(it - last_start - 1), slot(it - last_start), true, KK_STENCIL);
      if (it % K == 0 && it / K <= M - 2) save_ck(it / K);
    }
    download_traces(vd, shots, group, desc, on_device);
    // misfit and prescaled adjoint sources
    const int nblk = 64;
    ensure(vd, vd->d_partial, (size_t)nblk * S * sizeof(double), "misfit partials");
    {
      bool any_dense = false;
      for (const auto& d : desc) any_dense = any_dense || d.icd;
      cudaEvent_t ev = nullptr;
      vd->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
      if (any_dense) {
        k_vd_residual_dense<<<dim3(nblk, S), 256, 0, st>>>(R.ddesc);
        check_cuda(cudaGetLastError(), "residual launch");
        for (const auto& d : desc)
          if (d.icd) dense_invcov(vd->ctx, d.nt, d.nrec, d.icd, d.resid, const_cast<float*>(d.cres));
      }
      k_vd_misfit<<<dim3(nblk, S), 256, 0, st>>>(R.ddesc, vd->m0.as<float>(), vd->d_partial.as<double>());
      check_cuda(cudaGetLastError(), "misfit launch");
      k_vd_misfit_sum<<<1, 256, 0, st>>>(vd->d_partial.as<double>(), nblk * S, mout, first_group ? 0 : 1);
      check_cuda(cudaGetLastError(), "misfit sum launch");
      // CCTS shots: misfit and adjoint source from the cross-correlation time shift
      std::vector<int> kind(S), ntv(S), nrec(S);
      std::vector<double> mdt(S);
      std::vector<const float*> tr(S), obs(S);
      std::vector<float*> adj(S);
      std::vector<const long long*> rl(S);
      for (int k = 0; k < S; ++k) {
        const sw_acoustic_shot& s = shots[group[k].orig];
        kind[k] = s.misfit_kind;
        mdt[k] = s.misfit_dt;
        ntv[k] = desc[k].nt;
        nrec[k] = desc[k].nrec;
        tr[k] = desc[k].tr;
        obs[k] = desc[k].obs;
        adj[k] = desc[k].adj;
        rl[k] = desc[k].rec_lin;
      }
      ensure(vd, vd->d_ccts, (size_t)S * sizeof(CctsShot), "CCTS table");
      size_t smem = 0;
      const int crec = upload_ccts(vd->ctx, vd->d_ccts.as<CctsShot>(), kind, mdt, ntv, nrec, tr, obs, adj, rl, &smem);
      if (crec) {
        ensure(vd, vd->d_partial2, (size_t)crec * S * sizeof(double), "CCTS partials");
        k_ccts<<<dim3(crec, S), CCTS_THREADS, smem, st>>>(vd->d_ccts.as<CctsShot>(), vd->m0.as<float>(),
                                                          vd->d_partial2.as<double>());
        check_cuda(cudaGetLastError(), "CCTS misfit launch");
        k_vd_misfit_sum<<<1, 256, 0, st>>>(vd->d_partial2.as<double>(), crec * S, mout, 1);
        check_cuda(cudaGetLastError(), "CCTS misfit sum launch");
      }
      vd->ctx->prof.end(st, KK_OTHER, ev);
    }
    // adjoint with recompute, fused correlation and window flushes
    zero_state(vd, S, true);
    check_cuda(cudaMemsetAsync(vd->acc.p, 0, (size_t)S * 3 * F * sizeof(float), st), "window sums clear");
    check_cuda(cudaMemsetAsync(vd->tot.p, 0, (size_t)ngroups * 3 * F * sizeof(double), st), "totals clear");
    const int fblocks = (int)std::min<long long>((3 * (F / 4) + 255) / 256, 8192);
    for (int m = M - 1; m >= 0; --m) {
      const int t0 = m * K + 1, t1 = std::min((m + 1) * K, ntmax);
      if (m < M - 1) {
        load_ck(m);
        for (int t = t0; t <= t1; ++t)
          R.forward_step(active_count(group, t), t, slot(t - t0), slot(t - t0 + 1), false, KK_RECOMPUTE);
      }
      for (int it = t1; it >= t0; --it) R.adjoint_step(active_count(group, it), it, slot(it - t0 + 1), slot(it - t0));
      const int Aw = active_count(group, t0);
      if (Aw > 0) {
        cudaEvent_t ev = nullptr;
        vd->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
        k_vd_flush<<<fblocks, 256, 0, st>>>(g, Aw, gsize, vd->acc.as<float>(), vd->tot.as<double>());
        check_cuda(cudaGetLastError(), "window flush launch");
        check_cuda(cudaMemsetAsync(vd->acc.p, 0, (size_t)Aw * 3 * F * sizeof(float), st), "window sums clear");
        vd->ctx->prof.end(st, KK_OTHER, ev);
      }
    }
    // mute balls per group (= per shot when muting)
    std::vector<MuteBall> balls;
    std::vector<int> bptr(1, 0);
    if (mute) {
      const double hmax = std::max(vd->prm.h[0], vd->prm.h[1]);
      for (int k = 0; k < S; ++k) {
        const sw_acoustic_shot& s = shots[group[k].orig];
        for (int fam = 0; fam < 2; ++fam) {
          const int radius = fam == 0 ? vd->gp.mute_radius_src : vd->gp.mute_radius_rec;
          if (radius <= 0) continue;
          const double* pos = fam == 0 ? s.src_pos : s.rec_pos;
          const int npos = fam == 0 ? s.nsrc : s.nrec;
          for (int q = 0; q < npos; ++q) {
            MuteBall b{};
            for (int d = 0; d < 2; ++d) {
              const double x = pos[q + (long long)d * npos], h = vd->prm.h[d];
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
      upload(vd, vd->d_balls, balls, "mute balls");
      upload(vd, vd->d_ball_ptr, bptr, "mute balls");
    }
    {
      cudaEvent_t ev = nullptr;
      vd->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
      const int blocks = (int)std::min<long long>((np + 255) / 256, 8192);
      k_vd_reduce<<<blocks, 256, 0, st>>>(g, ngroups, vd->tot.as<double>(), vd->vp_d.as<double>(), vd->rho_d.as<double>(),
                                          vd->interp, vd->prm.h[0], vd->prm.h[1],
                                          mute ? vd->d_balls.as<MuteBall>() : nullptr,
                                          mute ? vd->d_ball_ptr.as<int>() : nullptr, out[0], out[1],
                                          first_group ? 0 : 1);
      check_cuda(cudaGetLastError(), "gradient reduction launch");
      vd->ctx->prof.end(st, KK_OTHER, ev);
    }
    check_cuda(cudaStreamSynchronize(st), "VD gradient group");
    first_group = false;
  }
  if (!on_device) {
    check_cuda(cudaMemcpyAsync(g_vp, out[0], np * sizeof(double), cudaMemcpyDeviceToHost, st), "gradient download");
    check_cuda(cudaMemcpyAsync(g_rho, out[1], np * sizeof(double), cudaMemcpyDeviceToHost, st), "gradient download");
  }
  if (misfit && (!on_device || mout != misfit))
    check_cuda(cudaMemcpyAsync(misfit, mout, sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               st), "misfit download");
  check_cuda(cudaStreamSynchronize(st), "VD gradient");
  vd->ctx->prof.resolve();
}

void vd_set_tuning(sw_acoustic_vd* vd, int tz) {
  if (tz != 0 && tz != 8 && tz != 16 && tz != 32) fail(SW_ERR_ARG, "tz must be 0, 8, 16 or 32");
  vd->tz = tz == 0 ? 8 : tz;
}
sw_ctx* vd_ctx(sw_acoustic_vd* vd) { return vd->ctx; }
sw_acoustic_vd* vd_new() { return new sw_acoustic_vd(); }
void vd_delete(sw_acoustic_vd* vd) { delete vd; }

}  // namespace swgb
