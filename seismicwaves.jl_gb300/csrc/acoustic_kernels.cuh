// Device kernels of the acoustic constant-density C-PML path (2D and 3D, FP32).
//
// One launch advances every active shot of a batch by one time step.  The
// psi strip update, the C-PML Laplacian, the xi update and the pressure
// update of SeismicWaves.jl's update_psi_x!/update_psi_y!/update_p_CPML!
// (src/models/acoustic/backends/shared/acoustic2D_xPU.jl:1-46,
// acoustic3D_xPU.jl:1-61, index maps of src/utils/fdgen.jl:137-215) are fused
// into a single pass over the grid:
//
//  * psi is double-buffered (read psi_in, write psi_out): each half-node value
//    is written by exactly one point and recomputed by its neighbour, so the
//    neighbour never sees a half-updated array;
//  * xi is owned by one point and updated in place (xi_in may differ from
//    xi_out on the first step after a checkpoint restore);
//  * optional side outputs: D = fact * lap (the second time difference the
//    gradient correlates with), and a checkpoint copy of the state read;
//  * the adjoint variant also accumulates the gradient correlation
//    g += lambda * D with Kahan compensation (correlate_gradient_xPU.jl:1-10).
//
// Time stepping in increment form.  The reference advances
//     p[n+1] = 2 p[n] - p[n-1] + fact * lap(p[n]);
// here the state is (p[n], d[n] = p[n] - p[n-1]) and a step is
//     d[n+1] = d[n] + fact * lap(p[n]),   p[n+1] = p[n] + d[n+1],
// the same recurrence in exact arithmetic.  In FP32 the three-level form
// rounds p every step and feeds that rounding back as a velocity error that
// grows linearly in time (1.4e-5 relative trace error after 3000 steps on an
// 801 x 801 model, against 1e-7 once the increment is carried separately).
// p is double-buffered (the stencil reads neighbours); d is updated in place.
//
// Layout: column-major with axis 0 (x) padded to a pitch P (multiple of 32
// floats); every thread owns four consecutive x points (one float4) and
// marches along the last axis keeping three planes of p in registers.
// Boundary nodes (first and last index of every axis) are never written by
// the stencil, exactly like the reference.
#pragma once

#include "internal.h"

namespace swgb {

enum StepMode { MODE_FWD = 0, MODE_FWD_D = 1, MODE_ADJ = 2 };

struct StepArgs {
  int n0, n1, n2;  // grid points per axis (n2 = 1 in 2D; the depth axis is n1 in 2D, n2 in 3D)
  int P;           // pitch of axis 0 in floats
  int halo;
  float ih[3], ih2[3];
  FieldArg pcur, pnew, din, dout;                  // p[n] (read), p[n+1] (write), d[n] -> d[n+1]
  FieldArg psi_in[3], psi_out[3], xi_in[3], xi_out[3];
  FieldArg ck_p, ck_d, ck_psi[3], ck_xi[3];        // checkpoint outputs (p == nullptr: none)
  FieldArg Dout;                                   // MODE_FWD_D: D = fact*lap output
  int d_first;                                     // MODE_FWD_D: shots >= d_first write D
  FieldArg dcorr, g, gc;                           // MODE_ADJ
  const float* fact;                               // shared by all shots
  const float* cpml;                               // per shot: N blocks [a, a_h, b, b_h]
  int cpml_stride;
  int nshots;
  int tiles_x, tiles_y, tiles_z, TZ;
};

struct StripIO {
  const float* psi_in;
  float* psi_out;
  float* ck_psi;
  const float* xi_in;
  float* xi_out;
  float* ck_xi;
  long long psi_base, psi_step, xi_base, xi_step;
  const float* a;
  const float* ah;
  const float* b;
  const float* bh;
};

__device__ __forceinline__ void ld4(float (&v)[4], const float* p) {
  const float4 t = __ldg(reinterpret_cast<const float4*>(p));
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ld4rw(float (&v)[4], const float* p) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void st4(float* p, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}

// Kahan-compensated g += y (compensation c holds the running rounding error;
// the sum is g - c).  Explicit round-to-nearest intrinsics keep the compiler
// from contracting or reassociating the compensation.
__device__ __forceinline__ void kahan_add(float& g, float& c, float y) {
  const float yy = __fsub_rn(y, c);
  const float t = __fadd_rn(g, yy);
  c = __fsub_rn(__fsub_rn(t, g), yy);
  g = t;
}

// C-PML term of one axis at point x (0-based) along an axis of n points.
// Without damping the term is d2 (the plain second derivative).  In a strip
// the two half-node memory variables psi around x are advanced (psi_out), the
// on-node variable xi is advanced, and d2 + dpsi + xi is returned.
__device__ __forceinline__ float cpml_axis_term(float d2, float pl, float p0, float pr, int x, int n,
                                                int halo, float ih, const StripIO& s) {
  int qr;
  bool first;
  if (x < halo) {
    qr = x;
    first = (x == 1);
  } else if (x >= n - halo) {
    qr = x + 1 - n + 2 * halo;
    first = (x == n - halo);
  } else {
    return d2;
  }
  const int ql = qr - 1;
  const long long il = s.psi_base + (long long)ql * s.psi_step;
  const long long ir = s.psi_base + (long long)qr * s.psi_step;
  const float oldl = s.psi_in[il];
  const float oldr = s.psi_in[ir];
  const float newl = s.bh[ql] * oldl + s.ah[ql] * ((p0 - pl) * ih);
  const float newr = s.bh[qr] * oldr + s.ah[qr] * ((pr - p0) * ih);
  s.psi_out[ir] = newr;
  if (s.ck_psi) s.ck_psi[ir] = oldr;
  if (first) {
    s.psi_out[il] = newl;
    if (s.ck_psi) s.ck_psi[il] = oldl;
  }
  const float dpsi = (newr - newl) * ih;
  const long long iq = s.xi_base + (long long)qr * s.xi_step;
  const float xo = s.xi_in[iq];
  if (s.ck_xi) s.ck_xi[iq] = xo;
  const float t = d2 + dpsi;
  const float xn = s.b[qr] * xo + s.a[qr] * t;
  s.xi_out[iq] = xn;
  return t + xn;
}

__device__ __forceinline__ float* fptr(const FieldArg& f, int shot) {
  return f.p ? f.p + (long long)shot * f.s : nullptr;
}

// ---------------------------------------------------------------------------
// 2D: axis 0 = x (n0 points), axis 1 = z (n1 points).  Block = 4 warps side by
// side in x (512 x points); tile = 512 x points x TZ rows.
// psi_0 / xi_0 layout: [z][q] (q fastest);  psi_1 / xi_1 layout: [q][P].
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(128) k_ac2d_step(const StepArgs A) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = A.nshots;
  const int shot = blockIdx.x % S;
  const int tile = blockIdx.x / S;
  const int txi = tile % A.tiles_x, tzi = tile / A.tiles_x;
  const int nx = A.n0, nz = A.n1, P = A.P, H = A.halo;
  const int z_begin = 1 + tzi * A.TZ;
  const int z_end = min(z_begin + A.TZ, nz - 1);
  const int wx0 = (txi * 4 + warp) * 128;
  if (z_begin >= z_end || wx0 >= P) return;  // warp-uniform
  const int x0 = wx0 + lane * 4;
  const bool inb = x0 < P;
  const int xa = inb ? x0 : P - 4;

  const float* __restrict__ pc = fptr(A.pcur, shot);
  float* __restrict__ pn = fptr(A.pnew, shot);
  const float* di = fptr(A.din, shot);
  float* dn = fptr(A.dout, shot);
  const float* __restrict__ fa = A.fact;
  const float* cp = A.cpml + (long long)shot * A.cpml_stride;
  const int na = 2 * H + 2, nh = 2 * H, L = 2 * na + 2 * nh;

  StripIO sx, sz;
  sx.psi_in = fptr(A.psi_in[0], shot);  sx.psi_out = fptr(A.psi_out[0], shot);
  sx.xi_in = fptr(A.xi_in[0], shot);    sx.xi_out = fptr(A.xi_out[0], shot);
  sx.ck_psi = fptr(A.ck_psi[0], shot);  sx.ck_xi = fptr(A.ck_xi[0], shot);
  sx.a = cp; sx.ah = cp + na; sx.b = cp + na + nh; sx.bh = cp + 2 * na + nh;
  sx.psi_step = 1; sx.xi_step = 1;
  sz.psi_in = fptr(A.psi_in[1], shot);  sz.psi_out = fptr(A.psi_out[1], shot);
  sz.xi_in = fptr(A.xi_in[1], shot);    sz.xi_out = fptr(A.xi_out[1], shot);
  sz.ck_psi = fptr(A.ck_psi[1], shot);  sz.ck_xi = fptr(A.ck_xi[1], shot);
  sz.a = cp + L; sz.ah = cp + L + na; sz.b = cp + L + na + nh; sz.bh = cp + L + 2 * na + nh;
  sz.psi_step = P; sz.xi_step = P;

  const bool xstrip = inb && (x0 < H || x0 + 3 >= nx - H);
  const bool vec_interior = (x0 >= 1) && (x0 + 3 <= nx - 2);
  float* ckp = fptr(A.ck_p, shot);
  float* ckd = fptr(A.ck_d, shot);
  float* Dw = nullptr;
  if (MODE == MODE_FWD_D && shot >= A.d_first) Dw = fptr(A.Dout, shot);
  const float* dcr = MODE == MODE_ADJ ? fptr(A.dcorr, shot) : nullptr;
  float* gg = MODE == MODE_ADJ ? fptr(A.g, shot) : nullptr;
  float* gcp = MODE == MODE_ADJ ? fptr(A.gc, shot) : nullptr;

  float rm[4], r0[4], rp[4];
  ld4(rm, pc + (long long)(z_begin - 1) * P + xa);
  ld4(r0, pc + (long long)z_begin * P + xa);
  for (int z = z_begin; z < z_end; ++z) {
    const long long row = (long long)z * P;
    ld4(rp, pc + row + P + xa);
    float left = __shfl_up_sync(FULL, r0[3], 1);
    float right = __shfl_down_sync(FULL, r0[0], 1);
    if (lane == 0) left = xa > 0 ? pc[row + xa - 1] : 0.f;
    if (lane == 31) right = xa + 4 < P ? pc[row + xa + 4] : 0.f;
    float o[4], f[4];
    ld4rw(o, di + row + xa);
    ld4(f, fa + row + xa);
    const bool zstrip = (z < H) || (z >= nz - H);
    sx.psi_base = (long long)z * nh;
    sx.xi_base = (long long)z * na;
    float outp[4], outd[4], outD[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float xm = e == 0 ? left : r0[e - 1];
      const float xp = e == 3 ? right : r0[e + 1];
      const float c = r0[e];
      float tx = (xm - 2.f * c + xp) * A.ih2[0];
      float tz = (rm[e] - 2.f * c + rp[e]) * A.ih2[1];
      const int x = x0 + e;
      const bool pin = inb && x >= 1 && x <= nx - 2;
      if (xstrip && pin) tx = cpml_axis_term(tx, xm, c, xp, x, nx, H, A.ih[0], sx);
      if (zstrip && pin) {
        sz.psi_base = x;
        sz.xi_base = x;
        tz = cpml_axis_term(tz, rm[e], c, rp[e], z, nz, H, A.ih[1], sz);
      }
      const float lap = tx + tz;
      outD[e] = f[e] * lap;
      outd[e] = o[e] + outD[e];
      outp[e] = c + outd[e];
    }
    if (inb) {
      if (ckp) {
        st4(ckp + row + x0, r0);
        st4(ckd + row + x0, o);
      }
      if (MODE == MODE_ADJ) {
        float dv[4], g4[4], c4[4];
        ld4(dv, dcr + row + x0);
        ld4rw(g4, gg + row + x0);
        ld4rw(c4, gcp + row + x0);
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (x0 + e >= 1 && x0 + e <= nx - 2) kahan_add(g4[e], c4[e], outp[e] * dv[e]);
        if (vec_interior) {
          st4(gg + row + x0, g4);
          st4(gcp + row + x0, c4);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (x0 + e >= 1 && x0 + e <= nx - 2) { gg[row + x0 + e] = g4[e]; gcp[row + x0 + e] = c4[e]; }
        }
      }
      if (vec_interior) {
        st4(pn + row + x0, outp);
        st4(dn + row + x0, outd);
        if (MODE == MODE_FWD_D && Dw) st4(Dw + row + x0, outD);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int x = x0 + e;
          if (x >= 1 && x <= nx - 2) {
            pn[row + x] = outp[e];
            dn[row + x] = outd[e];
            if (MODE == MODE_FWD_D && Dw) Dw[row + x] = outD[e];
          }
        }
      }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) { rm[e] = r0[e]; r0[e] = rp[e]; }
  }
}

// ---------------------------------------------------------------------------
// 3D: axes 0 = x, 1 = y, 2 = z.  Block = 4 warps, one y row each (128 x
// points per warp); tile = 128 x 4 y x TZ z.  y neighbours come through L1.
// psi_0/xi_0: [z][y][q];  psi_1/xi_1: [z][q][P];  psi_2/xi_2: [q][y][P].
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(128) k_ac3d_step(const StepArgs A) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = A.nshots;
  const int shot = blockIdx.x % S;
  int tile = blockIdx.x / S;
  const int txi = tile % A.tiles_x;
  tile /= A.tiles_x;
  const int tyi = tile % A.tiles_y, tzi = tile / A.tiles_y;
  const int nx = A.n0, ny = A.n1, nz = A.n2, P = A.P, H = A.halo;
  const int y = 1 + tyi * 4 + warp;
  const int z_begin = 1 + tzi * A.TZ;
  const int z_end = min(z_begin + A.TZ, nz - 1);
  const int wx0 = txi * 128;
  if (z_begin >= z_end || y > ny - 2) return;  // warp-uniform
  const int x0 = wx0 + lane * 4;
  const bool inb = x0 < P;
  const int xa = inb ? x0 : P - 4;
  const long long plane = (long long)P * ny;

  const float* __restrict__ pc = fptr(A.pcur, shot);
  float* __restrict__ pn = fptr(A.pnew, shot);
  const float* di = fptr(A.din, shot);
  float* dn = fptr(A.dout, shot);
  const float* __restrict__ fa = A.fact;
  const float* cp = A.cpml + (long long)shot * A.cpml_stride;
  const int na = 2 * H + 2, nh = 2 * H, L = 2 * na + 2 * nh;

  StripIO s0, s1, s2;
  StripIO* ss[3] = {&s0, &s1, &s2};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    StripIO& s = *ss[d];
    s.psi_in = fptr(A.psi_in[d], shot);  s.psi_out = fptr(A.psi_out[d], shot);
    s.xi_in = fptr(A.xi_in[d], shot);    s.xi_out = fptr(A.xi_out[d], shot);
    s.ck_psi = fptr(A.ck_psi[d], shot);  s.ck_xi = fptr(A.ck_xi[d], shot);
    s.a = cp + d * L; s.ah = cp + d * L + na; s.b = cp + d * L + na + nh; s.bh = cp + d * L + 2 * na + nh;
  }
  s0.psi_step = 1; s0.xi_step = 1;
  s1.psi_step = P; s1.xi_step = P;
  s2.psi_step = (long long)ny * P; s2.xi_step = (long long)ny * P;

  const bool xstrip = inb && (x0 < H || x0 + 3 >= nx - H);
  const bool ystrip = (y < H) || (y >= ny - H);
  const bool vec_interior = (x0 >= 1) && (x0 + 3 <= nx - 2);
  float* ckp = fptr(A.ck_p, shot);
  float* ckd = fptr(A.ck_d, shot);
  float* Dw = nullptr;
  if (MODE == MODE_FWD_D && shot >= A.d_first) Dw = fptr(A.Dout, shot);
  const float* dcr = MODE == MODE_ADJ ? fptr(A.dcorr, shot) : nullptr;
  float* gg = MODE == MODE_ADJ ? fptr(A.g, shot) : nullptr;
  float* gcp = MODE == MODE_ADJ ? fptr(A.gc, shot) : nullptr;

  const long long rowoff = (long long)y * P + xa;
  float rm[4], r0[4], rp[4];
  ld4(rm, pc + (long long)(z_begin - 1) * plane + rowoff);
  ld4(r0, pc + (long long)z_begin * plane + rowoff);
  for (int z = z_begin; z < z_end; ++z) {
    const long long base = (long long)z * plane;
    const long long idx = base + rowoff;
    ld4(rp, pc + idx + plane);
    float ym[4], yp[4];
    ld4(ym, pc + idx - P);
    ld4(yp, pc + idx + P);
    float left = __shfl_up_sync(FULL, r0[3], 1);
    float right = __shfl_down_sync(FULL, r0[0], 1);
    if (lane == 0) left = xa > 0 ? pc[idx - 1] : 0.f;
    if (lane == 31) right = xa + 4 < P ? pc[idx + 4] : 0.f;
    float o[4], f[4];
    ld4rw(o, di + idx);
    ld4(f, fa + idx);
    const bool zstrip = (z < H) || (z >= nz - H);
    s0.psi_base = ((long long)z * ny + y) * nh;
    s0.xi_base = ((long long)z * ny + y) * na;
    float outp[4], outd[4], outD[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float xm = e == 0 ? left : r0[e - 1];
      const float xp = e == 3 ? right : r0[e + 1];
      const float c = r0[e];
      float tx = (xm - 2.f * c + xp) * A.ih2[0];
      float ty = (ym[e] - 2.f * c + yp[e]) * A.ih2[1];
      float tz = (rm[e] - 2.f * c + rp[e]) * A.ih2[2];
      const int x = x0 + e;
      const bool pin = inb && x >= 1 && x <= nx - 2;
      if (xstrip && pin) tx = cpml_axis_term(tx, xm, c, xp, x, nx, H, A.ih[0], s0);
      if (ystrip && pin) {
        s1.psi_base = (long long)z * nh * P + x;
        s1.xi_base = (long long)z * na * P + x;
        ty = cpml_axis_term(ty, ym[e], c, yp[e], y, ny, H, A.ih[1], s1);
      }
      if (zstrip && pin) {
        s2.psi_base = (long long)y * P + x;
        s2.xi_base = (long long)y * P + x;
        tz = cpml_axis_term(tz, rm[e], c, rp[e], z, nz, H, A.ih[2], s2);
      }
      const float lap = (tx + ty) + tz;
      outD[e] = f[e] * lap;
      outd[e] = o[e] + outD[e];
      outp[e] = c + outd[e];
    }
    if (inb) {
      if (ckp) {
        st4(ckp + idx, r0);
        st4(ckd + idx, o);
      }
      if (MODE == MODE_ADJ) {
        float dv[4], g4[4], c4[4];
        ld4(dv, dcr + idx);
        ld4rw(g4, gg + idx);
        ld4rw(c4, gcp + idx);
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (x0 + e >= 1 && x0 + e <= nx - 2) kahan_add(g4[e], c4[e], outp[e] * dv[e]);
        if (vec_interior) {
          st4(gg + idx, g4);
          st4(gcp + idx, c4);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (x0 + e >= 1 && x0 + e <= nx - 2) { gg[idx + e] = g4[e]; gcp[idx + e] = c4[e]; }
        }
      }
      if (vec_interior) {
        st4(pn + idx, outp);
        st4(dn + idx, outd);
        if (MODE == MODE_FWD_D && Dw) st4(Dw + idx, outD);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int x = x0 + e;
          if (x >= 1 && x <= nx - 2) {
            pn[idx + e] = outp[e];
            dn[idx + e] = outd[e];
            if (MODE == MODE_FWD_D && Dw) Dw[idx + e] = outD[e];
          }
        }
      }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) { rm[e] = r0[e]; r0[e] = rp[e]; }
  }
}

}  // namespace swgb
