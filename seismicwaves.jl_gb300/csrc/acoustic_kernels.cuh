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
//  * the adjoint variants also accumulate the gradient correlation
//    g += lambda * D (correlate_gradient_xPU.jl:1-10): MODE_ADJW (the 2D
//    default) into a plain FP32 sum per shot that the host flushes into an
//    FP64 total every 32 steps, so no FP32 sum runs over more than 32 terms;
//    MODE_ADJ (3D, muted runs) with Kahan compensation.
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

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "internal.h"
#include "ff.cuh"

namespace swgb {

// MODE_ADJW (2D only): the adjoint with plain FP32 correlation sums per shot
// (no Kahan compensation), which the host flushes into FP64 totals every few
// steps (k_flush_grad).
enum StepMode { MODE_FWD = 0, MODE_FWD_D = 1, MODE_ADJ = 2, MODE_ADJW = 3 };

struct FieldArgE {  // int8 per-shot array (exponents of the FP16 D slots): shot k at p + k * s
  signed char* p;
  long long s;
};

struct Field64 {  // FP64 per-shot array: shot k at p + k * s
  double* p;
  long long s;
};

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
  int* err;                                        // set to 1 when a bounded wait gives up
  long long wait_cycles;                           // limit of one bounded wait (clock64 cycles)
  int withhold;  // TMA stencil test hook: block 0's producer never issues this stage (-1 = none)
  int pf;                                          // 2D stencil: rows ahead prefetched into L2 (0 = off)
  int dbf16;  // Dout / dcorr: 0 FP32, 1 BF16, 2 FP16 scaled by 2^e per row and 128-point x tile (3D)
  FieldArgE Dexp, dcorr_exp;  // dbf16 == 2: the exponents e of Dout / dcorr, [row][x tile]
  int ntx;                    // x tiles of 128 points per row of the exponent arrays
  // compensated step (k_ac_hp): low parts of p[n], p[n+1] and d (in place), of fact and of 1/h^2;
  // FP64 C-PML coefficients (stride cpml_stride), memory variables and 1/h
  FieldArg plo_cur, plo_new, dlo;
  const float* fact_lo;
  float ih2_lo[3];
  const double* cpml64;
  Field64 psi64_in[3], psi64_out[3], xi64[3];
  double ihd[3];
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

// The D slots (second time differences kept for the gradient) are FP32 or,
// with BF16 snapshots, __nv_bfloat16 arrays behind the same float* handle;
// idx counts elements either way.
__device__ __forceinline__ float* dptr(const FieldArg& f, int shot, int bf) {
  if (!f.p) return nullptr;
  if (bf) return reinterpret_cast<float*>(reinterpret_cast<__nv_bfloat16*>(f.p) + (long long)shot * f.s);
  return f.p + (long long)shot * f.s;
}
// FP16 D (dbf16 == 2): every 128-point x tile of a row is stored as
// round(D * 2^e) with e chosen from the tile's largest |D| so that it maps
// into [2^10, 2^11) (32x head room below FP16's largest value for the
// sources added afterwards; relative precision 2^-11 down to 2^-24 of the
// tile maximum).
__device__ __forceinline__ int dexp_of(float amax) {
  if (!(amax > 0.f)) return 0;
  const int ex = (int)((__float_as_uint(amax) >> 23) & 255u) - 127;  // amax in [2^ex, 2^(ex+1))
  return max(-100, min(100, 10 - ex));
}
__device__ __forceinline__ float pow2f(int e) { return __uint_as_float((unsigned)(e + 127) << 23); }
__device__ __forceinline__ float h_enc(float v, int e) {  // scaled and clamped to FP16's finite range
  return fminf(fmaxf(v * pow2f(e), -65504.f), 65504.f);
}
// e of one warp's tile (all lanes call it; lanes without points pass valid = false)
__device__ __forceinline__ int warp_dexp(const float (&v)[4], bool valid) {
  const float m = valid ? fmaxf(fmaxf(fabsf(v[0]), fabsf(v[1])), fmaxf(fabsf(v[2]), fabsf(v[3]))) : 0.f;
  return dexp_of(__uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(m))));
}

__device__ __forceinline__ void dld4(float (&v)[4], const float* p, long long idx, int bf, int e = 0) {
  if (bf == 2) {
    const uint2 u = __ldg(reinterpret_cast<const uint2*>(reinterpret_cast<const __half*>(p) + idx));
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
    const float s = pow2f(-e);
    v[0] = a.x * s; v[1] = a.y * s; v[2] = b.x * s; v[3] = b.y * s;
  } else if (bf) {
    const uint2 u = __ldg(reinterpret_cast<const uint2*>(reinterpret_cast<const __nv_bfloat16*>(p) + idx));
    const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.x));
    const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.y));
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  } else {
    ld4(v, p + idx);
  }
}
__device__ __forceinline__ void dst4(float* p, long long idx, const float (&v)[4], int bf, int e = 0) {
  if (bf == 2) {
    const __half2 a = __floats2half2_rn(h_enc(v[0], e), h_enc(v[1], e));
    const __half2 b = __floats2half2_rn(h_enc(v[2], e), h_enc(v[3], e));
    uint2 u;
    u.x = *reinterpret_cast<const unsigned*>(&a);
    u.y = *reinterpret_cast<const unsigned*>(&b);
    *reinterpret_cast<uint2*>(reinterpret_cast<__half*>(p) + idx) = u;
  } else if (bf) {
    const __nv_bfloat162 a = __floats2bfloat162_rn(v[0], v[1]);
    const __nv_bfloat162 b = __floats2bfloat162_rn(v[2], v[3]);
    uint2 u;
    u.x = *reinterpret_cast<const unsigned*>(&a);
    u.y = *reinterpret_cast<const unsigned*>(&b);
    *reinterpret_cast<uint2*>(reinterpret_cast<__nv_bfloat16*>(p) + idx) = u;
  } else {
    st4(p + idx, v);
  }
}
__device__ __forceinline__ void dst1(float* p, long long idx, float v, int bf, int e = 0) {
  if (bf == 2) reinterpret_cast<__half*>(p)[idx] = __float2half_rn(h_enc(v, e));
  else if (bf) reinterpret_cast<__nv_bfloat16*>(p)[idx] = __float2bfloat16_rn(v);
  else p[idx] = v;
}
__device__ __forceinline__ float dld1(const float* p, long long idx, int bf, int e = 0) {
  if (bf == 2) return __half2float(reinterpret_cast<const __half*>(p)[idx]) * pow2f(-e);
  if (bf) return __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(p)[idx]);
  return p[idx];
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

// Rounded FP32 operations that the compiler may not contract into FMAs: the
// stencil arithmetic below is spelled out with them so that every kernel
// that advances a point (one step per launch or two) rounds identically,
// whatever the surrounding code lets the compiler fuse.
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
// (l - 2c + r) * ih2: the second difference along one axis.  -2c is exact,
// so l - 2c as one fused multiply-add rounds exactly as the product followed
// by a rounded add (one instruction fewer per axis and point).
__device__ __forceinline__ float d2term(float l, float c, float r, float ih2) {
  return rmul(radd(__fmaf_rn(-2.f, c, l), r), ih2);
}

// One row of four interior points outside the damping strips advanced by one
// step: the arithmetic every stencil uses at such points (the general paths
// below add the C-PML terms and the boundary handling), straight-line for the
// warps whose whole row segment qualifies.
__device__ __forceinline__ void row4_interior(const float (&rm)[4], const float (&r0)[4], const float (&rp)[4],
                                              float left, float right, const float (&o)[4], const float (&f)[4],
                                              float ih2x, float ih2z, float (&outp)[4], float (&outd)[4],
                                              float (&outD)[4]) {
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const float xm = e == 0 ? left : r0[e - 1];
    const float xp = e == 3 ? right : r0[e + 1];
    const float c = r0[e];
    const float lap = radd(d2term(xm, c, xp, ih2x), d2term(rm[e], c, rp[e], ih2z));
    outD[e] = rmul(f[e], lap);
    outd[e] = radd(o[e], outD[e]);
    outp[e] = radd(c, outd[e]);
  }
}

// Points x (or rows z) in [lo, hi] are interior and outside the damping
// strips of an axis of n points with halo cells.
__device__ __forceinline__ int plain_lo(int H) { return H > 1 ? H : 1; }
__device__ __forceinline__ int plain_hi(int n, int H) { return (n - 1 - H) < (n - 2) ? (n - 1 - H) : (n - 2); }

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
  const float newl = radd(rmul(s.bh[ql], oldl), rmul(s.ah[ql], rmul(rsub(p0, pl), ih)));
  const float newr = radd(rmul(s.bh[qr], oldr), rmul(s.ah[qr], rmul(rsub(pr, p0), ih)));
  s.psi_out[ir] = newr;
  if (s.ck_psi) s.ck_psi[ir] = oldr;
  if (first) {
    s.psi_out[il] = newl;
    if (s.ck_psi) s.ck_psi[il] = oldl;
  }
  const float dpsi = rmul(rsub(newr, newl), ih);
  const long long iq = s.xi_base + (long long)qr * s.xi_step;
  const float xo = s.xi_in[iq];
  if (s.ck_xi) s.ck_xi[iq] = xo;
  const float t = radd(d2, dpsi);
  const float xn = radd(rmul(s.b[qr], xo), rmul(s.a[qr], t));
  s.xi_out[iq] = xn;
  return radd(t, xn);
}

// cpml_axis_term for four consecutive x points of an axis whose strip cell
// does not depend on x (the y and z axes of the 3D step): the same
// arithmetic per point, with psi, xi and their checkpoint copies moved as
// float4 (the base indices point at the first of the four points; the two
// outermost columns, which no point reads, get their values too).
__device__ __forceinline__ void cpml_axis_term4(float (&t)[4], const float (&pl)[4], const float (&p0)[4],
                                                const float (&pr)[4], int v, int n, int halo, float ih,
                                                const StripIO& s) {
  int qr;
  bool first;
  if (v < halo) {
    qr = v;
    first = (v == 1);
  } else if (v >= n - halo) {
    qr = v + 1 - n + 2 * halo;
    first = (v == n - halo);
  } else {
    return;
  }
  const int ql = qr - 1;
  const long long il = s.psi_base + (long long)ql * s.psi_step;
  const long long ir = s.psi_base + (long long)qr * s.psi_step;
  const long long iq = s.xi_base + (long long)qr * s.xi_step;
  const float bhl = s.bh[ql], ahl = s.ah[ql], bhr = s.bh[qr], ahr = s.ah[qr], bq = s.b[qr], aq = s.a[qr];
  float oldl[4], oldr[4], xo[4], newl[4], newr[4], xn[4];
  ld4rw(oldl, s.psi_in + il);
  ld4rw(oldr, s.psi_in + ir);
  ld4rw(xo, s.xi_in + iq);
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    newl[e] = radd(rmul(bhl, oldl[e]), rmul(ahl, rmul(rsub(p0[e], pl[e]), ih)));
    newr[e] = radd(rmul(bhr, oldr[e]), rmul(ahr, rmul(rsub(pr[e], p0[e]), ih)));
    const float dpsi = rmul(rsub(newr[e], newl[e]), ih);
    const float tt = radd(t[e], dpsi);
    xn[e] = radd(rmul(bq, xo[e]), rmul(aq, tt));
    t[e] = radd(tt, xn[e]);
  }
  st4(s.psi_out + ir, newr);
  if (s.ck_psi) st4(s.ck_psi + ir, oldr);
  if (first) {
    st4(s.psi_out + il, newl);
    if (s.ck_psi) st4(s.ck_psi + il, oldl);
  }
  if (s.ck_xi) st4(s.ck_xi + iq, xo);
  st4(s.xi_out + iq, xn);
}

// TMA prefetch of a contiguous global range into L2 (no registers, no
// completion to wait for).  Address 16-byte aligned, size a multiple of 16.
__device__ __forceinline__ void l2_prefetch(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

__device__ __forceinline__ float* fptr(const FieldArg& f, int shot) {
  return f.p ? f.p + (long long)shot * f.s : nullptr;
}

// ---------------------------------------------------------------------------
// 2D: axis 0 = x (n0 points), axis 1 = z (n1 points).  Block = 4 warps side by
// side in x (512 x points); tile = 512 x points x TZ rows.
// psi_0 / xi_0 layout: [z][q] (q fastest);  psi_1 / xi_1 layout: [q][P].
// ---------------------------------------------------------------------------
// One row of the 2D step at one thread's four x points: given p[n] of rows
// z-1, z, z+1 (rm, r0, rp) with the x neighbours of row z (left, right),
// d[n] and fact of row z, it advances the C-PML variables and writes p[n+1],
// d[n+1] and the side outputs (D, checkpoint copies) and, in the adjoint
// modes, the correlation term into the sums g4 (and compensations c4) of the
// row, which it stores.  Shared by the register-pipelined and the
// cp.async-staged kernels, which differ only in how rows reach registers.
template <int MODE>
struct Ac2dRow {
  int nx, nz, P, H, x0, dbf16;
  bool inb, xstrip, vec_interior, fastx;
  float ihx, ihz, ih2x, ih2z;
  StripIO sx, sz;
  float *pn, *dn, *ckp, *ckd, *Dw, *gg, *gcp;

  __device__ __forceinline__ void init(const StepArgs& A, int shot, int x0_) {
    nx = A.n0; nz = A.n1; P = A.P; H = A.halo; x0 = x0_; dbf16 = A.dbf16;
    ihx = A.ih[0]; ihz = A.ih[1]; ih2x = A.ih2[0]; ih2z = A.ih2[1];
    inb = x0 < P;
    const int na = 2 * H + 2, nh = 2 * H, L = 2 * na + 2 * nh;
    const float* cp = A.cpml + (long long)shot * A.cpml_stride;
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
    xstrip = inb && (x0 < H || x0 + 3 >= nx - H);
    vec_interior = (x0 >= 1) && (x0 + 3 <= nx - 2);
    // the warp's 128 points all interior and outside the x strips (warp-uniform)
    const int wx = x0 - 4 * (int)(threadIdx.x & 31);
    fastx = wx >= plain_lo(H) && wx + 127 <= plain_hi(nx, H);
    pn = fptr(A.pnew, shot);
    dn = fptr(A.dout, shot);
    ckp = fptr(A.ck_p, shot);
    ckd = fptr(A.ck_d, shot);
    Dw = (MODE == MODE_FWD_D && shot >= A.d_first) ? dptr(A.Dout, shot, A.dbf16) : nullptr;
    constexpr bool ADJ = MODE == MODE_ADJ || MODE == MODE_ADJW;
    gg = ADJ ? fptr(A.g, shot) : nullptr;
    gcp = MODE == MODE_ADJ ? fptr(A.gc, shot) : nullptr;
  }

  // XS (x strips split off): a lane whose four points meet an x strip
  // (xstrip) stores nothing here; the x-strip blocks of the launch
  // (xstrip_item) advance those points.  Every other lane's points lie
  // outside the x strips and inside the grid's
  // interior, so a row outside the z strips takes the interior path in every
  // warp and a z strip row needs only the z term.
  template <bool XS = false>
  __device__ __forceinline__ void update(int z, const float (&rm)[4], const float (&r0)[4], const float (&rp)[4],
                                         const float (&o)[4], const float (&f)[4], const float (&dv)[4],
                                         float (&g4)[4], float (&c4)[4], float left, float right) {
    const long long row = (long long)z * P;
    const bool zstrip = (z < H) || (z >= nz - H);
    sx.psi_base = (long long)z * (2 * H);
    sx.xi_base = (long long)z * (2 * H + 2);
    float outp[4], outd[4], outD[4];
    if ((XS || fastx) && z >= plain_lo(H) && z <= plain_hi(nz, H)) {
      row4_interior(rm, r0, rp, left, right, o, f, ih2x, ih2z, outp, outd, outD);
    } else if (XS) {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float c = r0[e];
        const float tx = d2term(e == 0 ? left : r0[e - 1], c, e == 3 ? right : r0[e + 1], ih2x);
        float tz = d2term(rm[e], c, rp[e], ih2z);
        if (zstrip && inb && !xstrip) {
          sz.psi_base = x0 + e;
          sz.xi_base = x0 + e;
          tz = cpml_axis_term(tz, rm[e], c, rp[e], z, nz, H, ihz, sz);
        }
        const float lap = radd(tx, tz);
        outD[e] = rmul(f[e], lap);
        outd[e] = radd(o[e], outD[e]);
        outp[e] = radd(c, outd[e]);
      }
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float xm = e == 0 ? left : r0[e - 1];
        const float xp = e == 3 ? right : r0[e + 1];
        const float c = r0[e];
        float tx = d2term(xm, c, xp, ih2x);
        float tz = d2term(rm[e], c, rp[e], ih2z);
        const int x = x0 + e;
        const bool pin = inb && x >= 1 && x <= nx - 2;
        if (xstrip && pin) tx = cpml_axis_term(tx, xm, c, xp, x, nx, H, ihx, sx);
        if (zstrip && pin) {
          sz.psi_base = x;
          sz.xi_base = x;
          tz = cpml_axis_term(tz, rm[e], c, rp[e], z, nz, H, ihz, sz);
        }
        const float lap = radd(tx, tz);
        outD[e] = rmul(f[e], lap);
        outd[e] = radd(o[e], outD[e]);
        outp[e] = radd(c, outd[e]);
      }
    }
    if (!inb || (XS && xstrip)) return;
    if (ckp) {
      st4(ckp + row + x0, r0);
      st4(ckd + row + x0, o);
    }
    if (MODE == MODE_ADJ) {
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
    if (MODE == MODE_ADJW) {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (x0 + e >= 1 && x0 + e <= nx - 2) g4[e] = __fmaf_rn(outp[e], dv[e], g4[e]);
      if (vec_interior) {
        st4(gg + row + x0, g4);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (x0 + e >= 1 && x0 + e <= nx - 2) gg[row + x0 + e] = g4[e];
      }
    }
    if (vec_interior) {
      st4(pn + row + x0, outp);
      st4(dn + row + x0, outd);
      if (MODE == MODE_FWD_D && Dw) dst4(Dw, row + x0, outD, dbf16);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int x = x0 + e;
        if (x >= 1 && x <= nx - 2) {
          pn[row + x] = outp[e];
          dn[row + x] = outd[e];
          if (MODE == MODE_FWD_D && Dw) dst1(Dw, row + x, outD[e], dbf16);
        }
      }
    }
  }
};

// The 4-point lane groups that meet an x strip (x0 < H or x0 + 3 >= nx - H,
// x0 = 0, 4, .. < P): nl groups x0 = 0 .. 4 (nl - 1) on the left, then the
// groups from x0 = xr up to the padded row end; ng in all.
__host__ __device__ __forceinline__ void xstrip_groups(int nx, int H, int P, int& nl, int& xr, int& ng) {
  nl = (H + 3) / 4;
  const int lo = nx - H - 3 > 0 ? nx - H - 3 : 0;
  xr = ((lo + 3) / 4) * 4;
  if (xr < 4 * nl) xr = 4 * nl;
  ng = nl + (P - xr > 0 ? (P - xr) / 4 : 0);
}

// The points that the main blocks of k_ac2d_step<.., XS = true> leave: work
// item t is one (lane group of the x strips, row, shot); it loads its rows
// and runs the general path of Ac2dRow (both strips per point), so every
// point is advanced by the same arithmetic as in the single-path kernel.
// Not inlined: its registers (and spills) stay out of the main blocks' path.
template <int MODE>
__device__ __noinline__ void xstrip_item(const StepArgs& A, long long t) {
  const int nx = A.n0, nz = A.n1, P = A.P, H = A.halo;
  int nl, xr, ng;
  xstrip_groups(nx, H, P, nl, xr, ng);
  const int g = (int)(t % ng);
  const long long rest = t / ng;
  const int z = 1 + (int)(rest % (nz - 2));
  const int shot = (int)(rest / (nz - 2));
  if (shot >= A.nshots) return;
  const int x0 = g < nl ? 4 * g : xr + 4 * (g - nl);
  const float* __restrict__ pc = fptr(A.pcur, shot);
  const float* di = fptr(A.din, shot);
  const long long row = (long long)z * P;
  float rm[4], r0[4], rp[4], o[4], f[4], dv[4] = {}, g4[4] = {}, c4[4] = {};
  ld4(rm, pc + row - P + x0);
  ld4(r0, pc + row + x0);
  ld4(rp, pc + row + P + x0);
  ld4rw(o, di + row + x0);
  ld4(f, A.fact + row + x0);
  const float left = x0 > 0 ? pc[row + x0 - 1] : 0.f;
  const float right = x0 + 4 < P ? pc[row + x0 + 4] : 0.f;
  Ac2dRow<MODE> R;
  R.init(A, shot, x0);
  R.fastx = false;
  constexpr bool ADJ = MODE == MODE_ADJ || MODE == MODE_ADJW;
  if (ADJ) {
    dld4(dv, dptr(A.dcorr, shot, A.dbf16), row + x0, A.dbf16);
    ld4rw(g4, R.gg + row + x0);
    if (MODE == MODE_ADJ) ld4rw(c4, R.gcp + row + x0);
  }
  R.update(z, rm, r0, rp, o, f, dv, g4, c4, left, right);
}

// Minimum resident blocks per SM for a block of NW warps: keeps the forward
// kernels at <= 64 registers (8 blocks of 4 warps, no spills; measured 4.1 /
// 4.5 TB/s forward / recompute against 3.8 / 4.3 at 7 blocks); the per-shot
// adjoint at <= 80 (6 blocks, 8 bytes spilled); the Kahan adjoint, which holds
// a second row of six arrays in registers, at 128.
template <int MODE, int NW>
struct Ac2dBounds {
  static constexpr int MINB = MODE == MODE_ADJ    ? (NW == 4 ? 4 : NW == 8 ? 2 : 1)
                              : MODE == MODE_ADJW ? (NW == 4 ? 6 : NW == 8 ? 3 : 1)
                                                  : (NW == 4 ? 8 : NW == 8 ? 4 : 2);
};

// XS: the lanes that meet an x strip store nothing in the main blocks (the
// first nshots x tiles_x x tiles_z); the blocks after them take the lane
// groups of the x strips, one per thread (xstrip_item), so that this work
// fills the tail of the launch.
template <int MODE, int NW, int DP = 1, bool XS = false>
__global__ void __launch_bounds__(32 * NW, (Ac2dBounds<MODE, NW>::MINB - (DP - 1))) k_ac2d_step(const StepArgs A) {
  constexpr unsigned FULL = 0xffffffffu;
  if constexpr (XS) {
    const long long nb_main = (long long)A.nshots * A.tiles_x * A.tiles_y * A.tiles_z;
    if ((long long)blockIdx.x >= nb_main) {
      xstrip_item<MODE>(A, ((long long)blockIdx.x - nb_main) * (32 * NW) + threadIdx.x);
      return;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int nwarps = NW;
  const int S = A.nshots;
  // block order: x tiles fastest (neighbouring CTAs stream one contiguous row
  // together), then shots (the shots of a row band share fact through L2)
  const int txi = blockIdx.x % A.tiles_x;
  const int rest = blockIdx.x / A.tiles_x;
  const int shot = rest % S, tzi = rest / S;
  const int nz = A.n1, P = A.P;
  const int z_begin = 1 + tzi * A.TZ;
  const int z_end = min(z_begin + A.TZ, nz - 1);
  const int wx0 = (txi * nwarps + warp) * 128;
  if (z_begin >= z_end || wx0 >= P) return;  // warp-uniform
  const int x0 = wx0 + lane * 4;
  const bool inb = x0 < P;
  const int xa = inb ? x0 : P - 4;

  const float* __restrict__ pc = fptr(A.pcur, shot);
  const float* di = fptr(A.din, shot);
  const float* __restrict__ fa = A.fact;
  Ac2dRow<MODE> R;
  R.init(A, shot, x0);
  constexpr bool ADJ = MODE == MODE_ADJ || MODE == MODE_ADJW;
  const float* dcr = ADJ ? dptr(A.dcorr, shot, A.dbf16) : nullptr;
  float* gg = R.gg;
  float* gcp = R.gcp;

  // The loads of row z+1 (p of row z+2, d, fact and for the adjoint D, g, gc)
  // are issued before the stores of row z, so each warp keeps two rows of
  // loads in flight instead of waiting on every row.
  float rm[4], r0[4], rp[4], o[4], f[4], dv[4], g4[4], c4[4];
  // The x neighbours of a lane's four points come from the neighbouring lanes
  // by shuffles; lane 0 (left) and lane 31 (right) read theirs from memory,
  // one value per row, loaded one row ahead (e0: row z) so that no row waits
  // on its edge load (DP == 1).
  const int eoff = lane == 0 ? xa - 1 : xa + 4;
  const bool eload = (lane == 0 && xa > 0) || (lane == 31 && xa + 4 < P);
  float e0 = 0.f;
  ld4(rm, pc + (long long)(z_begin - 1) * P + xa);
  ld4(r0, pc + (long long)z_begin * P + xa);
  if (DP == 1 && eload) e0 = pc[(long long)z_begin * P + eoff];
  {
    const long long row = (long long)z_begin * P;
    ld4(rp, pc + row + P + xa);
    ld4rw(o, di + row + xa);
    ld4(f, fa + row + xa);
    if (ADJ) {
      dld4(dv, dcr, row + xa, A.dbf16);
      ld4rw(g4, gg + row + xa);
      if (MODE == MODE_ADJ) ld4rw(c4, gcp + row + xa);
    }
  }
  // DP == 2 (forward kernels): a second row of loads in flight, issued one
  // iteration earlier (q* hold p of row z+2 and d, fact of row z+1).
  float qp[4], qo[4], qf[4];
  if constexpr (DP == 2) {
    if (z_begin + 1 < z_end) {
      const long long nrow = (long long)(z_begin + 1) * P;
      ld4(qp, pc + nrow + P + xa);
      ld4rw(qo, di + nrow + xa);
      ld4(qf, fa + nrow + xa);
    }
  }
  // one lane per warp asks the TMA unit to pull the warp's segments of a row
  // A.pf rows ahead into L2, so the register loads of that row later hit L2
  const unsigned seg = (unsigned)min(128, P - wx0) * 4u;
  for (int z = z_begin; z < z_end; ++z) {
    const long long row = (long long)z * P;
    if (A.pf > 0 && lane == 0 && z + A.pf < z_end) {
      const long long prow = row + (long long)A.pf * P + wx0;
      l2_prefetch(pc + prow + P, seg);
      l2_prefetch(di + prow, seg);
      if (ADJ) {
        if (!A.dbf16) l2_prefetch(dcr + prow, seg);
        l2_prefetch(gg + prow, seg);
        if (MODE == MODE_ADJ) l2_prefetch(gcp + prow, seg);
      }
    }
    float rpn[4], on[4], fn[4], dvn[4], g4n[4], c4n[4], en = 0.f;
    const bool more = z + 1 < z_end;
    if constexpr (DP == 2) {
      if (z + 2 < z_end) {
        const long long nrow = row + 2 * P;
        ld4(rpn, pc + nrow + P + xa);
        ld4rw(on, di + nrow + xa);
        ld4(fn, fa + nrow + xa);
      }
    } else if (more) {
      const long long nrow = row + P;
      if (eload) en = pc[nrow + eoff];
      ld4(rpn, pc + nrow + P + xa);
      ld4rw(on, di + nrow + xa);
      ld4(fn, fa + nrow + xa);
      if (ADJ) {
        dld4(dvn, dcr, nrow + xa, A.dbf16);
        ld4rw(g4n, gg + nrow + xa);
        if (MODE == MODE_ADJ) ld4rw(c4n, gcp + nrow + xa);
      }
    }
    float left = __shfl_up_sync(FULL, r0[3], 1);
    float right = __shfl_down_sync(FULL, r0[0], 1);
    if constexpr (DP == 2) {
      if (lane == 0) left = xa > 0 ? pc[row + xa - 1] : 0.f;
      if (lane == 31) right = xa + 4 < P ? pc[row + xa + 4] : 0.f;
    } else {
      if (lane == 0) left = e0;
      if (lane == 31) right = e0;
    }
    R.template update<XS>(z, rm, r0, rp, o, f, dv, g4, c4, left, right);
    if constexpr (DP == 1) e0 = en;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      rm[e] = r0[e];
      r0[e] = rp[e];
      if constexpr (DP == 2) {
        rp[e] = qp[e];
        o[e] = qo[e];
        f[e] = qf[e];
        qp[e] = rpn[e];
        qo[e] = on[e];
        qf[e] = fn[e];
      } else if (more) {
        rp[e] = rpn[e];
        o[e] = on[e];
        f[e] = fn[e];
        if (ADJ) { dv[e] = dvn[e]; g4[e] = g4n[e]; }
        if (MODE == MODE_ADJ) c4[e] = c4n[e];
      }
    }
  }
}


// ---------------------------------------------------------------------------
// 2D, two time steps per pass (temporal blocking) for the forward kinds and
// the adjoint.
//
// The one-step kernels move 16 bytes per point and step (read p and d, write
// them back); here one launch advances the state from step n to n+2 and moves
// the same 16 bytes once.  A warp covers 128 x points (4 per lane) and
// advances the first step on all of them, the second only on lanes 1..30
// (120 points): the first step of lanes 0 and 31 supplies the x neighbours of
// the second.  Along z the march runs the first step one row ahead of the
// second (rows zb-1 .. ze of the first step for rows zb .. ze-1 of the second),
// so a band's first and last rows come from the first step of its own halo.
// Every point the first step touches is computed by the same arithmetic
// wherever it is computed (neighbouring warps and bands repeat it), so the
// copies agree bit for bit; the two steps round exactly as two launches of the
// one-step kernel do (same rounded operations, see d2term / cpml_axis_term).
//
// State is double-buffered throughout (p, d, psi, xi read from one buffer,
// written to the other): a neighbour's repeated first step reads d and xi of
// points this warp owns.  The memory variables after the first step go to
// scratch strips (psi_mid, xi_mid); the second step reads them back from the
// same warp's earlier writes.  What lies between the two steps is done here:
// the sources of the first step are injected (same summation order as
// k_inject_record), and the pressure of receiver rows after the first step is
// kept in a small per-shot stash that the recording kernel reads.  The host
// pairs steps only where nothing else lies between them (no checkpoint state,
// snapshot or change of the active shots), and only for shots whose sources
// and receivers sit off the outermost grid lines.
//
// MODE_ADJW: two adjoint steps (it1 and it1 - 1) with the correlation of
// both: the first step's adjoint sources at the receivers are injected here
// (summed like k_adj_inject), and the per-shot FP32 sum g of a row is read
// once, takes lambda * D of the first step (with its injected share) and of
// the second, and is written once.  The injection of the second step is left
// to k_adj_inject, as after a one-step launch.
// ---------------------------------------------------------------------------
constexpr int PAIR_MAXSP = 4;  // unique source points per shot
constexpr int PAIR_MAXRR = 4;  // distinct receiver rows per shot
constexpr int PAIR_OUT = 120;  // x points a warp advances by both steps

struct PairShot {
  const float* tf;   // (nt, nsrc) scaled source time functions
  const float* adj;  // adjoint: (nt, nrec) prescaled adjoint sources
  int nt, nsp, nrr, pad;
  int sx[PAIR_MAXSP], sz[PAIR_MAXSP];  // unique source points (0-based)
  int k0[PAIR_MAXSP], k1[PAIR_MAXSP];  // their source ids: ids[k0 .. k1)
  int rrow[PAIR_MAXRR];                // receiver rows (0-based z), stash slot = index
};

struct PairArgs {
  FieldArg psi_mid[2], xi_mid[2];  // memory variables after the first step (scratch)
  FieldArg Dout2;                  // MODE_FWD_D: D of the second step (shots >= A.d_first)
  FieldArg stash;                  // [shot][k][P]: p after the first step on receiver row k (p == nullptr: none)
  FieldArg dcorr2;                 // MODE_ADJW: D the second step correlates with (A.dcorr: the first)
  const PairShot* shots;
  const int* ids;                  // source / receiver ids of the CSR ranges
  const int* ptr;                  // MODE_ADJW: CSR ranges of the unique receiver points
  const int* amap;                 // MODE_ADJW: [shot][k][P] CSR index of the receiver point at x on row k, or -1
  int it1;                         // 1-based index of the first step (the adjoint counts down: it1, it1 - 1)
};

// cp.async helpers (per-lane 4/8/16-byte copies into shared memory)
__device__ __forceinline__ void cpa16(void* smem, const void* g) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(g) : "memory");
}
__device__ __forceinline__ void cpa8(void* smem, const void* g) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(g) : "memory");
}
__device__ __forceinline__ void cpa4(void* smem, const void* g) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(g) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void sld4(float (&v)[4], const float4& s) {
  v[0] = s.x; v[1] = s.y; v[2] = s.z; v[3] = s.w;
}

// One row of four points advanced by one step (the arithmetic of
// Ac2dRow::update).  Points that are not advanced (act false, boundary nodes,
// padding) keep p and d; their D is 0.  mk(d) builds the C-PML strip
// descriptor of axis d only where a strip is met.
template <typename MK>
__device__ __forceinline__ void pair_row(const float (&rm)[4], const float (&r0)[4], const float (&rp)[4],
                                         float left, float right, const float (&o)[4], const float (&f)[4], int x0,
                                         int z, bool act, bool xstrip, bool fast, const StepArgs& A, MK&& mk,
                                         float (&outp)[4], float (&outd)[4], float (&outD)[4]) {
  if (fast) {  // warp-uniform: every point of the row segment interior and outside the strips
    row4_interior(rm, r0, rp, left, right, o, f, A.ih2[0], A.ih2[1], outp, outd, outD);
    return;
  }
  const int nx = A.n0, nz = A.n1, H = A.halo;
  const bool zin = z >= 1 && z <= nz - 2;
  const bool zstrip = z < H || z >= nz - H;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const float xm = e == 0 ? left : r0[e - 1];
    const float xp = e == 3 ? right : r0[e + 1];
    const float c = r0[e];
    const int x = x0 + e;
    const bool pin = act && zin && x >= 1 && x <= nx - 2;
    float tx = d2term(xm, c, xp, A.ih2[0]);
    float tz = d2term(rm[e], c, rp[e], A.ih2[1]);
    if (xstrip && pin) {
      StripIO s = mk(0);
      s.psi_base = (long long)z * (2 * H);
      s.xi_base = (long long)z * (2 * H + 2);
      tx = cpml_axis_term(tx, xm, c, xp, x, nx, H, A.ih[0], s);
    }
    if (zstrip && pin) {
      StripIO s = mk(1);
      s.psi_base = x;
      s.xi_base = x;
      tz = cpml_axis_term(tz, rm[e], c, rp[e], z, nz, H, A.ih[1], s);
    }
    const float lap = radd(tx, tz);
    const float D = rmul(f[e], lap);
    const float dd = radd(o[e], D);
    outD[e] = pin ? D : 0.f;
    outd[e] = pin ? dd : o[e];
    outp[e] = pin ? radd(c, dd) : c;
  }
}

// Stores four points of a row, interior x only (boundary nodes are never written).
__device__ __forceinline__ void pair_store(float* dst, long long row, int x0, int nx, bool vec, const float (&v)[4]) {
  if (vec) {
    st4(dst + row + x0, v);
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (x0 + e >= 1 && x0 + e <= nx - 2) dst[row + x0 + e] = v[e];
  }
}
__device__ __forceinline__ void pair_dstore(float* dst, long long row, int x0, int nx, bool vec, const float (&v)[4],
                                            int bf) {
  if (vec) {
    dst4(dst, row + x0, v, bf);
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (x0 + e >= 1 && x0 + e <= nx - 2) dst1(dst, row + x0 + e, v[e], bf);
  }
}

// Rows reach the warp through a per-warp shared-memory ring filled by
// cp.async: every lane copies its own 16-byte pieces of the rows PairRing::S-1
// iterations ahead (no registers held while they are in flight) and reads
// back only what it copied, so no barrier is needed; lanes 0 and 31 also copy
// the x neighbour beyond the warp.  Bundle j (iteration y = zb-1+j) holds p of
// row y+1, d and fact of row y and, in the adjoint, D of the first step and
// the sum g of row y and D of the second step of row y-1.
template <int MODE>
struct PairRing {
  static constexpr int NA = MODE == MODE_ADJW ? 6 : 3;  // arrays per bundle
  static constexpr int S = MODE == MODE_ADJW ? 3 : 4;   // bundles in the ring
};

// MB: resident blocks per SM the registers are bounded for (forward kinds:
// 6 blocks at <= 80 registers without spills; adjoint: 5 at <= 96).
template <int MODE, int NW, int MB>
__global__ void __launch_bounds__(32 * NW, MB) k_ac2d_pair(const StepArgs A, const PairArgs B) {
  constexpr bool ADJ = MODE == MODE_ADJW;
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int NA = PairRing<MODE>::NA, SR = PairRing<MODE>::S;
  __shared__ float4 ring[NW][SR][NA][32];
  __shared__ float hal[NW][SR][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = A.nshots;
  // block order as k_ac2d_step: x tiles fastest, then shots, then row bands
  const int txi = blockIdx.x % A.tiles_x;
  const int rest = blockIdx.x / A.tiles_x;
  const int shot = rest % S, tzi = rest / S;
  const int nx = A.n0, nz = A.n1, P = A.P, H = A.halo;
  const int zb = 1 + tzi * A.TZ;
  const int ze = min(zb + A.TZ, nz - 1);
  const int ox0 = (txi * NW + warp) * PAIR_OUT;  // first x point this warp advances by both steps
  if (zb >= ze || ox0 > nx - 2) return;          // warp-uniform
  const int x0 = ox0 - 4 + 4 * lane;
  const bool inb = x0 >= 0 && x0 < P;
  const int xa = min(max(x0, 0), P - 4);
  const bool own = inb && lane >= 1 && lane <= 30;
  const bool vec = x0 >= 1 && x0 + 3 <= nx - 2;
  const bool xstrip = inb && (x0 < H || x0 + 3 >= nx - H);
  // the warp's 128 points (both steps) interior and outside the x strips
  const bool fastx = ox0 - 4 >= plain_lo(H) && ox0 + 123 <= plain_hi(nx, H);
  const int zlo = plain_lo(H), zhi = plain_hi(nz, H);

  const float* __restrict__ pc = fptr(A.pcur, shot);
  const float* __restrict__ di = fptr(A.din, shot);
  const float* __restrict__ fa = A.fact;
  float* pn = fptr(A.pnew, shot);
  float* dn = fptr(A.dout, shot);
  float* ckp = fptr(A.ck_p, shot);
  float* ckd = fptr(A.ck_d, shot);
  const bool dw = MODE == MODE_FWD_D && shot >= A.d_first;
  float* Dw1 = dw ? dptr(A.Dout, shot, A.dbf16) : nullptr;
  float* Dw2 = dw ? dptr(B.Dout2, shot, A.dbf16) : nullptr;
  float* stash = B.stash.p ? B.stash.p + (long long)shot * B.stash.s : nullptr;
  const PairShot* T = B.shots + shot;
  const int nsp = ADJ ? 0 : T->nsp, nrr = (stash || ADJ) ? T->nrr : 0;
  const float* dc1 = ADJ ? dptr(A.dcorr, shot, A.dbf16) : nullptr;
  const float* dc2 = ADJ ? dptr(B.dcorr2, shot, A.dbf16) : nullptr;
  float* gg = ADJ ? fptr(A.g, shot) : nullptr;
  const int* am = ADJ ? B.amap + (long long)shot * PAIR_MAXRR * P : nullptr;

  const int na = 2 * H + 2, nh = 2 * H, L = 2 * na + 2 * nh;
  const float* cpb = A.cpml + (long long)shot * A.cpml_stride;
  // first step: psi, xi of step n -> scratch, with the checkpoint copies of step n
  auto mk1 = [&](int d) {
    StripIO s;
    const float* c = cpb + d * L;
    s.a = c; s.ah = c + na; s.b = c + na + nh; s.bh = c + 2 * na + nh;
    s.psi_in = fptr(A.psi_in[d], shot); s.psi_out = fptr(B.psi_mid[d], shot); s.ck_psi = fptr(A.ck_psi[d], shot);
    s.xi_in = fptr(A.xi_in[d], shot);   s.xi_out = fptr(B.xi_mid[d], shot);   s.ck_xi = fptr(A.ck_xi[d], shot);
    s.psi_step = d == 0 ? 1 : P;
    s.xi_step = s.psi_step;
    return s;
  };
  // second step: scratch -> psi, xi of step n+2
  auto mk2 = [&](int d) {
    StripIO s;
    const float* c = cpb + d * L;
    s.a = c; s.ah = c + na; s.b = c + na + nh; s.bh = c + 2 * na + nh;
    s.psi_in = fptr(B.psi_mid[d], shot); s.psi_out = fptr(A.psi_out[d], shot); s.ck_psi = nullptr;
    s.xi_in = fptr(B.xi_mid[d], shot);   s.xi_out = fptr(A.xi_out[d], shot);   s.ck_xi = nullptr;
    s.psi_step = d == 0 ? 1 : P;
    s.xi_step = s.psi_step;
    return s;
  };

  auto issue = [&](int j) {  // bundle j into slot j % SR; an empty group past the band
    const int yj = zb - 1 + j;
    if (yj <= ze) {
      const int sl = j % SR;
      const long long rj = (long long)yj * P;
      const bool nxt = yj + 1 <= nz - 1;
      if (inb) {
        if (nxt) cpa16(&ring[warp][sl][0][lane], pc + rj + P + x0);
        cpa16(&ring[warp][sl][1][lane], di + rj + x0);
        cpa16(&ring[warp][sl][2][lane], fa + rj + x0);
      }
      if constexpr (ADJ) {
        if (own && yj >= zb && yj < ze) {
          if (A.dbf16)
            cpa8(&ring[warp][sl][3][lane], reinterpret_cast<const __nv_bfloat16*>(dc1) + rj + x0);
          else
            cpa16(&ring[warp][sl][3][lane], dc1 + rj + x0);
          cpa16(&ring[warp][sl][4][lane], gg + rj + x0);
        }
        if (own && yj >= zb + 1) {
          if (A.dbf16)
            cpa8(&ring[warp][sl][5][lane], reinterpret_cast<const __nv_bfloat16*>(dc2) + rj - P + x0);
          else
            cpa16(&ring[warp][sl][5][lane], dc2 + rj - P + x0);
        }
      }
      if (nxt && lane == 0 && x0 >= 1) cpa4(&hal[warp][sl][0], pc + rj + P + x0 - 1);
      if (nxt && lane == 31 && x0 + 4 < P) cpa4(&hal[warp][sl][1], pc + rj + P + x0 + 4);
    }
    cpa_commit();
  };
  auto bundle_d = [&](float (&v)[4], const float4& slot) {  // D slot of a bundle, FP32 or BF16
    if (A.dbf16) {
      const uint2 u = *reinterpret_cast<const uint2*>(&slot);
      const float2 lo = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.x));
      const float2 hi = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.y));
      v[0] = lo.x; v[1] = lo.y; v[2] = hi.x; v[3] = hi.y;
    } else {
      sld4(v, slot);
    }
  };

  // p of step n at rows y-1, y, y+1 (rm, r0, rp) with the x neighbours of row
  // y beyond the warp (hl, hr), d and fact of row y; p of step n+1 at rows
  // y-2, y-1 (qm, q0), d of step n+1 and fact of row y-1
  float rm[4] = {0.f, 0.f, 0.f, 0.f}, r0[4], rp[4], o[4], f[4];
  float qm[4] = {0.f, 0.f, 0.f, 0.f}, q0[4] = {0.f, 0.f, 0.f, 0.f}, dq[4] = {0.f, 0.f, 0.f, 0.f},
        fq[4] = {0.f, 0.f, 0.f, 0.f};
  float g1[4] = {0.f, 0.f, 0.f, 0.f};  // adjoint: the sum g of row y-1 after its first step's correlation
  int y = zb - 1;
  if (y >= 1) ld4(rm, pc + (long long)(y - 1) * P + xa);
  ld4(r0, pc + (long long)y * P + xa);
  float hl = (lane == 0 && x0 >= 1) ? pc[(long long)y * P + x0 - 1] : 0.f;
  float hr = (lane == 31 && x0 + 4 < P) ? pc[(long long)y * P + x0 + 4] : 0.f;
#pragma unroll
  for (int q = 0; q < SR - 1; ++q) issue(q);
  for (int j = 0; y <= ze; ++y, ++j) {
    const long long row = (long long)y * P;
    cpa_wait<SR - 2>();  // bundle j has landed (bundles j+1 .. j+SR-2 may be in flight)
    __syncwarp();        // and the scratch strips written by the lanes' first step of the previous row
    const int sl = j % SR;
    sld4(rp, ring[warp][sl][0][lane]);
    sld4(o, ring[warp][sl][1][lane]);
    sld4(f, ring[warp][sl][2][lane]);
    const float nhl = hal[warp][sl][0], nhr = hal[warp][sl][1];
    // adjoint: D of both steps and the sum g, for the rows they are used on;
    // gn: the sum of row y after the first step (g1 holds row y-1's)
    const bool orow = y >= zb && y < ze;
    float dv1[4] = {0.f, 0.f, 0.f, 0.f}, dv2[4] = {0.f, 0.f, 0.f, 0.f}, gv[4] = {0.f, 0.f, 0.f, 0.f};
    float gn[4] = {0.f, 0.f, 0.f, 0.f};
    if constexpr (ADJ) {
      if (own && orow) {
        bundle_d(dv1, ring[warp][sl][3][lane]);
        sld4(gv, ring[warp][sl][4][lane]);
      }
      if (own && y >= zb + 1) bundle_d(dv2, ring[warp][sl][5][lane]);
    }
    // first step, row y
    float left = __shfl_up_sync(FULL, r0[3], 1);
    float right = __shfl_down_sync(FULL, r0[0], 1);
    if (lane == 0) left = hl;
    if (lane == 31) right = hr;
    float p1[4], d1[4], D1[4];
    pair_row(rm, r0, rp, left, right, o, f, x0, y, inb, xstrip, fastx && y >= zlo && y <= zhi, A, mk1, p1, d1, D1);
    if constexpr (ADJ) {
      // correlation of the first step on the band's rows (before its
      // injection, as the one-step kernel), then the first step's adjoint
      // sources at the receivers with their share lambda_add * D
      const bool cor = own && orow;
      if (cor) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          gn[e] = gv[e];
          if (x0 + e >= 1 && x0 + e <= nx - 2) gn[e] = __fmaf_rn(p1[e], dv1[e], gn[e]);
        }
      }
      for (int k = 0; k < nrr; ++k) {
        if (T->rrow[k] != y || !inb) continue;
        const int4 m = *reinterpret_cast<const int4*>(am + (long long)k * P + x0);
        const int mm[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (mm[e] < 0) continue;
          float acc = p1[e], add = 0.f;
          for (int jj = B.ptr[mm[e]]; jj < B.ptr[mm[e] + 1]; ++jj) {
            const float v = T->adj[(long long)(B.it1 - 1) + (long long)B.ids[jj] * T->nt];
            acc = radd(acc, v);
            add = radd(add, v);
          }
          p1[e] = acc;
          d1[e] = radd(d1[e], add);
          if (cor) gn[e] = __fmaf_rn(add, dv1[e], gn[e]);
        }
      }
    }
    for (int s = 0; s < nsp; ++s) {  // sources of the first step
      if (T->sz[s] != y) continue;
      const int dx = T->sx[s] - x0;
      if (dx < 0 || dx > 3 || !inb) continue;
      const int k0 = T->k0[s], k1 = T->k1[s];
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (e == dx) {
          float acc = p1[e], add = 0.f;
          for (int k = k0; k < k1; ++k) {
            const float v = T->tf[(long long)(B.it1 - 1) + (long long)B.ids[k] * T->nt];
            acc = radd(acc, v);
            add = radd(add, v);
          }
          p1[e] = acc;
          d1[e] = radd(d1[e], add);
          // k_inject_record adds to the stored D: with BF16 slots the stencil's
          // D is rounded to BF16 before the source is added
          const float Ds = A.dbf16 ? __bfloat162float(__float2bfloat16_rn(D1[e])) : D1[e];
          D1[e] = radd(Ds, add);
        }
    }
    if (own && orow) {  // outputs of the first step on the band's own rows
      if (ckp) {
        st4(ckp + row + x0, r0);
        st4(ckd + row + x0, o);
      }
      if (Dw1) pair_dstore(Dw1, row, x0, nx, vec, D1, A.dbf16);
      if (stash)
        for (int k = 0; k < nrr; ++k)
          if (T->rrow[k] == y) st4(stash + (long long)k * P + x0, p1);
    }
    // second step, row y-1
    if (y >= zb + 1) {
      const long long zrow = row - P;
      const float l2 = __shfl_up_sync(FULL, q0[3], 1);
      const float r2 = __shfl_down_sync(FULL, q0[0], 1);
      float p2[4], d2[4], D2[4];
      pair_row(qm, q0, p1, l2, r2, dq, fq, x0, y - 1, own, xstrip, fastx && y - 1 >= zlo && y - 1 <= zhi, A, mk2,
               p2, d2, D2);
      if (own) {
        pair_store(pn, zrow, x0, nx, vec, p2);
        pair_store(dn, zrow, x0, nx, vec, d2);
        if (Dw2) pair_dstore(Dw2, zrow, x0, nx, vec, D2, A.dbf16);
        if constexpr (ADJ) {  // correlation of the second step, then the row's sum goes back once
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (x0 + e >= 1 && x0 + e <= nx - 2) g1[e] = __fmaf_rn(p2[e], dv2[e], g1[e]);
          pair_store(gg, zrow, x0, nx, vec, g1);
        }
      }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if constexpr (ADJ) g1[e] = gn[e];
      qm[e] = q0[e];
      q0[e] = p1[e];
      dq[e] = d1[e];
      fq[e] = f[e];
      rm[e] = r0[e];
      r0[e] = rp[e];
    }
    hl = nhl;
    hr = nhr;
    issue(j + SR - 1);  // into the slot of bundle j-1, consumed in the previous iteration
  }
  cpa_wait<0>();
}

// ---------------------------------------------------------------------------
// 2D step with the rows staged through shared memory by cp.async.
//
// The register-pipelined kernel holds one row of loads in flight per warp,
// and a second register row costs more occupancy than it brings.  This
// variant keeps S-1 rows in flight without registers; on GB300 it measured
// slower all the same (64 shots of 2001 x 801: 3.75 / 4.23 / 4.71 TB/s
// forward / recompute / adjoint against 4.15 / 4.56 / 4.79), so more loads
// in flight are not what these kernels lack, and it stays a tuning variant
// (512).  Every lane copies its own 16-byte pieces of the rows ahead
// into a per-warp ring of S row bundles with cp.async (no registers held
// while in flight) and later reads back only what it copied itself, so no
// barrier is needed: cp.async.wait_group orders a lane's copies with its own
// reads.  Bundle k holds p of row k+1 (with the x neighbours x0-1 of lane 0
// and x0+4 of lane 31), d and fact of row k and, in the adjoint, D and the
// sums g (gc) of row k; S-1 bundles are in flight while row z is computed.
// Bundle z+S-1 reuses the slot of bundle z-1, whose values the row update of
// iteration z-1 has already consumed.
// ---------------------------------------------------------------------------
// Row arrays per bundle (p, d, fact [, D, g [, gc]]) and bundles in the ring:
// 24 KB of ring per 4-warp block for the forward kinds (8 blocks per SM),
// 30 / 36 KB for the adjoints (6 / 4 blocks per SM).
template <int MODE>
struct CpaRing {
  static constexpr int NA = MODE == MODE_ADJ ? 6 : MODE == MODE_ADJW ? 5 : 3;
  static constexpr int S = (MODE == MODE_ADJ || MODE == MODE_ADJW) ? 3 : 4;
};

template <int MODE, int NW>
__global__ void __launch_bounds__(32 * NW, Ac2dBounds<MODE, NW>::MINB) k_ac2d_cpa(const StepArgs A) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int NA = CpaRing<MODE>::NA, S = CpaRing<MODE>::S;
  constexpr bool ADJ = MODE == MODE_ADJ || MODE == MODE_ADJW;
  __shared__ float4 ring[NW][S][NA][32];
  __shared__ float halo[NW][S][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int txi = blockIdx.x % A.tiles_x;
  const int rest = blockIdx.x / A.tiles_x;
  const int shot = rest % A.nshots, tzi = rest / A.nshots;
  const int nz = A.n1, P = A.P;
  const int z_begin = 1 + tzi * A.TZ;
  const int z_end = min(z_begin + A.TZ, nz - 1);
  const int wx0 = (txi * NW + warp) * 128;
  if (z_begin >= z_end || wx0 >= P) return;  // warp-uniform
  const int x0 = wx0 + lane * 4;
  const int xa = x0 < P ? x0 : P - 4;
  const bool has_left = lane == 0 && xa > 0, has_right = lane == 31 && xa + 4 < P;

  const float* __restrict__ pc = fptr(A.pcur, shot);
  const float* di = fptr(A.din, shot);
  const float* __restrict__ fa = A.fact;
  Ac2dRow<MODE> R;
  R.init(A, shot, x0);
  const float* dcr = ADJ ? dptr(A.dcorr, shot, A.dbf16) : nullptr;

  auto issue = [&](int k) {  // bundle k into slot k % S; an empty group past the band
    if (k < z_end) {
      const int sl = k % S;
      const long long row = (long long)k * P;
      cpa16(&ring[warp][sl][0][lane], pc + row + P + xa);
      cpa16(&ring[warp][sl][1][lane], di + row + xa);
      cpa16(&ring[warp][sl][2][lane], fa + row + xa);
      if (has_left) cpa4(&halo[warp][sl][0], pc + row + P + xa - 1);
      if (has_right) cpa4(&halo[warp][sl][1], pc + row + P + xa + 4);
      if constexpr (ADJ) {
        if (A.dbf16)
          cpa8(&ring[warp][sl][3][lane], reinterpret_cast<const __nv_bfloat16*>(dcr) + row + xa);
        else
          cpa16(&ring[warp][sl][3][lane], dcr + row + xa);
        cpa16(&ring[warp][sl][4][lane], R.gg + row + xa);
        if constexpr (MODE == MODE_ADJ) cpa16(&ring[warp][sl][5][lane], R.gcp + row + xa);
      }
    }
    cpa_commit();
  };

  float rm[4], r0[4];
  ld4(rm, pc + (long long)(z_begin - 1) * P + xa);
  ld4(r0, pc + (long long)z_begin * P + xa);
  float hl = has_left ? pc[(long long)z_begin * P + xa - 1] : 0.f;
  float hr = has_right ? pc[(long long)z_begin * P + xa + 4] : 0.f;
#pragma unroll
  for (int q = 0; q < S - 1; ++q) issue(z_begin + q);
  for (int z = z_begin; z < z_end; ++z) {
    cpa_wait<S - 2>();  // bundle z has landed (bundles z+1 .. z+S-2 may be in flight)
    const int sl = z % S;
    float rp[4], o[4], f[4], dv[4], g4[4], c4[4];
    sld4(rp, ring[warp][sl][0][lane]);
    sld4(o, ring[warp][sl][1][lane]);
    sld4(f, ring[warp][sl][2][lane]);
    const float nhl = has_left ? halo[warp][sl][0] : 0.f;
    const float nhr = has_right ? halo[warp][sl][1] : 0.f;
    if constexpr (ADJ) {
      if (A.dbf16) {
        const uint2 u = *reinterpret_cast<const uint2*>(&ring[warp][sl][3][lane]);
        const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.x));
        const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.y));
        dv[0] = a.x; dv[1] = a.y; dv[2] = b.x; dv[3] = b.y;
      } else {
        sld4(dv, ring[warp][sl][3][lane]);
      }
      sld4(g4, ring[warp][sl][4][lane]);
      if constexpr (MODE == MODE_ADJ) sld4(c4, ring[warp][sl][5][lane]);
    }
    float left = __shfl_up_sync(FULL, r0[3], 1);
    float right = __shfl_down_sync(FULL, r0[0], 1);
    if (lane == 0) left = hl;
    if (lane == 31) right = hr;
    R.update(z, rm, r0, rp, o, f, dv, g4, c4, left, right);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      rm[e] = r0[e];
      r0[e] = rp[e];
    }
    hl = nhl;
    hr = nhr;
    issue(z + S - 1);
  }
  cpa_wait<0>();
}

// ---------------------------------------------------------------------------
// 2D adjoint step for a group of 4 shots with the correlation summed over the
// group before it is accumulated.  Warp w of a block runs shot 4*group + w
// over the same 128 x points and row band (the same per-shot arithmetic as
// k_ac2d_step<MODE_ADJ>); per row the four products lambda * D of a point are
// added in shot order and Kahan-accumulated once into the group's gradient
// pair (g, gc).  The per-point read-modify-write of the accumulator is thus
// shared by 4 shots (36 -> 24 bytes per shot and point); the fixed order
// keeps the result deterministic.  Warps of inactive shots (it > nt) only
// take part in the block barriers.
// ---------------------------------------------------------------------------
template <int MINB>
__global__ void __launch_bounds__(128, MINB) k_ac2d_adj_grp(const StepArgs A) {
  constexpr unsigned FULL = 0xffffffffu;
  __shared__ float4 prod[2][4][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = A.nshots;
  const int ngrp = (S + 3) / 4;
  const int txi = blockIdx.x % A.tiles_x;
  const int rest = blockIdx.x / A.tiles_x;
  const int grp = rest % ngrp, tzi = rest / ngrp;
  const int shot = grp * 4 + warp;
  const bool active = shot < S;
  const int nx = A.n0, nz = A.n1, P = A.P, H = A.halo;
  const int z_begin = 1 + tzi * A.TZ;
  const int z_end = min(z_begin + A.TZ, nz - 1);
  const int wx0 = txi * 128;
  if (z_begin >= z_end || wx0 >= P) return;  // block-uniform
  const int x0 = wx0 + lane * 4;
  const bool inb = x0 < P;
  const int xa = inb ? x0 : P - 4;
  const int sh = active ? shot : 0;

  const float* __restrict__ pc = fptr(A.pcur, sh);
  float* __restrict__ pn = fptr(A.pnew, sh);
  const float* di = fptr(A.din, sh);
  float* dn = fptr(A.dout, sh);
  const float* __restrict__ fa = A.fact;
  const float* dcr = dptr(A.dcorr, sh, A.dbf16);
  const float* cp = A.cpml + (long long)sh * A.cpml_stride;
  const int na = 2 * H + 2, nh = 2 * H, L = 2 * na + 2 * nh;
  StripIO sx, sz;
  sx.psi_in = fptr(A.psi_in[0], sh);  sx.psi_out = fptr(A.psi_out[0], sh);
  sx.xi_in = fptr(A.xi_in[0], sh);    sx.xi_out = fptr(A.xi_out[0], sh);
  sx.ck_psi = nullptr;                sx.ck_xi = nullptr;
  sx.a = cp; sx.ah = cp + na; sx.b = cp + na + nh; sx.bh = cp + 2 * na + nh;
  sx.psi_step = 1; sx.xi_step = 1;
  sz.psi_in = fptr(A.psi_in[1], sh);  sz.psi_out = fptr(A.psi_out[1], sh);
  sz.xi_in = fptr(A.xi_in[1], sh);    sz.xi_out = fptr(A.xi_out[1], sh);
  sz.ck_psi = nullptr;                sz.ck_xi = nullptr;
  sz.a = cp + L; sz.ah = cp + L + na; sz.b = cp + L + na + nh; sz.bh = cp + L + 2 * na + nh;
  sz.psi_step = P; sz.xi_step = P;
  const bool xstrip = inb && (x0 < H || x0 + 3 >= nx - H);
  const bool vec_interior = (x0 >= 1) && (x0 + 3 <= nx - 2);

  // the block's reduction: thread t owns point wx0 + t of the group accumulator
  const int xt = wx0 + threadIdx.x;
  const bool tin = xt >= 1 && xt <= nx - 2;
  float* gp = A.g.p + (long long)grp * A.g.s;
  float* gcp = A.gc.p + (long long)grp * A.gc.s;

  float rm[4], r0[4], rp[4], o[4], f[4], dv[4];
  if (active) {
    ld4(rm, pc + (long long)(z_begin - 1) * P + xa);
    ld4(r0, pc + (long long)z_begin * P + xa);
    const long long row = (long long)z_begin * P;
    ld4(rp, pc + row + P + xa);
    ld4rw(o, di + row + xa);
    ld4(f, fa + row + xa);
    dld4(dv, dcr, row + xa, A.dbf16);
  }
  float gv = 0.f, cv = 0.f;
  if (tin) {
    gv = gp[(long long)z_begin * P + xt];
    cv = gcp[(long long)z_begin * P + xt];
  }
  int par = 0;
  for (int z = z_begin; z < z_end; ++z) {
    const long long row = (long long)z * P;
    const bool more = z + 1 < z_end;
    float rpn[4], on[4], fn[4], dvn[4];
    float gvn = 0.f, cvn = 0.f;
    if (active && more) {
      const long long nrow = row + P;
      ld4(rpn, pc + nrow + P + xa);
      ld4rw(on, di + nrow + xa);
      ld4(fn, fa + nrow + xa);
      dld4(dvn, dcr, nrow + xa, A.dbf16);
    }
    if (tin && more) {
      gvn = gp[row + P + xt];
      cvn = gcp[row + P + xt];
    }
    float4 pr = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
      float left = __shfl_up_sync(FULL, r0[3], 1);
      float right = __shfl_down_sync(FULL, r0[0], 1);
      if (lane == 0) left = xa > 0 ? pc[row + xa - 1] : 0.f;
      if (lane == 31) right = xa + 4 < P ? pc[row + xa + 4] : 0.f;
      const bool zstrip = (z < H) || (z >= nz - H);
      sx.psi_base = (long long)z * nh;
      sx.xi_base = (long long)z * na;
      float outp[4], outd[4], prd[4];
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
        outd[e] = o[e] + f[e] * lap;
        outp[e] = c + outd[e];
        prd[e] = pin ? outp[e] * dv[e] : 0.f;
      }
      pr = make_float4(prd[0], prd[1], prd[2], prd[3]);
      if (inb) {
        if (vec_interior) {
          st4(pn + row + x0, outp);
          st4(dn + row + x0, outd);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int x = x0 + e;
            if (x >= 1 && x <= nx - 2) {
              pn[row + x] = outp[e];
              dn[row + x] = outd[e];
            }
          }
        }
      }
    }
    prod[par][warp][lane] = pr;
    __syncthreads();
    if (tin) {
      const float* pf = reinterpret_cast<const float*>(&prod[par][0][0]);
      const float sum = ((pf[threadIdx.x] + pf[128 + threadIdx.x]) + pf[256 + threadIdx.x]) + pf[384 + threadIdx.x];
      kahan_add(gv, cv, sum);
      gp[row + xt] = gv;
      gcp[row + xt] = cv;
    }
    par ^= 1;
    gv = gvn;
    cv = cvn;
    if (active) {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        rm[e] = r0[e];
        r0[e] = rp[e];
        if (more) {
          rp[e] = rpn[e];
          o[e] = on[e];
          f[e] = fn[e];
          dv[e] = dvn[e];
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// 3D: axes 0 = x, 1 = y, 2 = z.  Block = 4 warps, one y row each (128 x
// points per warp); tile = 128 x 4 y x TZ z.  y neighbours come through L1.
// psi_0/xi_0: [z][y][q];  psi_1/xi_1: [z][q][P];  psi_2/xi_2: [q][y][P].
// ---------------------------------------------------------------------------
// C-PML strip descriptor of axis d for one shot (built where it is needed).
__device__ __forceinline__ StripIO strip_io(const StepArgs& A, int d, int shot, long long step) {
  const int H = A.halo;
  const int na = 2 * H + 2, nh = 2 * H, L = 2 * na + 2 * nh;
  const float* cp = A.cpml + (long long)shot * A.cpml_stride + (long long)d * L;
  StripIO s;
  s.psi_in = fptr(A.psi_in[d], shot);
  s.psi_out = fptr(A.psi_out[d], shot);
  s.xi_in = fptr(A.xi_in[d], shot);
  s.xi_out = fptr(A.xi_out[d], shot);
  s.ck_psi = fptr(A.ck_psi[d], shot);
  s.ck_xi = fptr(A.ck_xi[d], shot);
  s.a = cp;
  s.ah = cp + na;
  s.b = cp + na + nh;
  s.bh = cp + 2 * na + nh;
  s.psi_step = step;
  s.xi_step = step;
  s.psi_base = 0;
  s.xi_base = 0;
  return s;
}

// Split of the (y, z) rows for the two-launch 3D step: per axis the rows
// [1, a) and [b, n-1) lie in (or next to) the C-PML strips, [a, b) outside.
__device__ __forceinline__ void split_axis(int n, int H, int& a, int& b) {
  a = min(max(H, 1), n - 1);
  b = max(n - max(H, 1), a);
}

// Work of one warp in the 3D step: (y row, z band) for a block index.
// REGION 0: the whole grid (tiles_y x tiles_z bands).  REGION 1: rows with y
// and z outside the C-PML strips (tiles_y x tiles_z over [a, b) of each).
// REGION 2: the z slabs (z in [1, a) or [b, nz-1), every y).  REGION 3: the
// y slabs (z in [a, b), y in [1, a) or [b, ny-1)).  Slabs are enumerated per
// x tile as (z band, y group) units.
template <int NW, int REGION>
__device__ __forceinline__ bool ac3d_work(const StepArgs& A, int tile, int warp, int& y, int& z_begin, int& z_end) {
  const int ny = A.n1, nz = A.n2, H = A.halo, TZ = A.TZ;
  if (REGION == 0) {
    const int tyi = tile % A.tiles_y, tzi = tile / A.tiles_y;
    y = 1 + tyi * NW + warp;
    z_begin = 1 + tzi * TZ;
    z_end = min(z_begin + TZ, nz - 1);
    return z_begin < z_end && y <= ny - 2;
  }
  int ay, by, az, bz;
  split_axis(ny, H, ay, by);
  split_axis(nz, H, az, bz);
  if (REGION == 1) {
    const int tyi = tile % A.tiles_y, tzi = tile / A.tiles_y;
    y = ay + tyi * NW + warp;
    z_begin = az + tzi * TZ;
    z_end = min(z_begin + TZ, bz);
    return z_begin < z_end && y < by;
  }
  const int gy_all = (ny - 2 + NW - 1) / NW;
  const int nb_lo = (az - 1 + TZ - 1) / TZ;
  if (REGION == 2) {
    const int kz = tile / gy_all, gy = tile % gy_all;
    y = 1 + gy * NW + warp;
    if (kz < nb_lo) {
      z_begin = 1 + kz * TZ;
      z_end = min(z_begin + TZ, az);
    } else {
      z_begin = bz + (kz - nb_lo) * TZ;
      z_end = min(z_begin + TZ, nz - 1);
    }
    return z_begin < z_end && y <= ny - 2;
  }
  const int gyl = (ay - 1 + NW - 1) / NW, gyh = (ny - 1 - by + NW - 1) / NW;
  if (gyl + gyh == 0) return false;
  const int kz = tile / (gyl + gyh), g = tile % (gyl + gyh);
  z_begin = az + kz * TZ;
  z_end = min(z_begin + TZ, bz);
  if (g < gyl) {
    y = 1 + g * NW + warp;
    return z_begin < z_end && y < ay;
  }
  y = by + (g - gyl) * NW + warp;
  return z_begin < z_end && y <= ny - 2;
}

template <int MODE, int NW, bool FAST = false, int REGION = 0, bool PIPE = true>
__device__ __forceinline__ void ac3d_body(const StepArgs& A) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = A.nshots;
  const int shot = blockIdx.x % S;
  int tile = blockIdx.x / S;
  const int txi = tile % A.tiles_x;
  tile /= A.tiles_x;
  const int nx = A.n0, ny = A.n1, nz = A.n2, P = A.P, H = A.halo;
  int y, z_begin, z_end;  // one y row per warp, NW rows per block
  if (!ac3d_work<NW, REGION>(A, tile, warp, y, z_begin, z_end)) return;  // warp-uniform
  const int wx0 = txi * 128;
  const int x0 = wx0 + lane * 4;
  const bool inb = x0 < P;
  const int xa = inb ? x0 : P - 4;
  const long long plane = (long long)P * ny;

  const float* __restrict__ pc = fptr(A.pcur, shot);
  float* __restrict__ pn = fptr(A.pnew, shot);
  const float* di = fptr(A.din, shot);
  float* dn = fptr(A.dout, shot);
  const float* __restrict__ fa = A.fact;
  const int na = 2 * H + 2, nh = 2 * H;

  const bool xstrip = inb && (x0 < H || x0 + 3 >= nx - H);
  // region 1: never in a y strip; region 3: always
  const bool ystrip = REGION == 3 || (REGION != 1 && ((y < H) || (y >= ny - H)));
  // the warp's 128 x points and its y row interior and outside the strips
  const bool fastxy = wx0 >= plain_lo(H) && wx0 + 127 <= plain_hi(nx, H) && y >= plain_lo(H) && y <= plain_hi(ny, H);
  const bool vec_interior = (x0 >= 1) && (x0 + 3 <= nx - 2);
  float* ckp = fptr(A.ck_p, shot);
  float* ckd = fptr(A.ck_d, shot);
  float* Dw = nullptr;
  if (MODE == MODE_FWD_D && shot >= A.d_first) Dw = dptr(A.Dout, shot, A.dbf16);
  const float* dcr = MODE == MODE_ADJ ? dptr(A.dcorr, shot, A.dbf16) : nullptr;
  float* gg = MODE == MODE_ADJ ? fptr(A.g, shot) : nullptr;
  float* gcp = MODE == MODE_ADJ ? fptr(A.gc, shot) : nullptr;

  // Software-pipelined z march: the loads of plane z+1 (p of z+2, the y
  // neighbours, d and fact) are issued before plane z is computed.  The
  // C-PML strip descriptors are built only where a strip is met (they would
  // otherwise hold ~60 registers for the whole kernel).
  const long long rowoff = (long long)y * P + xa;
  float rm[4], r0[4], rp[4], ym[4], yp[4], o[4], f[4];
  {
    const long long idx = (long long)z_begin * plane + rowoff;
    ld4(rm, pc + idx - plane);
    ld4(r0, pc + idx);
    if (PIPE) {
      ld4(rp, pc + idx + plane);
      ld4(ym, pc + idx - P);
      ld4(yp, pc + idx + P);
      ld4rw(o, di + idx);
      ld4(f, fa + idx);
    }
  }
  for (int z = z_begin; z < z_end; ++z) {
    const long long base = (long long)z * plane;
    const long long idx = base + rowoff;
    const bool more = PIPE && z + 1 < z_end;
    float rpn[4], ymn[4], ypn[4], on[4], fn[4];
    if (!PIPE) {  // no software pipeline: fewer registers, more resident warps
      ld4(rp, pc + idx + plane);
      ld4(ym, pc + idx - P);
      ld4(yp, pc + idx + P);
      ld4rw(o, di + idx);
      ld4(f, fa + idx);
    } else if (more) {
      const long long nidx = idx + plane;
      ld4(rpn, pc + nidx + plane);
      ld4(ymn, pc + nidx - P);
      ld4(ypn, pc + nidx + P);
      ld4rw(on, di + nidx);
      ld4(fn, fa + nidx);
    }
    float left = __shfl_up_sync(FULL, r0[3], 1);
    float right = __shfl_down_sync(FULL, r0[0], 1);
    if (lane == 0) left = xa > 0 ? pc[idx - 1] : 0.f;
    if (lane == 31) right = xa + 4 < P ? pc[idx + 4] : 0.f;
    // regions 1 and 3: never in a z strip; region 2: always
    const bool zstrip = REGION == 2 || (REGION != 1 && REGION != 3 && ((z < H) || (z >= nz - H)));
    float outp[4], outd[4], outD[4];
    if (FAST && fastxy && z >= plain_lo(H) && z <= plain_hi(nz, H)) {
      // warp-uniform: every point interior and outside the strips
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float xm = e == 0 ? left : r0[e - 1];
        const float xp = e == 3 ? right : r0[e + 1];
        const float c = r0[e];
        const float lap = radd(radd(d2term(xm, c, xp, A.ih2[0]), d2term(ym[e], c, yp[e], A.ih2[1])),
                               d2term(rm[e], c, rp[e], A.ih2[2]));
        outD[e] = rmul(f[e], lap);
        outd[e] = radd(o[e], outD[e]);
        outp[e] = radd(c, outd[e]);
      }
    } else {
      float tx[4], ty[4], tz[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float xm = e == 0 ? left : r0[e - 1];
        const float xp = e == 3 ? right : r0[e + 1];
        const float c = r0[e];
        tx[e] = d2term(xm, c, xp, A.ih2[0]);
        ty[e] = d2term(ym[e], c, yp[e], A.ih2[1]);
        tz[e] = d2term(rm[e], c, rp[e], A.ih2[2]);
        const int x = x0 + e;
        if (xstrip && inb && x >= 1 && x <= nx - 2) {
          StripIO s0 = strip_io(A, 0, shot, 1);
          s0.psi_base = ((long long)z * ny + y) * nh;
          s0.xi_base = ((long long)z * ny + y) * na;
          tx[e] = cpml_axis_term(tx[e], xm, c, xp, x, nx, H, A.ih[0], s0);
        }
      }
      // the y and z strips: the strip cell is the same for the four points
      // (it depends on y or z only), so their memory variables move as float4
      if (ystrip && inb) {
        StripIO s1 = strip_io(A, 1, shot, P);
        s1.psi_base = (long long)z * nh * P + xa;
        s1.xi_base = (long long)z * na * P + xa;
        cpml_axis_term4(ty, ym, r0, yp, y, ny, H, A.ih[1], s1);
      }
      if (zstrip && inb) {
        StripIO s2 = strip_io(A, 2, shot, (long long)ny * P);
        s2.psi_base = (long long)y * P + xa;
        s2.xi_base = (long long)y * P + xa;
        cpml_axis_term4(tz, rm, r0, rp, z, nz, H, A.ih[2], s2);
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float lap = radd(radd(tx[e], ty[e]), tz[e]);
        outD[e] = rmul(f[e], lap);
        outd[e] = radd(o[e], outD[e]);
        outp[e] = radd(r0[e], outd[e]);
      }
    }
    // FP16 D slots: the exponent of this warp's tile of row (y, z)
    const long long erow = ((long long)z * ny + y) * A.ntx + txi;
    int de = 0;
    if (MODE == MODE_FWD_D && A.dbf16 == 2 && Dw) {
      de = warp_dexp(outD, inb);
      if (lane == 0) A.Dexp.p[(long long)shot * A.Dexp.s + erow] = (signed char)de;
    }
    if (inb) {
      if (ckp) {
        st4(ckp + idx, r0);
        st4(ckd + idx, o);
      }
      if (MODE == MODE_ADJ) {
        float dv[4], g4[4], c4[4];
        dld4(dv, dcr, idx, A.dbf16, A.dbf16 == 2 ? A.dcorr_exp.p[(long long)shot * A.dcorr_exp.s + erow] : 0);
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
        if (MODE == MODE_FWD_D && Dw) dst4(Dw, idx, outD, A.dbf16, de);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int x = x0 + e;
          if (x >= 1 && x <= nx - 2) {
            pn[idx + e] = outp[e];
            dn[idx + e] = outd[e];
            if (MODE == MODE_FWD_D && Dw) dst1(Dw, idx + e, outD[e], A.dbf16, de);
          }
        }
      }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      rm[e] = r0[e];
      r0[e] = rp[e];
      if (more) {
        rp[e] = rpn[e];
        ym[e] = ymn[e];
        yp[e] = ypn[e];
        o[e] = on[e];
        f[e] = fn[e];
      }
    }
  }
}


// The gradient's forward / recompute (D output) and adjoint steps run faster
// at 6 resident blocks per SM (<= 85 registers: 23.3 against 22.0 Gpts/s on
// 16 shots of 400^3); the plain forward is fastest with the compiler's own
// register choice (1.96 against 1.76 TB/s).
template <int MODE, int NW = 4>
__global__ void __launch_bounds__(32 * NW, 24 / NW) k_ac3d_step(const StepArgs A) {
  ac3d_body<MODE, NW>(A);
}
template <int MODE, int NW = 4>
__global__ void __launch_bounds__(32 * NW) k_ac3d_fwd(const StepArgs A) {
  ac3d_body<MODE, NW, true>(A);
}
// Three-launch 3D step: rows outside the y and z strips (no y / z C-PML code,
// fewer registers), the z slabs (z strip code only where it applies), the y
// slabs.  Every point is computed by exactly one launch with the arithmetic
// of ac3d_body.
template <int MODE, int NW = 4>
__global__ void __launch_bounds__(32 * NW, 24 / NW) k_ac3d_inner(const StepArgs A) {
  ac3d_body<MODE, NW, false, 1>(A);
}
// the same without the software pipeline, at 8 resident blocks of 4 warps
template <int MODE, int NW = 4>
__global__ void __launch_bounds__(32 * NW, 32 / NW) k_ac3d_inner_np(const StepArgs A) {
  ac3d_body<MODE, NW, false, 1, false>(A);
}
// (the z slabs fit 6 blocks per SM without the software pipeline, 4 with it)
template <int MODE, int NW = 4, bool PIPE = true>
__global__ void __launch_bounds__(32 * NW, PIPE ? 16 / NW : 24 / NW) k_ac3d_zslab(const StepArgs A) {
  ac3d_body<MODE, NW, false, 2, PIPE>(A);
}
template <int MODE, int NW = 4, bool PIPE = true>
__global__ void __launch_bounds__(32 * NW, 16 / NW) k_ac3d_yslab(const StepArgs A) {
  ac3d_body<MODE, NW, false, 3, PIPE>(A);
}

// ---------------------------------------------------------------------------
// 2D, TMA pipeline with a dedicated producer warp.  Same arithmetic as
// k_ac2d_step.  A CTA has 4 consumer warps (512 x points, one float4 per
// thread) and 1 producer warp.  The producer streams the CTA's rows through a
// ring of TMA_NS shared-memory stages with cp.async.bulk copies (p row with a
// 4-float halo on each side, d, fact and, for the adjoint, D, g and its
// compensation); each stage has a "full" mbarrier (completed by the copies'
// transaction count) and an "empty" mbarrier (one arrival per consumer warp
// once it no longer reads the stage).  No block-wide barrier sits in the
// loop: warps only wait for data or for free slots.  Every wait is bounded
// (clock64); on expiry the warp raises A.err and leaves.
// ---------------------------------------------------------------------------
constexpr int TMA_W = 512;            // x points per CTA tile
constexpr int TMA_PROW = TMA_W + 8;   // p row in shared memory: 4 halo floats each side
constexpr long long TMA_TIMEOUT_CYCLES = 4000000000LL;  // default wait limit, ~2 s at 2 GHz

// Stage ring per mode: consumers hold 3 stages (p rows z-1, z, z+1), the rest
// are in flight.  7 stages of 6.2 KB (forward) and 4 CTAs per SM, 6 stages
// of 12.3 KB (adjoint) 3 CTAs.
template <int MODE>
struct TmaLayout {
  static constexpr int NAUX = MODE == MODE_ADJ ? 5 : 2;  // d, fact (+ D, g, gc)
  static constexpr int NS = MODE == MODE_ADJ ? 6 : 7;    // stage slots
  static constexpr int MIN_BLOCKS = MODE == MODE_ADJ ? 3 : 4;
  static constexpr int STAGE = TMA_PROW + NAUX * TMA_W;  // floats per stage (multiple of 4)
  static constexpr size_t BYTES = (size_t)NS * STAGE * sizeof(float) + 2 * NS * sizeof(unsigned long long);
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// returns false when the wait gave up after `limit` cycles
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* b, unsigned parity, long long limit) {
  if (mbar_try_wait(b, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(b, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes, unsigned long long* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(b))
               : "memory");
}

template <int MODE>
__global__ void __launch_bounds__(160, TmaLayout<MODE>::MIN_BLOCKS) k_ac2d_tma(const StepArgs A) {
  using Lay = TmaLayout<MODE>;
  constexpr int TMA_NS = Lay::NS;
  extern __shared__ __align__(128) float smem[];
  unsigned long long* full = reinterpret_cast<unsigned long long*>(smem + (size_t)TMA_NS * Lay::STAGE);
  unsigned long long* empty = full + TMA_NS;
  constexpr unsigned FULL = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int S = A.nshots;
  const int shot = blockIdx.x % S;
  const int tile = blockIdx.x / S;
  const int txi = tile % A.tiles_x, tzi = tile / A.tiles_x;
  const int nx = A.n0, nz = A.n1, P = A.P, H = A.halo;
  const int z_begin = 1 + tzi * A.TZ;
  const int z_end = min(z_begin + A.TZ, nz - 1);
  const int X0 = txi * TMA_W;
  if (z_begin >= z_end || X0 >= P) return;  // block-uniform
  const int rows = z_end - z_begin, nst = rows + 2;

  if (tid == 0) {
    for (int k = 0; k < TMA_NS; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], 4);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  const float* pc = fptr(A.pcur, shot);
  const float* di = fptr(A.din, shot);
  const float* dcr = MODE == MODE_ADJ ? dptr(A.dcorr, shot, A.dbf16) : nullptr;
  float* gg = MODE == MODE_ADJ ? fptr(A.g, shot) : nullptr;
  float* gcp = MODE == MODE_ADJ ? fptr(A.gc, shot) : nullptr;

  if (warp == 4) {
    // producer: stage j carries p row z_begin-1+j and the aux rows of z_begin+j-2
    if (lane != 0) return;
    const int gx0 = max(X0 - 4, 0), gx1 = min(X0 + TMA_W + 4, P);
    const int aw = min(TMA_W, P - X0);
    for (int j = 0; j < nst; ++j) {
      const int slot = j % TMA_NS;
      // test hook: stop before stage `withhold` (every copy issued so far is
      // consumed, so none is in flight when the consumers give up and leave)
      if (j == A.withhold && blockIdx.x == 0) return;
      if (j >= TMA_NS && !mbar_wait_bounded(&empty[slot], ((j / TMA_NS) - 1) & 1, A.wait_cycles)) {
        if (A.err) atomicExch(A.err, 1);
        return;
      }
      float* st = smem + (size_t)slot * Lay::STAGE;
      const int r = z_begin - 1 + j;
      const bool aux = j >= 2;
      unsigned bytes = (unsigned)(gx1 - gx0) * 4u;
      if (aux) bytes += (unsigned)aw * 4u * Lay::NAUX;
      mbar_arrive_expect_tx(&full[slot], bytes);
      tma_load_1d(st + (gx0 - (X0 - 4)), pc + (long long)r * P + gx0, (unsigned)(gx1 - gx0) * 4u, &full[slot]);
      if (aux) {
        const long long row = (long long)(r - 1) * P + X0;  // aux row z = r - 1
        float* a = st + TMA_PROW;
        tma_load_1d(a, di + row, aw * 4u, &full[slot]);
        tma_load_1d(a + TMA_W, A.fact + row, aw * 4u, &full[slot]);
        if (MODE == MODE_ADJ) {
          tma_load_1d(a + 2 * TMA_W, dcr + row, aw * 4u, &full[slot]);
          tma_load_1d(a + 3 * TMA_W, gg + row, aw * 4u, &full[slot]);
          tma_load_1d(a + 4 * TMA_W, gcp + row, aw * 4u, &full[slot]);
        }
      }
    }
    return;
  }

  // consumers
  const int x0 = X0 + 4 * tid;
  const bool inb = x0 < P;
  float* __restrict__ pn = fptr(A.pnew, shot);
  float* dn = fptr(A.dout, shot);
  const float* cp = A.cpml + (long long)shot * A.cpml_stride;
  const int na = 2 * H + 2, nh = 2 * H, L = 2 * na + 2 * nh;
  float* ckp = fptr(A.ck_p, shot);
  float* ckd = fptr(A.ck_d, shot);
  float* Dw = nullptr;
  if (MODE == MODE_FWD_D && shot >= A.d_first) Dw = dptr(A.Dout, shot, A.dbf16);
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
  const int so = 4 + 4 * tid;

  for (int k = 0; k < rows; ++k) {
    bool ok = true;
    if (k == 0) {
      ok = ok && mbar_wait_bounded(&full[0], 0, A.wait_cycles);
      ok = ok && mbar_wait_bounded(&full[1 % TMA_NS], 0, A.wait_cycles);
    }
    const int j2 = k + 2;
    ok = ok && mbar_wait_bounded(&full[j2 % TMA_NS], (j2 / TMA_NS) & 1, A.wait_cycles);
    if (!__all_sync(FULL, ok)) {
      if (lane == 0 && A.err) atomicExch(A.err, 1);
      return;
    }
    const float* sm_ = smem + (size_t)(k % TMA_NS) * Lay::STAGE;        // p row z-1
    const float* s0_ = smem + (size_t)((k + 1) % TMA_NS) * Lay::STAGE;  // p row z
    const float* sp_ = smem + (size_t)(j2 % TMA_NS) * Lay::STAGE;       // p row z+1, aux rows of z
    const int z = z_begin + k;
    const long long row = (long long)z * P;
    float rm[4], r0[4], rp[4], o[4], f[4];
    {
      const float4 a = *reinterpret_cast<const float4*>(sm_ + so);
      const float4 b = *reinterpret_cast<const float4*>(s0_ + so);
      const float4 c = *reinterpret_cast<const float4*>(sp_ + so);
      const float4 d = *reinterpret_cast<const float4*>(sp_ + TMA_PROW + 4 * tid);
      const float4 e = *reinterpret_cast<const float4*>(sp_ + TMA_PROW + TMA_W + 4 * tid);
      rm[0] = a.x; rm[1] = a.y; rm[2] = a.z; rm[3] = a.w;
      r0[0] = b.x; r0[1] = b.y; r0[2] = b.z; r0[3] = b.w;
      rp[0] = c.x; rp[1] = c.y; rp[2] = c.z; rp[3] = c.w;
      o[0] = d.x; o[1] = d.y; o[2] = d.z; o[3] = d.w;
      f[0] = e.x; f[1] = e.y; f[2] = e.z; f[3] = e.w;
    }
    float left = __shfl_up_sync(FULL, r0[3], 1);
    float right = __shfl_down_sync(FULL, r0[0], 1);
    if (lane == 0) left = s0_[so - 1];
    if (lane == 31) right = s0_[so + 4];
    float dv[4], g4[4], c4[4];
    if (MODE == MODE_ADJ) {
      const float4 dv4 = *reinterpret_cast<const float4*>(sp_ + TMA_PROW + 2 * TMA_W + 4 * tid);
      const float4 g4v = *reinterpret_cast<const float4*>(sp_ + TMA_PROW + 3 * TMA_W + 4 * tid);
      const float4 c4v = *reinterpret_cast<const float4*>(sp_ + TMA_PROW + 4 * TMA_W + 4 * tid);
      dv[0] = dv4.x; dv[1] = dv4.y; dv[2] = dv4.z; dv[3] = dv4.w;
      g4[0] = g4v.x; g4[1] = g4v.y; g4[2] = g4v.z; g4[3] = g4v.w;
      c4[0] = c4v.x; c4[1] = c4v.y; c4[2] = c4v.z; c4[3] = c4v.w;
    }
    // stage k (p row z-1) is no longer read by this warp
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[k % TMA_NS]);

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
        if (MODE == MODE_FWD_D && Dw) dst4(Dw, row + x0, outD, A.dbf16);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int x = x0 + e;
          if (x >= 1 && x <= nx - 2) {
            pn[row + x] = outp[e];
            dn[row + x] = outd[e];
            if (MODE == MODE_FWD_D && Dw) dst1(Dw, row + x, outD[e], A.dbf16);
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Compensated (double-FP32) forward step: sw_wavesim_set_precision(ws, 1).
//
// FP32 state loses about 1e-6 of relative trace accuracy over a few thousand
// steps, and most of it comes from the cancellation in the second
// differences (a smooth wave's p[x-1] - 2 p[x] + p[x+1] is a few percent of
// p, so its FP32 rounding is ~30 eps of the result), then from the FP32
// rounding of p, of the increment d and of fact = vp^2 dt^2.  This step keeps
// p and d as unevaluated sums hi + lo of two FP32 numbers and fact and 1/h^2
// as hi + lo pairs of their FP64 values, and evaluates the increment
// d[n+1] - d[n] = fact * lap(p) and both state updates with error-free
// transformations: Knuth's TwoSum, the FMA form of Dekker's TwoProduct
// (a*b - fl(a*b) = fma(a, b, -fl(a*b))) and Dekker's Fast2Sum
// renormalisation (the double-double arithmetic of Dekker 1971 and of the QD
// library of Hida, Li and Bailey), about 48 bits of significand.  In the
// C-PML strips (where sources and receivers often sit) the memory variables
// and coefficients are FP64 and their correction is evaluated in FP64.
// Same algorithm and update order as the FP32 step (k_ac2d_step / ac3d_body);
// checkpoints and the D slots get the rounded hi + lo values.
// ---------------------------------------------------------------------------
// p[l] - 2 p[c] + p[r] of compensated values, compensated
__device__ __forceinline__ ff ff_d2(float lh, float ll, float ch, float cl, float rh, float rl) {
  const ff s = two_sum(lh, rh);
  const ff t = two_sum(s.hi, __fmul_rn(-2.f, ch));  // -2 ch is exact
  const float lo = __fadd_rn(__fadd_rn(s.lo, t.lo), __fadd_rn(__fadd_rn(ll, rl), __fmul_rn(-2.f, cl)));
  return fast_two_sum(t.hi, lo);
}

// The C-PML correction of one axis (dpsi + xi) in FP64: the update of
// cpml_axis_term with FP64 memory variables and coefficients and the
// compensated pressures (hi + lo is exact in FP64), returned as an FP32 pair.
struct Strip64 {
  const double* psi_in;
  double* psi_out;
  float* ck_psi;
  const double* xi_in;
  double* xi_out;
  float* ck_xi;
  const double *a, *ah, *b, *bh;
  long long psi_step, xi_step, psi_base, xi_base;
};
__device__ __forceinline__ Strip64 strip64_io(const StepArgs& A, int d, int shot, long long step) {
  const int H = A.halo;
  const int na = 2 * H + 2, nh = 2 * H, L = 2 * na + 2 * nh;
  const double* cp = A.cpml64 + (long long)shot * A.cpml_stride + (long long)d * L;
  Strip64 s;
  s.psi_in = A.psi64_in[d].p + (long long)shot * A.psi64_in[d].s;
  s.psi_out = A.psi64_out[d].p + (long long)shot * A.psi64_out[d].s;
  s.xi_in = A.xi64[d].p + (long long)shot * A.xi64[d].s;
  s.xi_out = const_cast<double*>(s.xi_in);  // in place
  s.ck_psi = fptr(A.ck_psi[d], shot);
  s.ck_xi = fptr(A.ck_xi[d], shot);
  s.a = cp;
  s.ah = cp + na;
  s.b = cp + na + nh;
  s.bh = cp + 2 * na + nh;
  s.psi_step = step;
  s.xi_step = step;
  s.psi_base = 0;
  s.xi_base = 0;
  return s;
}
__device__ __forceinline__ double ff_d(ff a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ ff cpml_axis_corr64(ff d2, ff pl, ff p0, ff pr, int x, int n, int halo, double ih,
                                               const Strip64& s) {
  int qr;
  bool first;
  if (x < halo) {
    qr = x;
    first = (x == 1);
  } else if (x >= n - halo) {
    qr = x + 1 - n + 2 * halo;
    first = (x == n - halo);
  } else {
    return ff{0.f, 0.f};
  }
  const int ql = qr - 1;
  const long long il = s.psi_base + (long long)ql * s.psi_step;
  const long long ir = s.psi_base + (long long)qr * s.psi_step;
  const double P0 = ff_d(p0);
  const double oldl = s.psi_in[il];
  const double oldr = s.psi_in[ir];
  const double newl = s.bh[ql] * oldl + s.ah[ql] * ((P0 - ff_d(pl)) * ih);
  const double newr = s.bh[qr] * oldr + s.ah[qr] * ((ff_d(pr) - P0) * ih);
  s.psi_out[ir] = newr;
  if (s.ck_psi) s.ck_psi[ir] = (float)oldr;
  if (first) {
    s.psi_out[il] = newl;
    if (s.ck_psi) s.ck_psi[il] = (float)oldl;
  }
  const double dpsi = (newr - newl) * ih;
  const long long iq = s.xi_base + (long long)qr * s.xi_step;
  const double xo = s.xi_in[iq];
  if (s.ck_xi) s.ck_xi[iq] = (float)xo;
  const double xn = s.b[qr] * xo + s.a[qr] * (ff_d(d2) + dpsi);
  s.xi_out[iq] = xn;
  const double corr = dpsi + xn;
  const float hi = (float)corr;
  return ff{hi, (float)(corr - (double)hi)};
}

// One warp = 128 x points (4 per thread) of one row (2D) or of one y row
// (3D), marching a band of TZ rows of the last axis; 4 warps per block (2D:
// 512 x points; 3D: 4 y rows).  Forward modes only (MODE_FWD, MODE_FWD_D).
// The 2D kernel is bounded for six blocks per SM (80 registers, a few bytes
// of spills, faster than the unbounded allocation); a bound spills heavily in
// 3D.
template <int MODE, int NDIM>
__global__ void __launch_bounds__(128, NDIM == 2 ? 6 : 1) k_ac_hp(const StepArgs A) {
  static_assert(MODE == MODE_FWD || MODE == MODE_FWD_D, "compensated step: forward modes only");
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = A.nshots;
  const int shot = blockIdx.x % S;
  int tile = blockIdx.x / S;
  const int nx = A.n0, P = A.P, H = A.halo;
  const int nm = NDIM == 2 ? A.n1 : A.n2;  // marching axis
  const int ny = NDIM == 3 ? A.n1 : 1;
  int wx0, y = 0;
  if (NDIM == 2) {
    wx0 = (tile % A.tiles_x) * 512 + warp * 128;
    tile /= A.tiles_x;
  } else {
    wx0 = (tile % A.tiles_x) * 128;
    tile /= A.tiles_x;
    y = 1 + (tile % A.tiles_y) * 4 + warp;
    tile /= A.tiles_y;
  }
  const int z_begin = 1 + tile * A.TZ;
  const int z_end = min(z_begin + A.TZ, nm - 1);
  if (z_begin >= z_end || wx0 >= P || (NDIM == 3 && y > ny - 2)) return;  // warp-uniform
  const int x0 = wx0 + lane * 4;
  const bool inb = x0 < P;
  const int xa = inb ? x0 : P - 4;
  const long long plane = NDIM == 2 ? (long long)P : (long long)P * ny;  // stride of the marching axis
  const long long rowoff = NDIM == 2 ? xa : (long long)y * P + xa;

  const float* __restrict__ pc = fptr(A.pcur, shot);
  const float* __restrict__ pcl = fptr(A.plo_cur, shot);
  float* __restrict__ pn = fptr(A.pnew, shot);
  float* __restrict__ pnl = fptr(A.plo_new, shot);
  float* dd = fptr(A.dout, shot);  // in place: din == dout
  float* ddl = fptr(A.dlo, shot);
  const float* __restrict__ fh = A.fact;
  const float* __restrict__ fl = A.fact_lo;
  const int na = 2 * H + 2, nh = 2 * H;
  float* ckp = fptr(A.ck_p, shot);
  float* ckd = fptr(A.ck_d, shot);
  float* Dw = nullptr;
  if (MODE == MODE_FWD_D && shot >= A.d_first) Dw = dptr(A.Dout, shot, A.dbf16);
  const bool xstrip = inb && (x0 < H || x0 + 3 >= nx - H);
  const bool ystrip = NDIM == 3 && ((y < H) || (y >= ny - H));
  const int ax_m = NDIM - 1;  // index of the marching axis in ih / ih2
  const ff ih2x{A.ih2[0], A.ih2_lo[0]}, ih2m{A.ih2[ax_m], A.ih2_lo[ax_m]};
  const ff ih2y{A.ih2[1], A.ih2_lo[1]};

  float rmh[4], rml[4], r0h[4], r0l[4], rph[4], rpl[4];
  {
    const long long idx = (long long)z_begin * plane + rowoff;
    ld4(rmh, pc + idx - plane);
    ld4(rml, pcl + idx - plane);
    ld4(r0h, pc + idx);
    ld4(r0l, pcl + idx);
  }
  for (int z = z_begin; z < z_end; ++z) {
    const long long idx = (long long)z * plane + rowoff;
    ld4(rph, pc + idx + plane);
    ld4(rpl, pcl + idx + plane);
    float oh[4], ol[4], fa[4], fb[4];
    ld4rw(oh, dd + idx);
    ld4rw(ol, ddl + idx);
    ld4(fa, fh + idx);
    ld4(fb, fl + idx);
    float ymh[4], yml[4], yph[4], ypl[4];
    if (NDIM == 3) {
      ld4(ymh, pc + idx - P);
      ld4(yml, pcl + idx - P);
      ld4(yph, pc + idx + P);
      ld4(ypl, pcl + idx + P);
    }
    float lh = __shfl_up_sync(FULL, r0h[3], 1), ll = __shfl_up_sync(FULL, r0l[3], 1);
    float rh = __shfl_down_sync(FULL, r0h[0], 1), rl = __shfl_down_sync(FULL, r0l[0], 1);
    if (lane == 0) {
      lh = xa > 0 ? pc[idx - 1] : 0.f;
      ll = xa > 0 ? pcl[idx - 1] : 0.f;
    }
    if (lane == 31) {
      rh = xa + 4 < P ? pc[idx + 4] : 0.f;
      rl = xa + 4 < P ? pcl[idx + 4] : 0.f;
    }
    const bool mstrip = (z < H) || (z >= nm - H);
    float outph[4], outpl[4], outdh[4], outdl[4], outD[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float xmh = e == 0 ? lh : r0h[e - 1], xml = e == 0 ? ll : r0l[e - 1];
      const float xph = e == 3 ? rh : r0h[e + 1], xpl = e == 3 ? rl : r0l[e + 1];
      const float ch = r0h[e], cl = r0l[e];
      const int x = x0 + e;
      const bool pin = inb && x >= 1 && x <= nx - 2;
      ff dx = ff_d2(xmh, xml, ch, cl, xph, xpl);
      ff dm = ff_d2(rmh[e], rml[e], ch, cl, rph[e], rpl[e]);
      ff tx = ff_mul(dx, ih2x), tm = ff_mul(dm, ih2m);
      if (xstrip && pin) {
        Strip64 s0 = strip64_io(A, 0, shot, 1);
        if (NDIM == 2) {
          s0.psi_base = (long long)z * nh;
          s0.xi_base = (long long)z * na;
        } else {
          s0.psi_base = ((long long)z * ny + y) * nh;
          s0.xi_base = ((long long)z * ny + y) * na;
        }
        tx = ff_add(tx, cpml_axis_corr64(tx, ff{xmh, xml}, ff{ch, cl}, ff{xph, xpl}, x, nx, H, A.ihd[0], s0));
      }
      if (mstrip && pin) {
        Strip64 sm = strip64_io(A, ax_m, shot, plane);
        if (NDIM == 2) {
          sm.psi_base = x;
          sm.xi_base = x;
        } else {
          sm.psi_base = (long long)y * P + x;
          sm.xi_base = (long long)y * P + x;
        }
        tm = ff_add(tm, cpml_axis_corr64(tm, ff{rmh[e], rml[e]}, ff{ch, cl}, ff{rph[e], rpl[e]}, z, nm, H,
                                         A.ihd[ax_m], sm));
      }
      ff lap = ff_add(tx, tm);
      if (NDIM == 3) {
        ff ty = ff_mul(ff_d2(ymh[e], yml[e], ch, cl, yph[e], ypl[e]), ih2y);
        if (ystrip && pin) {
          Strip64 s1 = strip64_io(A, 1, shot, P);
          s1.psi_base = (long long)z * nh * P + x;
          s1.xi_base = (long long)z * na * P + x;
          ty = ff_add(ty, cpml_axis_corr64(ty, ff{ymh[e], yml[e]}, ff{ch, cl}, ff{yph[e], ypl[e]}, y, ny, H, A.ihd[1],
                                           s1));
        }
        lap = ff_add(lap, ty);
      }
      const ff D = ff_mul(ff{fa[e], fb[e]}, lap);
      const ff dn = ff_add(ff{oh[e], ol[e]}, D);
      const ff pnw = ff_add(ff{ch, cl}, dn);
      outD[e] = ff_round(D);
      outdh[e] = dn.hi;
      outdl[e] = dn.lo;
      outph[e] = pnw.hi;
      outpl[e] = pnw.lo;
    }
    int de = 0;  // FP16 D slots (3D): the exponent of this warp's tile
    if (MODE == MODE_FWD_D && A.dbf16 == 2 && Dw) {
      de = warp_dexp(outD, inb);
      const long long erow = ((long long)z * ny + y) * A.ntx + (wx0 >> 7);
      if (lane == 0) A.Dexp.p[(long long)shot * A.Dexp.s + erow] = (signed char)de;
    }
    if (inb) {
      if (ckp) {
        float cp4[4], cd4[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          cp4[e] = __fadd_rn(r0h[e], r0l[e]);
          cd4[e] = __fadd_rn(oh[e], ol[e]);
        }
        st4(ckp + idx, cp4);
        st4(ckd + idx, cd4);
      }
      if (x0 >= 1 && x0 + 3 <= nx - 2) {  // all four points interior: vector stores
        st4(pn + idx, outph);
        st4(pnl + idx, outpl);
        st4(dd + idx, outdh);
        st4(ddl + idx, outdl);
        if (MODE == MODE_FWD_D && Dw) dst4(Dw, idx, outD, A.dbf16, de);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int x = x0 + e;
          if (x >= 1 && x <= nx - 2) {
            pn[idx + e] = outph[e];
            pnl[idx + e] = outpl[e];
            dd[idx + e] = outdh[e];
            ddl[idx + e] = outdl[e];
            if (MODE == MODE_FWD_D && Dw) dst1(Dw, idx + e, outD[e], A.dbf16, de);
          }
        }
      }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      rmh[e] = r0h[e];
      rml[e] = r0l[e];
      r0h[e] = rph[e];
      r0l[e] = rpl[e];
    }
  }
}

}  // namespace swgb
