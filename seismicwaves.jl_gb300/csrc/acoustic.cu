// Acoustic constant-density C-PML path: shot tables, the batched forward and
// the batched gradient (forward with checkpoints, misfit and adjoint source,
// adjoint with recompute and fused correlation, reduction over shots).
//
// Reference behaviour restated here (SeismicWaves.jl v0.9.0):
//   run_swforward! / swforward_1shot!     src/apis/forward.jl:71-114, src/models/acoustic/acou_forward.jl:22-62
//   run_swgradient! / swgradient_1shot!   src/apis/gradient.jl:93-136, src/models/acoustic/acou_gradient.jl:4-95
//   inject_sources! / record_receivers!   src/models/acoustic/backends/shared/acoustic2D_xPU.jl:48-62
//   prescale_residuals!                   acoustic2D_xPU.jl:64-76
//   L2 misfit and dchi/du                 src/inversion/misfits/L2Misfit.jl:24-77
//   mutearoundpoint!                      src/utils/mute_grad.jl:13-80
//   LinearCheckpointer schedule           src/utils/checkpointers.jl:1-107
//
// Gradient schedule.  The reference stores p at every K-th step (width 2),
// psi and xi at every K-th step, and a buffer of K+1 fields that recover!
// refills by re-running K-1 forward steps whenever the adjoint loop reaches a
// checkpoint it = mK.  The correlation at adjoint step it needs the second
// time difference D(it-1) = p[it-2] - 2 p[it-1] + p[it], which the forward
// step that produces p[it] already knows exactly: D(it-1) = fact * lap(p[it-1])
// (+ the injected source).  So the forward (for the top segment) and the
// recompute write D directly (one field per step instead of three re-reads),
// the recompute runs K steps (m-1)K+1 .. mK from the checkpoint at (m-1)K,
// and checkpoints are written by the forward stencil itself in the step after
// they are reached (no copy kernels).  Recovery events fall on it = mK for
// every shot regardless of its nt, so shots with different record lengths
// share one schedule; a shot takes part in step it only while it <= nt.
//
// Correlation sums.  In 2D the adjoint stencil adds lambda * D into a plain
// FP32 sum per shot, which k_flush_grad adds into one FP64 total every 32
// adjoint steps (no FP32 sum runs over more than 32 terms); 3D, muted runs
// (which need each shot's own gradient) and the grouped 2D kernel of tuning
// variant 256 keep Kahan-compensated FP32 sums instead.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <sstream>

#include <cuda_bf16.h>

#include "acoustic_kernels.cuh"
#include "internal.h"
#include "ccts.cuh"

namespace swgb {

// ---------------------------------------------------------------------------
// Per-shot descriptor (device) and the small kernels around the stencil
// ---------------------------------------------------------------------------
struct ShotDesc {
  int nt, nsrc, nrec;
  int nsp, nrp;             // unique source / receiver points
  int last;                 // floor(nt/K)*K (gradient)
  long long sp_off, sp_ptr;  // unique source points: pts[sp_off + u], csr ptr[sp_ptr + u .. +1]
  long long rp_off, rp_ptr;  // unique receiver points
  long long rec_off;         // rec_lin[rec_off + r]
  const float* tf;           // (nt, nsrc)
  float* tr;                 // (nt, nrec)
  const float* obs;          // (nt, nrec)
  const float* ic;           // (nt) or nullptr
  const float* mask;         // (nt) or nullptr
  float* adj;                // (nt, nrec) adjoint source (prescaled)
  float* ring;               // 3 values per boundary injection point (see k_inject_record)
  const float* icd;          // dense inverse covariance (nt, nt) or nullptr
  float* resid;              // dense case: masked residuals (nt, nrec)
  const float* cres;         // dense case: C^-1 r (nt, nrec), from the dense product (dense.cu)
  int mkind;                 // 0 L2, 1 CCTS (k_ccts writes this shot's adjoint source)
};

// Boundary injection points.  The reference never updates the outermost grid
// nodes and rotates three pressure buffers, so a node on the boundary that
// receives an injection evolves as p[t] = p[t-3] + s[t].  The increment-form
// stencil keeps two pressure buffers, so such nodes carry their own 3-value
// ring (slot t mod 3 holds p[t-3] before the update) and are written here.
__device__ __forceinline__ float ring_update(float* ring, int slot, int it, float add, float* second_diff) {
  float* r = ring + 3 * slot;
  const float v = r[it % 3] + add;
  r[it % 3] = v;
  if (second_diff) *second_diff = v - 2.f * r[(it + 2) % 3] + r[(it + 1) % 3];
  return v;
}

// Sets (add = false) or adds to (add = true) the FP16 D value at lin and
// re-encodes the point's 128-point tile when the new tile maximum calls for
// another exponent (sources added after the stencil wrote the tile).
__device__ void d16_put(float* d, signed char* ex, long long lin, float v, bool add, int P) {
  __half* h = reinterpret_cast<__half*>(d);
  const long long row = lin / P;
  const int x = (int)(lin - row * P);
  const int ntx = (P + 127) / 128;
  signed char* ep = ex + row * ntx + (x >> 7);
  const int e = *ep;
  const long long t0 = row * P + (x & ~127), t1 = row * P + min((x | 127) + 1, P);
  const float nv = add ? __half2float(h[lin]) * pow2f(-e) + v : v;
  float m = fabsf(nv);
  for (long long q = t0; q < t1; ++q)
    if (q != lin) m = fmaxf(m, fabsf(__half2float(h[q]) * pow2f(-e)));
  const int e2 = dexp_of(m);
  if (e2 != e) {
    for (long long q = t0; q < t1; ++q)
      if (q != lin) h[q] = __float2half_rn(h_enc(__half2float(h[q]) * pow2f(-e), e2));
    *ep = (signed char)e2;
  }
  h[lin] = __float2half_rn(h_enc(nv, e2));
}

// inject_sources! + record_receivers! for every active shot: one block per
// shot.  Duplicated points are summed in source order by one thread, like the
// reference's serial loop.  Interior points add the source to p[n+1] and to
// the increment d[n+1] (and to D when the gradient keeps it).
// With two steps per stencil launch (k_ac2d_pair) the first step's pressure
// on the receiver rows is in the stash; it_stash > 0 records that step from it.
__global__ void k_inject_record(const ShotDesc* __restrict__ desc, const long long* __restrict__ pts,
                                const int* __restrict__ ptr, const int* __restrict__ ids,
                                const int* __restrict__ bslot, const long long* __restrict__ rec_lin,
                                FieldArg pnew, FieldArg dnew, FieldArg dfield, int d_first, int it, int record,
                                int dbf16, const int* __restrict__ rec_stash, FieldArg stash, int it_stash,
                                FieldArg plo, FieldArg dlo, FieldArgE dexp, int P) {
  const int shot = blockIdx.x;
  const ShotDesc D = desc[shot];
  if (it > D.nt) return;
  if (it_stash > 0) {
    const float* sp = stash.p + (long long)shot * stash.s;
    for (int r = threadIdx.x; r < D.nrec; r += blockDim.x)
      D.tr[(long long)(it_stash - 1) + (long long)r * D.nt] = sp[rec_stash[D.rec_off + r]];
  }
  float* pn = pnew.p + (long long)shot * pnew.s;
  float* dn = dnew.p + (long long)shot * dnew.s;
  float* dd = (dfield.p && shot >= d_first) ? dptr(dfield, shot, dbf16) : nullptr;
  float* dd16 = nullptr;  // FP16 D slots: updated below by one thread (tile exponents)
  if (dbf16 == 2) {
    dd16 = dd;
    dd = nullptr;
  }
  for (int u = threadIdx.x; u < D.nsp; u += blockDim.x) {
    const long long lin = pts[D.sp_off + u];
    float add = 0.f;
    const int k0 = ptr[D.sp_ptr + u], k1 = ptr[D.sp_ptr + u + 1];
    const int slot = bslot[D.sp_off + u];
    if (slot >= 0) {
      for (int k = k0; k < k1; ++k) add += D.tf[(long long)(it - 1) + (long long)ids[k] * D.nt];
      float sd;
      pn[lin] = ring_update(D.ring, slot, it, add, &sd);
      if (dd) dst1(dd, lin, sd, dbf16);
    } else if (plo.p) {  // compensated state: p and d get the sources without rounding
      float* pl = plo.p + (long long)shot * plo.s;
      float* dl = dlo.p + (long long)shot * dlo.s;
      ff pv{pn[lin], pl[lin]}, dv{dn[lin], dl[lin]}, av{0.f, 0.f};
      for (int k = k0; k < k1; ++k) {
        const ff v{D.tf[(long long)(it - 1) + (long long)ids[k] * D.nt], 0.f};
        pv = ff_add(pv, v);
        dv = ff_add(dv, v);
        av = ff_add(av, v);
      }
      pn[lin] = pv.hi;
      pl[lin] = pv.lo;
      dn[lin] = dv.hi;
      dl[lin] = dv.lo;
      if (dd) dst1(dd, lin, dld1(dd, lin, dbf16) + ff_round(av), dbf16);
    } else {
      float acc = pn[lin];
      for (int k = k0; k < k1; ++k) {
        const float v = D.tf[(long long)(it - 1) + (long long)ids[k] * D.nt];
        acc += v;
        add += v;
      }
      pn[lin] = acc;
      dn[lin] += add;
      if (dd) dst1(dd, lin, dld1(dd, lin, dbf16) + add, dbf16);
    }
  }
  if (dbf16 == 2) __syncthreads();  // block-uniform: the rings above are updated
  if (dd16 && threadIdx.x == 0) {
    signed char* ex = dexp.p + (long long)shot * dexp.s;
    for (int u = 0; u < D.nsp; ++u) {
      const long long lin = pts[D.sp_off + u];
      const int k0 = ptr[D.sp_ptr + u], k1 = ptr[D.sp_ptr + u + 1];
      float add = 0.f;
      for (int k = k0; k < k1; ++k) add += D.tf[(long long)(it - 1) + (long long)ids[k] * D.nt];
      const int slot = bslot[D.sp_off + u];
      if (slot >= 0)  // boundary node: D is the ring's second difference, read back from the ring
        d16_put(dd16, ex, lin, D.ring[3 * slot + it % 3] - 2.f * D.ring[3 * slot + (it + 2) % 3] +
                                     D.ring[3 * slot + (it + 1) % 3], false, P);
      else
        d16_put(dd16, ex, lin, add, true, P);
    }
  }
  if (!record) return;
  __syncthreads();
  const float* pnl = plo.p ? plo.p + (long long)shot * plo.s : nullptr;
  for (int r = threadIdx.x; r < D.nrec; r += blockDim.x) {
    const long long q = rec_lin[D.rec_off + r];
    D.tr[(long long)(it - 1) + (long long)r * D.nt] = pnl ? __fadd_rn(pn[q], pnl[q]) : pn[q];
  }
}

// Adjoint injection at the receivers (adjoint_onestep_CPML! -> inject_sources!
// with the prescaled residuals) and the matching correlation term: the fused
// stencil correlated interior lambda before injection, so g += a * D is added
// here (boundary nodes, which the stencil skips, add their full lambda * D).
__device__ void adj_inject_shot(const ShotDesc& D, const long long* __restrict__ pts, const int* __restrict__ ptr,
                                const int* __restrict__ ids, const int* __restrict__ bslot, float* lp, float* ld,
                                const float* dp, int dbf16, float* gp, float* cp, int it, const signed char* ex,
                                int P);

// One block per accumulator group (grp consecutive shots share one gradient
// pair); the group's shots are handled one after the other, so receivers of
// different shots on the same grid point never update the pair concurrently.
__global__ void k_adj_inject(const ShotDesc* __restrict__ desc, const long long* __restrict__ pts,
                             const int* __restrict__ ptr, const int* __restrict__ ids,
                             const int* __restrict__ bslot, FieldArg lam, FieldArg lamd, FieldArg dcorr, FieldArg g,
                             FieldArg gc, int it, int nshots, int grp, int dbf16, FieldArgE dexp, int P) {
  float* gp = g.p + (long long)blockIdx.x * g.s;
  float* cp = gc.p ? gc.p + (long long)blockIdx.x * gc.s : nullptr;  // null: plain FP32 sums
  for (int j = 0; j < grp; ++j) {
    const int shot = blockIdx.x * grp + j;
    if (shot >= nshots) break;
    if (j > 0) __syncthreads();
    adj_inject_shot(desc[shot], pts, ptr, ids, bslot, lam.p + (long long)shot * lam.s,
                    lamd.p + (long long)shot * lamd.s, dptr(dcorr, shot, dbf16), dbf16, gp, cp, it,
                    dexp.p ? dexp.p + (long long)shot * dexp.s : nullptr, P);
  }
}

__device__ void adj_inject_shot(const ShotDesc& D, const long long* __restrict__ pts, const int* __restrict__ ptr,
                                const int* __restrict__ ids, const int* __restrict__ bslot, float* lp, float* ld,
                                const float* dp, int dbf16, float* gp, float* cp, int it, const signed char* ex,
                                int P) {
  if (it > D.nt) return;
  for (int u = threadIdx.x; u < D.nrp; u += blockDim.x) {
    const long long lin = pts[D.rp_off + u];
    const int k0 = ptr[D.rp_ptr + u], k1 = ptr[D.rp_ptr + u + 1];
    const int slot = bslot[D.rp_off + u];
    float add = 0.f, corr;
    if (slot >= 0) {
      // the adjoint iterates it = nt..1; its ring is indexed by the adjoint step count
      for (int k = k0; k < k1; ++k) add += D.adj[(long long)(it - 1) + (long long)ids[k] * D.nt];
      const float v = ring_update(D.ring, slot, D.nt - it + 1, add, nullptr);
      lp[lin] = v;
      corr = v;
    } else {
      float acc = lp[lin];
      for (int k = k0; k < k1; ++k) {
        const float v = D.adj[(long long)(it - 1) + (long long)ids[k] * D.nt];
        acc += v;
        add += v;
      }
      lp[lin] = acc;
      ld[lin] += add;
      corr = add;
    }
    // FP16 D slots: the exponent of the point's 128-point tile
    const int e = ex ? ex[(lin / P) * ((P + 127) / 128) + ((lin % P) >> 7)] : 0;
    if (cp) {
      float gv = gp[lin], cv = cp[lin];
      kahan_add(gv, cv, corr * dld1(dp, lin, dbf16, e));
      gp[lin] = gv;
      cp[lin] = cv;
    } else {
      gp[lin] = __fmaf_rn(corr, dld1(dp, lin, dbf16, e), gp[lin]);
    }
  }
}

// Plain FP32 correlation sums of the first S shots (MODE_ADJW) added into the
// FP64 total; called every few adjoint steps so that no FP32 sum runs over
// more than that many terms (the host clears the sums right after).  Four
// consecutive points per thread; the shot loop only loads, so the loads of
// several shots are in flight together.
__global__ void k_flush_grad(const float* __restrict__ g, long long F, int S, double* __restrict__ tot) {
  const long long F4 = F / 4;  // F is a multiple of 4 (padded pitch)
  const float4* g4 = reinterpret_cast<const float4*>(g);
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < F4; q += (long long)gridDim.x * blockDim.x) {
    double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
#pragma unroll 8
    for (int k = 0; k < S; ++k) {
      const float4 v = __ldg(g4 + (long long)k * F4 + q);
      t0 += (double)v.x;
      t1 += (double)v.y;
      t2 += (double)v.z;
      t3 += (double)v.w;
    }
    double* o = tot + 4 * q;
    o[0] += t0;
    o[1] += t1;
    o[2] += t2;
    o[3] += t3;
  }
}

// grad[c] (+)= 2/vp^3 * (1/dt^2) * total[c] (the MODE_ADJW counterpart of k_reduce_grad).
__global__ void k_reduce_grad_tot(const double* __restrict__ tot, const float* __restrict__ vp, int n0, long long npts,
                                  int P, double inv_dt2, double* __restrict__ out, int accumulate) {
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < npts;
       c += (long long)gridDim.x * blockDim.x) {
    const long long rowi = c / n0;
    const long long lin = rowi * P + (c - rowi * n0);
    const double v = (double)vp[c];
    const double val = (2.0 / (v * v * v)) * inv_dt2 * tot[lin];
    out[c] = accumulate ? out[c] + val : val;
  }
}

// Masked residuals of the shots with a dense inverse covariance (the input of
// the dense product C^-1 r).  gridDim = (blocks per shot, shots).
__global__ void k_residual_dense(const ShotDesc* __restrict__ desc) {
  const ShotDesc& D = desc[blockIdx.y];
  if (!D.icd) return;
  const long long total = (long long)D.nt * D.nrec;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    float res = D.tr[q] - D.obs[q];
    if (D.mask) res *= D.mask[q % D.nt];
    D.resid[q] = res;
  }
}

// Residuals, window mask, C^-1 r, misfit (FP64) and the prescaled adjoint
// source -C^-1 r * fact(rec).  gridDim = (blocks per shot, shots).
__global__ void k_misfit_adjsrc(const ShotDesc* __restrict__ desc, const long long* __restrict__ rec_lin,
                                const float* __restrict__ fact, double* __restrict__ partial) {
  const int shot = blockIdx.y;
  const ShotDesc D = desc[shot];
  const long long total = D.mkind == 1 ? 0 : (long long)D.nt * D.nrec;  // CCTS shots: k_ccts
  double acc = 0.0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int t = (int)(q % D.nt);
    const int r = (int)(q / D.nt);
    float res = D.tr[q] - D.obs[q];
    if (D.mask) res *= D.mask[t];
    const float cres = D.cres ? D.cres[q] : (D.ic ? D.ic[t] * res : res);
    acc += (double)res * (double)cres;
    D.adj[q] = (-cres) * fact[rec_lin[D.rec_off + r]];
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

__global__ void k_misfit_sum(const double* __restrict__ partial, int nblk, int nshots, double* out,
                             int accumulate) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < nblk * nshots; i += blockDim.x) acc += partial[i];
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = (accumulate ? *out : 0.0) + 0.5 * red[0];
}

// mutearoundpoint!: multiplies g (and its Kahan compensation) by r/rmax inside
// the ball around each listed point, sequentially over the points of a shot.
struct MutePoint {
  int shot;
  int lo[3], hi[3];
  double pos[3];
};
__global__ void k_mute(const MutePoint* __restrict__ mp, const int* __restrict__ shot_ptr, int N, int n0, int n1,
                       int n2, int P, double h0, double h1, double h2, double rmax, FieldArg g, FieldArg gc) {
  const int shot = blockIdx.x;
  float* gp = g.p + (long long)shot * g.s;
  float* cp = gc.p + (long long)shot * gc.s;
  const double h[3] = {h0, h1, h2};
  const int n[3] = {n0, n1, n2};
  for (int k = shot_ptr[shot]; k < shot_ptr[shot + 1]; ++k) {
    const MutePoint m = mp[k];
    const int e0 = m.hi[0] - m.lo[0] + 1, e1 = m.hi[1] - m.lo[1] + 1, e2 = N == 3 ? m.hi[2] - m.lo[2] + 1 : 1;
    const int cnt = e0 * e1 * e2;
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
      int I[3];
      I[0] = m.lo[0] + t % e0;
      I[1] = m.lo[1] + (t / e0) % e1;
      I[2] = N == 3 ? m.lo[2] + t / (e0 * e1) : 1;
      bool inb = true;
      double r2 = 0.0;
      for (int d = 0; d < N; ++d) {
        if (I[d] < 1 || I[d] > n[d]) inb = false;
        const double xc = (I[d] - 1) * h[d];
        r2 += (m.pos[d] - xc) * (m.pos[d] - xc);
      }
      if (!inb) continue;
      const double r = sqrt(r2);
      if (r <= rmax) {
        const float att = (float)(r / rmax);
        const long long lin = N == 3 ? ((long long)(I[2] - 1) * n1 + (I[1] - 1)) * P + (I[0] - 1)
                                     : (long long)(I[1] - 1) * P + (I[0] - 1);
        gp[lin] *= att;
        cp[lin] *= att;
      }
    }
    __syncthreads();
  }
}

// grad[c] (+)= 2/vp^3 * (1/dt^2) * sum_s (g_s - c_s)  in FP64, unpadded
// column-major output.  g accumulates lambda * D with D = p[t-2] - 2 p[t-1] + p[t];
// the 1/dt^2 of correlate_gradient! (correlate_gradient_xPU.jl:1-10) and the
// 2/vp^3 rescaling of swgradient_1shot! (acou_gradient.jl:93) are applied here once.
__global__ void k_reduce_grad(const float* __restrict__ g, const float* __restrict__ gc, long long fstride,
                              int nshots, const float* __restrict__ vp, int n0, long long npts, int P,
                              double inv_dt2, double* __restrict__ out, int accumulate) {
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < npts;
       c += (long long)gridDim.x * blockDim.x) {
    const long long rowi = c / n0;
    const long long lin = rowi * P + (c - rowi * n0);
    double s = 0.0;
    for (int k = 0; k < nshots; ++k) {
      const long long q = (long long)k * fstride + lin;
      s += (double)g[q] - (double)gc[q];
    }
    const double v = (double)vp[c];
    const double val = (2.0 / (v * v * v)) * inv_dt2 * s;
    out[c] = accumulate ? out[c] + val : val;
  }
}

// BF16 checkpoints.  The (p, d) pair of a checkpoint is staged in FP32 (the
// stencil writes it there), then each field of each shot is stored as BF16
// with its own power-of-two scale (2^-e with e the exponent of the field's
// largest |value|, so the stored values lie in (-2, 2)); recovery expands it
// back into the FP32 stage.  gridDim.y = 2 * shots (field-major per shot).
__global__ void k_ck_absmax(const float* __restrict__ stage, long long F, unsigned int* __restrict__ maxbits) {
  const int q = blockIdx.y;  // shot * 2 + field
  const float* x = stage + (long long)q * F;
  float mx = 0.0f;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < F; c += (long long)gridDim.x * blockDim.x)
    mx = fmaxf(mx, fabsf(x[c]));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxbits + q, __float_as_uint(mx));
}

__device__ __forceinline__ int ck_exponent(unsigned int bits) {
  const float mx = __uint_as_float(bits);
  return (mx > 0.0f && mx < 3.0e38f) ? ilogbf(mx) : 0;
}

__global__ void k_ck_pack(const float* __restrict__ stage, long long F, const unsigned int* __restrict__ maxbits,
                          __nv_bfloat16* __restrict__ dst, long long shot_stride, float* __restrict__ inv_scale) {
  const int q = blockIdx.y;
  const int shot = q >> 1, f = q & 1;
  const int e = ck_exponent(maxbits[q]);
  const float sc = ldexpf(1.0f, -e);
  const float* x = stage + (long long)q * F;
  __nv_bfloat16* y = dst + (long long)shot * shot_stride + (long long)f * F;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < F; c += (long long)gridDim.x * blockDim.x)
    y[c] = __float2bfloat16_rn(x[c] * sc);
  if (blockIdx.x == 0 && threadIdx.x == 0) inv_scale[q] = ldexpf(1.0f, e);
}

__global__ void k_ck_unpack(const __nv_bfloat16* __restrict__ src, long long shot_stride, long long F,
                            const float* __restrict__ inv_scale, float* __restrict__ stage) {
  const int q = blockIdx.y;
  const int shot = q >> 1, f = q & 1;
  const float is = inv_scale[q];
  const __nv_bfloat16* x = src + (long long)shot * shot_stride + (long long)f * F;
  float* y = stage + (long long)q * F;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < F; c += (long long)gridDim.x * blockDim.x)
    y[c] = __bfloat162float(x[c]) * is;
}

// fact = dt^2 vp^2 into the padded layout; vp kept unpadded (float).
__global__ void k_set_fact(const float* __restrict__ vp, int n0, long long npts, int P, double dt2,
                           float* __restrict__ fact, float* __restrict__ fact_lo) {
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < npts;
       c += (long long)gridDim.x * blockDim.x) {
    const long long rowi = c / n0;
    const double v = (double)vp[c];
    const double f = dt2 * v * v;
    const float hi = (float)f;
    fact[rowi * P + (c - rowi * n0)] = hi;
    if (fact_lo) fact_lo[rowi * P + (c - rowi * n0)] = (float)(f - (double)hi);  // compensated step
  }
}

// fact from FP64 velocities: the FP32 rounding of vp for the kernels that
// take vp, fact = dt^2 vp^2 in FP64 split into its FP32 rounding and (with a
// low-part buffer) the remainder.
__global__ void k_set_fact64(const double* __restrict__ vp64, int n0, long long npts, int P, double dt2,
                             float* __restrict__ vp, float* __restrict__ fact, float* __restrict__ fact_lo) {
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < npts;
       c += (long long)gridDim.x * blockDim.x) {
    const long long rowi = c / n0;
    const double v = vp64[c];
    const double f = dt2 * v * v;
    const float hi = (float)f;
    vp[c] = (float)v;
    fact[rowi * P + (c - rowi * n0)] = hi;
    if (fact_lo) fact_lo[rowi * P + (c - rowi * n0)] = (float)(f - (double)hi);
  }
}

}  // namespace swgb

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using namespace swgb;

struct sw_wavesim {
  sw_ctx* ctx = nullptr;
  sw_acoustic_params prm{};
  bool gradient = false;
  sw_grad_params gp{};
  int N = 2;
  int n[3] = {1, 1, 1};
  int P = 0;
  long long F = 0;           // floats per field (padded)
  long long npts = 0;        // unpadded points
  long long psz[3] = {0, 0, 0}, xsz[3] = {0, 0, 0};
  long long strip_total = 0;  // sum psi + sum xi (floats)
  bool has_vp = false;
  DevMem vp, fact;
  // capacity (shots) of the state buffers
  int cap = 0;
  DevMem pb[2], db, psi[2][3], xi[3];     // forward state: p ping-pong, increment d, psi ping-pong, xi
  DevMem db2, xi2[3];                     // second d / xi buffers (two-step launches write state n+2 apart)
  DevMem psim[3], xim[3];                 // memory variables between the two steps of a two-step launch
  DevMem d_pair, d_recstash, d_stash;     // two-step launches: per-shot source / receiver-row table,
                                          // receiver -> stash index, first-step pressure of receiver rows
  bool pair_on = false;                   // 2D: two time steps per launch where possible (tuning variant)
  bool split3d = true;                    // 3D: inner rows and strip rows as two launches (variant bit 16: one)
  bool inner_np = false;                  // 3D: the three launches without the software pipeline (variant bit 17)
  bool xsplit = true;                     // 2D 4-warp stencil: x strips as extra blocks (variant bit 18: not)
  int pair_tz = 0;                        // rows per block of the two-step kernel (0 = heuristic)
  int pair_occ = 0;                       // resident-block bound of the two-step kernel (0 = default, 1, 2)
  bool pair_ok = false;                   // the current group's shots allow two-step launches
  DevMem adb2, axi2[3];                   // second adjoint d / xi buffers (two-step adjoint launches)
  DevMem d_amap;                          // [shot][k][P]: receiver point (CSR index) at x on receiver row k, or -1
  bool pair_adj_ok = false;               // ... and two-step adjoint launches
  DevMem ab[2], adb, apsi[2][3], axi[3];  // adjoint state
  DevMem g, gc;
  DevMem dbuf;                         // D slots
  DevMem dexp;                         // FP16 D slots (snapshot_bf16 3): exponent per row and 128-point x tile
  long long d_slots = 0;
  DevMem ck;                           // checkpoint slots (with BF16 snapshots: the psi / xi strips only)
  long long ck_slots = 0;
  DevMem ck16, ck_scale, ck_max, ck_stage;  // BF16 (p, d) per slot and shot, their scales, FP32 stage
  DevMem zero;                         // zero state (one shot, stride 0)
  // tables
  DevMem d_desc, d_pts, d_ptr, d_ids, d_bslot, d_rec, d_tf, d_tr, d_obs, d_ic, d_mask, d_adj, d_cpml, d_partial, d_mis;
  DevMem d_ccts, d_partial2;  // CCTS descriptors and per-trace misfit terms
  DevMem d_ring;  // boundary-injection rings (3 floats per point)
  DevMem d_icd, d_dres;  // dense inverse covariances; residuals and C^-1 r of those shots
  DevMem d_mute, d_mute_ptr;
  int tile_tz = 0;  // 0 = heuristic
  int precision = 0;                          // 1: compensated (double-FP32) forward steps (k_ac_hp)
  DevMem plo[2], dlo, fact_lo;                 // their low parts of p (ping-pong), d and fact
  DevMem vp64;                                 // FP64 vp of sw_wavesim_set_vp64 (fact's low part comes from it)
  DevMem psi64[2][3], xi64[3], d_cpml64;       // compensated step: FP64 C-PML memory variables, coefficients
  int hp_cap = 0;                              // shots the low-part buffers hold
  long long wait_cycles = TMA_TIMEOUT_CYCLES;  // limit of one bounded device-side wait
  int withhold = -1;                           // test hook of the TMA stencil (StepArgs::withhold)
  int kind_tz[3] = {0, 0, 0};  // band height per stencil kind (forward, recompute, adjoint); 0 = tile_tz
  int variant = 0;  // 2D stencil: 0 = register-pipelined, 1 = TMA
  int pf = 0;       // 2D stencil: L2 prefetch distance in rows (0 = off)
  bool cpa = false; // 2D stencil (4 warps): rows staged through shared memory by cp.async
  int grp = 1;      // shots per gradient accumulator in the adjoint (4: shot sum fused, 1: per shot)
  bool adj_plain = true;   // 2D: per-shot adjoint with plain FP32 sums flushed to FP64 (MODE_ADJW);
                           // false: the grouped Kahan adjoint (k_ac2d_adj_grp) for 4+ shots
  bool adjw = false;       // the current gradient call uses MODE_ADJW
  DevMem tot64;            // MODE_ADJW: FP64 gradient total (padded layout)
  // CUDA graphs of a group's whole time loop, keyed by what the captured launches depend on
  long long gen = 0;  // bumped whenever a device buffer the kernels see is (re)allocated
  bool use_graphs = true;
  std::map<std::vector<long long>, cudaGraphExec_t> graphs;
  std::map<std::vector<long long>, int> graph_uses;  // calls per key (a key is captured on its second call)
  DevMem d_gout, d_mout;  // gradient / misfit of the host-buffer path (stable addresses for the graphs)
  // snapshots requested by the current forward call (snapevery = 0: none)
  int snapevery = 0;
  float* const* snap_out = nullptr;  // per caller shot: host buffer of nt/snapevery fields
  void drop_graphs() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    graph_uses.clear();
  }
  ~sw_wavesim() { drop_graphs(); }
};

namespace {

struct HostShot {
  int orig;  // index in the caller's array
  int nt;
};

inline long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

void ensure(sw_wavesim* ws, DevMem& m, size_t bytes, const char* what) {
  if (m.bytes >= bytes && m.p) return;
  m.release();
  dev_alloc(m, bytes, what, ws->ctx->stream);
  ++ws->gen;
}

// Runs `work` (the device work of one group: launches, memsets, no host
// synchronisation and no allocation) through a CUDA graph: captured on the
// second call with `key` (one-off calls run directly), replayed afterwards;
// at most 32 graphs are kept per simulation, later keys run directly.  Launch-bound cases (small grids, single
// shots) gain the most.  Work runs directly instead when profiling (the
// per-kernel events belong to single launches), when the caller's stream is
// itself being captured (the launches then join the caller's graph), for the
// TMA stencil variant, or when graphs are switched off.
template <typename Work>
void run_graph(sw_wavesim* ws, std::vector<long long> key, Work&& work) {
  cudaStream_t st = ws->ctx->stream;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  check_cuda(cudaStreamIsCapturing(st, &cs), "cudaStreamIsCapturing");
  if (!ws->use_graphs || ws->ctx->prof.on || cs != cudaStreamCaptureStatusNone || (ws->variant & 3) == 1) {
    work();
    return;
  }
  key.push_back(ws->gen);
  auto it = ws->graphs.find(key);
  if (it == ws->graphs.end()) {
    if (ws->graph_uses.size() > 4096) ws->graph_uses.clear();
    if (++ws->graph_uses[key] < 2 || ws->graphs.size() >= 32) {
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
    it = ws->graphs.emplace(key, ex).first;
  }
  check_cuda(cudaGraphLaunch(it->second, st), "graph launch");
}

std::vector<long long> group_key(const sw_wavesim* ws, const std::vector<HostShot>& group, bool grad) {
  std::vector<long long> k = {grad ? 1 : 0, ws->grp, ws->variant, ws->tile_tz, ws->pf, ws->adjw ? 1 : 0,
                              ws->cpa ? 1 : 0, ws->pair_ok ? 1 : 0, ws->pair_adj_ok ? 1 : 0, ws->pair_tz,
                              ws->pair_occ, ws->kind_tz[0], ws->kind_tz[1], ws->kind_tz[2], ws->precision,
                              ws->split3d ? 1 : 0, ws->inner_np ? 1 : 0, ws->xsplit ? 1 : 0,
                              (long long)group.size()};
  for (const auto& h : group) k.push_back(h.nt);
  return k;
}

template <typename T>
void upload(sw_wavesim* ws, DevMem& m, const std::vector<T>& v, const char* what) {
  const size_t bytes = std::max<size_t>(v.size() * sizeof(T), 16);
  ensure(ws, m, bytes, what);
  if (!v.empty())
    check_cuda(cudaMemcpyAsync(m.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, ws->ctx->stream), what);
}

struct Tables {
  std::vector<ShotDesc> desc;
  std::vector<long long> pts, rec;
  std::vector<int> ptr, ids;
  std::vector<int> bslot;  // per unique point: ring slot (boundary node) or -1
  int nring = 0;
  std::vector<HostShot> order;  // sorted by nt descending
  int max_nt = 0;
  std::vector<PairShot> pair;    // two-step launches: per shot sources and receiver rows
  std::vector<int> recstash;     // per receiver: stash index k * P + x (k = its row's slot)
  bool pair_ok = false;
  std::vector<int> amap;         // adjoint: receiver point on each receiver row, per x
  bool pair_adj_ok = false;
};

long long lin_of(const sw_wavesim* ws, const int* I) {  // 1-based -> padded linear
  if (ws->N == 2) return (long long)(I[1] - 1) * ws->P + (I[0] - 1);
  return ((long long)(I[2] - 1) * ws->n[1] + (I[1] - 1)) * ws->P + (I[0] - 1);
}

// Unique grid points of a list of positions (CSR of the position ids, in
// order).  Points on the outermost grid lines get consecutive ring slots
// starting at slot_base; returns the number of slots used.
int unique_points(const sw_wavesim* ws, const int32_t* idx, int npos, Tables& T, long long& off,
                  long long& ptr_off, int& nunique, int slot_base) {
  std::vector<long long> lin(npos);
  std::vector<char> bnd(npos, 0);
  for (int p = 0; p < npos; ++p) {
    int I[3] = {1, 1, 1};
    for (int d = 0; d < ws->N; ++d) {
      I[d] = idx[p + (long long)d * npos];
      if (I[d] == 1 || I[d] == ws->n[d]) bnd[p] = 1;
    }
    lin[p] = lin_of(ws, I);
  }
  // unique points in order of first appearance; ids listed in position order
  std::vector<long long> uniq;
  std::vector<std::vector<int>> members;
  for (int p = 0; p < npos; ++p) {
    auto it = std::find(uniq.begin(), uniq.end(), lin[p]);
    if (it == uniq.end()) {
      uniq.push_back(lin[p]);
      members.push_back({p});
    } else {
      members[it - uniq.begin()].push_back(p);
    }
  }
  off = (long long)T.pts.size();
  ptr_off = (long long)T.ptr.size();
  nunique = (int)uniq.size();
  int nr = 0;
  for (size_t u = 0; u < uniq.size(); ++u) {
    T.pts.push_back(uniq[u]);
    T.bslot.push_back(bnd[members[u][0]] ? slot_base + nr++ : -1);
    T.ptr.push_back((int)T.ids.size());
    for (int m : members[u]) T.ids.push_back(m);
  }
  T.ptr.push_back((int)T.ids.size());
  return nr;
}

void validate_shot(const sw_wavesim* ws, const sw_acoustic_shot& s, int k, bool grad) {
  std::ostringstream os;
  if (s.nt < 1) { os << "shot " << k << ": nt must be positive"; fail(SW_ERR_ARG, os.str()); }
  if (s.nsrc < 1) { os << "shot " << k << ": there must be at least one source"; fail(SW_ERR_ARG, os.str()); }
  if (s.nrec < 1) { os << "shot " << k << ": there must be at least one receiver"; fail(SW_ERR_ARG, os.str()); }
  if (!s.src_idx || !s.rec_idx || !s.srctf || !s.traces || !s.cpml) {
    os << "shot " << k << ": missing array";
    fail(SW_ERR_ARG, os.str());
  }
  auto chk = [&](const int32_t* idx, int np, const char* what) {
    for (int p = 0; p < np; ++p)
      for (int d = 0; d < ws->N; ++d) {
        const int v = idx[p + (long long)d * np];
        if (v < 1 || v > ws->n[d]) {
          std::ostringstream e;
          e << "shot " << k << ": " << what << " " << p + 1 << " index " << v << " outside 1.." << ws->n[d]
            << " on axis " << d + 1;
          fail(SW_ERR_ARG, e.str());
        }
      }
  };
  chk(s.src_idx, s.nsrc, "source");
  chk(s.rec_idx, s.nrec, "receiver");
  if (grad) {
    if (!s.observed) { os << "shot " << k << ": gradient needs observed data"; fail(SW_ERR_ARG, os.str()); }
    const int K = ws->gp.check_freq;
    if (K >= s.nt) {
      os << "shot " << k << ": checkpointing frequency must be smaller than the number of timesteps";
      fail(SW_ERR_ARG, os.str());
    }
    if (K > 1) {
      for (int p = 0; p < s.nsrc; ++p)
        for (int d = 0; d < ws->N; ++d) {
          const int v = s.src_idx[p + (long long)d * s.nsrc];
          if (v == 1 || v == ws->n[d]) {
            std::ostringstream e;
            e << "shot " << k << ": source " << p + 1
              << " lies on the outermost grid line; with check_freq > 1 the reference's recompute reads a "
                 "stale buffer there, so no well-defined gradient exists (use check_freq = 1 or move the source)";
            fail(SW_ERR_UNSUPPORTED, e.str());
          }
        }
    }
    for (int w = 0; w < s.nwin; ++w) {
      const int a = s.windows[2 * w], b = s.windows[2 * w + 1];
      if (!(1 <= a && a <= b && b <= s.nt)) {
        os << "shot " << k << ": windows indices must be between 1 and maximum number of timesteps";
        fail(SW_ERR_ARG, os.str());
      }
    }
    validate_misfit_kind(s, k);
  }
}

// Builds and uploads the shot tables for shots[first .. first+count) in the
// sorted order; bulk arrays are uploaded (host) or referenced (device).
void build_tables(sw_wavesim* ws, const sw_acoustic_shot* shots, const std::vector<HostShot>& group,
                  bool on_device, bool grad, Tables& T) {
  cudaStream_t st = ws->ctx->stream;
  const int S = (int)group.size();
  T.desc.assign(S, ShotDesc{});
  T.pts.clear(); T.rec.clear(); T.ptr.clear(); T.ids.clear(); T.bslot.clear();
  T.nring = 0;
  std::vector<int> ring_off(S);
  long long tf_total = 0, tr_total = 0, ic_total = 0, mask_total = 0, icd_total = 0, dres_total = 0;
  for (int k = 0; k < S; ++k) {
    const sw_acoustic_shot& s = shots[group[k].orig];
    tf_total += (long long)s.nt * s.nsrc;
    tr_total += (long long)s.nt * s.nrec;
    if (s.invcov_diag) ic_total += s.nt;
    if (grad && s.invcov && s.misfit_kind == 0) {
      icd_total += (long long)s.nt * s.nt;
      dres_total += (long long)s.nt * s.nrec;
    }
    if (s.nwin > 0) mask_total += s.nt;
  }
  // device staging
  if (!on_device) ensure(ws, ws->d_tf, std::max<long long>(tf_total, 4) * sizeof(float), "srctf");
  ensure(ws, ws->d_tr, std::max<long long>(tr_total, 4) * sizeof(float), "traces");
  if (grad) {
    if (!on_device) {
      ensure(ws, ws->d_obs, std::max<long long>(tr_total, 4) * sizeof(float), "observed");
      ensure(ws, ws->d_ic, std::max<long long>(ic_total, 4) * sizeof(float), "invcov");
    }
    ensure(ws, ws->d_mask, std::max<long long>(mask_total, 4) * sizeof(float), "window mask");
    ensure(ws, ws->d_adj, std::max<long long>(tr_total, 4) * sizeof(float), "adjoint source");
    if (dres_total) {
      if (!on_device) ensure(ws, ws->d_icd, icd_total * sizeof(float), "dense inverse covariance");
      ensure(ws, ws->d_dres, 2 * dres_total * sizeof(float), "dense residuals");
    }
  }
  long long icd_o = 0, dres_o = 0;
  const int na = 2 * ws->prm.halo + 2, nh = 2 * ws->prm.halo;
  const int cstride = ws->N * (2 * na + 2 * nh);
  std::vector<float> cpml((size_t)S * cstride);
  std::vector<double> cpml64(ws->precision == 1 ? (size_t)S * cstride : 0);
  std::vector<float> masks;
  long long tf_o = 0, tr_o = 0, ic_o = 0;
  for (int k = 0; k < S; ++k) {
    const sw_acoustic_shot& s = shots[group[k].orig];
    ShotDesc& D = T.desc[k];
    D.nt = s.nt; D.nsrc = s.nsrc; D.nrec = s.nrec;
    D.last = grad ? (s.nt / ws->gp.check_freq) * ws->gp.check_freq : 0;
    // ring slots are relative to this shot's part of the ring array:
    // boundary source points first, then boundary receiver points
    const int nsb = unique_points(ws, s.src_idx, s.nsrc, T, D.sp_off, D.sp_ptr, D.nsp, 0);
    const int nrb = unique_points(ws, s.rec_idx, s.nrec, T, D.rp_off, D.rp_ptr, D.nrp, nsb);
    ring_off[k] = T.nring;
    T.nring += nsb + nrb;
    D.rec_off = (long long)T.rec.size();
    for (int r = 0; r < s.nrec; ++r) {
      int I[3] = {1, 1, 1};
      for (int d = 0; d < ws->N; ++d) I[d] = s.rec_idx[r + (long long)d * s.nrec];
      T.rec.push_back(lin_of(ws, I));
    }
    std::memcpy(&cpml[(size_t)k * cstride], s.cpml, sizeof(float) * cstride);
    if (ws->precision == 1)  // FP64 coefficients of the compensated step (the FP32 ones widened if absent)
      for (int q = 0; q < cstride; ++q) cpml64[(size_t)k * cstride + q] = s.cpml64 ? s.cpml64[q] : (double)s.cpml[q];
    const long long ntf = (long long)s.nt * s.nsrc, ntr = (long long)s.nt * s.nrec;
    if (on_device) {
      D.tf = s.srctf;
      D.obs = s.observed;
      D.ic = s.invcov_diag;
    } else {
      float* tfp = ws->d_tf.as<float>() + tf_o;
      check_cuda(cudaMemcpyAsync(tfp, s.srctf, ntf * sizeof(float), cudaMemcpyHostToDevice, st), "srctf upload");
      D.tf = tfp;
      if (grad) {
        float* op = ws->d_obs.as<float>() + tr_o;
        check_cuda(cudaMemcpyAsync(op, s.observed, ntr * sizeof(float), cudaMemcpyHostToDevice, st), "observed upload");
        D.obs = op;
        if (s.invcov_diag) {
          float* ip = ws->d_ic.as<float>() + ic_o;
          check_cuda(cudaMemcpyAsync(ip, s.invcov_diag, s.nt * sizeof(float), cudaMemcpyHostToDevice, st), "invcov upload");
          D.ic = ip;
          ic_o += s.nt;
        }
      }
    }
    D.tr = ws->d_tr.as<float>() + tr_o;
    D.mkind = grad ? s.misfit_kind : 0;
    if (grad && s.invcov && s.misfit_kind == 0) {
      if (on_device) {
        D.icd = s.invcov;
      } else {
        float* cp = ws->d_icd.as<float>() + icd_o;
        check_cuda(cudaMemcpyAsync(cp, s.invcov, (size_t)s.nt * s.nt * sizeof(float), cudaMemcpyHostToDevice, st),
                   "invcov upload");
        D.icd = cp;
        icd_o += (long long)s.nt * s.nt;
      }
      D.resid = ws->d_dres.as<float>() + dres_o;
      D.cres = ws->d_dres.as<float>() + dres_total + dres_o;
      dres_o += (long long)s.nt * s.nrec;
    }
    if (grad) {
      D.adj = ws->d_adj.as<float>() + tr_o;
      if (s.nwin > 0) {
        const size_t mo = masks.size();
        masks.resize(mo + s.nt, 0.f);
        for (int w = 0; w < s.nwin; ++w)
          for (int t = s.windows[2 * w] - 1; t <= s.windows[2 * w + 1] - 1; ++t) masks[mo + t] = 1.f;
        D.mask = ws->d_mask.as<float>() + mo;
      }
    }
    tf_o += ntf;
    tr_o += ntr;
  }
  // Two-step launches (2D): every shot's source points and receivers off the
  // outermost grid lines (no boundary ring), at most PAIR_MAXSP unique source
  // points and PAIR_MAXRR receiver rows per shot.
  T.pair.assign(S, PairShot{});
  T.recstash.assign(T.rec.size(), 0);
  T.pair_ok = ws->N == 2 && ws->pair_on && (ws->variant & 3) == 0 && !ws->cpa && ws->precision == 0;
  for (int k = 0; k < S && T.pair_ok; ++k) {
    const ShotDesc& D = T.desc[k];
    PairShot& ps = T.pair[k];
    ps.tf = D.tf;
    ps.nt = D.nt;
    ps.nsp = D.nsp;
    if (D.nsp > PAIR_MAXSP) { T.pair_ok = false; break; }
    for (int u = 0; u < D.nsp; ++u) {
      const long long lin = T.pts[D.sp_off + u];
      if (T.bslot[D.sp_off + u] >= 0) T.pair_ok = false;
      ps.sx[u] = (int)(lin % ws->P);
      ps.sz[u] = (int)(lin / ws->P);
      ps.k0[u] = T.ptr[D.sp_ptr + u];
      ps.k1[u] = T.ptr[D.sp_ptr + u + 1];
    }
    ps.nrr = 0;
    for (int r = 0; r < D.nrec && T.pair_ok; ++r) {
      const long long lin = T.rec[D.rec_off + r];
      const int z = (int)(lin / ws->P), x = (int)(lin % ws->P);
      if (z < 1 || z > ws->n[1] - 2) { T.pair_ok = false; break; }
      int slot = -1;
      for (int q = 0; q < ps.nrr; ++q)
        if (ps.rrow[q] == z) slot = q;
      if (slot < 0) {
        if (ps.nrr == PAIR_MAXRR) { T.pair_ok = false; break; }
        slot = ps.nrr++;
        ps.rrow[slot] = z;
      }
      T.recstash[D.rec_off + r] = slot * ws->P + x;
    }
  }
  // two-step adjoint launches: the receiver points (the adjoint sources) off
  // the outermost grid lines too; per receiver row a map x -> point
  T.pair_adj_ok = T.pair_ok && grad;
  if (T.pair_adj_ok) {
    T.amap.assign((size_t)S * PAIR_MAXRR * ws->P, -1);
    for (int k = 0; k < S && T.pair_adj_ok; ++k) {
      const ShotDesc& D = T.desc[k];
      T.pair[k].adj = D.adj;
      for (int u = 0; u < D.nrp; ++u) {
        const long long lin = T.pts[D.rp_off + u];
        const int z = (int)(lin / ws->P), x = (int)(lin % ws->P);
        if (T.bslot[D.rp_off + u] >= 0) { T.pair_adj_ok = false; break; }
        int slot = -1;
        for (int q = 0; q < T.pair[k].nrr; ++q)
          if (T.pair[k].rrow[q] == z) slot = q;
        if (slot < 0) { T.pair_adj_ok = false; break; }
        T.amap[((size_t)k * PAIR_MAXRR + slot) * ws->P + x] = (int)(D.rp_ptr + u);
      }
    }
  }
  if (T.pair_adj_ok) upload(ws, ws->d_amap, T.amap, "adjoint receiver map");
  ws->pair_adj_ok = T.pair_adj_ok;
  if (T.pair_ok) {
    upload(ws, ws->d_pair, T.pair, "two-step shot table");
    upload(ws, ws->d_recstash, T.recstash, "receiver stash table");
    ensure(ws, ws->d_stash, (size_t)S * PAIR_MAXRR * ws->P * sizeof(float), "receiver-row stash");
  }
  ws->pair_ok = T.pair_ok;
  ensure(ws, ws->d_ring, (size_t)std::max(3 * T.nring, 4) * sizeof(float), "boundary rings");
  for (int k = 0; k < S; ++k) T.desc[k].ring = ws->d_ring.as<float>() + 3LL * ring_off[k];
  upload(ws, ws->d_desc, T.desc, "shot descriptors");
  upload(ws, ws->d_bslot, T.bslot, "boundary slots");
  upload(ws, ws->d_pts, T.pts, "point table");
  upload(ws, ws->d_ptr, T.ptr, "point csr");
  upload(ws, ws->d_ids, T.ids, "point ids");
  upload(ws, ws->d_rec, T.rec, "receiver table");
  upload(ws, ws->d_cpml, cpml, "cpml coefficients");
  if (ws->precision == 1) upload(ws, ws->d_cpml64, cpml64, "cpml coefficients (FP64)");
  if (!masks.empty())
    check_cuda(cudaMemcpyAsync(ws->d_mask.p, masks.data(), masks.size() * sizeof(float), cudaMemcpyHostToDevice, st),
               "mask upload");
}

size_t per_shot_bytes(const sw_wavesim* ws, bool grad, int max_nt);

// Exponent array of the FP16 D slots: per slot rows x x-tiles bytes, slots of a shot contiguous.
long long dexp_slot(const sw_wavesim* ws) {
  long long rows = 1;
  for (int d = 1; d < ws->N; ++d) rows *= ws->n[d];
  return rows * ((ws->P + 127) / 128);
}
// The exponents of the D slot that `D` (a dslot_arg result) points to.
FieldArgE dexp_for(const sw_wavesim* ws, const FieldArg& D) {
  if (!D.p || ws->gp.snapshot_bf16 != 3) return FieldArgE{nullptr, 0};
  const long long off = reinterpret_cast<const __half*>(D.p) - ws->dbuf.as<__half>();
  const long long Fe = dexp_slot(ws);
  return FieldArgE{ws->dexp.as<signed char>() + (off / ws->F) * Fe, ws->d_slots * Fe};
}


// Device memory held by the per-shot buffers (counted back into the budget of
// plan_groups and ensure_state).
size_t owned_bytes(const sw_wavesim* ws) {
  size_t owned = 0;
  for (int b = 0; b < 2; ++b) owned += ws->pb[b].bytes + ws->ab[b].bytes + ws->plo[b].bytes;
  owned += ws->db.bytes + ws->adb.bytes + ws->g.bytes + ws->gc.bytes + ws->dbuf.bytes + ws->ck.bytes + ws->dlo.bytes;
  owned += ws->db2.bytes + ws->adb2.bytes + ws->ck16.bytes + ws->ck_stage.bytes;
  for (int d = 0; d < 3; ++d) owned += ws->psi64[0][d].bytes + ws->psi64[1][d].bytes + ws->xi64[d].bytes;
  for (int k = 0; k < 2; ++k)
    for (int d = 0; d < 3; ++d) owned += ws->psi[k][d].bytes + ws->apsi[k][d].bytes;
  return owned;
}

void ensure_state(sw_wavesim* ws, int S, bool grad, int max_nt) {
  const long long F = ws->F;
  cudaStream_t st = ws->ctx->stream;
  // A gradient group smaller than the state capacity (left by a larger
  // forward batch) gets state sized to the group when the gradient buffers
  // of the whole capacity would not fit.
  bool shrink = false;
  if (grad && S < ws->cap) {
    size_t free_b = 0, total_b = 0;
    check_cuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    shrink = (double)per_shot_bytes(ws, true, max_nt) * ws->cap > 0.85 * (double)(free_b + owned_bytes(ws));
  }
  if (shrink) {
    ws->dbuf.release();
    ws->ck.release();
    ws->ck16.release();
    ws->ck_stage.release();
    for (int b = 0; b < 2; ++b) ws->plo[b].release();
    ws->dlo.release();
    for (int d = 0; d < 3; ++d) {
      ws->psi64[0][d].release();
      ws->psi64[1][d].release();
      ws->xi64[d].release();
    }
    ws->hp_cap = 0;
    ws->cap = 0;
  }
  if (S > ws->cap) {
    for (int b = 0; b < 2; ++b) dev_alloc(ws->pb[b], (size_t)S * F * sizeof(float), "pressure field", st);
    dev_alloc(ws->db, (size_t)S * F * sizeof(float), "pressure increment", st);
    for (int k = 0; k < 2; ++k)
      for (int d = 0; d < ws->N; ++d) dev_alloc(ws->psi[k][d], (size_t)S * ws->psz[d] * sizeof(float), "psi", st);
    for (int d = 0; d < ws->N; ++d) dev_alloc(ws->xi[d], (size_t)S * ws->xsz[d] * sizeof(float), "xi", st);
    if (ws->N == 2) {  // two-step launches
      dev_alloc(ws->db2, (size_t)S * F * sizeof(float), "pressure increment (second buffer)", st);
      for (int d = 0; d < ws->N; ++d) {
        dev_alloc(ws->xi2[d], (size_t)S * ws->xsz[d] * sizeof(float), "xi (second buffer)", st);
        dev_alloc(ws->psim[d], (size_t)S * ws->psz[d] * sizeof(float), "psi between two steps", st);
        dev_alloc(ws->xim[d], (size_t)S * ws->xsz[d] * sizeof(float), "xi between two steps", st);
      }
    }
    if (ws->gradient) {
      for (int b = 0; b < 2; ++b) dev_alloc(ws->ab[b], (size_t)S * F * sizeof(float), "adjoint field", st);
      dev_alloc(ws->adb, (size_t)S * F * sizeof(float), "adjoint increment", st);
      for (int k = 0; k < 2; ++k)
        for (int d = 0; d < ws->N; ++d) dev_alloc(ws->apsi[k][d], (size_t)S * ws->psz[d] * sizeof(float), "adjoint psi", st);
      for (int d = 0; d < ws->N; ++d) dev_alloc(ws->axi[d], (size_t)S * ws->xsz[d] * sizeof(float), "adjoint xi", st);
      dev_alloc(ws->g, (size_t)S * F * sizeof(float), "gradient", st);
      dev_alloc(ws->gc, (size_t)S * F * sizeof(float), "gradient compensation", st);
      if (ws->N == 2) {  // two-step adjoint launches
        dev_alloc(ws->adb2, (size_t)S * F * sizeof(float), "adjoint increment (second buffer)", st);
        for (int d = 0; d < ws->N; ++d)
          dev_alloc(ws->axi2[d], (size_t)S * ws->xsz[d] * sizeof(float), "adjoint xi (second buffer)", st);
      }
    }
    ws->cap = S;
    ws->d_slots = 0;
    ws->ck_slots = 0;
    ++ws->gen;
  }
  if (ws->precision == 1 && ws->hp_cap < ws->cap) {
    for (int b = 0; b < 2; ++b) dev_alloc(ws->plo[b], (size_t)ws->cap * F * sizeof(float), "pressure low part", st);
    dev_alloc(ws->dlo, (size_t)ws->cap * F * sizeof(float), "increment low part", st);
    for (int d = 0; d < ws->N; ++d) {
      for (int k = 0; k < 2; ++k)
        dev_alloc(ws->psi64[k][d], (size_t)ws->cap * ws->psz[d] * sizeof(double), "psi (FP64)", st);
      dev_alloc(ws->xi64[d], (size_t)ws->cap * ws->xsz[d] * sizeof(double), "xi (FP64)", st);
    }
    ws->hp_cap = ws->cap;
    ++ws->gen;
  }
  if (grad) {
    const int K = ws->gp.check_freq;
    const long long dslots = K == 1 ? max_nt : K;
    if (dslots > ws->d_slots) {
      ws->dbuf.release();
      const size_t esz = ws->gp.snapshot_bf16 >= 1 ? sizeof(__nv_bfloat16) : sizeof(float);
      dev_alloc(ws->dbuf, (size_t)ws->cap * dslots * F * esz, "D buffer", st);
      if (ws->gp.snapshot_bf16 == 3) {
        dev_alloc(ws->dexp, (size_t)ws->cap * dslots * dexp_slot(ws), "D exponents", st);
        check_cuda(cudaMemsetAsync(ws->dexp.p, 0, ws->dexp.bytes, st), "D exponents");
      }
      ws->d_slots = dslots;
      ++ws->gen;
    }
    const long long cks = K == 1 ? 0 : max_nt / K;
    if (cks > ws->ck_slots) {
      ws->ck.release();
      const bool bf = ws->gp.snapshot_bf16 == 2;
      const long long slot = bf ? ws->strip_total : 2 * F + ws->strip_total;
      dev_alloc(ws->ck, (size_t)ws->cap * cks * slot * sizeof(float), "checkpoints", st);
      if (bf) {
        ws->ck16.release();
        dev_alloc(ws->ck16, (size_t)ws->cap * cks * 2 * F * sizeof(__nv_bfloat16), "BF16 checkpoints", st);
        dev_alloc(ws->ck_scale, (size_t)ws->cap * cks * 2 * sizeof(float), "checkpoint scales", st);
        dev_alloc(ws->ck_max, (size_t)ws->cap * 2 * sizeof(unsigned), "checkpoint maxima", st);
        dev_alloc(ws->ck_stage, (size_t)ws->cap * 2 * F * sizeof(float), "checkpoint stage", st);
      }
      ws->ck_slots = cks;
      ++ws->gen;
    }
    if (!ws->zero.p) {
      dev_alloc(ws->zero, (size_t)(2 * F + ws->strip_total) * sizeof(float), "zero state", st);
      ++ws->gen;
    }
  }
}

// Device memory (bytes) one shot needs in a batch.
size_t per_shot_bytes(const sw_wavesim* ws, bool grad, int max_nt) {
  // p ping-pong + increment, two psi buffers and xi; the same for the adjoint, plus g and its compensation
  long long floats = 3 * ws->F + ws->strip_total;
  for (int d = 0; d < ws->N; ++d) floats += ws->psz[d];
  if (ws->gradient) floats = 2 * floats + 2 * ws->F;
  if (ws->N == 2) floats += ws->F + 2 * ws->strip_total;  // second d / xi buffers, scratch strips
  if (ws->N == 2 && ws->gradient) floats += ws->F + ws->strip_total;  // second adjoint d / xi buffers
  if (ws->precision == 1) {  // low parts of p (two buffers) and d; FP64 psi (two buffers) and xi
    floats += 3 * ws->F;
    for (int d = 0; d < ws->N; ++d) floats += 4 * ws->psz[d] + 2 * ws->xsz[d];
  }
  if (grad) {
    const int K = ws->gp.check_freq;
    const long long dsl = (K == 1 ? (long long)max_nt : K) * ws->F;
    floats += ws->gp.snapshot_bf16 >= 1 ? (dsl + 1) / 2 : dsl;  // BF16 D slots take half
    if (K > 1) {
      if (ws->gp.snapshot_bf16 == 2)  // BF16 (p, d) = one float's worth per point, plus the FP32 stage
        floats += (long long)(max_nt / K) * (ws->F + ws->strip_total) + 2 * ws->F;
      else
        floats += (long long)(max_nt / K) * (2 * ws->F + ws->strip_total);
    }
  }
  return (size_t)floats * sizeof(float);
}

struct StepCtx {
  sw_wavesim* ws;
  int TZ;
  int tiles_x, tiles_y, tiles_z;
};

// Warps per block of the register-pipelined 2D stencil (variant 0: 4, 2: 8, 3: 16).
int block_warps(const sw_wavesim* ws) { return (ws->variant & 3) == 2 ? 8 : (ws->variant & 3) == 3 ? 16 : 4; }
// 3D: y rows (warps) per block, 4 or (variant 2) 8.
int block_rows3d(const sw_wavesim* ws) { return (ws->variant & 3) == 2 ? 8 : 4; }

enum { TZ_FORWARD = 0, TZ_RECOMPUTE = 1, TZ_ADJOINT = 2 };

StepCtx make_step_ctx(sw_wavesim* ws, int S, int kind = TZ_FORWARD) {
  StepCtx c{ws, 0, 0, 1, 0};
  const int sms = ws->ctx->num_sms > 0 ? ws->ctx->num_sms : 148;
  const int nint = ws->n[ws->N - 1] - 2;  // interior extent of the marching axis
  if (ws->N == 2) {
    const int w = 128 * block_warps(ws);
    c.tiles_x = (int)((ws->P + w - 1) / w);
  } else {
    c.tiles_x = (int)((ws->P + 127) / 128);
    const int nw = block_rows3d(ws);
    c.tiles_y = (ws->n[1] - 2 + nw - 1) / nw;
  }
  int TZ = ws->kind_tz[kind] > 0 ? ws->kind_tz[kind] : ws->tile_tz;
  if (TZ <= 0) {
    if (ws->N == 2 && (ws->variant & 3) != 1) {
      // register-pipelined 2D stencil: short bands keep every SM at full
      // occupancy with a negligible tail (8 rows measured best on GB300 for
      // 64 shots of 2001 x 801: 55.6 Gpts/s against 48.4 at 64 rows); small
      // batches take 4-row bands to fill the GPU
      TZ = (long long)S * c.tiles_x * ((nint + 7) / 8) < 4LL * sms ? 4 : 8;
    } else {
      // aim for >= ~8 blocks per SM in total, with TZ in [tz_min, 64]
      TZ = 64;
      const int tz_min = (ws->N == 2 && (ws->variant & 3) == 1) ? 16 : 8;
      while (TZ > tz_min) {
        const long long blocks = (long long)S * c.tiles_x * c.tiles_y * ((nint + TZ - 1) / TZ);
        if (blocks >= 8LL * sms) break;
        TZ /= 2;
      }
    }
  }
  c.TZ = TZ;
  c.tiles_z = (nint + TZ - 1) / TZ;
  return c;
}

// Compensated forward step (k_ac_hp): 2D blocks of 512 x points, 3D blocks of
// 128 x points and 4 y rows; bands of 32 rows, shorter while the launch would
// have fewer than 8 blocks per SM, 4 rows at least.
StepCtx make_hp_ctx(sw_wavesim* ws, int S) {
  StepCtx c{ws, 0, 0, 1, 0};
  const int sms = ws->ctx->num_sms > 0 ? ws->ctx->num_sms : 148;
  if (ws->N == 2) {
    c.tiles_x = (int)((ws->P + 511) / 512);
  } else {
    c.tiles_x = (int)((ws->P + 127) / 128);
    c.tiles_y = (ws->n[1] - 2 + 3) / 4;
  }
  const int nint = ws->n[ws->N - 1] - 2;
  int TZ = 32;
  while (TZ > 4 && (long long)S * c.tiles_x * c.tiles_y * ((nint + TZ - 1) / TZ) < 8LL * sms) TZ /= 2;
  c.TZ = TZ;
  c.tiles_z = (nint + TZ - 1) / TZ;
  return c;
}

// Two-step launches: warps of PAIR_OUT x points, 4 per block; bands of 32
// rows (the band halo of the first step repeats 2 of every 34 rows), shorter
// bands where 32-row ones would leave the GPU with less than two waves of
// blocks (small batches), 4 rows at least.
StepCtx make_pair_ctx(sw_wavesim* ws, int S) {
  StepCtx c{ws, 0, 0, 1, 0};
  const int warps = (ws->n[0] - 2) / PAIR_OUT + 1;
  c.tiles_x = (warps + 3) / 4;
  int TZ = ws->pair_tz;
  if (TZ <= 0) {
    const int sms = ws->ctx->num_sms > 0 ? ws->ctx->num_sms : 148;
    TZ = 32;
    while (TZ > 4 && (long long)S * c.tiles_x * ((ws->n[1] - 2 + TZ - 1) / TZ) < 2LL * 6 * sms) TZ /= 2;
  }
  c.TZ = TZ;
  c.tiles_z = (ws->n[1] - 2 + c.TZ - 1) / c.TZ;
  return c;
}

// Algorithmic bytes of one two-step launch: per interior point and shot R
// p[n], d[n], W p[n+2], d[n+2] (16 B for both steps), fact once for the
// launch, per strip cell and axis R psi/xi of step n and W those of step n+2;
// the D slots of both steps; checkpoint copies of step n; adjoint: R D of
// both steps and R/W the per-shot FP32 correlation sum once.
double pair_bytes(const sw_wavesim* ws, int S, int n_dwrite, bool ckpt, bool adjoint = false) {
  double pts = (double)(ws->n[0] - 2) * (ws->n[1] - 2);
  double strip = 0.0;
  const int H = ws->prm.halo;
  for (int d = 0; d < 2; ++d) {
    double w = 0.0;
    for (int x = 1; x <= ws->n[d] - 2; ++x) w += (x < H || x >= ws->n[d] - H) ? 1.0 : 0.0;
    strip += w * (double)(ws->n[1 - d] - 2);
  }
  const double dsz = (ws->gradient && ws->gp.snapshot_bf16 >= 1) ? 2.0 : 4.0;
  double b = (16.0 * S + 4.0) * pts + 16.0 * strip * S + 2.0 * dsz * pts * n_dwrite;
  if (ckpt) b += 8.0 * pts * S + 8.0 * strip * S;
  if (adjoint) b += (2.0 * dsz + 8.0) * pts * S;
  return b;
}

// Extra bytes of a compensated forward launch: per interior point and shot R
// plo[n], W plo[n+1], R/W dlo; the low part of fact once for the launch.
double hp_extra_bytes(const sw_wavesim* ws, int S) {
  double pts = 1.0;
  for (int d = 0; d < ws->N; ++d) pts *= (double)(ws->n[d] - 2);
  return (16.0 * S + 4.0) * pts;
}

// Algorithmic bytes of one stencil launch (FP32 words): per interior point and
// shot R p[n], R d[n], W p[n+1], W d[n+1]; fact is read once for all shots of
// the launch; per damping-strip cell and axis R/W psi and R/W xi; D write
// (forward of the gradient), R D + RMW g and its compensation (adjoint);
// checkpoint copies of p, d, psi, xi.
double stencil_bytes(const sw_wavesim* ws, int S, int mode, int n_dwrite, bool ckpt, int ngroups = -1) {
  double pts = 1.0;
  for (int d = 0; d < ws->N; ++d) pts *= (double)(ws->n[d] - 2);
  double strip = 0.0;  // interior points inside the damping strips, summed over axes
  const int H = ws->prm.halo;
  for (int d = 0; d < ws->N; ++d) {
    double w = 0.0;
    for (int x = 1; x <= ws->n[d] - 2; ++x) w += (x < H || x >= ws->n[d] - H) ? 1.0 : 0.0;
    double other = 1.0;
    for (int e = 0; e < ws->N; ++e)
      if (e != d) other *= (double)(ws->n[e] - 2);
    strip += w * other;
  }
  double b = (16.0 * S + 4.0) * pts + 16.0 * strip * S;
  if (mode == MODE_FWD_D) b += 4.0 * pts * n_dwrite;
  if (mode == MODE_ADJ) b += ngroups < 0 ? 20.0 * pts * S : (4.0 * S + 16.0 * ngroups) * pts;
  if (mode == MODE_ADJW) b += 12.0 * pts * S;  // R D, RMW the plain sum
  if (ckpt) b += 8.0 * pts * S + 8.0 * strip * S;
  return b;
}

// The stencil moves p, d, D, g and the checkpoint copies of p and d with
// 16-byte vector accesses: refuse to launch on a misaligned base or stride.
void check_vector_alignment(const StepArgs& a) {
  auto ok = [](const FieldArg& f) {
    return f.p == nullptr || ((reinterpret_cast<uintptr_t>(f.p) % 16) == 0 && f.s % 4 == 0);
  };
  const FieldArg* vec[] = {&a.pcur, &a.pnew, &a.din, &a.dout, &a.ck_p, &a.ck_d, &a.Dout, &a.dcorr, &a.g, &a.gc};
  for (const FieldArg* f : vec)
    if (!ok(*f)) fail(SW_ERR_CUDA, "internal error: misaligned field handed to the stencil");
  if (a.P % 4 != 0 || reinterpret_cast<uintptr_t>(a.fact) % 16 != 0)
    fail(SW_ERR_CUDA, "internal error: misaligned pitch or fact");
}

template <int MODE>
void enable_tma_smem() {
  static int done_for_device = -1;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (done_for_device == dev) return;
  check_cuda(cudaFuncSetAttribute(k_ac2d_tma<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)TmaLayout<MODE>::BYTES),
             "shared memory attribute");
  done_for_device = dev;
}

// The cp.async-staged stencil keeps its row ring in shared memory (24-36 KB
// per block): ask for the largest shared-memory carveout so that the
// occupancy of its launch bounds is reached.
template <int MODE>
void enable_cpa_carveout() {
  static int done_for_device = -1;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (done_for_device == dev) return;
  check_cuda(cudaFuncSetAttribute(k_ac2d_cpa<MODE, 4>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared),
             "shared memory carveout");
  done_for_device = dev;
}

// The two-step kernels keep a row ring in shared memory (25 / 37 KB per
// block): ask for the largest carveout so the occupancy of their launch
// bounds is reached.
template <int MODE, int MB>
void enable_pair_carveout() {
  static int done_for_device = -1;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (done_for_device == dev) return;
  check_cuda(cudaFuncSetAttribute(k_ac2d_pair<MODE, 4, MB>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared),
             "shared memory carveout");
  done_for_device = dev;
}

// The 2D one-step stencil of 4-warp blocks with the x strips split off:
// `blocks` main blocks for the lanes outside the x strips, then one block
// per 128 lane groups of the x strips (rows x shots), which run in the tail
// of the launch (79.5 against 78.4 Gpts/s as a second launch on the 64-shot
// headline).  Returns the number of kernels launched.
template <int MODE>
int launch_2d_xsplit(long long blocks, cudaStream_t st, const StepArgs& a) {
  int nl, xr, ng;
  xstrip_groups(a.n0, a.halo, a.P, nl, xr, ng);
  const long long items = (long long)ng * (a.n1 - 2) * a.nshots;
  k_ac2d_step<MODE, 4, 1, true><<<(unsigned)(blocks + (items + 127) / 128), 128, 0, st>>>(a);
  return 1;
}

template <int MODE, int MB>
void launch_pair(long long blocks, cudaStream_t st, const StepArgs& a, const PairArgs& b) {
  enable_pair_carveout<MODE, MB>();
  k_ac2d_pair<MODE, 4, MB><<<(unsigned)blocks, 128, 0, st>>>(a, b);
}

// Grid of the two-launch 3D step (the host side of ac3d_work): per axis the
// rows [1, a) and [b, n-1) hold the C-PML strips.
struct Split3d {
  int tiles_y1, tiles_z1;  // region 1: y groups x z bands over [a, b) x [a, b)
  int zslab_units;         // region 2: (z band, y group) units per x tile
  int yslab_units;         // region 3: the same for the y slabs
};
void split_axis_host(int n, int H, int& a, int& b) {
  a = std::min(std::max(H, 1), n - 1);
  b = std::max(n - std::max(H, 1), a);
}
Split3d split3d(const sw_wavesim* ws, int TZ, int NW) {
  const int ny = ws->n[1], nz = ws->n[2], H = ws->prm.halo;
  int ay, by, az, bz;
  split_axis_host(ny, H, ay, by);
  split_axis_host(nz, H, az, bz);
  Split3d r;
  r.tiles_y1 = (by - ay + NW - 1) / NW;
  r.tiles_z1 = (bz - az + TZ - 1) / TZ;
  if (r.tiles_y1 == 0 || r.tiles_z1 == 0) r.tiles_y1 = r.tiles_z1 = 0;
  const int gy_all = (ny - 2 + NW - 1) / NW;
  const int nb_lo = (az - 1 + TZ - 1) / TZ, nb_hi = (nz - 1 - bz + TZ - 1) / TZ;
  const int gyl = (ay - 1 + NW - 1) / NW, gyh = (ny - 1 - by + NW - 1) / NW;
  r.zslab_units = (nb_lo + nb_hi) * gy_all;
  r.yslab_units = ((bz - az + TZ - 1) / TZ) * (gyl + gyh);
  return r;
}

struct Launcher {
  sw_wavesim* ws;
  cudaStream_t st;
  template <int MODE>
  void step(const StepArgs& a0, const StepCtx& c, double bytes, bool recompute = false) {
    StepArgs a = a0;
    if (a.dbf16 == 2) {  // the exponents of the FP16 D slots read / written
      a.Dexp = dexp_for(ws, a.Dout);
      a.dcorr_exp = dexp_for(ws, a.dcorr);
    }
    check_vector_alignment(a);
    const long long blocks = (long long)a.nshots * c.tiles_x * c.tiles_y * c.tiles_z;
    cudaEvent_t ev = nullptr;
    const int kind = (MODE == MODE_ADJ || MODE == MODE_ADJW) ? KK_ADJOINT : (recompute ? KK_RECOMPUTE : KK_STENCIL);
    ws->ctx->prof.begin(st, kind, bytes, &ev);
    int nk = 1;  // kernels launched for this step
    if constexpr (MODE == MODE_FWD || MODE == MODE_FWD_D) {
      if (ws->precision == 1 && !recompute) {  // compensated forward (context from make_hp_ctx)
        if (ws->N == 2)
          k_ac_hp<MODE, 2><<<(unsigned)blocks, 128, 0, st>>>(a);
        else
          k_ac_hp<MODE, 3><<<(unsigned)blocks, 128, 0, st>>>(a);
        check_cuda(cudaGetLastError(), "compensated stencil launch");
        ws->ctx->prof.end(st, kind, ev);
        return;
      }
    }
    if constexpr (MODE == MODE_ADJW) {  // 2D register-pipelined or cp.async-staged stencil only
      const int nw = block_warps(ws);
      if (nw == 4 && ws->cpa) {
        enable_cpa_carveout<MODE>();
        k_ac2d_cpa<MODE, 4><<<(unsigned)blocks, 128, 0, st>>>(a);
      } else if (nw == 4 && ws->xsplit)
        nk = launch_2d_xsplit<MODE>(blocks, st, a);
      else if (nw == 4)
        k_ac2d_step<MODE, 4><<<(unsigned)blocks, 128, 0, st>>>(a);
      else if (nw == 8)
        k_ac2d_step<MODE, 8><<<(unsigned)blocks, 256, 0, st>>>(a);
      else
        k_ac2d_step<MODE, 16><<<(unsigned)blocks, 512, 0, st>>>(a);
    } else if (ws->N == 2 && (ws->variant & 3) == 1) {
      enable_tma_smem<MODE>();
      k_ac2d_tma<MODE><<<(unsigned)blocks, 160, TmaLayout<MODE>::BYTES, st>>>(a);
    } else if (ws->N == 2) {
      const int nw = block_warps(ws);
      bool launched = false;
      if (nw == 4 && ws->cpa) {
        enable_cpa_carveout<MODE>();
        k_ac2d_cpa<MODE, 4><<<(unsigned)blocks, 128, 0, st>>>(a);
        launched = true;
      }
      if constexpr (MODE != MODE_ADJ) {
        if (!launched && nw == 4 && (ws->variant & 4)) {
          k_ac2d_step<MODE, 4, 2><<<(unsigned)blocks, 128, 0, st>>>(a);
          launched = true;
        }
      }
      if (launched) {
      } else if (nw == 4 && ws->xsplit)
        nk = launch_2d_xsplit<MODE>(blocks, st, a);
      else if (nw == 4)
        k_ac2d_step<MODE, 4><<<(unsigned)blocks, 128, 0, st>>>(a);
      else if (nw == 8)
        k_ac2d_step<MODE, 8><<<(unsigned)blocks, 256, 0, st>>>(a);
      else
        k_ac2d_step<MODE, 16><<<(unsigned)blocks, 512, 0, st>>>(a);
    } else if (ws->split3d) {
      // rows outside the y / z strips, the z slabs, the y slabs (k_ac3d_inner, k_ac3d_zslab, k_ac3d_yslab)
      const int nw = block_rows3d(ws);
      const Split3d sp = split3d(ws, c.TZ, nw);
      StepArgs a1 = a;
      a1.tiles_y = sp.tiles_y1;
      a1.tiles_z = sp.tiles_z1;
      const long long b1 = (long long)a.nshots * c.tiles_x * sp.tiles_y1 * sp.tiles_z1;
      // the slabs are thin: shorter bands while a slab launch would fill less
      // than two waves of 4 blocks per SM (small batches), 4 rows at least
      const int sms = ws->ctx->num_sms > 0 ? ws->ctx->num_sms : 148;
      int tzs = c.TZ;
      Split3d ss = sp;
      while (tzs > 4 && (long long)a.nshots * c.tiles_x * std::min(ss.zslab_units, ss.yslab_units) < 8LL * sms) {
        tzs /= 2;
        ss = split3d(ws, tzs, nw);
      }
      StepArgs a2 = a;
      a2.TZ = tzs;
      const long long b2 = (long long)a.nshots * c.tiles_x * ss.zslab_units;
      const long long b3 = (long long)a.nshots * c.tiles_x * ss.yslab_units;
      nk = (b1 > 0) + (b2 > 0) + (b3 > 0);
      if (b1 > 0 && ws->inner_np) {
        if (nw == 8) k_ac3d_inner_np<MODE, 8><<<(unsigned)b1, 256, 0, st>>>(a1);
        else k_ac3d_inner_np<MODE><<<(unsigned)b1, 128, 0, st>>>(a1);
      } else if (b1 > 0) {
        if (nw == 8) k_ac3d_inner<MODE, 8><<<(unsigned)b1, 256, 0, st>>>(a1);
        else k_ac3d_inner<MODE><<<(unsigned)b1, 128, 0, st>>>(a1);
      }
      if (b2 > 0 && ws->inner_np) {
        if (nw == 8) k_ac3d_zslab<MODE, 8, false><<<(unsigned)b2, 256, 0, st>>>(a2);
        else k_ac3d_zslab<MODE, 4, false><<<(unsigned)b2, 128, 0, st>>>(a2);
      } else if (b2 > 0) {
        if (nw == 8) k_ac3d_zslab<MODE, 8><<<(unsigned)b2, 256, 0, st>>>(a2);
        else k_ac3d_zslab<MODE><<<(unsigned)b2, 128, 0, st>>>(a2);
      }
      if (b3 > 0 && ws->inner_np) {
        if (nw == 8) k_ac3d_yslab<MODE, 8, false><<<(unsigned)b3, 256, 0, st>>>(a2);
        else k_ac3d_yslab<MODE, 4, false><<<(unsigned)b3, 128, 0, st>>>(a2);
      } else if (b3 > 0) {
        if (nw == 8) k_ac3d_yslab<MODE, 8><<<(unsigned)b3, 256, 0, st>>>(a2);
        else k_ac3d_yslab<MODE><<<(unsigned)b3, 128, 0, st>>>(a2);
      }
    } else {
      const int nw = block_rows3d(ws);
      if constexpr (MODE == MODE_FWD) {
        if (nw == 8) k_ac3d_fwd<MODE_FWD, 8><<<(unsigned)blocks, 256, 0, st>>>(a);
        else k_ac3d_fwd<MODE_FWD><<<(unsigned)blocks, 128, 0, st>>>(a);
      } else {
        if (nw == 8) k_ac3d_step<MODE, 8><<<(unsigned)blocks, 256, 0, st>>>(a);
        else k_ac3d_step<MODE><<<(unsigned)blocks, 128, 0, st>>>(a);
      }
    }
    check_cuda(cudaGetLastError(), "stencil launch");
    ws->ctx->prof.end(st, kind, ev, nk);
  }
  // two time steps in one launch (2D)
  template <int MODE>
  void pair(const StepArgs& a, const PairArgs& b, double bytes, bool recompute = false) {
    check_vector_alignment(a);
    if (reinterpret_cast<uintptr_t>(b.Dout2.p) % 16 != 0 || reinterpret_cast<uintptr_t>(b.dcorr2.p) % 16 != 0 ||
        (b.stash.p && b.stash.s % 4 != 0))
      fail(SW_ERR_CUDA, "internal error: misaligned field handed to the two-step stencil");
    const long long blocks = (long long)a.nshots * a.tiles_x * a.tiles_y * a.tiles_z;
    cudaEvent_t ev = nullptr;
    const int kind = MODE == MODE_ADJW ? KK_ADJOINT : recompute ? KK_RECOMPUTE : KK_STENCIL;
    ws->ctx->prof.begin(st, kind, bytes, &ev);
    // resident blocks per SM: forward kinds 6 (default), 4 or 7; adjoint 5, 3 or 4
    if constexpr (MODE == MODE_ADJW) {
      if (ws->pair_occ == 1)
        launch_pair<MODE, 3>(blocks, st, a, b);
      else if (ws->pair_occ == 2)
        launch_pair<MODE, 4>(blocks, st, a, b);
      else
        launch_pair<MODE, 5>(blocks, st, a, b);
    } else {
      if (ws->pair_occ == 1)
        launch_pair<MODE, 4>(blocks, st, a, b);
      else if (ws->pair_occ == 2)
        launch_pair<MODE, 7>(blocks, st, a, b);
      else
        launch_pair<MODE, 6>(blocks, st, a, b);
    }
    check_cuda(cudaGetLastError(), "two-step stencil launch");
    ws->ctx->prof.end(st, kind, ev);
  }
};

StepArgs base_args(sw_wavesim* ws, const StepCtx& c, int S) {
  StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n0 = ws->n[0];
  a.n1 = ws->n[1];
  a.n2 = ws->N == 3 ? ws->n[2] : 1;
  a.P = ws->P;
  a.halo = ws->prm.halo;
  for (int d = 0; d < ws->N; ++d) {
    const double ih = 1.0 / ws->prm.h[d];
    a.ih[d] = (float)ih;
    a.ih2[d] = (float)(ih * ih);
  }
  a.fact = ws->fact.as<float>();
  a.cpml = ws->d_cpml.as<float>();
  a.cpml_stride = ws->N * (2 * (2 * ws->prm.halo + 2) + 2 * (2 * ws->prm.halo));
  a.nshots = S;
  a.tiles_x = c.tiles_x;
  a.tiles_y = c.tiles_y;
  a.tiles_z = c.tiles_z;
  a.TZ = c.TZ;
  a.err = ws->ctx->err.as<int>();
  if (ws->precision == 1) {
    a.fact_lo = ws->fact_lo.as<float>();
    a.cpml64 = ws->d_cpml64.as<double>();
    for (int d = 0; d < ws->N; ++d) a.ihd[d] = 1.0 / ws->prm.h[d];
    for (int d = 0; d < ws->N; ++d) {
      const double ih2 = 1.0 / (ws->prm.h[d] * ws->prm.h[d]);
      a.ih2[d] = (float)ih2;
      a.ih2_lo[d] = (float)(ih2 - (double)(float)ih2);
    }
  }
  a.wait_cycles = ws->wait_cycles;
  a.withhold = ws->withhold;
  a.pf = ws->pf;
  a.dbf16 = (ws->gradient && ws->gp.snapshot_bf16 >= 1) ? (ws->gp.snapshot_bf16 == 3 ? 2 : 1) : 0;
  a.ntx = (int)((ws->P + 127) / 128);
  return a;
}

// D slot `k` of every shot (the slots of a shot are contiguous; FP32 or BF16 elements).
FieldArg dslot_arg(const sw_wavesim* ws, long long k) {
  const long long off = k * ws->F;
  float* p = ws->gp.snapshot_bf16 >= 1 ? reinterpret_cast<float*>(ws->dbuf.as<__nv_bfloat16>() + off)
                                       : ws->dbuf.as<float>() + off;
  return FieldArg{p, ws->d_slots * ws->F};
}

FieldArg fa(const DevMem& m, long long stride) { return FieldArg{m.as<float>(), stride}; }

int active_count(const std::vector<HostShot>& g, int it) {
  int k = 0;
  while (k < (int)g.size() && g[k].nt >= it) ++k;
  return k;
}

void zero_state(sw_wavesim* ws, int S, bool adjoint) {
  cudaStream_t st = ws->ctx->stream;
  DevMem* b = adjoint ? ws->ab : ws->pb;
  for (int k = 0; k < 2; ++k) check_cuda(cudaMemsetAsync(b[k].p, 0, (size_t)S * ws->F * sizeof(float), st), "reset");
  check_cuda(cudaMemsetAsync((adjoint ? ws->adb : ws->db).p, 0, (size_t)S * ws->F * sizeof(float), st), "reset d");
  for (int k = 0; k < 2; ++k)
    for (int d = 0; d < ws->N; ++d)
      check_cuda(cudaMemsetAsync((adjoint ? ws->apsi : ws->psi)[k][d].p, 0, (size_t)S * ws->psz[d] * sizeof(float), st),
                 "reset psi");
  for (int d = 0; d < ws->N; ++d)
    check_cuda(cudaMemsetAsync((adjoint ? ws->axi : ws->xi)[d].p, 0, (size_t)S * ws->xsz[d] * sizeof(float), st),
               "reset xi");
  DevMem& d2 = adjoint ? ws->adb2 : ws->db2;
  if (d2.p) {
    check_cuda(cudaMemsetAsync(d2.p, 0, (size_t)S * ws->F * sizeof(float), st), "reset d");
    for (int d = 0; d < ws->N; ++d)
      check_cuda(cudaMemsetAsync((adjoint ? ws->axi2 : ws->xi2)[d].p, 0, (size_t)S * ws->xsz[d] * sizeof(float), st),
                 "reset xi");
  }
  if (!adjoint && ws->precision == 1) {
    for (int k = 0; k < 2; ++k)
      check_cuda(cudaMemsetAsync(ws->plo[k].p, 0, (size_t)S * ws->F * sizeof(float), st), "reset p low part");
    check_cuda(cudaMemsetAsync(ws->dlo.p, 0, (size_t)S * ws->F * sizeof(float), st), "reset d low part");
    for (int d = 0; d < ws->N; ++d) {
      for (int k = 0; k < 2; ++k)
        check_cuda(cudaMemsetAsync(ws->psi64[k][d].p, 0, (size_t)S * ws->psz[d] * sizeof(double), st), "reset psi");
      check_cuda(cudaMemsetAsync(ws->xi64[d].p, 0, (size_t)S * ws->xsz[d] * sizeof(double), st), "reset xi");
    }
  }
  check_cuda(cudaMemsetAsync(ws->d_ring.p, 0, ws->d_ring.bytes, st), "reset rings");
}

// Download traces of a group back to the caller (host or device pointers).
void download_traces(sw_wavesim* ws, const sw_acoustic_shot* shots, const std::vector<HostShot>& group,
                     bool on_device) {
  cudaStream_t st = ws->ctx->stream;
  long long o = 0;
  for (const HostShot& h : group) {
    const sw_acoustic_shot& s = shots[h.orig];
    const long long n = (long long)s.nt * s.nrec;
    check_cuda(cudaMemcpyAsync(s.traces, ws->d_tr.as<float>() + o, n * sizeof(float),
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st),
               "traces download");
    o += n;
  }
}

void launch_inject(sw_wavesim* ws, int Sa, const FieldArg& pnew, const FieldArg& dnew, const FieldArg& Dw,
                   int d_first, int it, int record, int it_stash = 0, const FieldArg& plo = FieldArg{nullptr, 0},
                   const FieldArg& dlo = FieldArg{nullptr, 0}) {
  cudaStream_t st = ws->ctx->stream;
  cudaEvent_t ev = nullptr;
  ws->ctx->prof.begin(st, KK_SRCREC, 0.0, &ev);
  const FieldArg stash{ws->d_stash.as<float>(), (long long)PAIR_MAXRR * ws->P};
  k_inject_record<<<Sa, 128, 0, st>>>(ws->d_desc.as<ShotDesc>(), ws->d_pts.as<long long>(), ws->d_ptr.as<int>(),
                                      ws->d_ids.as<int>(), ws->d_bslot.as<int>(), ws->d_rec.as<long long>(), pnew,
                                      dnew, Dw, d_first, it, record,
                                      (ws->gradient && ws->gp.snapshot_bf16 >= 1) ? (ws->gp.snapshot_bf16 == 3 ? 2 : 1) : 0,
                                      ws->d_recstash.as<int>(), stash, it_stash, plo, dlo, dexp_for(ws, Dw), ws->P);
  check_cuda(cudaGetLastError(), "inject/record launch");
  ws->ctx->prof.end(st, KK_SRCREC, ev);
}

// BF16 checkpoint slot `slot`: the staged (p, d) of the S first shots.
void pack_checkpoint(sw_wavesim* ws, int S, int slot) {
  cudaStream_t st = ws->ctx->stream;
  const long long F = ws->F;
  const long long sstride16 = ws->ck_slots * 2 * F;  // one shot's slots are contiguous
  cudaEvent_t ev = nullptr;
  ws->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
  check_cuda(cudaMemsetAsync(ws->ck_max.p, 0, (size_t)S * 2 * sizeof(unsigned), st), "checkpoint max clear");
  const dim3 grid((unsigned)std::min<long long>((F + 255) / 256, 256), 2 * S);
  k_ck_absmax<<<grid, 256, 0, st>>>(ws->ck_stage.as<float>(), F, ws->ck_max.as<unsigned>());
  check_cuda(cudaGetLastError(), "checkpoint max launch");
  k_ck_pack<<<grid, 256, 0, st>>>(ws->ck_stage.as<float>(), F, ws->ck_max.as<unsigned>(),
                                  ws->ck16.as<__nv_bfloat16>() + (long long)slot * 2 * F, sstride16,
                                  ws->ck_scale.as<float>() + (long long)slot * 2 * ws->cap);
  check_cuda(cudaGetLastError(), "checkpoint pack launch");
  ws->ctx->prof.end(st, KK_OTHER, ev);
}

void unpack_checkpoint(sw_wavesim* ws, int S, int slot) {
  cudaStream_t st = ws->ctx->stream;
  const long long F = ws->F;
  const long long sstride16 = ws->ck_slots * 2 * F;
  cudaEvent_t ev = nullptr;
  ws->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
  const dim3 grid((unsigned)std::min<long long>((F + 255) / 256, 256), 2 * S);
  k_ck_unpack<<<grid, 256, 0, st>>>(ws->ck16.as<__nv_bfloat16>() + (long long)slot * 2 * F, sstride16, F,
                                    ws->ck_scale.as<float>() + (long long)slot * 2 * ws->cap,
                                    ws->ck_stage.as<float>());
  check_cuda(cudaGetLastError(), "checkpoint unpack launch");
  ws->ctx->prof.end(st, KK_OTHER, ev);
}

// Forward state buffers.  A launch reads state (p, d, psi, xi) from buffers
// (p, d, k, x) and writes the other p and psi buffers; a two-step launch also
// writes the other d and xi buffers (its repeated first steps at band and
// warp edges read d and xi of points other warps update), a one-step launch
// updates d and xi in place.  The adjoint state uses the same scheme.
struct FwdState {
  int p = 0, d = 0, k = 0, x = 0;
};

void set_io(sw_wavesim* ws, StepArgs& a, FwdState& s, bool two, bool adjoint) {
  const long long F = ws->F;
  const int dn = two ? 1 - s.d : s.d, xn = two ? 1 - s.x : s.x;
  DevMem* pb = adjoint ? ws->ab : ws->pb;
  DevMem* db[2] = {adjoint ? &ws->adb : &ws->db, adjoint ? &ws->adb2 : &ws->db2};
  a.pcur = fa(pb[s.p], F);
  a.pnew = fa(pb[1 - s.p], F);
  if (!adjoint && ws->precision == 1) {
    a.plo_cur = fa(ws->plo[s.p], F);
    a.plo_new = fa(ws->plo[1 - s.p], F);
    a.dlo = fa(ws->dlo, F);
    for (int d = 0; d < ws->N; ++d) {
      a.psi64_in[d] = Field64{ws->psi64[s.k][d].as<double>(), ws->psz[d]};
      a.psi64_out[d] = Field64{ws->psi64[1 - s.k][d].as<double>(), ws->psz[d]};
      a.xi64[d] = Field64{ws->xi64[d].as<double>(), ws->xsz[d]};
    }
  }
  a.din = fa(*db[s.d], F);
  a.dout = fa(*db[dn], F);
  for (int d = 0; d < ws->N; ++d) {
    DevMem* xb[2] = {adjoint ? &ws->axi[d] : &ws->xi[d], adjoint ? &ws->axi2[d] : &ws->xi2[d]};
    DevMem(*ps)[3] = adjoint ? ws->apsi : ws->psi;
    a.psi_in[d] = fa(ps[s.k][d], ws->psz[d]);
    a.psi_out[d] = fa(ps[1 - s.k][d], ws->psz[d]);
    a.xi_in[d] = fa(*xb[s.x], ws->xsz[d]);
    a.xi_out[d] = fa(*xb[xn], ws->xsz[d]);
  }
  s.p = 1 - s.p;
  s.k = 1 - s.k;
  s.d = dn;
  s.x = xn;
  // the second d / xi buffers exist for 2D simulations only
  bool ok = a.din.p && a.dout.p;
  for (int d = 0; d < ws->N; ++d) ok = ok && a.xi_in[d].p && a.xi_out[d].p;
  if (!ok) fail(SW_ERR_CUDA, "internal error: state buffer missing for this launch");
}

PairArgs pair_args(sw_wavesim* ws, int it1) {
  PairArgs b;
  std::memset(&b, 0, sizeof(b));
  for (int d = 0; d < 2; ++d) {
    b.psi_mid[d] = fa(ws->psim[d], ws->psz[d]);
    b.xi_mid[d] = fa(ws->xim[d], ws->xsz[d]);
  }
  b.shots = ws->d_pair.as<PairShot>();
  b.ids = ws->d_ids.as<int>();
  b.it1 = it1;
  return b;
}

// Forward of one group: all shots step together.  Gradient mode (grad = true)
// also writes checkpoints and the top-segment D.  Consecutive steps run as one
// two-step launch where nothing happens between them (see k_ac2d_pair).
void forward_group(sw_wavesim* ws, const std::vector<HostShot>& group, bool grad) {
  const int S = (int)group.size();
  cudaStream_t st = ws->ctx->stream;
  zero_state(ws, S, false);
  const int max_nt = group.front().nt;
  const int K = grad ? ws->gp.check_freq : 0;
  const long long F = ws->F;
  const bool bf16 = grad && ws->gp.snapshot_bf16 == 2;
  const long long slot = bf16 ? ws->strip_total : 2 * F + ws->strip_total;
  FwdState sta;
  Launcher L{ws, st};
  // D(it-1) is kept at step it by shots >= d_first: every shot when K == 1,
  // else the shots whose top segment (after their last checkpoint) holds it-1
  auto d_first_of = [&](int it, int Sa) {
    if (K == 1) return 0;
    for (int k = 0; k < Sa; ++k)
      if (it - 1 >= group[k].nt / K * K) return k;
    return Sa;
  };
  auto dslot_of = [&](int it) -> long long { return K == 1 ? it - 1 : (it - 1) % K; };
  const bool snap = !grad && ws->snapevery > 0;
  for (int it = 1; it <= max_nt;) {
    const int Sa = active_count(group, it);
    const int d_first = grad ? d_first_of(it, Sa) : Sa;
    // two steps (it, it+1) when state `it` needs no checkpoint or snapshot and
    // the active shots and D writers stay the same
    bool two = ws->pair_ok && it + 1 <= max_nt && active_count(group, it + 1) == Sa &&
               !(snap && it % ws->snapevery == 0);
    if (two && grad) two = !(K > 1 && it % K == 0) && d_first_of(it + 1, Sa) == d_first;
    const StepCtx c = two ? make_pair_ctx(ws, Sa) : ws->precision == 1 ? make_hp_ctx(ws, Sa) : make_step_ctx(ws, Sa);
    StepArgs a = base_args(ws, c, Sa);
    set_io(ws, a, sta, two, false);
    int ck_slot = -1;
    bool ckpt = false;
    if (grad) {
      // checkpoint m = (it-1)/K holds the state (p, d, psi, xi) after step mK
      if (K > 1 && (it - 1) % K == 0 && (it - 1) / K >= 1) {
        const int m = (it - 1) / K;
        float* base = ws->ck.as<float>() + (long long)(m - 1) * slot;
        const long long sstride = ws->ck_slots * slot;
        long long off = 0;
        if (bf16) {  // p and d go to the FP32 stage, packed to BF16 after the step
          a.ck_p = FieldArg{ws->ck_stage.as<float>(), 2 * F};
          a.ck_d = FieldArg{ws->ck_stage.as<float>() + F, 2 * F};
          ck_slot = m - 1;
        } else {
          a.ck_p = FieldArg{base, sstride};
          a.ck_d = FieldArg{base + F, sstride};
          off = 2 * F;
        }
        for (int d = 0; d < ws->N; ++d) { a.ck_psi[d] = FieldArg{base + off, sstride}; off += ws->psz[d]; }
        for (int d = 0; d < ws->N; ++d) { a.ck_xi[d] = FieldArg{base + off, sstride}; off += ws->xsz[d]; }
        ckpt = true;
      }
      a.Dout = dslot_arg(ws, dslot_of(it));
      a.d_first = d_first;
    }
    const int n_dwrite = grad ? Sa - d_first : 0;
    if (two) {
      PairArgs b = pair_args(ws, it);
      b.Dout2 = grad ? dslot_arg(ws, dslot_of(it + 1)) : FieldArg{nullptr, 0};
      b.stash = FieldArg{ws->d_stash.as<float>(), (long long)PAIR_MAXRR * ws->P};
      const double bytes = pair_bytes(ws, Sa, n_dwrite, ckpt);
      if (grad)
        L.pair<MODE_FWD_D>(a, b, bytes);
      else
        L.pair<MODE_FWD>(a, b, bytes);
      launch_inject(ws, Sa, a.pnew, a.dout, grad ? b.Dout2 : FieldArg{nullptr, 0}, d_first, it + 1, 1, it);
    } else {
      double bytes = stencil_bytes(ws, Sa, grad ? MODE_FWD_D : MODE_FWD, n_dwrite, ckpt);
      if (ws->precision == 1) bytes += hp_extra_bytes(ws, Sa);
      // steps before the top segment write no D: the plain forward kernel does the same work
      // without the D store path
      if (grad && n_dwrite > 0)
        L.step<MODE_FWD_D>(a, c, bytes);
      else
        L.step<MODE_FWD>(a, c, bytes);
      launch_inject(ws, Sa, a.pnew, a.dout, grad ? a.Dout : FieldArg{nullptr, 0}, d_first, it, 1, 0, a.plo_new,
                    a.dlo);
    }
    if (ck_slot >= 0) pack_checkpoint(ws, Sa, ck_slot);
    const int it_end = two ? it + 1 : it;
    if (snap && it_end % ws->snapevery == 0) {
      // savesnapshot!("pcur" => p[it]): unpadded copy into the caller's buffer of each active shot
      const long long rows = (long long)ws->n[1] * (ws->N == 3 ? ws->n[2] : 1);
      for (int k = 0; k < Sa; ++k) {
        float* dst = ws->snap_out[group[k].orig] + (long long)(it_end / ws->snapevery - 1) * ws->npts;
        check_cuda(cudaMemcpy2DAsync(dst, (size_t)ws->n[0] * sizeof(float), a.pnew.p + (long long)k * a.pnew.s,
                                     (size_t)ws->P * sizeof(float), (size_t)ws->n[0] * sizeof(float), (size_t)rows,
                                     cudaMemcpyDefault, st),
                   "snapshot copy");
      }
    }
    it = it_end + 1;
  }
}

void adjoint_group(sw_wavesim* ws, const std::vector<HostShot>& group) {
  const int S = (int)group.size();
  cudaStream_t st = ws->ctx->stream;
  const int max_nt = group.front().nt;
  const int K = ws->gp.check_freq;
  const long long F = ws->F;
  const bool bf16 = ws->gp.snapshot_bf16 == 2;
  const long long slot = bf16 ? ws->strip_total : 2 * F + ws->strip_total;
  Launcher L{ws, st};
  zero_state(ws, S, true);
  check_cuda(cudaMemsetAsync(ws->g.p, 0, (size_t)S * F * sizeof(float), st), "reset g");
  check_cuda(cudaMemsetAsync(ws->gc.p, 0, (size_t)S * F * sizeof(float), st), "reset gc");
  if (ws->adjw) check_cuda(cudaMemsetAsync(ws->tot64.p, 0, (size_t)F * sizeof(double), st), "reset total");
  FwdState ast;  // adjoint state buffers (p = lambda, d, psi, xi), as the forward's
  for (int it = max_nt; it >= 1;) {
    const int Sa = active_count(group, it);
    if (K > 1 && it % K == 0) {
      // recover segment m: forward steps (m-1)K+1 .. mK from the checkpoint at (m-1)K
      const int m = it / K;
      const StepCtx c = make_step_ctx(ws, Sa, TZ_RECOMPUTE);
      float* cbase;
      long long cstride;
      if (m - 1 >= 1) {
        cbase = ws->ck.as<float>() + (long long)(m - 2) * slot;
        cstride = ws->ck_slots * slot;
      } else {
        cbase = ws->zero.as<float>();
        cstride = 0;
      }
      FieldArg ck_p{cbase, cstride}, ck_d{cbase + F, cstride}, ck_psi[3], ck_xi[3];
      long long off = 2 * F;
      if (bf16 && m - 1 >= 1) {  // expand the BF16 (p, d) into the FP32 stage; strips stay in the slot
        unpack_checkpoint(ws, Sa, m - 2);
        ck_p = FieldArg{ws->ck_stage.as<float>(), 2 * F};
        ck_d = FieldArg{ws->ck_stage.as<float>() + F, 2 * F};
        off = 0;
      }
      for (int d = 0; d < ws->N; ++d) { ck_psi[d] = FieldArg{cbase + off, cstride}; off += ws->psz[d]; }
      for (int d = 0; d < ws->N; ++d) { ck_xi[d] = FieldArg{cbase + off, cstride}; off += ws->xsz[d]; }
      // the first launch reads the checkpoint and writes p / psi buffers 0 and
      // d / xi buffer 0 (one step, in place) or 1 (two steps; 2D only)
      FwdState rs{1, 0, 1, 0};
      const StepCtx cp2 = make_pair_ctx(ws, Sa);
      for (int t = (m - 1) * K + 1; t <= m * K;) {
        const bool first = t == (m - 1) * K + 1;
        const bool two = ws->pair_ok && t + 1 <= m * K;
        StepArgs a = base_args(ws, two ? cp2 : c, Sa);
        set_io(ws, a, rs, two, false);
        if (first) {
          a.pcur = ck_p;
          a.din = ck_d;
          for (int d = 0; d < ws->N; ++d) {
            a.psi_in[d] = ck_psi[d];
            a.xi_in[d] = ck_xi[d];
          }
        }
        a.Dout = dslot_arg(ws, (t - 1) % K);
        a.d_first = 0;
        if (two) {
          PairArgs b = pair_args(ws, t);
          b.Dout2 = dslot_arg(ws, t % K);
          L.pair<MODE_FWD_D>(a, b, pair_bytes(ws, Sa, Sa, false), true);
          launch_inject(ws, Sa, a.pnew, a.dout, b.Dout2, 0, t + 1, 0);
          t += 2;
        } else {
          L.step<MODE_FWD_D>(a, c, stencil_bytes(ws, Sa, MODE_FWD_D, Sa, false), true);
          launch_inject(ws, Sa, a.pnew, a.dout, a.Dout, 0, t, 0);
          t += 1;
        }
      }
    }
    // adjoint step it with the fused correlation against D(it-1); two steps
    // (it, it-1) in one launch when no recompute and no flush of the FP32 sums
    // falls between them and the active shots stay the same
    const bool two = ws->pair_adj_ok && ws->adjw && it - 1 >= 1 && active_count(group, it - 1) == Sa &&
                     !(K > 1 && (it - 1) % K == 0) && (it - 1) % 32 != 0;
    const StepCtx c = two ? make_pair_ctx(ws, Sa) : make_step_ctx(ws, Sa, TZ_ADJOINT);
    StepArgs a = base_args(ws, c, Sa);
    set_io(ws, a, ast, two, true);
    const long long dslot = K == 1 ? it - 1 : (it - 1) % K;
    a.dcorr = dslot_arg(ws, dslot);
    a.g = fa(ws->g, F);
    a.gc = ws->adjw ? FieldArg{nullptr, 0} : fa(ws->gc, F);
    FieldArg dcorr_last = a.dcorr;  // the D of the step whose injection follows
    if (two) {
      PairArgs b = pair_args(ws, it);
      b.dcorr2 = dslot_arg(ws, K == 1 ? it - 2 : (it - 2) % K);
      b.ptr = ws->d_ptr.as<int>();
      b.amap = ws->d_amap.as<int>();
      L.pair<MODE_ADJW>(a, b, pair_bytes(ws, Sa, 0, false, true));
      dcorr_last = b.dcorr2;
    } else if (ws->adjw) {
      L.step<MODE_ADJW>(a, c, stencil_bytes(ws, Sa, MODE_ADJW, 0, false));
    } else if (ws->grp == 4) {
      // 4 shots per block (one per warp) over 128-wide tiles; the correlation is
      // summed over the group before its single Kahan update
      StepArgs b = a;
      b.tiles_x = (int)((ws->P + 127) / 128);
      const int ngrp = (Sa + 3) / 4;
      const long long blocks = (long long)ngrp * b.tiles_x * b.tiles_z;
      check_vector_alignment(b);
      cudaEvent_t ev0 = nullptr;
      ws->ctx->prof.begin(st, KK_ADJOINT, stencil_bytes(ws, Sa, MODE_ADJ, 0, false, ngrp), &ev0);
      if (ws->variant & 8)
        k_ac2d_adj_grp<5><<<(unsigned)blocks, 128, 0, st>>>(b);
      else
        k_ac2d_adj_grp<4><<<(unsigned)blocks, 128, 0, st>>>(b);
      check_cuda(cudaGetLastError(), "adjoint stencil launch");
      ws->ctx->prof.end(st, KK_ADJOINT, ev0);
    } else {
      L.step<MODE_ADJ>(a, c, stencil_bytes(ws, Sa, MODE_ADJ, 0, false));
    }
    const int it_last = two ? it - 1 : it;  // the step whose adjoint sources are injected now
    cudaEvent_t ev = nullptr;
    ws->ctx->prof.begin(st, KK_SRCREC, 0.0, &ev);
    k_adj_inject<<<(Sa + ws->grp - 1) / ws->grp, 128, 0, st>>>(
        ws->d_desc.as<ShotDesc>(), ws->d_pts.as<long long>(), ws->d_ptr.as<int>(), ws->d_ids.as<int>(),
        ws->d_bslot.as<int>(), a.pnew, a.dout, dcorr_last, a.g, a.gc, it_last, Sa, ws->grp, a.dbf16,
        dexp_for(ws, dcorr_last), ws->P);
    check_cuda(cudaGetLastError(), "adjoint inject launch");
    ws->ctx->prof.end(st, KK_SRCREC, ev);
    if (ws->adjw && (it_last - 1) % 32 == 0) {  // at most 32 terms per FP32 sum
      ws->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
      const long long blocks = std::min<long long>((F / 4 + 255) / 256, 8192);
      k_flush_grad<<<(unsigned)blocks, 256, 0, st>>>(ws->g.as<float>(), F, S, ws->tot64.as<double>());
      check_cuda(cudaGetLastError(), "gradient flush launch");
      check_cuda(cudaMemsetAsync(ws->g.p, 0, (size_t)S * F * sizeof(float), st), "gradient sums clear");
      ws->ctx->prof.end(st, KK_OTHER, ev);
    }
    it = it_last - 1;
  }
}

std::vector<std::vector<HostShot>> plan_groups(sw_wavesim* ws, const std::vector<HostShot>& order, bool grad) {
  size_t free_b = 0, total_b = 0;
  check_cuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
  // keep the buffers already allocated in the budget
  const double budget = 0.85 * (double)(free_b + owned_bytes(ws));
  std::vector<std::vector<HostShot>> groups;
  size_t i = 0;
  while (i < order.size()) {
    const int max_nt = order[i].nt;  // sorted descending: the first of a group is the longest
    const size_t per = per_shot_bytes(ws, grad, max_nt);
    size_t cnt = (size_t)std::max(1.0, std::floor(budget / (double)per));
    cnt = std::min(cnt, order.size() - i);
    groups.emplace_back(order.begin() + i, order.begin() + i + cnt);
    i += cnt;
  }
  return groups;
}

std::vector<HostShot> sorted_order(int nshots, const sw_acoustic_shot* shots) {
  std::vector<HostShot> order(nshots);
  for (int k = 0; k < nshots; ++k) order[k] = HostShot{k, shots[k].nt};
  std::stable_sort(order.begin(), order.end(), [](const HostShot& a, const HostShot& b) { return a.nt > b.nt; });
  return order;
}

}  // namespace

// ---------------------------------------------------------------------------
// Entry points used by api.cu
// ---------------------------------------------------------------------------
namespace swgb {

// Raised by kernels whose bounded waits gave up: report it and re-arm the flag.
void check_timeout(sw_wavesim* ws) {
  int flag = 0;
  check_cuda(cudaMemcpy(&flag, ws->ctx->err.p, sizeof(int), cudaMemcpyDeviceToHost), "error flag");
  if (flag) {
    check_cuda(cudaMemset(ws->ctx->err.p, 0, sizeof(int)), "error flag");
    fail(SW_ERR_TIMEOUT, "a device-side wait on a data pipeline stage timed out");
  }
}

void wavesim_init(sw_wavesim* ws, sw_ctx* ctx, const sw_acoustic_params* p, int gradient, const sw_grad_params* gp) {
  if (!p) fail(SW_ERR_ARG, "params is NULL");
  if (p->ndim != 2 && p->ndim != 3) fail(SW_ERR_ARG, "Only 2D and 3D acoustic simulations are supported");
  if (p->halo < 0) fail(SW_ERR_ARG, "CPML halo size must be non-negative!");
  if (!(p->dt > 0)) fail(SW_ERR_ARG, "Timestep size must be positive!");
  for (int d = 0; d < p->ndim; ++d) {
    if (p->n[d] <= 0) fail(SW_ERR_ARG, "All numbers of grid points must be positive!");
    if (!(p->h[d] > 0)) fail(SW_ERR_ARG, "All grid spacings must be positive!");
    const bool cpml_axis = !(p->freetop && d == p->ndim - 1);
    if (cpml_axis && p->n[d] < 2 * p->halo + 3) {
      std::ostringstream os;
      os << "Number grid points in the dimensions with C-PML boundaries must be at least 2*halo+3 = "
         << 2 * p->halo + 3 << "!";
      fail(SW_ERR_ARG, os.str());
    }
    if (!cpml_axis && p->n[d] < 2 * p->halo + 3) {
      std::ostringstream os;
      os << "the free-surface axis needs at least 2*halo+3 = " << 2 * p->halo + 3
         << " grid points in this backend (its two damping strips must not overlap)";
      fail(SW_ERR_UNSUPPORTED, os.str());
    }
  }
  ws->ctx = ctx;
  if (!ctx->err.p) dev_alloc(ctx->err, sizeof(int), "error flag", ctx->stream);
  ws->prm = *p;
  ws->gradient = gradient != 0;
  if (ws->gradient) {
    ws->gp = gp ? *gp : sw_grad_params{1, 0, 0, 0, 0};
    if (ws->gp.check_freq < 1) fail(SW_ERR_ARG, "check_freq must be positive");
    if (ws->gp.mute_radius_src < 0 || ws->gp.mute_radius_rec < 0)
      fail(SW_ERR_ARG, "mutearoundpoint!(): The smoothing radius must be positive.");
    if (ws->gp.snapshot_bf16 < 0 || ws->gp.snapshot_bf16 > 3) fail(SW_ERR_ARG, "snapshot_bf16 must be 0, 1, 2 or 3");
    if (ws->gp.snapshot_bf16 == 3 && p->ndim != 3)
      fail(SW_ERR_UNSUPPORTED, "snapshot_bf16 = 3 (FP16 recompute buffer) is available for 3D simulations");
  }
  ws->N = p->ndim;
  for (int d = 0; d < 3; ++d) ws->n[d] = d < p->ndim ? p->n[d] : 1;
  ws->P = (int)round_up(ws->n[0], 32);
  ws->F = (long long)ws->P * ws->n[1] * (ws->N == 3 ? ws->n[2] : 1);
  ws->npts = (long long)ws->n[0] * ws->n[1] * (ws->N == 3 ? ws->n[2] : 1);
  const int H = p->halo;
  ws->strip_total = 0;
  for (int d = 0; d < ws->N; ++d) {
    long long ps = 1, xs = 1;
    for (int e = 0; e < ws->N; ++e) {
      const long long ext = e == 0 ? ws->P : ws->n[e];
      ps *= e == d ? 2 * H : ext;
      xs *= e == d ? 2 * H + 2 : ext;
    }
    // multiples of 32 floats keep every array that follows in a checkpoint slot
    // 128-byte aligned (the stencil moves p and d with 16-byte vector accesses)
    ws->psz[d] = round_up(std::max<long long>(ps, 1), 32);
    ws->xsz[d] = round_up(std::max<long long>(xs, 1), 32);
    ws->strip_total += ws->psz[d] + ws->xsz[d];
  }
  dev_alloc(ws->vp, (size_t)ws->npts * sizeof(float), "vp", ws->ctx->stream);
  dev_alloc(ws->fact, (size_t)ws->F * sizeof(float), "fact", ws->ctx->stream);
}

void wavesim_set_vp(sw_wavesim* ws, const float* vp, bool on_device) {
  if (!vp) fail(SW_ERR_ARG, "vp is NULL");
  cudaStream_t st = ws->ctx->stream;
  if (!on_device) {
    for (long long c = 0; c < ws->npts; ++c)
      if (!(vp[c] > 0)) fail(SW_ERR_ARG, "Pressure velocity material property must be positive!");
  }
  check_cuda(cudaMemcpyAsync(ws->vp.p, vp, ws->npts * sizeof(float),
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st),
             "vp upload");
  ws->vp64.release();  // the FP32 values are the model now
  const double dt = ws->prm.dt;
  cudaEvent_t ev = nullptr;
  ws->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
  k_set_fact<<<std::min<long long>((ws->npts + 255) / 256, 4096), 256, 0, st>>>(
      ws->vp.as<float>(), ws->n[0], ws->npts, ws->P, dt * dt, ws->fact.as<float>(),
      ws->precision == 1 ? ws->fact_lo.as<float>() : nullptr);
  check_cuda(cudaGetLastError(), "fact launch");
  ws->ctx->prof.end(st, KK_OTHER, ev);
  ws->has_vp = true;
}

void launch_fact64(sw_wavesim* ws) {
  cudaStream_t st = ws->ctx->stream;
  cudaEvent_t ev = nullptr;
  ws->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
  k_set_fact64<<<std::min<long long>((ws->npts + 255) / 256, 4096), 256, 0, st>>>(
      ws->vp64.as<double>(), ws->n[0], ws->npts, ws->P, ws->prm.dt * ws->prm.dt, ws->vp.as<float>(),
      ws->fact.as<float>(), ws->precision == 1 ? ws->fact_lo.as<float>() : nullptr);
  check_cuda(cudaGetLastError(), "fact launch");
  ws->ctx->prof.end(st, KK_OTHER, ev);
}

void wavesim_set_vp64(sw_wavesim* ws, const double* vp, bool on_device) {
  if (!vp) fail(SW_ERR_ARG, "vp is NULL");
  cudaStream_t st = ws->ctx->stream;
  if (!on_device) {
    for (long long c = 0; c < ws->npts; ++c)
      if (!(vp[c] > 0)) fail(SW_ERR_ARG, "Pressure velocity material property must be positive!");
  }
  if (!ws->vp64.p) dev_alloc(ws->vp64, (size_t)ws->npts * sizeof(double), "vp (FP64)", st);
  check_cuda(cudaMemcpyAsync(ws->vp64.p, vp, ws->npts * sizeof(double),
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st),
             "vp upload");
  launch_fact64(ws);
  ws->has_vp = true;
}

void acoustic_forward(sw_wavesim* ws, int nshots, const sw_acoustic_shot* shots, bool on_device) {
  if (!ws->has_vp) fail(SW_ERR_STATE, "material properties not set (sw_wavesim_set_vp)");
  if (nshots < 1 || !shots) fail(SW_ERR_ARG, "no shots");
  for (int k = 0; k < nshots; ++k) validate_shot(ws, shots[k], k, false);
  const std::vector<HostShot> order = sorted_order(nshots, shots);
  for (const auto& group : plan_groups(ws, order, false)) {
    ensure_state(ws, (int)group.size(), false, group.front().nt);
    Tables T;
    build_tables(ws, shots, group, on_device, false, T);
    if (ws->snapevery > 0)
      forward_group(ws, group, false);  // host copies inside the loop: no graph
    else
      run_graph(ws, group_key(ws, group, false), [&] { forward_group(ws, group, false); });
    download_traces(ws, shots, group, on_device);
  }
  check_cuda(cudaStreamSynchronize(ws->ctx->stream), "forward");
  check_timeout(ws);
  ws->ctx->prof.resolve();
}

void acoustic_forward_snapshots(sw_wavesim* ws, int nshots, const sw_acoustic_shot* shots, bool on_device,
                                int snapevery, float* const* snapshots) {
  if (snapevery < 1 || !snapshots) fail(SW_ERR_ARG, "snapevery must be positive and snapshots non-NULL");
  for (int k = 0; k < nshots; ++k) {
    if (shots && snapevery >= shots[k].nt)
      fail(SW_ERR_ARG, "Checkpointing frequency must be smaller than the number of timesteps!");
    if (!snapshots[k]) fail(SW_ERR_ARG, "snapshot buffer is NULL");
  }
  ws->snapevery = snapevery;
  ws->snap_out = snapshots;
  try {
    acoustic_forward(ws, nshots, shots, on_device);
  } catch (...) {
    ws->snapevery = 0;
    ws->snap_out = nullptr;
    throw;
  }
  ws->snapevery = 0;
  ws->snap_out = nullptr;
}

void acoustic_gradient(sw_wavesim* ws, int nshots, const sw_acoustic_shot* shots, bool on_device, double* grad,
                       double* misfit) {
  if (!ws->gradient) fail(SW_ERR_STATE, "The wavesim object was not built for gradient computations.");
  if (!ws->has_vp) fail(SW_ERR_STATE, "material properties not set (sw_wavesim_set_vp)");
  if (nshots < 1 || !shots) fail(SW_ERR_ARG, "no shots");
  if (!grad) fail(SW_ERR_ARG, "grad output is NULL");
  for (int k = 0; k < nshots; ++k) validate_shot(ws, shots[k], k, true);
  const bool mute = ws->gp.mute_radius_src > 0 || ws->gp.mute_radius_rec > 0;
  if (mute)
    for (int k = 0; k < nshots; ++k) {
      const sw_acoustic_shot& s = shots[k];
      if ((ws->gp.mute_radius_src > 0 && !s.src_pos) || (ws->gp.mute_radius_rec > 0 && !s.rec_pos))
        fail(SW_ERR_ARG, "muting needs src_pos / rec_pos");
      auto chk = [&](const double* pos, int np) {
        for (int p = 0; p < np; ++p)
          for (int d = 0; d < ws->N; ++d) {
            const double x = pos[p + (long long)d * np], ext = ws->prm.h[d] * (ws->n[d] - 1);
            if (!(0.0 <= x && x <= ext)) fail(SW_ERR_ARG, "mutearoundpoint!(): The point lies outside the grid");
          }
      };
      if (ws->gp.mute_radius_src > 0) chk(s.src_pos, s.nsrc);
      if (ws->gp.mute_radius_rec > 0) chk(s.rec_pos, s.nrec);
    }
  cudaStream_t st = ws->ctx->stream;
  const std::vector<HostShot> order = sorted_order(nshots, shots);
  double* gout = grad;
  double* mout = misfit;
  if (!on_device) {
    ensure(ws, ws->d_gout, (size_t)ws->npts * sizeof(double), "gradient output");
    gout = ws->d_gout.as<double>();
  }
  if (!on_device || !mout) {
    ensure(ws, ws->d_mout, sizeof(double), "misfit output");
    mout = ws->d_mout.as<double>();
  }
  if (ws->gp.snapshot_bf16 >= 1 && ws->N == 2 && (ws->variant & 3) == 1)
    fail(SW_ERR_UNSUPPORTED, "BF16 snapshots are not available with the TMA stencil variant");
  // the shot sum is fused into the 2D adjoint for batches of 4 or more shots,
  // unless per-shot muting needs each shot's gradient
  ws->adjw = !mute && ws->N == 2 && (ws->variant & 3) != 1 && ws->adj_plain;
  ws->grp = (!ws->adjw && !mute && ws->N == 2 && (ws->variant & 3) != 1 && nshots >= 4) ? 4 : 1;
  const int nblk = 64;
  bool first_group = true;
  for (const auto& group : plan_groups(ws, order, true)) {
    const int S = (int)group.size();
    const int max_nt = group.front().nt;
    ensure_state(ws, S, true, max_nt);
    if (ws->adjw) ensure(ws, ws->tot64, (size_t)ws->F * sizeof(double), "gradient total");
    Tables T;
    build_tables(ws, shots, group, on_device, true, T);
    ensure(ws, ws->d_partial, (size_t)nblk * S * sizeof(double), "misfit partials");
    const bool accumulate = !first_group;
    bool any_dense = false;
    for (const auto& h : group) any_dense = any_dense || (shots[h.orig].invcov && shots[h.orig].misfit_kind == 0);
    size_t ccts_smem = 0;
    int ccts_rec = 0;
    {
      std::vector<int> kind(S), nt(S), nrec(S);
      std::vector<double> mdt(S);
      std::vector<const float*> tr(S), obs(S);
      std::vector<float*> adj(S);
      std::vector<const long long*> rl(S);
      for (int k = 0; k < S; ++k) {
        const sw_acoustic_shot& s = shots[group[k].orig];
        kind[k] = s.misfit_kind;
        mdt[k] = s.misfit_dt;
        nt[k] = T.desc[k].nt;
        nrec[k] = T.desc[k].nrec;
        tr[k] = T.desc[k].tr;
        obs[k] = T.desc[k].obs;
        adj[k] = T.desc[k].adj;
        rl[k] = ws->d_rec.as<long long>() + T.desc[k].rec_off;
      }
      ensure(ws, ws->d_ccts, (size_t)S * sizeof(CctsShot), "CCTS table");
      ccts_rec = upload_ccts(ws->ctx, ws->d_ccts.as<CctsShot>(), kind, mdt, nt, nrec, tr, obs, adj, rl, &ccts_smem);
      if (ccts_rec) ensure(ws, ws->d_partial2, (size_t)ccts_rec * S * sizeof(double), "CCTS partials");
    }
    auto misfit_and_adjsrc = [&] {
      cudaEvent_t ev = nullptr;
      if (any_dense) {  // C^-1 r of the shots with a dense inverse covariance (dense.cu)
        k_residual_dense<<<dim3(nblk, S), 256, 0, st>>>(ws->d_desc.as<ShotDesc>());
        check_cuda(cudaGetLastError(), "residual launch");
        for (int k = 0; k < S; ++k)
          if (T.desc[k].icd)
            dense_invcov(ws->ctx, T.desc[k].nt, T.desc[k].nrec, T.desc[k].icd, T.desc[k].resid,
                         const_cast<float*>(T.desc[k].cres));
      }
      ws->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
      k_misfit_adjsrc<<<dim3(nblk, S), 256, 0, st>>>(ws->d_desc.as<ShotDesc>(), ws->d_rec.as<long long>(),
                                                     ws->fact.as<float>(), ws->d_partial.as<double>());
      check_cuda(cudaGetLastError(), "misfit launch");
      ws->ctx->prof.end(st, KK_OTHER, ev);
      ws->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
      k_misfit_sum<<<1, 256, 0, st>>>(ws->d_partial.as<double>(), nblk, S, mout, accumulate ? 1 : 0);
      check_cuda(cudaGetLastError(), "misfit sum launch");
      if (ccts_rec) {
        k_ccts<<<dim3(ccts_rec, S), CCTS_THREADS, ccts_smem, st>>>(ws->d_ccts.as<CctsShot>(), ws->fact.as<float>(),
                                                                   ws->d_partial2.as<double>());
        check_cuda(cudaGetLastError(), "CCTS misfit launch");
        k_misfit_sum<<<1, 256, 0, st>>>(ws->d_partial2.as<double>(), ccts_rec, S, mout, 1);
        check_cuda(cudaGetLastError(), "CCTS misfit sum launch");
      }
      ws->ctx->prof.end(st, KK_OTHER, ev);
    };
    auto reduce = [&] {
      cudaEvent_t ev = nullptr;
      ws->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
      const long long blocks = std::min<long long>((ws->npts + 255) / 256, 8192);
      if (ws->adjw) {
        k_reduce_grad_tot<<<(unsigned)blocks, 256, 0, st>>>(ws->tot64.as<double>(), ws->vp.as<float>(), ws->n[0],
                                                            ws->npts, ws->P, 1.0 / (ws->prm.dt * ws->prm.dt), gout,
                                                            accumulate ? 1 : 0);
        check_cuda(cudaGetLastError(), "gradient reduction launch");
        ws->ctx->prof.end(st, KK_OTHER, ev);
        return;
      }
      k_reduce_grad<<<(unsigned)blocks, 256, 0, st>>>(ws->g.as<float>(), ws->gc.as<float>(), ws->F,
                                                      (S + ws->grp - 1) / ws->grp,
                                                      ws->vp.as<float>(), ws->n[0], ws->npts, ws->P,
                                                      1.0 / (ws->prm.dt * ws->prm.dt), gout, accumulate ? 1 : 0);
      check_cuda(cudaGetLastError(), "gradient reduction launch");
      ws->ctx->prof.end(st, KK_OTHER, ev);
    };
    if (!mute) {
      // the whole group -- forward, misfit (with the dense C^-1 products),
      // adjoint, shot sum -- as one graph
      std::vector<long long> key = group_key(ws, group, true);
      for (const auto& h : group) key.push_back(shots[h.orig].misfit_kind);
      for (int k = 0; k < S; ++k)  // the dense products' operands are launch arguments
        if (T.desc[k].icd) key.insert(key.end(), {k, T.desc[k].nrec, (long long)(uintptr_t)T.desc[k].icd});
      key.insert(key.end(), {accumulate ? 1 : 0, (long long)(uintptr_t)gout, (long long)(uintptr_t)mout});
      run_graph(ws, key, [&] {
        forward_group(ws, group, true);
        misfit_and_adjsrc();
        adjoint_group(ws, group);
        reduce();
      });
      download_traces(ws, shots, group, on_device);
      first_group = false;
      continue;
    }
    forward_group(ws, group, true);
    download_traces(ws, shots, group, on_device);
    misfit_and_adjsrc();
    adjoint_group(ws, group);
    {
      // sources first, then receivers, like the reference; rmax depends on the radius
      double hmax = 0;
      for (int d = 0; d < ws->N; ++d) hmax = std::max(hmax, ws->prm.h[d]);
      for (int fam = 0; fam < 2; ++fam) {
        const int radius = fam == 0 ? ws->gp.mute_radius_src : ws->gp.mute_radius_rec;
        if (radius <= 0) continue;
        std::vector<MutePoint> pts;
        std::vector<int> ptr(S + 1, 0);
        for (int k = 0; k < S; ++k) {
          const sw_acoustic_shot& s = shots[group[k].orig];
          const double* pos = fam == 0 ? s.src_pos : s.rec_pos;
          const int np = fam == 0 ? s.nsrc : s.nrec;
          for (int p = 0; p < np; ++p) {
            MutePoint m{};
            m.shot = k;
            for (int d = 0; d < ws->N; ++d) {
              const double x = pos[p + (long long)d * np], h = ws->prm.h[d];
              const int ijk = (int)std::round((x - std::fmod(x, h)) / h) + 1;  // floor(Int, div(x, h)) + 1
              m.lo[d] = ijk - radius;
              m.hi[d] = ijk + radius;
              m.pos[d] = x;
            }
            pts.push_back(m);
          }
          ptr[k + 1] = (int)pts.size();
        }
        upload(ws, ws->d_mute, pts, "mute points");
        upload(ws, ws->d_mute_ptr, ptr, "mute csr");
        cudaEvent_t ev = nullptr;
        ws->ctx->prof.begin(st, KK_OTHER, 0.0, &ev);
        k_mute<<<S, 256, 0, st>>>(ws->d_mute.as<MutePoint>(), ws->d_mute_ptr.as<int>(), ws->N, ws->n[0], ws->n[1],
                                  ws->n[2], ws->P, ws->prm.h[0], ws->prm.h[1], ws->prm.h[2], radius * hmax,
                                  fa(ws->g, ws->F), fa(ws->gc, ws->F));
        check_cuda(cudaGetLastError(), "mute launch");
        ws->ctx->prof.end(st, KK_OTHER, ev);
        check_cuda(cudaStreamSynchronize(st), "mute");
      }
    }
    reduce();
    first_group = false;
  }
  if (!on_device) {
    check_cuda(cudaMemcpyAsync(grad, gout, ws->npts * sizeof(double), cudaMemcpyDeviceToHost, st), "grad download");
    if (misfit) check_cuda(cudaMemcpyAsync(misfit, mout, sizeof(double), cudaMemcpyDeviceToHost, st), "misfit download");
  }
  check_cuda(cudaStreamSynchronize(st), "gradient");
  check_timeout(ws);
  ws->ctx->prof.resolve();
}

void wavesim_set_tuning(sw_wavesim* ws, int tz, int variant) {
  ws->tile_tz = tz;
  ws->variant = variant % 16;
  ws->pf = (variant / 16) % 16;
  ws->adj_plain = (variant & 256) == 0;
  ws->cpa = (variant & 512) != 0;
  ws->pair_on = (variant & 1024) != 0;
  static const int pair_tz[8] = {0, 8, 16, 32, 64, 128, 4, 0};
  ws->pair_tz = pair_tz[(variant >> 11) & 7];
  ws->pair_occ = (variant >> 14) & 3;
  ws->split3d = (variant & 65536) == 0;
  ws->inner_np = (variant & 131072) != 0;
  ws->xsplit = (variant & 262144) == 0;
}
void wavesim_set_band_heights(sw_wavesim* ws, int tz_forward, int tz_recompute, int tz_adjoint) {
  ws->kind_tz[TZ_FORWARD] = tz_forward;
  ws->kind_tz[TZ_RECOMPUTE] = tz_recompute;
  ws->kind_tz[TZ_ADJOINT] = tz_adjoint;
}
void wavesim_set_precision(sw_wavesim* ws, int mode) {
  if (mode == ws->precision) return;
  ws->precision = mode;
  ws->drop_graphs();
  if (mode == 1 && !ws->fact_lo.p) {
    cudaStream_t st = ws->ctx->stream;
    dev_alloc(ws->fact_lo, (size_t)ws->F * sizeof(float), "fact low part", st);
    check_cuda(cudaMemsetAsync(ws->fact_lo.p, 0, (size_t)ws->F * sizeof(float), st), "fact low part");
    if (ws->has_vp && ws->vp64.p) {
      launch_fact64(ws);
    } else if (ws->has_vp) {
      k_set_fact<<<std::min<long long>((ws->npts + 255) / 256, 4096), 256, 0, st>>>(
          ws->vp.as<float>(), ws->n[0], ws->npts, ws->P, ws->prm.dt * ws->prm.dt, ws->fact.as<float>(),
          ws->fact_lo.as<float>());
      check_cuda(cudaGetLastError(), "fact launch");
    }
    check_cuda(cudaStreamSynchronize(st), "set precision");
  }
}
void wavesim_set_wait_test(sw_wavesim* ws, long long wait_cycles, int withhold) {
  ws->wait_cycles = wait_cycles;
  ws->withhold = withhold;
}
void wavesim_use_graphs(sw_wavesim* ws, bool on) {
  ws->use_graphs = on;
  if (!on) ws->drop_graphs();
}
sw_ctx* wavesim_ctx(sw_wavesim* ws) { return ws->ctx; }
sw_wavesim* wavesim_new() { return new sw_wavesim(); }
void wavesim_delete(sw_wavesim* ws) { delete ws; }

}  // namespace swgb
