// SPDX-License-Identifier: MIT
//
// TEST INFRASTRUCTURE ONLY -- the CPU oracle for the swgb300 acoustic path.
//
// This file restates, in plain C++ (FP64 and FP32 instantiations, OpenMP over
// the slowest axis), the algorithm SeismicWaves.jl v0.9.0 runs for the
// acoustic constant-density C-PML simulation.  It is used by the test suite
// as the checker and by bench.py as the timed CPU baseline.  Nothing in the
// product path links or calls it.
//
// What it follows (paths relative to the SeismicWaves.jl source tree):
//   C-PML coefficients ........ src/models/cpmlcoeffs.jl:18-100,
//                               src/models/acoustic/acou_init_bc.jl:7-40
//   psi strips ................ src/models/acoustic/backends/shared/acoustic2D_xPU.jl:1-25,
//                               acoustic3D_xPU.jl:1-38, via src/utils/fdgen.jl:137-161
//   pressure / xi update ...... acoustic2D_xPU.jl:27-46, acoustic3D_xPU.jl:40-61,
//                               via src/utils/fdgen.jl:163-215 (fdcoeffs(2,2) = [1,-2,1])
//   injection / recording ..... acoustic2D_xPU.jl:48-62, acoustic3D_xPU.jl:63-79
//   residual prescaling ....... acoustic2D_xPU.jl:64-76
//   one step + buffer rotation  acoustic2D_xPU.jl:78-169, acoustic3D_xPU.jl:96-218
//   forward driver ............ src/models/acoustic/acou_forward.jl:22-62 (swforward_1shot!)
//   gradient driver ........... src/models/acoustic/acou_gradient.jl:4-95 (swgradient_1shot!, CD)
//   linear checkpointer ....... src/utils/checkpointers.jl:1-107
//   correlation ............... src/models/acoustic/backends/shared/correlate_gradient_xPU.jl:1-10
//   L2 misfit / adjoint source  src/inversion/misfits/L2Misfit.jl:24-77
//   gradient muting ........... src/utils/mute_grad.jl:13-80
//
// Parity status: the reference publishes no golden vectors and Julia is not
// available to run it, so this restatement is pinned by re-running the
// reference's own known-answer tests against it (analytical Green's
// functions, source/receiver reversal, checkpoint equivalence, misfit
// consistency) -- see tests/test_oracle_*.py.  Trace-level agreement with the
// Julia program itself is unpinned.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_common.h"

namespace {

using oracle::cpml_axis;
using oracle::LinearCheckpointer;
using oracle::mute_around_point;
using oracle::Snap;

// ---------------------------------------------------------------------------
// Acoustic constant-density simulation state, N = 2 or 3, element type T.
// Column-major (x fastest); all indices below are the reference's 1-based ones.
// ---------------------------------------------------------------------------
template <typename T>
struct AcousticSim {
  int N, halo, nthreads;
  int n[3];
  long st[3];        // strides of the grid
  T inv_h[3];        // _dx, _dy, _dz
  T inv_h2[3];       // _dx^2 ...
  long npts;
  std::vector<T> fact;
  // three rotating pressure buffers (pold, pcur, pnew roles by index)
  std::vector<T> buf[3];
  int iold = 0, icur = 1, inew = 2;
  std::vector<T> psi[3], xi[3];       // per axis
  long pst[3][3], xst[3][3];           // strides of psi_d / xi_d arrays
  std::vector<T> ca[3], cah[3], cb[3], cbh[3];  // C-PML coefficients per axis

  AcousticSim(int N_, const int* n_, const double* h, int halo_, int nthreads_)
      : N(N_), halo(halo_), nthreads(nthreads_) {
    for (int d = 0; d < 3; ++d) n[d] = d < N ? n_[d] : 1;
    st[0] = 1; st[1] = n[0]; st[2] = (long)n[0] * n[1];
    npts = (long)n[0] * n[1] * n[2];
    for (int d = 0; d < N; ++d) {
      inv_h[d] = (T)(1.0 / (T)h[d]);
      inv_h2[d] = inv_h[d] * inv_h[d];
    }
    fact.assign(npts, T(0));
    for (auto& b : buf) b.assign(npts, T(0));
    for (int d = 0; d < N; ++d) {
      int dp[3], dx[3];
      for (int e = 0; e < 3; ++e) { dp[e] = n[e]; dx[e] = n[e]; }
      dp[d] = 2 * halo; dx[d] = 2 * (halo + 1);
      pst[d][0] = 1; pst[d][1] = dp[0]; pst[d][2] = (long)dp[0] * dp[1];
      xst[d][0] = 1; xst[d][1] = dx[0]; xst[d][2] = (long)dx[0] * dx[1];
      psi[d].assign((long)dp[0] * dp[1] * dp[2], T(0));
      xi[d].assign((long)dx[0] * dx[1] * dx[2], T(0));
    }
  }

  void set_cpml(int d, const double* blk) {
    const int na = 2 * (halo + 1), nh = 2 * halo;
    ca[d].assign(na, 0); cah[d].assign(nh, 0); cb[d].assign(na, 0); cbh[d].assign(nh, 0);
    for (int k = 0; k < na; ++k) { ca[d][k] = (T)blk[k]; cb[d][k] = (T)blk[na + nh + k]; }
    for (int k = 0; k < nh; ++k) { cah[d][k] = (T)blk[na + k]; cbh[d][k] = (T)blk[2 * na + nh + k]; }
  }

  void reset_fields() {  // reset!(model.grid; except=["fact"])
    for (auto& b : buf) std::fill(b.begin(), b.end(), T(0));
    for (int d = 0; d < N; ++d) {
      std::fill(psi[d].begin(), psi[d].end(), T(0));
      std::fill(xi[d].begin(), xi[d].end(), T(0));
    }
    iold = 0; icur = 1; inew = 2;
  }

  inline long lin(const int* I) const {  // 1-based multi-index -> linear
    return (long)(I[0] - 1) + (long)(I[1] - 1) * st[1] + (long)(I[2] - 1) * st[2];
  }

  // update_psi_d!: acoustic2D_xPU.jl:1-25 via fdgen.jl:137-161 (halfgrid)
  void update_psi(int d) {
    const T* p = buf[icur].data();
    T* ps = psi[d].data();
    const T* a = cah[d].data();
    const T* b = cbh[d].data();
    const int nd = n[d];
    // iterate over all grid points with axis-d index in the strip range 1..2halo
    int lo[3] = {1, 1, 1}, hi[3] = {n[0], n[1], n[2]};
    lo[d] = 1; hi[d] = 2 * halo;
    const int outer = N - 1;  // parallelise over the slowest axis of the strip
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int io = lo[outer]; io <= hi[outer]; ++io) {
      int I[3];
      I[outer] = io;
      const int mlo = N == 3 ? lo[1] : 1, mhi = N == 3 ? hi[1] : 1;
      for (int im = mlo; im <= mhi; ++im) {
        if (N == 3) I[1] = im;
        for (int ix = lo[0]; ix <= hi[0]; ++ix) {
          I[0] = ix;
          if (N == 2) I[2] = 1;
          int J[3] = {I[0], I[1], I[2]};
          const int i = I[d];
          const int ii = i > halo ? nd - halo - 1 + (i - halo) : i;
          J[d] = ii;
          const long c = lin(J);
          // deriv 1, order 2 on the half grid: (-p[ii] + p[ii+1]) * _d
          const T dA = (T(-1) * p[c] + T(1) * p[c + st[d]]) * inv_h[d];
          int k;
          if (ii <= halo) {
            k = ii;
          } else if (ii >= nd - halo) {
            k = ii - (nd - halo) + 1 + halo;
          } else {
            continue;
          }
          int K[3] = {J[0], J[1], J[2]};
          K[d] = k;
          const long q = (long)(K[0] - 1) * pst[d][0] + (long)(K[1] - 1) * pst[d][1] + (long)(K[2] - 1) * pst[d][2];
          ps[q] = b[k - 1] * ps[q] + a[k - 1] * dA;
        }
      }
    }
  }

  // One axis term of the C-PML Laplacian, fdgen.jl:163-193
  inline T axis_term(int d, const T* p, const int* I, long c) {
    const int i = I[d];
    const int nd = n[d];
    const long s = st[d];
    const T d2 = (T(1) * p[c - s] + T(-2) * p[c] + T(1) * p[c + s]) * inv_h2[d];
    int k;
    if (i <= halo) {
      k = i;
    } else if (i >= nd - halo + 1) {
      k = i - (nd - halo) + 1 + halo;
    } else {
      return d2;
    }
    int K[3] = {I[0], I[1], I[2]};
    K[d] = k - 1;
    const long qp = (long)(K[0] - 1) * pst[d][0] + (long)(K[1] - 1) * pst[d][1] + (long)(K[2] - 1) * pst[d][2];
    const T dpsi = (T(-1) * psi[d][qp] + T(1) * psi[d][qp + pst[d][d]]) * inv_h[d];
    K[d] = k;
    const long qx = (long)(K[0] - 1) * xst[d][0] + (long)(K[1] - 1) * xst[d][1] + (long)(K[2] - 1) * xst[d][2];
    T& x = xi[d][qx];
    x = cb[d][k - 1] * x + ca[d][k - 1] * (d2 + dpsi);
    return d2 + dpsi + x;
  }

  // update_p_CPML!: acoustic2D_xPU.jl:27-46 / acoustic3D_xPU.jl:40-61
  void update_p() {
    const T* pc = buf[icur].data();
    const T* po = buf[iold].data();
    T* pn = buf[inew].data();
    const T* f = fact.data();
    const int outer = N - 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int io = 2; io <= n[outer] - 1; ++io) {
      int I[3] = {1, 1, 1};
      I[outer] = io;
      const int mlo = N == 3 ? 2 : 1, mhi = N == 3 ? n[1] - 1 : 1;
      for (int im = mlo; im <= mhi; ++im) {
        if (N == 3) I[1] = im;
        for (int ix = 2; ix <= n[0] - 1; ++ix) {
          I[0] = ix;
          const long c = lin(I);
          T lap = axis_term(0, pc, I, c);
          lap = lap + axis_term(1, pc, I, c);
          if (N == 3) lap = lap + axis_term(2, pc, I, c);
          pn[c] = T(2) * pc[c] - po[c] + f[c] * lap;
        }
      }
    }
  }

  // forward_onestep_CPML! (acoustic2D_xPU.jl:78-126): psi, p/xi, inject, record, rotate
  void step(int it, int nsrc, const long* src_lin, const T* srctf, int ntf,
            int nrec, const long* rec_lin, T* traces, int ntr) {
    for (int d = 0; d < N; ++d) update_psi(d);
    update_p();
    T* pn = buf[inew].data();
    for (int s = 0; s < nsrc; ++s) pn[src_lin[s]] += srctf[(long)(it - 1) + (long)s * ntf];
    if (traces)
      for (int r = 0; r < nrec; ++r) traces[(long)(it - 1) + (long)r * ntr] = pn[rec_lin[r]];
    // grid.fields["pold"] = pcur; pcur = pnew; pnew = pold (old pold buffer)
    const int o = iold;
    iold = icur; icur = inew; inew = o;
  }
};

// Field snapshot used by the checkpointer: p, or (psi_1..psi_N), or (xi_1..xi_N)
template <typename T>
struct ShotArgs {
  int nt, nsrc, nrec;
  std::vector<long> src_lin, rec_lin;
  std::vector<T> srctf;  // (nt, nsrc)
};

template <typename T>
void prepare_sim(AcousticSim<T>& sim, const double* vp, double dt, const double* cpml) {
  const long np = sim.npts;
  const T tdt = (T)dt;
  for (long c = 0; c < np; ++c) {
    const T v = (T)vp[c];
    sim.fact[c] = (tdt * tdt) * (v * v);  // precompute_fact!: dt^2 .* vp.^2
  }
  const int na = 2 * (sim.halo + 1), nh = 2 * sim.halo;
  for (int d = 0; d < sim.N; ++d) sim.set_cpml(d, cpml + (long)d * (2 * na + 2 * nh));
}

template <typename T>
Snap<T> snap_p(const AcousticSim<T>& s, int which) { return Snap<T>{s.buf[which]}; }

template <typename T>
int run_forward(int N, const int* n, const double* h, double dt, int halo, const double* vp,
                const double* cpml, int nt, int nsrc, const int* src_idx, const double* srctf,
                int nrec, const int* rec_idx, double* traces, int nthreads, int snapevery = 0,
                double* snaps = nullptr) {
  AcousticSim<T> sim(N, n, h, halo, nthreads);
  prepare_sim(sim, vp, dt, cpml);
  std::vector<long> sl(nsrc), rl(nrec);
  for (int s = 0; s < nsrc; ++s) {
    int I[3] = {1, 1, 1};
    for (int d = 0; d < N; ++d) I[d] = src_idx[s + (long)d * nsrc];
    sl[s] = sim.lin(I);
  }
  for (int r = 0; r < nrec; ++r) {
    int I[3] = {1, 1, 1};
    for (int d = 0; d < N; ++d) I[d] = rec_idx[r + (long)d * nrec];
    rl[r] = sim.lin(I);
  }
  std::vector<T> tf((long)nt * nsrc), tr((long)nt * nrec, T(0));
  for (long q = 0; q < (long)nt * nsrc; ++q) tf[q] = (T)srctf[q];
  sim.reset_fields();
  for (int it = 1; it <= nt; ++it) {
    sim.step(it, nsrc, sl.data(), tf.data(), nt, nrec, rl.data(), tr.data(), nt);
    // savesnapshot!("pcur" => p[it]) (acou_forward.jl:54-57, snapshotter.jl:35-41)
    if (snaps && snapevery > 0 && it % snapevery == 0) {
      double* o = snaps + (long)(it / snapevery - 1) * sim.npts;
      for (long c = 0; c < sim.npts; ++c) o[c] = (double)sim.buf[sim.icur][c];
    }
  }
  for (long q = 0; q < (long)nt * nrec; ++q) traces[q] = (double)tr[q];
  return 0;
}

template <typename T>
int run_gradient(int N, const int* n, const double* h, double dt, int halo, const double* vp,
                 const double* cpml, int nt, int nsrc, const int* src_idx, const double* srctf,
                 int nrec, const int* rec_idx, const double* observed, const double* invcov,
                 int invcov_kind, int nwin, const int* windows, int check_freq,
                 int mute_src, int mute_rec, const double* src_pos, const double* rec_pos,
                 double* traces_out, double* grad_out, double* misfit_out, int nthreads, int misfit_kind,
                 double misfit_dt) {
  if (check_freq < 1 || check_freq >= nt) return 1;  // LinearCheckpointer assertion
  AcousticSim<T> sim(N, n, h, halo, nthreads);
  prepare_sim(sim, vp, dt, cpml);
  AcousticSim<T> adj(N, n, h, halo, nthreads);
  adj.fact = sim.fact;
  for (int d = 0; d < N; ++d) { adj.ca[d] = sim.ca[d]; adj.cah[d] = sim.cah[d]; adj.cb[d] = sim.cb[d]; adj.cbh[d] = sim.cbh[d]; }
  std::vector<long> sl(nsrc), rl(nrec);
  for (int s = 0; s < nsrc; ++s) {
    int I[3] = {1, 1, 1};
    for (int d = 0; d < N; ++d) I[d] = src_idx[s + (long)d * nsrc];
    sl[s] = sim.lin(I);
  }
  for (int r = 0; r < nrec; ++r) {
    int I[3] = {1, 1, 1};
    for (int d = 0; d < N; ++d) I[d] = rec_idx[r + (long)d * nrec];
    rl[r] = sim.lin(I);
  }
  const long np = sim.npts;
  std::vector<T> tf((long)nt * nsrc), tr((long)nt * nrec, T(0));
  for (long q = 0; q < (long)nt * nsrc; ++q) tf[q] = (T)srctf[q];

  auto snap_psi = [&](AcousticSim<T>& s) { Snap<T> o; for (int d = 0; d < N; ++d) o.push_back(s.psi[d]); return o; };
  auto snap_xi = [&](AcousticSim<T>& s) { Snap<T> o; for (int d = 0; d < N; ++d) o.push_back(s.xi[d]); return o; };

  // acou_models.jl:159-173: checkpointer built with zero fields, -1 and 0 saved
  std::map<std::string, Snap<T>> proto;
  proto["pcur"] = snap_p(sim, sim.icur);
  proto["psi"] = snap_psi(sim);
  proto["xi"] = snap_xi(sim);
  LinearCheckpointer<T> ck(nt, check_freq, proto);
  ck.save("pcur", snap_p(sim, sim.iold), -1);
  ck.save("pcur", snap_p(sim, sim.icur), 0);
  ck.save("psi", snap_psi(sim), 0);
  ck.save("xi", snap_xi(sim), 0);

  // swgradient_1shot!: reset, forward with checkpoints
  sim.reset_fields();
  adj.reset_fields();
  ck.reset();
  std::vector<T> grad(np, T(0));
  for (int it = 1; it <= nt; ++it) {
    sim.step(it, nsrc, sl.data(), tf.data(), nt, nrec, rl.data(), tr.data(), nt);
    ck.save("pcur", snap_p(sim, sim.icur), it);
    ck.save("psi", snap_psi(sim), it);
    ck.save("xi", snap_xi(sim), it);
  }
  for (long q = 0; q < (long)nt * nrec; ++q) traces_out[q] = (double)tr[q];

  // residuals, window mask, C^-1 r (L2Misfit.jl:64-77), misfit (:24-42)
  std::vector<double> res((long)nt * nrec), cres((long)nt * nrec, 0.0);
  for (int r = 0; r < nrec; ++r)
    for (int t = 0; t < nt; ++t) {
      const long q = t + (long)r * nt;
      res[q] = (double)tr[q] - observed[q];
    }
  if (nwin > 0) {
    std::vector<double> mask(nt, 0.0);
    for (int w = 0; w < nwin; ++w)
      for (int t = windows[2 * w] - 1; t <= windows[2 * w + 1] - 1; ++t) mask[t] = 1.0;
    for (int r = 0; r < nrec; ++r)
      for (int t = 0; t < nt; ++t) res[t + (long)r * nt] *= mask[t];
  }
  for (int r = 0; r < nrec; ++r)
    for (int t = 0; t < nt; ++t) {
      const long q = t + (long)r * nt;
      if (invcov_kind == 0) cres[q] = res[q];
      else if (invcov_kind == 1) cres[q] = invcov[t] * res[q];
      else {
        double acc = 0;
        for (int u = 0; u < nt; ++u) acc += invcov[t + (long)u * nt] * res[u + (long)r * nt];
        cres[q] = acc;
      }
    }
  double msf = 0;
  for (long q = 0; q < (long)nt * nrec; ++q) msf += res[q] * cres[q];
  *misfit_out = msf / 2;
  if (misfit_kind == 1) {  // CCTSMisfit: dchi/du per trace instead
    std::vector<double> syn(nt);
    double m = 0.0;
    for (int r = 0; r < nrec; ++r) {
      for (int t = 0; t < nt; ++t) syn[t] = (double)tr[t + (long)r * nt];
      m += oracle::ccts_trace(observed + (long)r * nt, syn.data(), nt, misfit_dt, cres.data() + (long)r * nt);
    }
    *misfit_out = m;
  }

  // adjoint source = -dchi/du, prescaled by fact at the receivers (acoustic2D_xPU.jl:64-76)
  std::vector<T> adjsrc((long)nt * nrec);
  for (int r = 0; r < nrec; ++r)
    for (int t = 0; t < nt; ++t) {
      const long q = t + (long)r * nt;
      adjsrc[q] = (T)(-cres[q]);
      adjsrc[q] *= sim.fact[rl[r]];
    }

  const T _dt2 = (T)(T(1) / ((T)dt * (T)dt));
  for (int it = nt; it >= 1; --it) {
    // adjoint_onestep_CPML!: receivers act as sources of the adjoint field
    adj.step(it, nrec, rl.data(), adjsrc.data(), nt, 0, nullptr, nullptr, nt);
    if (!ck.issaved("pcur", it - 2)) {
      ck.initrecover();
      sim.buf[sim.iold] = ck.getsaved("pcur", ck.curr_checkpoint - 1)[0];
      sim.buf[sim.icur] = ck.getsaved("pcur", ck.curr_checkpoint)[0];
      const Snap<T>& ps = ck.getsaved("psi", ck.curr_checkpoint);
      const Snap<T>& xs = ck.getsaved("xi", ck.curr_checkpoint);
      for (int d = 0; d < N; ++d) { sim.psi[d] = ps[d]; sim.xi[d] = xs[d]; }
      const int start = ck.curr_checkpoint + 1, end = ck.curr_checkpoint + ck.K - 1;
      for (int rit = start; rit <= end; ++rit) {
        sim.step(rit, nsrc, sl.data(), tf.data(), nt, 0, nullptr, nullptr, nt);
        ck.buffer[rit - start + 1] = snap_p(sim, sim.icur);
      }
    }
    const std::vector<T>& p0 = ck.getsaved("pcur", it - 2)[0];
    const std::vector<T>& p1 = ck.getsaved("pcur", it - 1)[0];
    const std::vector<T>& p2 = ck.getsaved("pcur", it)[0];
    const T* lam = adj.buf[adj.icur].data();
    // correlate_gradient_kernel!: grad += adjcur * (pcur - 2 pold + pveryold) * _dt2
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (long c = 0; c < np; ++c)
      grad[c] = grad[c] + (lam[c] * (p0[c] - T(2) * p1[c] + p2[c]) * _dt2);
  }
  std::vector<double> g(np);
  for (long c = 0; c < np; ++c) g[c] = (double)grad[c];
  for (int s = 0; s < nsrc && mute_src > 0; ++s) {
    double pt[3];
    for (int d = 0; d < N; ++d) pt[d] = src_pos[s + (long)d * nsrc];
    mute_around_point(g.data(), N, n, h, pt, mute_src);
  }
  for (int r = 0; r < nrec && mute_rec > 0; ++r) {
    double pt[3];
    for (int d = 0; d < N; ++d) pt[d] = rec_pos[r + (long)d * nrec];
    mute_around_point(g.data(), N, n, h, pt, mute_rec);
  }
  for (long c = 0; c < np; ++c) {
    const T v = (T)vp[c];
    grad_out[c] = (double)((T(2) / (v * v * v)) * (T)g[c]);
  }
  return 0;
}

}  // namespace

extern "C" {

int oracle_version() { return 1; }

int oracle_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// Coefficient block per axis (length 4*halo+4 + 4*halo = 2*(2(halo+1)) + 2*(2halo)):
// a[2(halo+1)], a_h[2halo], b[2(halo+1)], b_h[2halo]
void oracle_cpml_axis(double vel_max, double dt, int halo, double rcoef, double h, double f0,
                      int freetop_axis, double* out) {
  cpml_axis(vel_max, dt, halo, rcoef, h, f0, freetop_axis != 0, out);
}

int oracle_acoustic_forward(int use_f32, int N, const int* n, const double* h, double dt, int halo,
                            const double* vp, const double* cpml, int nt, int nsrc, const int* src_idx,
                            const double* srctf, int nrec, const int* rec_idx, double* traces,
                            int nthreads) {
  if (N != 2 && N != 3) return 1;
  if (use_f32)
    return run_forward<float>(N, n, h, dt, halo, vp, cpml, nt, nsrc, src_idx, srctf, nrec, rec_idx, traces, nthreads);
  return run_forward<double>(N, n, h, dt, halo, vp, cpml, nt, nsrc, src_idx, srctf, nrec, rec_idx, traces, nthreads);
}

int oracle_acoustic_forward_snap(int N, const int* n, const double* h, double dt, int halo, const double* vp,
                                 const double* cpml, int nt, int nsrc, const int* src_idx, const double* srctf,
                                 int nrec, const int* rec_idx, double* traces, int nthreads, int snapevery,
                                 double* snaps) {
  if (N != 2 && N != 3) return 1;
  return run_forward<double>(N, n, h, dt, halo, vp, cpml, nt, nsrc, src_idx, srctf, nrec, rec_idx, traces, nthreads,
                             snapevery, snaps);
}

int oracle_acoustic_gradient(int use_f32, int N, const int* n, const double* h, double dt, int halo,
                             const double* vp, const double* cpml, int nt, int nsrc, const int* src_idx,
                             const double* srctf, int nrec, const int* rec_idx, const double* observed,
                             const double* invcov, int invcov_kind, int nwin, const int* windows,
                             int check_freq, int mute_src, int mute_rec, const double* src_pos,
                             const double* rec_pos, double* traces_out, double* grad_out,
                             double* misfit_out, int nthreads, int misfit_kind, double misfit_dt) {
  if (N != 2 && N != 3) return 1;
  if (use_f32)
    return run_gradient<float>(N, n, h, dt, halo, vp, cpml, nt, nsrc, src_idx, srctf, nrec, rec_idx, observed,
                               invcov, invcov_kind, nwin, windows, check_freq, mute_src, mute_rec, src_pos,
                               rec_pos, traces_out, grad_out, misfit_out, nthreads, misfit_kind, misfit_dt);
  return run_gradient<double>(N, n, h, dt, halo, vp, cpml, nt, nsrc, src_idx, srctf, nrec, rec_idx, observed,
                              invcov, invcov_kind, nwin, windows, check_freq, mute_src, mute_rec, src_pos,
                              rec_pos, traces_out, grad_out, misfit_out, nthreads, misfit_kind, misfit_dt);
}

}  // extern "C"
