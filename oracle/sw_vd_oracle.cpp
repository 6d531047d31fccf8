// SPDX-License-Identifier: MIT
//
// TEST INFRASTRUCTURE ONLY -- the CPU oracle for the swgb300 variable-density
// acoustic 2D path.
//
// Plain C++ restatement (FP64 and FP32 instantiations, OpenMP over rows) of
// what SeismicWaves.jl v0.9.0 runs for AcousticVDStaggeredCPMLWaveSimulation
// in 2D: the staggered 4th-order pressure-velocity scheme with C-PML, its
// forward modelling and its gradient with respect to vp and rho.  The test
// suite uses it as the checker and bench.py as the timed CPU baseline; nothing
// in the product links it.
//
// What it follows (paths relative to the SeismicWaves.jl source tree):
//   update_p_CPML!, update_vx_CPML!, update_vy_CPML!,
//   inject_sources!, record_receivers! .. src/models/acoustic/backends/shared/acoustic2D_VD_xPU.jl:1-78
//   staggered derivative and its boundary rules  src/utils/fdgen.jl:44-135 (fdcoeffs(1, 4) =
//                                      [1/24, -27/24, 27/24, -1/24], a point outside its array counts 0)
//   C-PML memory variables ........... src/utils/fdgen.jl:137-161 (the dtilde operator, halfgrid true / false)
//   forward / adjoint step ........... acoustic2D_VD_xPU.jl:80-169
//   gradient correlations ............ acoustic2D_VD_xPU.jl:171-192, correlate_gradient_xPU.jl:12-21
//   material factors ................. src/models/acoustic/acou_models.jl:283-300 (fact_m0 = vp^2 rho dt,
//                                      fact_m1_stag = interp(1/rho) dt)
//   source scaling ................... src/models/acoustic/acou_forward.jl:66-80 (done by the caller)
//   forward driver ................... acou_forward.jl:83-125
//   gradient driver .................. src/models/acoustic/acou_gradient.jl:97-202, checkpointer set-up
//                                      acou_models.jl:402-414 (pcur buffered with width 1)
//   back-interpolation ............... src/utils/interpolations.jl:1-47
//   L2 misfit ........................ src/inversion/misfits/L2Misfit.jl:24-77
//
// Parity status: the reference has no golden vectors for this simulation.
// Its tests pin an analytical 2D Green's function (1 % integrated error),
// "gradient != 0", misfit consistency and checkpoint equivalence
// (test/test_analytical_vs_numerical_acoustic_variable_density.jl,
// test/test_gradient_acoustic_variable_density.jl), which the test suite
// re-runs against this restatement.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_common.h"

namespace {

using oracle::back_interp;
using oracle::interp_at;
using oracle::LinearCheckpointer;
using oracle::mute_around_point;
using oracle::Snap;

template <typename T>
struct Arr2 {
  int n1 = 0, n2 = 0;
  std::vector<T> v;
  void init(int a, int b) { n1 = a; n2 = b; v.assign((size_t)a * (size_t)b, T(0)); }
  T& operator()(int i, int j) { return v[(size_t)(i - 1) + (size_t)(j - 1) * (size_t)n1]; }
  T operator()(int i, int j) const { return v[(size_t)(i - 1) + (size_t)(j - 1) * (size_t)n1]; }
  T at0(int i, int j) const {  // 0 outside the array (the boundary rules of fdgen.jl:72-120)
    if (i < 1 || i > n1 || j < 1 || j > n2) return T(0);
    return (*this)(i, j);
  }
  void zero() { std::fill(v.begin(), v.end(), T(0)); }
};

// 4th-order staggered first derivative over the points k0 .. k0+3 of one axis
// (fdidxs(1, 4) = I-1 .. I+2 with k0 = I-1), missing points 0.
template <typename T>
inline T d4(T f1, T f2, T f3, T f4, T inv) {
  const T c1 = T(1) / T(24), c2 = T(27) / T(24);
  return (c1 * f1 - c2 * f2 + c2 * f3 - c1 * f4) * inv;
}

template <typename T>
inline T dx_at(const Arr2<T>& A, int I, int j, T inv) {
  return d4(A.at0(I - 1, j), A.at0(I, j), A.at0(I + 1, j), A.at0(I + 2, j), inv);
}
template <typename T>
inline T dz_at(const Arr2<T>& A, int i, int J, T inv) {
  return d4(A.at0(i, J - 1), A.at0(i, J), A.at0(i, J + 1), A.at0(i, J + 2), inv);
}

// The dtilde operator of fdgen.jl:137-161 along one axis: I = index of the
// derivative along the axis, nA = size of the differentiated array along it.
// halfgrid = true: cells idim = I <= halo or >= nA - halo; halfgrid = false:
// idim = I + 1 <= halo + 1 or >= nA + 1 - halo.  Returns the coefficient index
// (1-based) or 0 outside the strips.
inline int cpml_index(int I, int nA, int halo, bool halfgrid) {
  const int plusone = halfgrid ? 0 : 1;
  const int idim = I + plusone;
  const int ndim = nA + plusone;
  if (idim <= halo + plusone) return idim;
  if (idim >= ndim - halo) return idim - (ndim - halo) + 1 + (halo + plusone);
  return 0;
}

template <typename T>
struct VDSim {
  int nx, nz, halo, nthreads;
  T dt, _dx, _dz;
  Arr2<T> p, vx, vz;
  Arr2<T> m0, m1x, m1z;  // fact_m0, fact_m1_stag
  Arr2<T> psi_x, psi_z, xi_x, xi_z;
  std::vector<T> ax, axh, bx, bxh, az, azh, bz, bzh;

  VDSim(int nx_, int nz_, const double* h, double dt_, int halo_, int nthreads_)
      : nx(nx_), nz(nz_), halo(halo_), nthreads(nthreads_) {
    dt = (T)dt_;
    _dx = T(1) / (T)h[0];
    _dz = T(1) / (T)h[1];
    p.init(nx, nz); vx.init(nx - 1, nz); vz.init(nx, nz - 1);
    m0.init(nx, nz); m1x.init(nx - 1, nz); m1z.init(nx, nz - 1);
    // acou_models.jl:379-389: psi for the velocities (2 halo), xi for the pressure (2 (halo + 1))
    psi_x.init(2 * halo, nz); psi_z.init(nx, 2 * halo);
    xi_x.init(2 * (halo + 1), nz); xi_z.init(nx, 2 * (halo + 1));
  }

  void set_cpml(const double* blk, int d) {
    const int na = 2 * (halo + 1), nh = 2 * halo;
    std::vector<T> a(na), ah(nh), b(na), bh(nh);
    for (int k = 0; k < na; ++k) { a[k] = (T)blk[k]; b[k] = (T)blk[na + nh + k]; }
    for (int k = 0; k < nh; ++k) { ah[k] = (T)blk[na + k]; bh[k] = (T)blk[2 * na + nh + k]; }
    if (d == 0) { ax = a; axh = ah; bx = b; bxh = bh; } else { az = a; azh = ah; bz = b; bzh = bh; }
  }

  // precompute_fact!, acou_models.jl:292-300
  void set_material(const double* vp, const double* rho, int method) {
    std::vector<double> m(rho, rho + (size_t)nx * nz);
    for (auto& x : m) x = 1.0 / x;
    for (int j = 1; j <= nz; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t c = (size_t)(i - 1) + (size_t)(j - 1) * nx;
        m0(i, j) = (T)(vp[c] * vp[c] * rho[c] * (double)dt);
      }
    for (int j = 1; j <= nz; ++j)
      for (int i = 1; i <= nx - 1; ++i) m1x(i, j) = (T)(interp_at(m.data(), nx, i, j, 1, 0, method) * (double)dt);
    for (int j = 1; j <= nz - 1; ++j)
      for (int i = 1; i <= nx; ++i) m1z(i, j) = (T)(interp_at(m.data(), nx, i, j, 0, 1, method) * (double)dt);
  }

  void reset_fields() {
    p.zero(); vx.zero(); vz.zero();
    psi_x.zero(); psi_z.zero(); xi_x.zero(); xi_z.zero();
  }

  // update_p_CPML!, acoustic2D_VD_xPU.jl:17-37, on (2:nx-1, 2:nz-1)
  void update_p() {
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 2; j <= nz - 1; ++j)
      for (int i = 2; i <= nx - 1; ++i) {
        T dvx = dx_at(vx, i - 1, j, _dx);
        int k = cpml_index(i - 1, nx - 1, halo, false);
        if (k) {
          xi_x(k, j) = bx[k - 1] * xi_x(k, j) + ax[k - 1] * dvx;
          dvx = dvx + xi_x(k, j);
        }
        T dvz = dz_at(vz, i, j - 1, _dz);
        k = cpml_index(j - 1, nz - 1, halo, false);
        if (k) {
          xi_z(i, k) = bz[k - 1] * xi_z(i, k) + az[k - 1] * dvz;
          dvz = dvz + xi_z(i, k);
        }
        p(i, j) -= m0(i, j) * (dvx + dvz);
      }
  }

  // update_vx_CPML! (1:nx-1, 1:nz) and update_vy_CPML! (1:nx, 1:nz-1), :39-77
  void update_v() {
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 1; j <= nz; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        T d = dx_at(p, i, j, _dx);
        const int k = cpml_index(i, nx, halo, true);
        if (k) {
          psi_x(k, j) = bxh[k - 1] * psi_x(k, j) + axh[k - 1] * d;
          d = d + psi_x(k, j);
        }
        vx(i, j) -= m1x(i, j) * d;
      }
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 1; j <= nz - 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        T d = dz_at(p, i, j, _dz);
        const int k = cpml_index(j, nz, halo, true);
        if (k) {
          psi_z(i, k) = bzh[k - 1] * psi_z(i, k) + azh[k - 1] * d;
          d = d + psi_z(i, k);
        }
        vz(i, j) -= m1z(i, j) * d;
      }
  }

  Snap<T> snap_p() const { return Snap<T>{p.v}; }
  Snap<T> snap_v() const { return Snap<T>{vx.v, vz.v}; }
  Snap<T> snap_psi() const { return Snap<T>{psi_x.v, psi_z.v}; }
  Snap<T> snap_xi() const { return Snap<T>{xi_x.v, xi_z.v}; }
  void load(const Snap<T>& sp, const Snap<T>& sv, const Snap<T>& sps, const Snap<T>& sxi) {
    p.v = sp[0]; vx.v = sv[0]; vz.v = sv[1];
    psi_x.v = sps[0]; psi_z.v = sps[1]; xi_x.v = sxi[0]; xi_z.v = sxi[1];
  }
};

struct VDShot {
  int nt, nsrc, nrec;
  std::vector<int> src, rec;  // 1-based (i, j) pairs
  std::vector<double> tf;     // (nt, nsrc), already scaled (possrcrec_scaletf)
};

// forward_onestep_CPML!, acoustic2D_VD_xPU.jl:80-125: p update, injection,
// velocity updates, recording.
template <typename T>
void forward_step(VDSim<T>& s, const VDShot& sh, int it, T* tr) {
  s.update_p();
  for (int q = 0; q < sh.nsrc; ++q) s.p(sh.src[2 * q], sh.src[2 * q + 1]) += (T)sh.tf[(size_t)(it - 1) + (size_t)q * sh.nt];
  s.update_v();
  if (tr)
    for (int r = 0; r < sh.nrec; ++r) tr[(size_t)(it - 1) + (size_t)r * sh.nt] = s.p(sh.rec[2 * r], sh.rec[2 * r + 1]);
}

// adjoint_onestep_CPML!, :127-169: velocity updates, p update, injection of the
// adjoint sources at the receivers.
template <typename T>
void adjoint_step(VDSim<T>& s, const VDShot& sh, int it, const std::vector<T>& adj) {
  s.update_v();
  s.update_p();
  for (int r = 0; r < sh.nrec; ++r) s.p(sh.rec[2 * r], sh.rec[2 * r + 1]) += adj[(size_t)(it - 1) + (size_t)r * sh.nt];
}

template <typename T>
void setup(VDSim<T>& s, const double* vp, const double* rho, int method, const double* cpml) {
  s.set_material(vp, rho, method);
  const int blk = 2 * (2 * (s.halo + 1)) + 2 * (2 * s.halo);
  s.set_cpml(cpml, 0);
  s.set_cpml(cpml + blk, 1);
}

template <typename T>
int run_forward(const int* n, const double* h, double dt, int halo, const double* vp, const double* rho, int method,
                const double* cpml, const VDShot& sh, double* traces, int nthreads, int snapevery = 0,
                double* snaps = nullptr) {
  VDSim<T> s(n[0], n[1], h, dt, halo, nthreads);
  setup(s, vp, rho, method, cpml);
  std::vector<T> tr((size_t)sh.nt * sh.nrec, T(0));
  const size_t np = (size_t)n[0] * n[1], nvx = (size_t)(n[0] - 1) * n[1], nvz = (size_t)n[0] * (n[1] - 1);
  for (int it = 1; it <= sh.nt; ++it) {
    forward_step(s, sh, it, tr.data());
    if (snaps && snapevery > 0 && it % snapevery == 0) {
      // savesnapshot!("pcur", "vcur"), acou_forward.jl:118-121: [p, vx, vz] per snapshot
      double* o = snaps + (size_t)(it / snapevery - 1) * (np + nvx + nvz);
      for (size_t c = 0; c < np; ++c) o[c] = (double)s.p.v[c];
      for (size_t c = 0; c < nvx; ++c) o[np + c] = (double)s.vx.v[c];
      for (size_t c = 0; c < nvz; ++c) o[np + nvx + c] = (double)s.vz.v[c];
    }
  }
  for (size_t q = 0; q < tr.size(); ++q) traces[q] = (double)tr[q];
  return 0;
}

template <typename T>
int run_gradient(const int* n, const double* h, double dt, int halo, const double* vp, const double* rho, int method,
                 const double* cpml, const VDShot& sh, const double* observed, const double* invcov, int invcov_kind,
                 int nwin, const int* windows, int check_freq, int mute_src, int mute_rec, const double* src_pos,
                 const double* rec_pos, double* traces_out, double* g_vp, double* g_rho, double* misfit_out,
                 int nthreads, int misfit_kind, double misfit_dt) {
  const int nt = sh.nt, nx = n[0], nz = n[1];
  if (check_freq < 1 || check_freq >= nt) return 1;  // LinearCheckpointer assertion
  VDSim<T> sim(nx, nz, h, dt, halo, nthreads), adj(nx, nz, h, dt, halo, nthreads);
  setup(sim, vp, rho, method, cpml);
  setup(adj, vp, rho, method, cpml);

  // acou_models.jl:402-414: checkpoints of pcur (width 1, buffered), vcur, psi, xi
  std::map<std::string, Snap<T>> proto;
  proto["pcur"] = sim.snap_p();
  proto["vcur"] = sim.snap_v();
  proto["psi"] = sim.snap_psi();
  proto["xi"] = sim.snap_xi();
  LinearCheckpointer<T> ck(nt, check_freq, proto, "pcur", 1);
  ck.save("pcur", sim.snap_p(), 0);
  ck.save("vcur", sim.snap_v(), 0);
  ck.save("psi", sim.snap_psi(), 0);
  ck.save("xi", sim.snap_xi(), 0);

  sim.reset_fields();
  adj.reset_fields();
  ck.reset();
  std::vector<T> tr((size_t)nt * sh.nrec, T(0));
  for (int it = 1; it <= nt; ++it) {
    forward_step(sim, sh, it, tr.data());
    // savecheckpoint! copies nothing unless it is a checkpoint or lies in the buffered tail
    if (it % check_freq == 0 || it >= ck.last_checkpoint) ck.save("pcur", sim.snap_p(), it);
    if (it % check_freq == 0) {
      ck.save("vcur", sim.snap_v(), it);
      ck.save("psi", sim.snap_psi(), it);
      ck.save("xi", sim.snap_xi(), it);
    }
  }
  for (size_t q = 0; q < tr.size(); ++q) traces_out[q] = (double)tr[q];

  // residuals, windows, C^-1, misfit (L2Misfit.jl:24-77)
  const long ntot = (long)nt * sh.nrec;
  std::vector<double> res(ntot), cres(ntot, 0.0);
  for (long q = 0; q < ntot; ++q) res[q] = (double)tr[q] - observed[q];
  if (nwin > 0) {
    std::vector<double> mask(nt, 0.0);
    for (int w = 0; w < nwin; ++w)
      for (int t = windows[2 * w] - 1; t <= windows[2 * w + 1] - 1; ++t) mask[t] = 1.0;
    for (int r = 0; r < sh.nrec; ++r)
      for (int t = 0; t < nt; ++t) res[t + (long)r * nt] *= mask[t];
  }
  for (int r = 0; r < sh.nrec; ++r)
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
  for (long q = 0; q < ntot; ++q) msf += res[q] * cres[q];
  *misfit_out = msf / 2;
  if (misfit_kind == 1) {  // CCTSMisfit (CCTSMisfit.jl:17-61): dchi/du per trace instead
    std::vector<double> syn(nt);
    double m = 0.0;
    for (int r = 0; r < sh.nrec; ++r) {
      for (int t = 0; t < nt; ++t) syn[t] = (double)tr[t + (long)r * nt];
      m += oracle::ccts_trace(observed + (long)r * nt, syn.data(), nt, misfit_dt, cres.data() + (long)r * nt);
    }
    *misfit_out = m;
  }
  // adjoint source -C^-1 r, prescaled by fact_m0 at the receivers (acou_gradient.jl:146-150)
  std::vector<T> adjsrc(ntot);
  for (int r = 0; r < sh.nrec; ++r) {
    const T f = sim.m0(sh.rec[2 * r], sh.rec[2 * r + 1]);
    for (int t = 0; t < nt; ++t) {
      const long q = t + (long)r * nt;
      adjsrc[q] = (T)(-cres[q]);
      adjsrc[q] *= f;
    }
  }

  Arr2<T> g0, g1x, g1z;
  g0.init(nx, nz); g1x.init(nx - 1, nz); g1z.init(nx, nz - 1);
  const T _dt = T(1) / sim.dt;
  for (int it = nt; it >= 1; --it) {
    adjoint_step(adj, sh, it, adjsrc);
    if (!ck.issaved("pcur", it - 1)) {
      ck.initrecover();
      const int c = ck.curr_checkpoint;
      sim.load(ck.getsaved("pcur", c), ck.getsaved("vcur", c), ck.getsaved("psi", c), ck.getsaved("xi", c));
      // recover!: steps c+1 .. c+K-1 refill the buffer (pcur only)
      for (int rit = c + 1; rit <= c + ck.K - 1; ++rit) {
        forward_step(sim, sh, rit, (T*)nullptr);
        ck.buffer[rit - c] = sim.snap_p();
      }
    }
    Arr2<T> pc, po;
    pc.n1 = po.n1 = nx;
    pc.n2 = po.n2 = nz;
    pc.v = ck.getsaved("pcur", it)[0];
    po.v = ck.getsaved("pcur", it - 1)[0];
    // correlate_gradient_m0!: g0 -= adjp (pcur - pold) / dt
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 1; j <= nz; ++j)
      for (int i = 1; i <= nx; ++i) g0(i, j) = g0(i, j) - (adj.p(i, j) * (pc(i, j) - po(i, j)) * _dt);
    // correlate_gradient_m1!: g1 += adjv * d(pcur) on the staggered grids
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 1; j <= nz; ++j)
      for (int i = 1; i <= nx - 1; ++i) g1x(i, j) = g1x(i, j) + adj.vx(i, j) * dx_at(pc, i, j, sim._dx);
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 1; j <= nz - 1; ++j)
      for (int i = 1; i <= nx; ++i) g1z(i, j) = g1z(i, j) + adj.vz(i, j) * dz_at(pc, i, j, sim._dz);
  }
  // acou_gradient.jl:178-201: back-interpolation of the m1 gradients, muting, chain rule
  const size_t np = (size_t)nx * nz;
  std::vector<double> m(rho, rho + np), G0(np), G1(np, 0.0);
  for (auto& x : m) x = 1.0 / x;
  for (size_t c = 0; c < np; ++c) G0[c] = (double)g0.v[c];
  std::vector<double> dx(g1x.v.begin(), g1x.v.end()), dz(g1z.v.begin(), g1z.v.end());
  back_interp(m.data(), nx, nz, dx.data(), nx - 1, 1, 0, method, G1.data());
  back_interp(m.data(), nx, nz, dz.data(), nx, 0, 1, method, G1.data());
  const int nn[2] = {nx, nz};
  for (double* g : {G0.data(), G1.data()}) {
    for (int s = 0; s < sh.nsrc && mute_src > 0; ++s) {
      const double pt[2] = {src_pos[s], src_pos[s + sh.nsrc]};
      mute_around_point(g, 2, nn, h, pt, mute_src);
    }
    for (int r = 0; r < sh.nrec && mute_rec > 0; ++r) {
      const double pt[2] = {rec_pos[r], rec_pos[r + sh.nrec]};
      mute_around_point(g, 2, nn, h, pt, mute_rec);
    }
  }
  for (size_t c = 0; c < np; ++c) {
    g_vp[c] = -2.0 * G0[c] / (vp[c] * vp[c] * vp[c] * rho[c]);
    g_rho[c] = -G0[c] / (vp[c] * vp[c] * rho[c] * rho[c]) - G1[c] / rho[c];
  }
  return 0;
}

VDShot make_shot(int nt, int nsrc, const int* src_idx, const double* srctf, int nrec, const int* rec_idx) {
  VDShot s;
  s.nt = nt;
  s.nsrc = nsrc;
  s.nrec = nrec;
  s.src.resize(2 * nsrc);
  s.rec.resize(2 * nrec);
  for (int q = 0; q < nsrc; ++q) { s.src[2 * q] = src_idx[q]; s.src[2 * q + 1] = src_idx[q + nsrc]; }
  for (int r = 0; r < nrec; ++r) { s.rec[2 * r] = rec_idx[r]; s.rec[2 * r + 1] = rec_idx[r + nrec]; }
  s.tf.assign(srctf, srctf + (size_t)nt * nsrc);
  return s;
}

bool bad_indices(const int* n, const VDShot& s) {
  for (int q = 0; q < s.nsrc + s.nrec; ++q) {
    const int i = q < s.nsrc ? s.src[2 * q] : s.rec[2 * (q - s.nsrc)];
    const int j = q < s.nsrc ? s.src[2 * q + 1] : s.rec[2 * (q - s.nsrc) + 1];
    if (i < 1 || i > n[0] || j < 1 || j > n[1]) return true;
  }
  return false;
}

}  // namespace

extern "C" {

// swforward_1shot! of the VD simulation for one shot.  src_idx / rec_idx are
// (n, 2) column-major 1-based grid indices; srctf (nt, nsrc) is already scaled
// by dt vp(src)^2 rho(src) / (dx dz).  snapevery > 0 fills snaps with
// floor(nt / snapevery) blocks [p (nx, nz), vx (nx-1, nz), vz (nx, nz-1)].
int oracle_vd_forward(int use_f32, const int* n, const double* h, double dt, int halo, const double* vp,
                      const double* rho, int method, const double* cpml, int nt, int nsrc, const int* src_idx,
                      const double* srctf, int nrec, const int* rec_idx, double* traces, int nthreads, int snapevery,
                      double* snaps) {
  if (n[0] < 4 || n[1] < 4) return 1;
  const VDShot sh = make_shot(nt, nsrc, src_idx, srctf, nrec, rec_idx);
  if (bad_indices(n, sh)) return 2;
  if (use_f32) return run_forward<float>(n, h, dt, halo, vp, rho, method, cpml, sh, traces, nthreads, snapevery, snaps);
  return run_forward<double>(n, h, dt, halo, vp, rho, method, cpml, sh, traces, nthreads, snapevery, snaps);
}

// swgradient_1shot! of the VD simulation plus calcmisfit for one shot.
// invcov_kind: 0 identity, 1 diagonal (nt), 2 dense (nt, nt).  misfit_kind 1:
// CCTSMisfit with time step misfit_dt (windows and invcov then unused).
int oracle_vd_gradient(int use_f32, const int* n, const double* h, double dt, int halo, const double* vp,
                       const double* rho, int method, const double* cpml, int nt, int nsrc, const int* src_idx,
                       const double* srctf, int nrec, const int* rec_idx, const double* observed,
                       const double* invcov, int invcov_kind, int nwin, const int* windows, int check_freq,
                       int mute_src, int mute_rec, const double* src_pos, const double* rec_pos, double* traces_out,
                       double* g_vp, double* g_rho, double* misfit_out, int nthreads, int misfit_kind,
                       double misfit_dt) {
  if (n[0] < 4 || n[1] < 4) return 1;
  const VDShot sh = make_shot(nt, nsrc, src_idx, srctf, nrec, rec_idx);
  if (bad_indices(n, sh)) return 2;
  if (use_f32)
    return run_gradient<float>(n, h, dt, halo, vp, rho, method, cpml, sh, observed, invcov, invcov_kind, nwin, windows,
                               check_freq, mute_src, mute_rec, src_pos, rec_pos, traces_out, g_vp, g_rho, misfit_out,
                               nthreads, misfit_kind, misfit_dt);
  return run_gradient<double>(n, h, dt, halo, vp, rho, method, cpml, sh, observed, invcov, invcov_kind, nwin, windows,
                              check_freq, mute_src, mute_rec, src_pos, rec_pos, traces_out, g_vp, g_rho, misfit_out,
                              nthreads, misfit_kind, misfit_dt);
}

}  // extern "C"
