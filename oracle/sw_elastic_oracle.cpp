// SPDX-License-Identifier: MIT
//
// TEST INFRASTRUCTURE ONLY -- the CPU oracle for the swgb300 elastic path.
//
// Plain C++ restatement (FP64 and FP32 instantiations, OpenMP over rows) of
// what SeismicWaves.jl v0.9.0 runs for the isotropic elastic 2D (P-SV) C-PML
// simulation and its gradient.  The test suite uses it as the checker and
// bench.py as the timed CPU baseline; nothing in the product links it.
//
// What it follows (paths relative to the SeismicWaves.jl source tree):
//   stress / displacement updates .. src/models/elastic/backends/shared/elastic2D_iso_xPU.jl:1-79
//   4th-order staggered derivatives  src/models/elastic/backends/shared/freesurface_derivatives_4th_mirror.jl:1-234
//   C-PML memory variables ......... src/utils/fdgenerated.jl:177-199 (the dtilde-4th operator)
//   injection / recording .......... elastic2D_iso_xPU.jl:81-118
//   one step + field swap .......... elastic2D_iso_xPU.jl:120-357, adjoint step :359-448
//   material interpolation ......... src/models/elastic/ela_models.jl:156-173, src/utils/interpolations.jl:1-47
//   sinc source/receiver spreading . src/utils/utils.jl:62-214 (besseli(0, x) by its power series,
//                                    Abramowitz & Stegun 9.6.10)
//   forward driver ................. src/models/elastic/ela_forward.jl:4-159
//   gradient driver ................ src/models/elastic/ela_gradient.jl:4-362,
//                                    checkpointer set-up ela_models.jl:370-383
//   correlation .................... src/models/elastic/backends/shared/correlate_gradient_xPU.jl:1-83
//   L2 misfit, 3-D traces .......... src/inversion/misfits/L2Misfit.jl:44-95
//   C-PML coefficients ............. src/models/elastic/ela_init_bc.jl:7-40 (same axis formula as acoustic)
//
// Parity status: the reference has no elastic golden vectors; its elastic
// tests pin only "gradient != 0", misfit consistency and checkpoint
// equivalence (test/test_gradient_elastic_homogeneous.jl), which the test
// suite re-runs against this restatement.  Trace-level parity with the Julia
// program itself is unpinned.

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

// Column-major 2-D array with the reference's 1-based indexing.
template <typename T>
struct Arr2 {
  int n1 = 0, n2 = 0;
  std::vector<T> v;
  void init(int a, int b) { n1 = a; n2 = b; v.assign((size_t)a * (size_t)b, T(0)); }
  T& operator()(int i, int j) { return v[(size_t)(i - 1) + (size_t)(j - 1) * (size_t)n1]; }
  T operator()(int i, int j) const { return v[(size_t)(i - 1) + (size_t)(j - 1) * (size_t)n1]; }
  void zero() { std::fill(v.begin(), v.end(), T(0)); }
};

// (1/24 f1 - 27/24 f2 + 27/24 f3 - 1/24 f4) * inv, freesurface_derivatives_4th_mirror.jl:2-7
template <typename T>
inline T d4(T f1, T f2, T f3, T f4, T inv) {
  const T c1 = T(1) / T(24), c2 = T(27) / T(24);
  return (c1 * f1 - c2 * f2 + c2 * f3 - c1 * f4) * inv;
}

// The dtilde-4th operator of fdgenerated.jl:178-195: the C-PML memory variable
// update on the strip cell selected by the reference's two index maps.  A cell
// is written only when its value changes: the "full" maps send the last left
// point and the first right point to the same cell, whose coefficient a is 0,
// so that cell stays 0 and concurrent rows never write it.
template <typename T, typename Cell>
inline T cpml_apply(int ndim, int Idir, bool half, T dv, const std::vector<T>& a, const std::vector<T>& b,
                    int halo, Cell cell) {
  const int plusone = half ? 1 : 0;
  const int idim = Idir + plusone;
  const int iidim = Idir - (ndim - halo) + 1 + (halo + plusone);
  int k = 0;
  if (idim <= halo + plusone) k = idim;
  else if (idim >= ndim - halo) k = iidim;
  else return dv;
  T& p = cell(k);
  const T nv = b[k - 1] * p + a[k - 1] * dv;
  if (nv != p) p = nv;
  return dv + p;
}

// One point table (sinc spreading of one position, or one nearest grid point).
struct Pts {
  std::vector<int> i, j;
  std::vector<double> c;
};

template <typename T>
struct ElasticSim {
  int nx, nz, halo;
  bool freetop;
  T dt, _dx, _dz;
  int nthreads;
  Arr2<T> sxx, szz, sxz;
  Arr2<T> ux[3], uz[3];
  int iold = 0, icur = 1, inew = 2;
  Arr2<T> lam, mu, rho_i, rho_j, mu_ij;
  // psi arrays, ela_models.jl:276-299
  Arr2<T> psi_sxx_x, psi_sxz_x, psi_szz_z, psi_sxz_z, psi_ux_x, psi_uz_x, psi_ux_z, psi_uz_z;
  std::vector<T> ax, axh, bx, bxh, az, azh, bz, bzh;

  ElasticSim(int nx_, int nz_, const double* h, double dt_, int halo_, bool freetop_, int nthreads_)
      : nx(nx_), nz(nz_), halo(halo_), freetop(freetop_), nthreads(nthreads_) {
    dt = (T)dt_;
    _dx = T(1) / (T)h[0];
    _dz = T(1) / (T)h[1];
    sxx.init(nx, nz); szz.init(nx, nz); sxz.init(nx - 1, nz - 1);
    for (int b = 0; b < 3; ++b) { ux[b].init(nx - 1, nz); uz[b].init(nx, nz - 1); }
    lam.init(nx, nz); mu.init(nx, nz); rho_i.init(nx - 1, nz); rho_j.init(nx, nz - 1); mu_ij.init(nx - 1, nz - 1);
    psi_sxx_x.init(2 * halo, nz);
    psi_sxz_x.init(2 * (halo + 1), nz - 1);
    psi_szz_z.init(nx, 2 * halo);
    psi_sxz_z.init(nx - 1, 2 * (halo + 1));
    psi_ux_x.init(2 * (halo + 1), nz);
    psi_uz_x.init(2 * halo, nz - 1);
    psi_ux_z.init(nx - 1, 2 * halo);
    psi_uz_z.init(nx, 2 * (halo + 1));
  }

  void set_cpml(const double* blk, int d) {
    const int na = 2 * (halo + 1), nh = 2 * halo;
    std::vector<T> a(na), ah(nh), b(na), bh(nh);
    for (int k = 0; k < na; ++k) { a[k] = (T)blk[k]; b[k] = (T)blk[na + nh + k]; }
    for (int k = 0; k < nh; ++k) { ah[k] = (T)blk[na + k]; bh[k] = (T)blk[2 * na + nh + k]; }
    if (d == 0) { ax = a; axh = ah; bx = b; bxh = bh; } else { az = a; azh = ah; bz = b; bzh = bh; }
  }

  void reset_fields() {
    sxx.zero(); szz.zero(); sxz.zero();
    for (int b = 0; b < 3; ++b) { ux[b].zero(); uz[b].zero(); }
    psi_sxx_x.zero(); psi_sxz_x.zero(); psi_szz_z.zero(); psi_sxz_z.zero();
    psi_ux_x.zero(); psi_uz_x.zero(); psi_ux_z.zero(); psi_uz_z.zero();
  }

  Snap<T> snap_u() const { return Snap<T>{ux[icur].v, uz[icur].v}; }
  Snap<T> snap_uold() const { return Snap<T>{ux[iold].v, uz[iold].v}; }
  Snap<T> snap_psi() const {
    return Snap<T>{psi_sxx_x.v, psi_sxz_x.v, psi_szz_z.v, psi_sxz_z.v,
                   psi_ux_x.v, psi_uz_x.v, psi_ux_z.v, psi_uz_z.v};
  }
  void load_psi(const Snap<T>& s) {
    psi_sxx_x.v = s[0]; psi_sxz_x.v = s[1]; psi_szz_z.v = s[2]; psi_sxz_z.v = s[3];
    psi_ux_x.v = s[4]; psi_uz_x.v = s[5]; psi_ux_z.v = s[6]; psi_uz_z.v = s[7];
  }

  // ---- derivative wrappers, freesurface_derivatives_4th_mirror.jl:72-234 ----
  T dsxx_dx(int i, int j) const {
    const Arr2<T>& f = sxx;
    if (i == 1) return d4(T(0), f(i, j), f(i + 1, j), f(i + 2, j), _dx);
    if (i == nx - 1) return d4(f(i - 1, j), f(i, j), f(i + 1, j), T(0), _dx);
    return d4(f(i - 1, j), f(i, j), f(i + 1, j), f(i + 2, j), _dx);
  }
  T dszz_dz(int i, int j) const {
    const Arr2<T>& f = szz;
    if (j == 1) {
      if (freetop) return d4(-f(i, j + 1), f(i, j), f(i, j + 1), f(i, j + 2), _dz);
      return d4(T(0), f(i, j), f(i, j + 1), f(i, j + 2), _dz);
    }
    if (j == nz - 1) return d4(f(i, j - 1), f(i, j), f(i, j + 1), T(0), _dz);
    return d4(f(i, j - 1), f(i, j), f(i, j + 1), f(i, j + 2), _dz);
  }
  T dsxz_dx(int i, int j) const {
    const Arr2<T>& f = sxz;
    if (i == 1) return d4(T(0), T(0), f(i, j), f(i + 1, j), _dx);
    if (i == 2) return d4(T(0), f(i - 1, j), f(i, j), f(i + 1, j), _dx);
    if (i == nx - 1) return d4(f(i - 2, j), f(i - 1, j), f(i, j), T(0), _dx);
    if (i == nx) return d4(f(i - 2, j), f(i - 1, j), T(0), T(0), _dx);
    return d4(f(i - 2, j), f(i - 1, j), f(i, j), f(i + 1, j), _dx);
  }
  T dsxz_dz(int i, int j) const {
    const Arr2<T>& f = sxz;
    if (j == 1) {
      if (freetop) return d4(-f(i, j + 1), -f(i, j), f(i, j), f(i, j + 1), _dz);
      return d4(T(0), T(0), f(i, j), f(i, j + 1), _dz);
    }
    if (j == 2) {
      if (freetop) return d4(-f(i, j - 1), f(i, j - 1), f(i, j), f(i, j + 1), _dz);
      return d4(T(0), f(i, j - 1), f(i, j), f(i, j + 1), _dz);
    }
    if (j == nz - 1) return d4(f(i, j - 2), f(i, j - 1), f(i, j), T(0), _dz);
    if (j == nz) return d4(f(i, j - 2), f(i, j - 1), T(0), T(0), _dz);
    return d4(f(i, j - 2), f(i, j - 1), f(i, j), f(i, j + 1), _dz);
  }
  T dux_dx(const Arr2<T>& u, int i, int j) const {
    if (i == 1) return d4(T(0), T(0), u(i, j), u(i + 1, j), _dx);
    if (i == 2) return d4(T(0), u(i - 1, j), u(i, j), u(i + 1, j), _dx);
    if (i == nx - 1) return d4(u(i - 2, j), u(i - 1, j), u(i, j), T(0), _dx);
    if (i == nx) return d4(u(i - 2, j), u(i - 1, j), T(0), T(0), _dx);
    return d4(u(i - 2, j), u(i - 1, j), u(i, j), u(i + 1, j), _dx);
  }
  T duz_dz(const Arr2<T>& ux_, const Arr2<T>& uz_, int i, int j) const {
    if (j == 1) {
      if (freetop) {
        const T d = dux_dx(ux_, i, j);
        return (-lam(i, j) / (lam(i, j) + T(2) * mu(i, j))) * d;
      }
      return d4(T(0), T(0), uz_(i, j), uz_(i, j + 1), _dz);
    }
    if (j == 2) {
      if (freetop) return d4(uz_(i, j - 1), uz_(i, j - 1), uz_(i, j), uz_(i, j + 1), _dz);
      return d4(T(0), uz_(i, j - 1), uz_(i, j), uz_(i, j + 1), _dz);
    }
    if (j == nz - 1) return d4(uz_(i, j - 2), uz_(i, j - 1), uz_(i, j), T(0), _dz);
    if (j == nz) return d4(uz_(i, j - 2), uz_(i, j - 1), T(0), T(0), _dz);
    return d4(uz_(i, j - 2), uz_(i, j - 1), uz_(i, j), uz_(i, j + 1), _dz);
  }
  T dux_dz(const Arr2<T>& u, int i, int j) const {
    if (j == 1) {
      if (freetop) return d4(u(i, j + 1), u(i, j), u(i, j + 1), u(i, j + 2), _dz);
      return d4(T(0), u(i, j), u(i, j + 1), u(i, j + 2), _dz);
    }
    if (j == nz - 1) return d4(u(i, j - 1), u(i, j), u(i, j + 1), T(0), _dz);
    return d4(u(i, j - 1), u(i, j), u(i, j + 1), u(i, j + 2), _dz);
  }
  T duz_dx(const Arr2<T>& u, int i, int j) const {
    if (i == 1) return d4(T(0), u(i, j), u(i + 1, j), u(i + 2, j), _dx);
    if (i == nx - 1) return d4(u(i - 1, j), u(i, j), u(i + 1, j), T(0), _dx);
    return d4(u(i - 1, j), u(i, j), u(i + 1, j), u(i + 2, j), _dx);
  }

  // ---- kernels, elastic2D_iso_xPU.jl:1-79 ----
  void update_sxx_szz() {
    const Arr2<T>& uxc = ux[icur];
    const Arr2<T>& uzc = uz[icur];
    const int jlo = freetop ? 1 : 2;
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = jlo; j <= nz - 1; ++j)
      for (int i = 2; i <= nx - 1; ++i) {
        const T dux = dux_dx(uxc, i, j);
        const T duz = duz_dz(uxc, uzc, i, j);
        const T duxc = cpml_apply(nx - 1, i - 1, true, dux, ax, bx, halo, [&](int k) -> T& { return psi_ux_x(k, j); });
        const T duzc = cpml_apply(nz - 1, j - 1, true, duz, az, bz, halo, [&](int k) -> T& { return psi_uz_z(i, k); });
        const T l = lam(i, j), m = mu(i, j);
        sxx(i, j) = (l + T(2) * m) * duxc + l * duzc;
        if (j == 1) szz(i, j) = T(0);
        else szz(i, j) = l * duxc + (l + T(2) * m) * duzc;
      }
  }
  void update_sxz() {
    const Arr2<T>& uxc = ux[icur];
    const Arr2<T>& uzc = uz[icur];
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 1; j <= nz - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        const T dzx = duz_dx(uzc, i, j);
        const T dxz = dux_dz(uxc, i, j);
        const T dzxc = cpml_apply(nx, i, false, dzx, axh, bxh, halo, [&](int k) -> T& { return psi_uz_x(k, j); });
        const T dxzc = cpml_apply(nz, j, false, dxz, azh, bzh, halo, [&](int k) -> T& { return psi_ux_z(i, k); });
        sxz(i, j) = mu_ij(i, j) * (dzxc + dxzc);
      }
  }
  void update_u() {
    Arr2<T>& uxn = ux[inew];
    Arr2<T>& uzn = uz[inew];
    const Arr2<T>& uxc = ux[icur];
    const Arr2<T>& uzc = uz[icur];
    const Arr2<T>& uxo = ux[iold];
    const Arr2<T>& uzo = uz[iold];
    const T dt2 = dt * dt;
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 1; j <= nz; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        const T d1 = dsxx_dx(i, j);
        const T d2 = dsxz_dz(i, j);
        const T d1c = cpml_apply(nx, i, false, d1, axh, bxh, halo, [&](int k) -> T& { return psi_sxx_x(k, j); });
        const T d2c = cpml_apply(nz - 1, j - 1, true, d2, az, bz, halo, [&](int k) -> T& { return psi_sxz_z(i, k); });
        const T o = uxo(i, j);  // uold and unew may be one array (field swap below)
        uxn(i, j) = T(2) * uxc(i, j) - o + dt2 / rho_i(i, j) * (d1c + d2c);
      }
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 1; j <= nz - 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        const T d1 = dsxz_dx(i, j);
        const T d2 = dszz_dz(i, j);
        const T d1c = cpml_apply(nx - 1, i - 1, true, d1, ax, bx, halo, [&](int k) -> T& { return psi_sxz_x(k, j); });
        const T d2c = cpml_apply(nz, j, false, d2, azh, bzh, halo, [&](int k) -> T& { return psi_szz_z(i, k); });
        const T o = uzo(i, j);
        uzn(i, j) = T(2) * uzc(i, j) - o + dt2 / rho_j(i, j) * (d1c + d2c);
      }
  }
  // grid.fields swap of elastic2D_iso_xPU.jl:233-236: uold <- ucur, ucur <- unew,
  // unew <- (the new) uold, so from the second step on unew and uold are one array.
  void swap() {
    const int o = icur, c = inew;
    iold = o; icur = c; inew = o;
  }
};

// ---------------------------------------------------------------------------
// Material set-up: precomp_elaprop!, ela_models.jl:156-173 with the
// interpolations of interpolations.jl:30-43 (0 = arithmetic, 1 = harmonic).
// ---------------------------------------------------------------------------
template <typename T>
void set_material(ElasticSim<T>& sim, const double* lam, const double* mu, const double* rho, int irho, int imu) {
  const int nx = sim.nx, nz = sim.nz;
  for (int j = 1; j <= nz; ++j)
    for (int i = 1; i <= nx; ++i) {
      sim.lam(i, j) = (T)lam[(size_t)(i - 1) + (size_t)(j - 1) * nx];
      sim.mu(i, j) = (T)mu[(size_t)(i - 1) + (size_t)(j - 1) * nx];
    }
  for (int j = 1; j <= nz; ++j)
    for (int i = 1; i <= nx - 1; ++i) sim.rho_i(i, j) = (T)interp_at(rho, nx, i, j, 1, 0, irho);
  for (int j = 1; j <= nz - 1; ++j)
    for (int i = 1; i <= nx; ++i) sim.rho_j(i, j) = (T)interp_at(rho, nx, i, j, 0, 1, irho);
  for (int j = 1; j <= nz - 1; ++j)
    for (int i = 1; i <= nx - 1; ++i) sim.mu_ij(i, j) = (T)interp_at(mu, nx, i, j, 1, 1, imu);
}

// ---------------------------------------------------------------------------
// Sinc spreading, utils.jl:62-214
// ---------------------------------------------------------------------------
inline double bessel_i0(double x) {
  // I0(x) = sum_k ((x/2)^(2k)) / (k!)^2  (A&S 9.6.10), summed until the terms vanish
  const double q = 0.25 * x * x;
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 500; ++k) {
    term *= q / ((double)k * (double)k);
    sum += term;
    if (term < sum * 1e-18) break;
  }
  return sum;
}

inline double kaiser(double x, double r, double beta) {
  if (!(-r <= x && x <= r)) return 0.0;
  const double t = x / r;
  return bessel_i0(beta * std::sqrt(1.0 - t * t)) / bessel_i0(beta);
}

inline double sinc_n(double t) {  // Julia's normalised sinc
  if (t == 0.0) return 1.0;
  if (t == std::nearbyint(t)) return 0.0;  // sinpi at an integer is exactly 0
  return std::sin(M_PI * t) / (M_PI * t);
}

inline int findnearest(double x, double xstart, double dx, int n) {
  int best = 1;
  double bd = std::fabs(x - xstart);
  for (int k = 2; k <= n; ++k) {
    const double d = std::fabs(x - (xstart + (k - 1) * dx));
    if (d < bd) { bd = d; best = k; }
  }
  return best;
}

// coeffsinc1D: indices (1-based) and coefficients, duplicates summed in order of
// first appearance (the Dict of the reference; the order of the pairs is free)
inline void coeffsinc1d(double x0, double dx, int n, int r, double beta, double xstart, bool mirror,
                        double xbl, double xbr, std::vector<int>& idx_out, std::vector<double>& c_out) {
  const int i0 = findnearest(x0, xstart, dx, n);
  std::vector<int> idxs;
  std::vector<double> cs;
  for (int idx = i0 - r - 1; idx <= i0 + r + 1; ++idx) {
    const double xc = (idx - 1) * dx + xstart;
    const double coe = kaiser(xc - x0, r * dx, beta) * sinc_n((xc - x0) / dx);
    if (!(std::fabs(coe) <= 1e-15)) { idxs.push_back(idx); cs.push_back(coe); }
  }
  idx_out.clear(); c_out.clear();
  for (size_t q = 0; q < idxs.size(); ++q) {
    const double xc = (idxs[q] - 1) * dx + xstart;
    int id = idxs[q];
    double c = cs[q];
    if (xc < xbl) { id = findnearest(xbl + (xbl - xc), xstart, dx, n); if (mirror) c = -c; }
    else if (xc > xbr) { id = findnearest(xbr - (xc - xbr), xstart, dx, n); if (mirror) c = -c; }
    auto it = std::find(idx_out.begin(), idx_out.end(), id);
    if (it == idx_out.end()) { idx_out.push_back(id); c_out.push_back(c); }
    else c_out[it - idx_out.begin()] += c;
  }
}

// spread_positions for one position: tensor product, x index fastest
inline Pts spread_one(const int* n, const double* h, const double* pos, const double* shift, bool mirror,
                      int r, double beta) {
  std::vector<int> ix, iz;
  std::vector<double> cx, cz;
  const double ext0 = h[0] * (n[0] - 1), ext1 = h[1] * (n[1] - 1);
  coeffsinc1d(pos[0], h[0], n[0], r, beta, shift[0], mirror, 0.0, ext0, ix, cx);
  coeffsinc1d(pos[1], h[1], n[1], r, beta, shift[1], mirror, 0.0, ext1, iz, cz);
  Pts p;
  for (size_t b = 0; b < iz.size(); ++b)
    for (size_t a = 0; a < ix.size(); ++a) {
      p.i.push_back(ix[a]); p.j.push_back(iz[b]); p.c.push_back(cx[a] * cz[b]);
    }
  return p;
}

// ---------------------------------------------------------------------------
// Shot description shared by forward and gradient
// ---------------------------------------------------------------------------
struct ElShot {
  int nt, kind, nsrc, nrec;
  std::vector<double> srctf;    // MT: (nt, nsrc); force: (nt, 2, nsrc)
  std::vector<double> momtens;  // (3, nsrc)
  std::vector<Pts> src[2], rec[2];
};

// tables packed as: cnt[table * nitems + item], then (i, j) pairs and coefs in
// the order table 0 item 0.., table 1 item 0..
inline void unpack_tables(int nitems, const int* cnt, const int* ij, const double* coef, std::vector<Pts>* out) {
  long q = 0;
  for (int t = 0; t < 2; ++t) {
    out[t].assign(nitems, Pts());
    for (int s = 0; s < nitems; ++s) {
      const int c = cnt[t * nitems + s];
      for (int k = 0; k < c; ++k, ++q) {
        out[t][s].i.push_back(ij[2 * q]);
        out[t][s].j.push_back(ij[2 * q + 1]);
        out[t][s].c.push_back(coef[q]);
      }
    }
  }
}

template <typename T>
struct Runner {
  ElasticSim<T>& sim;
  const ElShot& sh;
  std::vector<T> tf, mt;

  Runner(ElasticSim<T>& s, const ElShot& shot) : sim(s), sh(shot) {
    tf.resize(sh.srctf.size());
    for (size_t q = 0; q < tf.size(); ++q) tf[q] = (T)sh.srctf[q];
    mt.resize(sh.momtens.size());
    for (size_t q = 0; q < mt.size(); ++q) mt[q] = (T)sh.momtens[q];
  }

  // inject_external_sources2D_u{x,z}!: u += coe * tf / rho * dt^2
  void inject_force(Arr2<T>& ux, Arr2<T>& uz, const std::vector<Pts>* tab, const T* f, int nt, int nitems, int it) {
    const T dt2 = sim.dt * sim.dt;
    for (int s = 0; s < nitems; ++s) {
      const Pts& px = tab[0][s];
      for (size_t p = 0; p < px.c.size(); ++p) {
        const T v = f[(it - 1) + (size_t)nt * (0 + 2 * (size_t)s)];
        ux(px.i[p], px.j[p]) += (T)px.c[p] * v / sim.rho_i(px.i[p], px.j[p]) * dt2;
      }
      const Pts& pz = tab[1][s];
      for (size_t p = 0; p < pz.c.size(); ++p) {
        const T v = f[(it - 1) + (size_t)nt * (1 + 2 * (size_t)s)];
        uz(pz.i[p], pz.j[p]) += (T)pz.c[p] * v / sim.rho_j(pz.i[p], pz.j[p]) * dt2;
      }
    }
  }

  // forward_onestep_CPML! (both source kinds), elastic2D_iso_xPU.jl:120-357
  void step(int it, T* traces) {
    sim.update_sxx_szz();
    sim.update_sxz();
    if (sh.kind == 0) {  // inject_momten_sources2D_*
      for (int s = 0; s < sh.nsrc; ++s) {
        const T stf = tf[(it - 1) + (size_t)sh.nt * s];
        const T Mxx = mt[3 * s], Mzz = mt[3 * s + 1], Mxz = mt[3 * s + 2];
        const Pts& a = sh.src[0][s];
        for (size_t p = 0; p < a.c.size(); ++p) {
          sim.sxx(a.i[p], a.j[p]) += Mxx * (T)a.c[p] * stf;
          sim.szz(a.i[p], a.j[p]) += Mzz * (T)a.c[p] * stf;
        }
        const Pts& b = sh.src[1][s];
        for (size_t p = 0; p < b.c.size(); ++p) sim.sxz(b.i[p], b.j[p]) += Mxz * (T)b.c[p] * stf;
      }
    }
    sim.update_u();
    if (sh.kind == 1) inject_force(sim.ux[sim.inew], sim.uz[sim.inew], sh.src, tf.data(), sh.nt, sh.nsrc, it);
    if (traces) {  // record_receivers2D_u{x,z}! + the per-receiver sum
      for (int r = 0; r < sh.nrec; ++r)
        for (int c = 0; c < 2; ++c) {
          const Pts& pr = sh.rec[c][r];
          const Arr2<T>& u = c == 0 ? sim.ux[sim.inew] : sim.uz[sim.inew];
          T acc = T(0);
          for (size_t p = 0; p < pr.c.size(); ++p) acc += (T)pr.c[p] * u(pr.i[p], pr.j[p]);
          traces[(it - 1) + (size_t)sh.nt * (c + 2 * (size_t)r)] = acc;
        }
    }
    sim.swap();
  }

  // adjoint_onestep_CPML!, elastic2D_iso_xPU.jl:359-448 (residuals as forces at the receivers)
  void adjoint_step(int it, const T* res) {
    sim.update_sxx_szz();
    sim.update_sxz();
    sim.update_u();
    inject_force(sim.ux[sim.inew], sim.uz[sim.inew], sh.rec, res, sh.nt, sh.nrec, it);
    sim.swap();
  }
};

template <typename T>
ElShot make_shot(int nt, int kind, int nsrc, const double* srctf, const double* momtens, const int* src_cnt,
                 const int* src_ij, const double* src_coef, int nrec, const int* rec_cnt, const int* rec_ij,
                 const double* rec_coef) {
  ElShot sh;
  sh.nt = nt; sh.kind = kind; sh.nsrc = nsrc; sh.nrec = nrec;
  sh.srctf.assign(srctf, srctf + (size_t)nt * nsrc * (kind == 1 ? 2 : 1));
  if (kind == 0) sh.momtens.assign(momtens, momtens + 3 * (size_t)nsrc);
  unpack_tables(nsrc, src_cnt, src_ij, src_coef, sh.src);
  unpack_tables(nrec, rec_cnt, rec_ij, rec_coef, sh.rec);
  return sh;
}

template <typename T>
int run_forward(const int* n, const double* h, double dt, int halo, int freetop, const double* lam,
                const double* mu, const double* rho, int irho, int imu, const double* cpml, const ElShot& sh,
                double* traces, int nthreads, int snapevery = 0, double* snaps = nullptr) {
  ElasticSim<T> sim(n[0], n[1], h, dt, halo, freetop != 0, nthreads);
  set_material(sim, lam, mu, rho, irho, imu);
  const int blk = 2 * (2 * (halo + 1)) + 2 * (2 * halo);
  sim.set_cpml(cpml, 0);
  sim.set_cpml(cpml + blk, 1);
  sim.reset_fields();
  Runner<T> run(sim, sh);
  std::vector<T> tr((size_t)sh.nt * 2 * sh.nrec, T(0));
  const long sblk = (long)(n[0] - 1) * n[1] + (long)n[0] * (n[1] - 1) + 2L * n[0] * n[1] + (long)(n[0] - 1) * (n[1] - 1);
  for (int it = 1; it <= sh.nt; ++it) {
    run.step(it, tr.data());
    // savesnapshot!("ucur" => ..., "σ" => ...) (ela_forward.jl:74-78): ux, uz, sxx, szz, sxz
    if (snaps && snapevery > 0 && it % snapevery == 0) {
      double* o = snaps + (long)(it / snapevery - 1) * sblk;
      for (const std::vector<T>* v : {&sim.ux[sim.icur].v, &sim.uz[sim.icur].v, &sim.sxx.v, &sim.szz.v, &sim.sxz.v})
        for (T x : *v) *o++ = (double)x;
    }
  }
  for (size_t q = 0; q < tr.size(); ++q) traces[q] = (double)tr[q];
  return 0;
}

template <typename T>
int run_gradient(const int* n, const double* h, double dt, int halo, int freetop, const double* lam,
                 const double* mu, const double* rho, int irho, int imu, const double* cpml, const ElShot& sh,
                 const double* observed, const double* invcov, int invcov_kind, int nwin, const int* windows,
                 int check_freq, int mute_src, int mute_rec, const double* src_pos, const double* rec_pos,
                 double* traces_out, double* g_rho, double* g_lam, double* g_mu, double* misfit_out,
                 int nthreads, int ccts, double ccts_dt) {
  const int nt = sh.nt, nx = n[0], nz = n[1];
  if (check_freq < 1 || check_freq >= nt) return 1;  // LinearCheckpointer assertion
  ElasticSim<T> sim(nx, nz, h, dt, halo, freetop != 0, nthreads);
  ElasticSim<T> adj(nx, nz, h, dt, halo, freetop != 0, nthreads);
  for (ElasticSim<T>* s : {&sim, &adj}) {
    set_material(*s, lam, mu, rho, irho, imu);
    const int blk = 2 * (2 * (halo + 1)) + 2 * (2 * halo);
    s->set_cpml(cpml, 0);
    s->set_cpml(cpml + blk, 1);
  }
  Runner<T> fw(sim, sh), bw(adj, sh);

  // ela_models.jl:370-383: checkpointer over ucur (width 2, buffered) and psi
  std::map<std::string, Snap<T>> proto;
  proto["ucur"] = sim.snap_u();
  proto["psi"] = sim.snap_psi();
  LinearCheckpointer<T> ck(nt, check_freq, proto, "ucur");
  ck.save("ucur", sim.snap_uold(), -1);
  ck.save("ucur", sim.snap_u(), 0);
  ck.save("psi", sim.snap_psi(), 0);

  sim.reset_fields();
  adj.reset_fields();
  ck.reset();
  std::vector<T> tr((size_t)nt * 2 * sh.nrec, T(0));
  for (int it = 1; it <= nt; ++it) {
    fw.step(it, tr.data());
    ck.save("ucur", sim.snap_u(), it);
    ck.save("psi", sim.snap_psi(), it);
  }
  for (size_t q = 0; q < tr.size(); ++q) traces_out[q] = (double)tr[q];

  // residuals (nt, 2, nrec), windows, C^-1 per component, misfit
  const long ntot = (long)nt * 2 * sh.nrec;
  std::vector<double> res(ntot), cres(ntot, 0.0);
  for (long q = 0; q < ntot; ++q) res[q] = (double)tr[q] - observed[q];
  if (nwin > 0) {
    std::vector<double> mask(nt, 0.0);
    for (int w = 0; w < nwin; ++w)
      for (int t = windows[2 * w] - 1; t <= windows[2 * w + 1] - 1; ++t) mask[t] = 1.0;
    for (long c = 0; c < 2L * sh.nrec; ++c)
      for (int t = 0; t < nt; ++t) res[t + c * nt] *= mask[t];
  }
  for (long c = 0; c < 2L * sh.nrec; ++c)
    for (int t = 0; t < nt; ++t) {
      const long q = t + c * nt;
      if (invcov_kind == 0) cres[q] = res[q];
      else if (invcov_kind == 1) cres[q] = invcov[t] * res[q];
      else {
        double acc = 0;
        for (int u = 0; u < nt; ++u) acc += invcov[t + (long)u * nt] * res[u + c * nt];
        cres[q] = acc;
      }
    }
  double msf = 0;
  for (long q = 0; q < ntot; ++q) msf += res[q] * cres[q];
  *misfit_out = msf / 2;
  if (ccts) {  // CCTSMisfit{T,3}: per receiver and component, dtau^2/2 and dtau/N ds/dt (CCTSMisfit.jl:30-44, :63-80)
    std::vector<double> syn(nt);
    msf = 0;
    for (long c = 0; c < 2L * sh.nrec; ++c) {
      for (int t = 0; t < nt; ++t) syn[t] = (double)tr[t + c * nt];
      msf += oracle::ccts_trace(observed + c * nt, syn.data(), nt, ccts_dt, cres.data() + c * nt);
    }
    *misfit_out = msf;
  }
  std::vector<T> adjsrc(ntot);
  for (long q = 0; q < ntot; ++q) adjsrc[q] = (T)(-cres[q]);

  // gradient accumulators (ela_models.jl:353-368)
  Arr2<T> gl, gm, gri, grj, gmij;
  gl.init(nx, nz); gm.init(nx, nz); gri.init(nx - 1, nz); grj.init(nx, nz - 1); gmij.init(nx - 1, nz - 1);
  const T _dt2 = T(1) / (sim.dt * sim.dt);
  const bool ft = freetop != 0;
  for (int it = nt; it >= 1; --it) {
    bw.adjoint_step(it, adjsrc.data());
    if (!ck.issaved("ucur", it - 2)) {
      ck.initrecover();
      const Snap<T>& u0 = ck.getsaved("ucur", ck.curr_checkpoint - 1);
      const Snap<T>& u1 = ck.getsaved("ucur", ck.curr_checkpoint);
      sim.ux[sim.iold].v = u0[0]; sim.uz[sim.iold].v = u0[1];
      sim.ux[sim.icur].v = u1[0]; sim.uz[sim.icur].v = u1[1];
      sim.load_psi(ck.getsaved("psi", ck.curr_checkpoint));
      const int start = ck.curr_checkpoint + 1, end = ck.curr_checkpoint + ck.K - 1;
      for (int rit = start; rit <= end; ++rit) {
        fw.step(rit, nullptr);
        ck.buffer[rit - start + 1] = sim.snap_u();
      }
    }
    const Snap<T>& s0 = ck.getsaved("ucur", it - 2);
    const Snap<T>& s1 = ck.getsaved("ucur", it - 1);
    const Snap<T>& s2 = ck.getsaved("ucur", it);
    const Arr2<T>& aux = adj.ux[adj.icur];
    const Arr2<T>& auz = adj.uz[adj.icur];
    // correlate_gradient_rho_kernel! on the ux and uz grids
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 1; j <= nz; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        const size_t c = (size_t)(i - 1) + (size_t)(j - 1) * (nx - 1);
        const T v = aux(i, j) * (s0[0][c] - T(2) * s1[0][c] + s2[0][c]) * _dt2;
        if (j == 1 && ft) gri(i, j) += v / T(2);
        else gri(i, j) += v;
      }
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 1; j <= nz - 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t c = (size_t)(i - 1) + (size_t)(j - 1) * nx;
        grj(i, j) += auz(i, j) * (s0[1][c] - T(2) * s1[1][c] + s2[1][c]) * _dt2;
      }
    Arr2<T> fux, fuz;
    fux.n1 = nx - 1; fux.n2 = nz; fux.v = s1[0];
    fuz.n1 = nx; fuz.n2 = nz - 1; fuz.v = s1[1];
    const int jlo = ft ? 1 : 2;
    // correlate_gradient_lambda_mu_kernel!
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = jlo; j <= nz - 1; ++j)
      for (int i = 2; i <= nx - 1; ++i) {
        const T exx = sim.dux_dx(fux, i, j);
        const T exx_a = sim.dux_dx(aux, i, j);
        const T ezz = sim.duz_dz(fux, fuz, i, j);
        const T ezz_a = sim.duz_dz(aux, auz, i, j);
        const T div = exx + ezz, div_a = exx_a + ezz_a;
        if (j == 1 && ft) {
          gl(i, j) += div * div_a / T(2);
          gm(i, j) += (exx * exx_a + ezz * ezz_a);
        } else {
          gl(i, j) += div * div_a;
          gm(i, j) += T(2) * (exx * exx_a + ezz * ezz_a);
        }
      }
    // correlate_gradient_mu_ihalf_jhalf_kernel!
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int j = 1; j <= nz - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        const T exz = (sim.duz_dx(fuz, i, j) + sim.dux_dz(fux, i, j)) / T(2);
        const T exz_a = (sim.duz_dx(auz, i, j) + sim.dux_dz(aux, i, j)) / T(2);
        gmij(i, j) += T(2) * (exz * exz_a + exz * exz_a);
      }
  }
  // ela_gradient.jl:155-180: back-interpolation, then muting per position
  const size_t np = (size_t)nx * nz;
  std::vector<double> vr(np, 0.0), vl(np), vm(np);
  for (size_t c = 0; c < np; ++c) { vl[c] = (double)gl.v[c]; vm[c] = (double)gm.v[c]; }
  std::vector<double> dri(gri.v.begin(), gri.v.end()), drj(grj.v.begin(), grj.v.end()),
      dmij(gmij.v.begin(), gmij.v.end());
  back_interp(rho, nx, nz, dri.data(), nx - 1, 1, 0, irho, vr.data());
  back_interp(rho, nx, nz, drj.data(), nx, 0, 1, irho, vr.data());
  back_interp(mu, nx, nz, dmij.data(), nx - 1, 1, 1, imu, vm.data());
  const int nn[2] = {nx, nz};
  for (double* g : {vr.data(), vl.data(), vm.data()}) {
    for (int s = 0; s < sh.nsrc && mute_src > 0; ++s) {
      const double pt[2] = {src_pos[s], src_pos[s + sh.nsrc]};
      mute_around_point(g, 2, nn, h, pt, mute_src);
    }
    for (int r = 0; r < sh.nrec && mute_rec > 0; ++r) {
      const double pt[2] = {rec_pos[r], rec_pos[r + sh.nrec]};
      mute_around_point(g, 2, nn, h, pt, mute_rec);
    }
  }
  std::memcpy(g_rho, vr.data(), np * sizeof(double));
  std::memcpy(g_lam, vl.data(), np * sizeof(double));
  std::memcpy(g_mu, vm.data(), np * sizeof(double));
  return 0;
}

}  // namespace

extern "C" {

// spread_positions for npos positions (positions (npos, 2), column-major).
// Returns the total number of entries; when cnt/ij/coef are non-null, fills
// cnt[npos] and the concatenated (i, j) pairs and coefficients (capacity cap).
long oracle_spread_positions(const int* n, const double* h, int npos, const double* positions,
                             const double* shift, int mirror, int r, double beta, int* cnt, int* ij,
                             double* coef, long cap) {
  long q = 0;
  for (int p = 0; p < npos; ++p) {
    const double pos[2] = {positions[p], positions[p + npos]};
    Pts t = spread_one(n, h, pos, shift, mirror != 0, r, beta);
    if (cnt) cnt[p] = (int)t.c.size();
    for (size_t k = 0; k < t.c.size(); ++k, ++q)
      if (ij && q < cap) { ij[2 * q] = t.i[k]; ij[2 * q + 1] = t.j[k]; coef[q] = t.c[k]; }
  }
  return q;
}

double oracle_bessel_i0(double x) { return bessel_i0(x); }

// interp (interpolations.jl:1-43) of an (nx, nz) array to the half points of
// the axes with di / dj = 1; out is (nx - di, nz - dj).  method 0 arithmetic, 1 harmonic.
void oracle_interp(const double* m, int nx, int nz, int di, int dj, int method, double* out) {
  for (int j = 1; j <= nz - dj; ++j)
    for (int i = 1; i <= nx - di; ++i)
      out[(size_t)(i - 1) + (size_t)(j - 1) * (nx - di)] = interp_at(m, nx, i, j, di, dj, method);
}

// back_interp (interpolations.jl:15-28): g is (nx - di, nz - dj); res (nx, nz) is added to.
void oracle_back_interp(const double* m, int nx, int nz, const double* g, int di, int dj, int method, double* res) {
  back_interp(m, nx, nz, g, nx - di, di, dj, method, res);
}

int oracle_elastic_forward(int use_f32, const int* n, const double* h, double dt, int halo, int freetop,
                           const double* lam, const double* mu, const double* rho, int irho, int imu,
                           const double* cpml, int nt, int kind, int nsrc, const double* srctf,
                           const double* momtens, const int* src_cnt, const int* src_ij, const double* src_coef,
                           int nrec, const int* rec_cnt, const int* rec_ij, const double* rec_coef,
                           double* traces, int nthreads) {
  if (n[0] < 5 || n[1] < 5 || (kind != 0 && kind != 1)) return 1;
  ElShot sh = make_shot<double>(nt, kind, nsrc, srctf, momtens, src_cnt, src_ij, src_coef, nrec, rec_cnt,
                                rec_ij, rec_coef);
  if (use_f32)
    return run_forward<float>(n, h, dt, halo, freetop, lam, mu, rho, irho, imu, cpml, sh, traces, nthreads);
  return run_forward<double>(n, h, dt, halo, freetop, lam, mu, rho, irho, imu, cpml, sh, traces, nthreads);
}

int oracle_elastic_forward_snap(const int* n, const double* h, double dt, int halo, int freetop, const double* lam,
                                const double* mu, const double* rho, int irho, int imu, const double* cpml, int nt,
                                int kind, int nsrc, const double* srctf, const double* momtens, const int* src_cnt,
                                const int* src_ij, const double* src_coef, int nrec, const int* rec_cnt,
                                const int* rec_ij, const double* rec_coef, double* traces, int nthreads,
                                int snapevery, double* snaps) {
  if (n[0] < 5 || n[1] < 5 || (kind != 0 && kind != 1)) return 1;
  ElShot sh = make_shot<double>(nt, kind, nsrc, srctf, momtens, src_cnt, src_ij, src_coef, nrec, rec_cnt,
                                rec_ij, rec_coef);
  return run_forward<double>(n, h, dt, halo, freetop, lam, mu, rho, irho, imu, cpml, sh, traces, nthreads,
                             snapevery, snaps);
}

int oracle_elastic_gradient(int use_f32, const int* n, const double* h, double dt, int halo, int freetop,
                            const double* lam, const double* mu, const double* rho, int irho, int imu,
                            const double* cpml, int nt, int kind, int nsrc, const double* srctf,
                            const double* momtens, const int* src_cnt, const int* src_ij,
                            const double* src_coef, int nrec, const int* rec_cnt, const int* rec_ij,
                            const double* rec_coef, const double* observed, const double* invcov,
                            int invcov_kind, int nwin, const int* windows, int check_freq, int mute_src,
                            int mute_rec, const double* src_pos, const double* rec_pos, double* traces_out,
                            double* g_rho, double* g_lam, double* g_mu, double* misfit_out, int nthreads,
                            int ccts, double ccts_dt) {
  if (n[0] < 5 || n[1] < 5 || (kind != 0 && kind != 1)) return 1;
  ElShot sh = make_shot<double>(nt, kind, nsrc, srctf, momtens, src_cnt, src_ij, src_coef, nrec, rec_cnt,
                                rec_ij, rec_coef);
  if (use_f32)
    return run_gradient<float>(n, h, dt, halo, freetop, lam, mu, rho, irho, imu, cpml, sh, observed, invcov,
                               invcov_kind, nwin, windows, check_freq, mute_src, mute_rec, src_pos, rec_pos,
                               traces_out, g_rho, g_lam, g_mu, misfit_out, nthreads, ccts, ccts_dt);
  return run_gradient<double>(n, h, dt, halo, freetop, lam, mu, rho, irho, imu, cpml, sh, observed, invcov,
                              invcov_kind, nwin, windows, check_freq, mute_src, mute_rec, src_pos, rec_pos,
                              traces_out, g_rho, g_lam, g_mu, misfit_out, nthreads, ccts, ccts_dt);
}

}  // extern "C"
