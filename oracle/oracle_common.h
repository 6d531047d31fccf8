// SPDX-License-Identifier: MIT
//
// TEST INFRASTRUCTURE ONLY -- pieces shared by the acoustic and elastic CPU
// oracles (sw_oracle.cpp, sw_elastic_oracle.cpp): C-PML coefficients, the
// linear checkpointer and gradient muting, restated from SeismicWaves.jl
// v0.9.0 (paths relative to its source tree).
#pragma once

#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------------------
// C-PML coefficients, cpmlcoeffs.jl:18-100 (K = 1, npower = 2)
// ---------------------------------------------------------------------------
inline void kab_side(int halo, double dt, double d0, double alpha_max, bool halfgrid,
              std::vector<double>& a_l, std::vector<double>& a_r,
              std::vector<double>& b_l, std::vector<double>& b_r) {
  const int nk = halfgrid ? halo : halo + 1;
  const double shift = halfgrid ? 0.5 : 0.0;
  a_l.assign(nk, 0.0); a_r.assign(nk, 0.0); b_l.assign(nk, 0.0); b_r.assign(nk, 0.0);
  for (int k = 0; k < nk; ++k) {
    // dist = LinRange(shift, nk + shift - 1, nk) -> shift + k
    const double dist_r = shift + k;
    const double dist_l = shift + (nk - 1 - k);  // reverse(dist)
    const double nl = halo != 0 ? dist_l / halo : dist_l;
    const double nr = halo != 0 ? dist_r / halo : dist_r;
    const double dl = d0 * (nl * nl), dr = d0 * (nr * nr);
    const double al = alpha_max * (1.0 - nl), ar = alpha_max * (1.0 - nr);
    b_l[k] = std::exp(-(dl + al) * dt);
    b_r[k] = std::exp(-(dr + ar) * dt);
    a_l[k] = dl * (b_l[k] - 1.0) / (dl + al);
    a_r[k] = dr * (b_r[k] - 1.0) / (dr + ar);
  }
}

// Output block per axis: a[2(halo+1)], a_h[2halo], b[2(halo+1)], b_h[2halo]
inline void cpml_axis(double vel_max, double dt, int halo, double rcoef, double h,
               double f0, bool freetop_axis, double* out) {
  const double thickness = h * halo;
  const double alpha_max = M_PI * f0;
  double d0 = -(2.0 + 1.0) * vel_max * std::log(rcoef) / (2.0 * thickness);
  if (halo == 0) d0 = 0.0;
  std::vector<double> al, ar, bl, br, ahl, ahr, bhl, bhr;
  kab_side(halo, dt, d0, alpha_max, false, al, ar, bl, br);
  kab_side(halo, dt, d0, alpha_max, true, ahl, ahr, bhl, bhr);
  const int na = 2 * (halo + 1), nh = 2 * halo;
  double* a = out;
  double* a_h = a + na;
  double* b = a_h + nh;
  double* b_h = b + na;
  for (int k = 0; k < halo + 1; ++k) { a[k] = al[k]; a[halo + 1 + k] = ar[k]; b[k] = bl[k]; b[halo + 1 + k] = br[k]; }
  for (int k = 0; k < halo; ++k) { a_h[k] = ahl[k]; a_h[halo + k] = ahr[k]; b_h[k] = bhl[k]; b_h[halo + k] = bhr[k]; }
  if (freetop_axis) {  // acou_init_bc.jl:32-39: first half of the last axis undamped
    for (int k = 0; k < na / 2; ++k) { a[k] = 0.0; b[k] = 1.0; }
    for (int k = 0; k < nh / 2; ++k) { a_h[k] = 0.0; b_h[k] = 1.0; }
  }
}

// ---------------------------------------------------------------------------
// Half-point interpolation and its chain rule, interpolations.jl:1-47
// ---------------------------------------------------------------------------
// Value at the half point whose lower corner is node (i, j) (1-based): the
// average over the 2 (di + dj = 1) or 4 corners, arithmetic (method 0) or
// harmonic (method 1).
inline double interp_at(const double* m, int nx, int i, int j, int di, int dj, int method) {
  // (i, j) 1-based lower corner; averages over the 2 or 4 corners
  double s = 0;
  int cnt = 0;
  for (int b = 0; b <= dj; ++b)
    for (int a = 0; a <= di; ++a) {
      const double v = m[(size_t)(i - 1 + a) + (size_t)(j - 1 + b) * nx];
      s += method == 1 ? 1.0 / v : v;
      ++cnt;
    }
  s /= cnt;
  return method == 1 ? 1.0 / s : s;
}

// back_interp, interpolations.jl:15-47: chain rule of the half-point
// interpolation back onto the (nx, nz) nodes.
inline void back_interp(const double* m, int nx, int nz, const double* g, int gx, int di, int dj, int method,
                        double* res) {
  const int gz = nz - dj;
  const double w0 = 1.0 / double((di + 1) * (dj + 1));
  for (int j = 1; j <= gz; ++j)
    for (int i = 1; i <= gx; ++i) {
      const double gv = g[(size_t)(i - 1) + (size_t)(j - 1) * gx];
      const double itp = method == 1 ? interp_at(m, nx, i, j, di, dj, 1) : 0.0;
      for (int pb = 0; pb <= dj; ++pb)
        for (int pa = 0; pa <= di; ++pa) {
          const size_t c = (size_t)(i - 1 + pa) + (size_t)(j - 1 + pb) * nx;
          double w = w0;
          if (method == 1) w = itp * itp / (m[c] * m[c]) * w0;
          res[c] += gv * w;
        }
    }
}

// ---------------------------------------------------------------------------
// CCTSMisfit for one trace, CCTSMisfit.jl:17-61 (scalar receivers).
// xcorr(u, v) (DSP.jl: conv(u, reverse(v)), length 2 nt - 1) has at 1-based
// index k the value sum_i u[i] v[i - (k - nt)]; the reference takes the first
// k of the largest |xcorr(observed, synthetic)| and dtau = (k - (nt - 1)) dt.
// Returns dtau^2 / 2 and writes dchi/du = dtau / N * ds/dt with ds/dt the
// central difference (first sample (s[2] - 0) / 2dt, last sample 0) and N the
// trapezoidal integral of (ds/dt)^2 over the times dt, 2 dt, ..., nt dt
// (NumericalIntegration.integrate).
// ---------------------------------------------------------------------------
inline double ccts_trace(const double* obs, const double* syn, int nt, double dt, double* dchi) {
  int kbest = 1;
  double best = -1.0;
  for (int k = 1; k <= 2 * nt - 1; ++k) {
    const int L = k - nt;
    double c = 0.0;
    for (int i = std::max(1, 1 + L); i <= std::min(nt, nt + L); ++i) c += obs[i - 1] * syn[i - 1 - L];
    if (std::fabs(c) > best) { best = std::fabs(c); kbest = k; }
  }
  const double dtau = (double)(kbest - (nt - 1)) * dt;
  std::vector<double> ds(nt, 0.0);
  for (int t = 2; t <= nt - 1; ++t) ds[t - 1] = (syn[t] - syn[t - 2]) / (2.0 * dt);
  if (nt >= 2) ds[0] = (syn[1] - 0.0) / (2.0 * dt);
  double norm = 0.0;
  for (int t = 1; t <= nt - 1; ++t) norm += dt * (ds[t - 1] * ds[t - 1] + ds[t] * ds[t]) / 2.0;
  for (int t = 0; t < nt; ++t) dchi[t] = (dtau / norm) * ds[t];
  return dtau * dtau / 2.0;
}

template <typename T>
using Snap = std::vector<std::vector<T>>;

// LinearCheckpointer, checkpointers.jl:1-107.  One field (`bname`: "pcur" for
// the acoustic paths, "ucur" for the elastic one) is buffered in a K+1 buffer
// and checkpointed with width `bwidth` (2 for the constant-density acoustic and
// the elastic simulations, 1 for the variable-density one); the others are
// checkpointed with width 1.
template <typename T>
struct LinearCheckpointer {
  int nt, K, last_checkpoint, curr_checkpoint;
  std::map<int, std::map<std::string, Snap<T>>> checkpoints;
  std::vector<Snap<T>> buffer;  // buffers[bname], K+1 entries

  std::string bname;
  int bwidth;

  LinearCheckpointer(int nt_, int K_, const std::map<std::string, Snap<T>>& proto,
                     const std::string& buffered = "pcur", int buffered_width = 2)
      : nt(nt_), K(K_), bname(buffered), bwidth(buffered_width) {
    last_checkpoint = (nt / K) * K;
    curr_checkpoint = last_checkpoint;
    for (int it = 0; it <= nt + 1; ++it) {
      if (it % K != 0) continue;
      for (auto& kv : proto) {
        const int w = kv.first == bname ? bwidth : 1;
        for (int itw = it; itw >= it - w + 1; --itw) {
          Snap<T> z = kv.second;
          for (auto& v : z) std::fill(v.begin(), v.end(), T(0));
          checkpoints[itw][kv.first] = z;
        }
      }
    }
    Snap<T> z = proto.at(bname);
    for (auto& v : z) std::fill(v.begin(), v.end(), T(0));
    buffer.assign(K + 1, z);
  }

  void save(const std::string& name, const Snap<T>& f, int it) {
    const int w = name == bname ? bwidth : 1;
    for (int itw = it; itw <= it + w - 1; ++itw)
      if (itw % K == 0) checkpoints[it][name] = f;
    if (name == bname && it >= last_checkpoint) buffer[it - last_checkpoint] = f;
  }
  bool isbuffered(const std::string& name, int it) const {
    return name == bname && curr_checkpoint <= it && it <= curr_checkpoint + K;
  }
  bool ischeckpointed(const std::string& name, int it) const {
    auto c = checkpoints.find(it);
    return c != checkpoints.end() && c->second.count(name);
  }
  bool issaved(const std::string& name, int it) const { return isbuffered(name, it) || ischeckpointed(name, it); }
  const Snap<T>& getsaved(const std::string& name, int it) const {
    if (ischeckpointed(name, it)) return checkpoints.at(it).at(name);
    return buffer.at(it - curr_checkpoint);
  }
  void initrecover() {
    const int old = curr_checkpoint;
    curr_checkpoint -= K;
    buffer[0] = checkpoints.at(curr_checkpoint).at(bname);
    buffer[K] = checkpoints.at(old).at(bname);
  }
  void reset() { curr_checkpoint = last_checkpoint; }
};

// mutearoundpoint!, mute_grad.jl:13-80 (radius in grid points, positions in metres)
inline void mute_around_point(double* g, int N, const int* n, const double* h, const double* pt, int radius) {
  if (radius == 0) return;
  double hmax = 0;
  for (int d = 0; d < N; ++d) hmax = std::max(hmax, h[d]);
  const double rmax = radius * hmax;
  int lo[3] = {1, 1, 1}, hi[3] = {1, 1, 1};
  for (int d = 0; d < N; ++d) {
    // ijkpt = floor(Int, div(x, h)) + 1 with Julia's float div (truncated quotient)
    const double q = std::round((pt[d] - std::fmod(pt[d], h[d])) / h[d]);
    const int ijk = (int)q + 1;
    lo[d] = ijk - radius; hi[d] = ijk + radius;
  }
  for (int k = lo[2]; k <= hi[2]; ++k)
    for (int j = lo[1]; j <= hi[1]; ++j)
      for (int i = lo[0]; i <= hi[0]; ++i) {
        const int I[3] = {i, j, k};
        bool inb = true;
        double r2 = 0;
        for (int d = 0; d < N; ++d) {
          if (!(1 <= I[d] && I[d] <= n[d])) { inb = false; break; }
          const double x = (I[d] - 1) * h[d];
          r2 += (pt[d] - x) * (pt[d] - x);
        }
        if (!inb) continue;
        const double r = std::sqrt(r2);
        if (r <= rmax) {
          const long c = (long)(i - 1) + (long)(j - 1) * n[0] + (long)(k - 1) * n[0] * (N == 3 ? n[1] : 1);
          g[c] *= r / rmax;
        }
      }
}

}  // namespace oracle
