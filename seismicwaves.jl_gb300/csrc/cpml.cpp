// C-PML damping coefficients on the host, the quantities
// compute_CPML_coefficientsAxis! / calc_Kab_CPML_axis produce
// (SeismicWaves.jl src/models/cpmlcoeffs.jl:18-100) with the free-surface
// override of src/models/acoustic/acou_init_bc.jl:32-39.
//
// Profile: d(r) = d0 r^2 with d0 = -3 vmax ln(R) / (2 L), L = halo*h;
// alpha(r) = pi f0 (1 - r); K = 1; b = exp(-(d + alpha) dt);
// a = d (b - 1) / (d + alpha).  r is the normalised distance into the layer,
// sampled on grid nodes (halo+1 values per side) and on half nodes (halo per
// side); the left side lists r from the outer edge inwards.
#include <cmath>
#include <vector>

#include "internal.h"

namespace swgb {

namespace {

void side(int halo, int count, double offset, double dt, double d0, double alpha_max, double* left,
          double* right, double* bleft, double* bright) {
  for (int k = 0; k < count; ++k) {
    const double r_right = halo ? (offset + k) / halo : (offset + k);
    const double r_left = halo ? (offset + (count - 1 - k)) / halo : (offset + (count - 1 - k));
    const double dr = d0 * r_right * r_right, dl = d0 * r_left * r_left;
    const double ar = alpha_max * (1.0 - r_right), al = alpha_max * (1.0 - r_left);
    const double br = std::exp(-(dr + ar) * dt), bl = std::exp(-(dl + al) * dt);
    bright[k] = br;
    bleft[k] = bl;
    right[k] = dr * (br - 1.0) / (dr + ar);
    left[k] = dl * (bl - 1.0) / (dl + al);
  }
}

}  // namespace

void cpml_axis_coefficients(double vel_max, double dt, int halo, double rcoef, double h, double f0,
                            bool freetop_axis, double* a, double* a_h, double* b, double* b_h) {
  const double alpha_max = M_PI * f0;
  const double d0 = halo == 0 ? 0.0 : -3.0 * vel_max * std::log(rcoef) / (2.0 * (h * halo));
  const int na = halo + 1, nh = halo;
  // on-grid nodes: distances 0..halo ; half nodes: 0.5..halo-0.5
  side(halo, na, 0.0, dt, d0, alpha_max, a, a + na, b, b + na);
  side(halo, nh, 0.5, dt, d0, alpha_max, a_h, a_h + nh, b_h, b_h + nh);
  if (freetop_axis) {
    for (int k = 0; k < na; ++k) { a[k] = 0.0; b[k] = 1.0; }
    for (int k = 0; k < nh; ++k) { a_h[k] = 0.0; b_h[k] = 1.0; }
  }
}

}  // namespace swgb
