// Host-side helpers of the GR entry points shared by the translation units
// that take a pic_gr_metric: the metric's validity check and the
// QKerrSchild constants in the grid's real_t.
#pragma once

#include <cmath>
#include <limits>

#include "ctx_internal.cuh"
#include "gr_metric.cuh"

namespace pic_internal {

using pic::kInvPiSqr;
using pic::kPi;
using pic::kSmallAngleGR;
using pic::QKS;

inline int gr_check(const pic_ctx* c, const pic_gr_metric* g) {
  if (!c || !g) return PIC_ERR_ARG;
  if (c->grid.dim != 2) return PIC_ERR_UNSUPPORTED;
  // the stretching theta(eta) is monotone for -1/2 < h < 1 (d theta / d eta
  // = 1 + 2h at the axes and 1 - h at the equator), and the reference's
  // closed-form inverse is real for h >= 0 (a square root of h^3 times a
  // factor positive for h < 1)
  if (!(g->h >= 0.0 && g->h < 1.0)) return PIC_ERR_ARG;
  if (!(g->x1min > g->r0) || !(g->x1max > g->x1min) || !(g->x2max > g->x2min)) return PIC_ERR_ARG;
  if (!(g->a >= 0.0 && g->a < 1.0)) return PIC_ERR_ARG;
  return PIC_OK;
}

// eta -> theta of the angle stretching (qkerr_schild.h:858-869), in real_t
template <typename real>
inline real qks_eta2theta(real h, real eta) {
  if (std::fabs(h) <= std::numeric_limits<real>::epsilon()) return eta;
  return eta + (real)2 * h * eta * ((real)kPi - (real)2 * eta) * ((real)kPi - eta) *
                 (real)kInvPiSqr;
}

// theta -> eta: the real root of the cubic theta = eta + 2 h eta (pi - 2 eta)
// (pi - eta) / pi^2 by Cardano's formula (qkerr_schild.h:886-912). The
// formula and its operation order are the reference's, so that eta_min and
// deta, and with them every metric value, round as the reference's do: the
// square and cube of h and the square of theta are real_t products, the
// rest is double. h = 0 is the identity.
template <typename real>
inline real qks_theta2eta(real h, real theta) {
  if (std::fabs(h) <= std::numeric_limits<real>::epsilon()) return theta;
  constexpr double pi = kPi, two_pi = 6.28318530717958647692, sqrt3 = 1.73205080756887729352;
  // pi^(2/3), pi^(1/3), 2^(2/3), 3^(1/3), 2^(1/3), (3 pi)^(2/3)
  constexpr double p23 = 2.14502939711102560008, p13 = 1.46459188756152326302;
  constexpr double t23 = 1.58740105196819947475, r13 = 1.442249570307408382321;
  constexpr double t13 = 1.2599210498948731647672, tp23 = 4.46184094890142313715794;
  const real   h2 = h * h, h3 = h * h * h, th2 = theta * theta;
  const double q  = (4.0 - h) * ((pi + h * two_pi) * (pi + h * two_pi)) -
                   108.0 * h * pi * theta + 108.0 * h * th2;
  const double R  = std::pow(-9.0 * h2 * (pi - 2.0 * theta) + sqrt3 * std::sqrt(h3 * q),
                             1.0 / 3.0);
  return (real)(p23 * (6.0 * p13 + 2.0 * t13 * (h - (real)1) * tp23 / R + t23 * r13 * R / h) /
                12.0);
}

// QKerrSchild's constructor (qkerr_schild.h:76-94) in real_t arithmetic,
// with the code coordinates of the pusher's polar clamp (gr.hpp:352-364):
// theta in [SMALL_ANGLE_GR, pi - SMALL_ANGLE_GR], the upper bound formed in
// double from the real_t lower one, as the pusher forms it
template <typename real>
inline QKS<double> make_qks(const pic_ctx* c, const pic_gr_metric* g) {
  QKS<double> m;
  const real  a = (real)g->a, r0 = (real)g->r0, h = (real)g->h;
  const real  chi_min = (real)std::log((real)g->x1min - r0);
  const real  eta_min = qks_theta2eta<real>(h, (real)g->x2min);
  const real  dchi    = ((real)std::log((real)g->x1max - r0) - chi_min) / (real)c->grid.n[0];
  const real  deta    = (qks_theta2eta<real>(h, (real)g->x2max) - eta_min) / (real)c->grid.n[1];
  const real  deta_inv = (real)1 / deta;
  m.a = a, m.r0 = r0, m.h0 = h, m.chi_min = chi_min, m.eta_min = eta_min;
  m.dchi = dchi, m.deta = deta, m.dchi_inv = (real)1 / dchi, m.deta_inv = deta_inv;
  m.small_angle = (double)qks_eta2theta<real>(h, (real)0.5 * deta) < 1e-3;
  const real small = (real)kSmallAngleGR;
  const real large = (real)(kPi - (double)small);
  m.x2_small = (qks_theta2eta<real>(h, small) - eta_min) * deta_inv;
  m.x2_large = (qks_theta2eta<real>(h, large) - eta_min) * deta_inv;
  return m;
}

}  // namespace pic_internal
