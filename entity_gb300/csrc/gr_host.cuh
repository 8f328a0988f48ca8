// Host-side helpers of the GR entry points shared by the translation units
// that take a pic_gr_metric: the metric's validity check and the
// QKerrSchild constants in the grid's real_t.
#pragma once

#include <cmath>

#include "ctx_internal.cuh"
#include "gr_metric.cuh"

namespace pic_internal {

using pic::QKS;

inline int gr_check(const pic_ctx* c, const pic_gr_metric* g) {
  if (!c || !g) return PIC_ERR_ARG;
  if (c->grid.dim != 2) return PIC_ERR_UNSUPPORTED;
  if (g->h != 0.0) return PIC_ERR_UNSUPPORTED;
  if (!(g->x1min > g->r0) || !(g->x1max > g->x1min) || !(g->x2max > g->x2min)) return PIC_ERR_ARG;
  if (!(g->a >= 0.0 && g->a < 1.0)) return PIC_ERR_ARG;
  return PIC_OK;
}

// QKerrSchild's constructor (qkerr_schild.h:76-92) in real_t arithmetic
template <typename real>
inline QKS<double> make_qks(const pic_ctx* c, const pic_gr_metric* g) {
  QKS<double> m;
  const real  a = (real)g->a, r0 = (real)g->r0;
  const real  chi_min = (real)std::log((real)g->x1min - r0);
  const real  eta_min = (real)g->x2min;
  const real  dchi    = ((real)std::log((real)g->x1max - r0) - chi_min) / (real)c->grid.n[0];
  const real  deta    = ((real)g->x2max - eta_min) / (real)c->grid.n[1];
  m.a = a, m.r0 = r0, m.h0 = (real)g->h, m.chi_min = chi_min, m.eta_min = eta_min;
  m.dchi = dchi, m.deta = deta, m.dchi_inv = (real)1 / dchi, m.deta_inv = (real)1 / deta;
  m.small_angle = (double)((real)0.5 * deta) < 1e-3;
  return m;
}

}  // namespace pic_internal
