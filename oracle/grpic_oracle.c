/*
 * CPU oracle for the GR particle-in-cell path (TEST INFRASTRUCTURE ONLY).
 * See grpic_oracle.h for the contract; each function restates the cited
 * reference kernel in its operation order.
 */
#include "grpic_oracle.h"
#include "inject_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef ORC_SINGLE
typedef float real;
#define EPS_REAL FLT_EPSILON
#else
typedef double real;
#define EPS_REAL DBL_EPSILON
#endif

/* src/global/utils/numeric.h:91-103 */
#define ORC_PI             3.14159265358979323846
#define ORC_INV_PI         0.31830988618379067154
#define ORC_PI_SQR         9.86960440108935861882
#define ORC_INV_PI_SQR     0.10132118364233777144
#define ORC_SMALL_ANGLE    1e-3
#define ORC_SMALL_ANGLE_GR 1e-5

static const float  EPS_f = FLT_EPSILON;
static const double EPS_d = DBL_EPSILON;

#define MR   float
#define MSUF _f
#define MFN  f
#include "grpic_metric.inc"
#undef MR
#undef MSUF
#undef MFN

#define MR   double
#define MSUF _d
#define MFN
#include "grpic_metric.inc"
#undef MR
#undef MSUF
#undef MFN

#define EBI(g, i, j, c) \
  ((int64_t)(i) * (g)->em_s[0] + (int64_t)(j) * (g)->em_s[1] + (int64_t)(c) * (g)->em_s[3])
#define JI(g, i, j, c) \
  ((int64_t)(i) * (g)->cur_s[0] + (int64_t)(j) * (g)->cur_s[1] + (int64_t)(c) * (g)->cur_s[3])

/* the metric type of the oracle's own precision */
#ifdef ORC_SINGLE
typedef float mreal;
#define MT     qks_f
#define MK(q)  qks_make_f(q)
#define M_(fn) fn##_f
#else
typedef double mreal;
#define MT     qks_d
#define MK(q)  qks_make_d(q)
#define M_(fn) fn##_d
#endif

/* QKerrSchild::eta2theta (qkerr_schild.h:858-869), in real_t */
static real qks_eta2theta(real h, real eta) {
  if (fabs((double)h) <= (double)EPS_REAL) return eta;
  return eta + (real)2 * h * eta * ((real)ORC_PI - (real)2 * eta) * ((real)ORC_PI - eta) *
                 (real)ORC_INV_PI_SQR;
}

/* QKerrSchild::theta2eta (qkerr_schild.h:883-912): Cardano's root of the
 * cubic; h^2, h^3 and theta^2 are real_t products, the rest double */
static real qks_theta2eta(real h, real theta) {
  if (fabs((double)h) <= (double)EPS_REAL) return theta;
  const real   h2 = h * h, h3 = h * h * h, th2 = theta * theta;
  const double pp = ORC_PI + h * 6.28318530717958647692;
  const double q  = (4.0 - h) * (pp * pp) - 108.0 * h * ORC_PI * theta + 108.0 * h * th2;
  const double R  = pow(-9.0 * h2 * (ORC_PI - 2.0 * theta) + 1.73205080756887729352 * sqrt(h3 * q),
                        1.0 / 3.0);
  /* pi^(2/3), pi^(1/3), 2^(1/3), (3 pi)^(2/3), 2^(2/3), 3^(1/3) */
  return (real)(2.14502939711102560008 *
                (6.0 * 1.46459188756152326302 +
                 2.0 * 1.2599210498948731647672 * (h - (real)1) * 4.46184094890142313715794 / R +
                 1.58740105196819947475 * 1.442249570307408382321 * R / h) /
                12.0);
}

void orc_gr_convert_x2(const orc_qks* q, int to_code, const double* in, int64_t n, double* out) {
  const real h = (real)q->h, eta_min = (real)q->eta_min, deta = (real)q->deta;
  const real deta_inv = (real)q->deta_inv;
  for (int64_t k = 0; k < n; ++k) {
    const real x = (real)in[k];
    out[k] = to_code ? (double)((qks_theta2eta(h, x) - eta_min) * deta_inv)
                     : (double)qks_eta2theta(h, x * deta + eta_min);
  }
}

double orc_qks_theta2eta(double h, double theta) { return qks_theta2eta((real)h, (real)theta); }
double orc_qks_eta2theta(double h, double eta) { return qks_eta2theta((real)h, (real)eta); }

void orc_qks_init(orc_qks* q, int n1, int n2, double x1min, double x1max, double x2min,
                  double x2max, double a, double r0, double h) {
  /* QKerrSchild::QKerrSchild (qkerr_schild.h:76-94), in real_t */
  const real ar = (real)a, r0r = (real)r0, hr = (real)h;
  q->a   = ar;
  q->rh  = (real)((real)1 + (real)sqrt((double)((real)1 - ar * ar)));
  q->r0  = r0r;
  q->h   = hr;
  const real chi_min  = (real)log((double)((real)x1min - r0r));
  const real eta_min  = qks_theta2eta(hr, (real)x2min);
  const real dchi     = ((real)log((double)((real)x1max - r0r)) - chi_min) / (real)n1;
  const real deta     = (qks_theta2eta(hr, (real)x2max) - eta_min) / (real)n2;
  const real deta_inv = (real)1 / deta;
  q->chi_min  = chi_min;
  q->eta_min  = eta_min;
  q->dchi     = dchi;
  q->deta     = deta;
  q->dchi_inv = (real)1 / dchi;
  q->deta_inv = deta_inv;
  q->small_angle = (double)qks_eta2theta(hr, (real)0.5 * deta) < ORC_SMALL_ANGLE;
  /* gr.hpp:352-364: small is real_t, large = PI - small in double, both
   * converted through metric.convert<2, Ph, Cd> (qkerr_schild.h:636-640) */
  const real small = (real)ORC_SMALL_ANGLE_GR;
  const real large = (real)(ORC_PI - (double)small);
  q->x2_small = (qks_theta2eta(hr, small) - eta_min) * deta_inv;
  q->x2_large = (qks_theta2eta(hr, large) - eta_min) * deta_inv;
}

void orc_gr_metric(const orc_qks* q, const double* x, int64_t n, double* out) {
  const MT m = MK(q);
  for (int64_t k = 0; k < n; ++k) {
    const mreal xp[2] = { (mreal)x[2 * k], (mreal)x[2 * k + 1] };
    double*     o     = out + k * ORC_GR_NQ;
    o[0]  = M_(h_11)(&m, xp);
    o[1]  = M_(h_22)(&m, xp);
    o[2]  = M_(h_33)(&m, xp);
    o[3]  = M_(h_13)(&m, xp);
    o[4]  = M_(h11)(&m, xp);
    o[5]  = M_(h22)(&m, xp);
    o[6]  = M_(h33)(&m, xp);
    o[7]  = M_(h13)(&m, xp);
    o[8]  = M_(alpha)(&m, xp);
    o[9]  = M_(beta1)(&m, xp);
    o[10] = M_(sqrt_det_h)(&m, xp);
    o[11] = M_(sqrt_det_h_tilde)(&m, xp);
    o[12] = M_(dr_alpha)(&m, xp);
    o[13] = M_(dt_alpha)(&m, xp);
    o[14] = M_(dr_beta1)(&m, xp);
    o[15] = M_(dt_beta1)(&m, xp);
    o[16] = M_(dr_h11)(&m, xp);
    o[17] = M_(dr_h22)(&m, xp);
    o[18] = M_(dr_h33)(&m, xp);
    o[19] = M_(dr_h13)(&m, xp);
    o[20] = M_(dt_h11)(&m, xp);
    o[21] = M_(dt_h22)(&m, xp);
    o[22] = M_(dt_h33)(&m, xp);
    o[23] = M_(dt_h13)(&m, xp);
  }
}

void orc_gr_transform(const orc_qks* q, int kind, const double* x, const double* v, int64_t n,
                      double* out) {
  const MT m = MK(q);
  for (int64_t k = 0; k < n; ++k) {
    const mreal xp[2] = { (mreal)x[2 * k], (mreal)x[2 * k + 1] };
    const mreal vi[3] = { (mreal)v[3 * k], (mreal)v[3 * k + 1], (mreal)v[3 * k + 2] };
    mreal       vo[3];
    if (kind == 0) M_(d_to_u)(&m, xp, vi, vo);
    else if (kind == 1) M_(u_to_t)(&m, xp, vi, vo);
    else if (kind == 2) M_(d_to_t)(&m, xp, vi, vo);
    else M_(t_to_d)(&m, xp, vi, vo);
    for (int c = 0; c < 3; ++c) out[3 * k + c] = vo[c];
  }
}

/* from_Xi_to_i_di (gr.hpp:34-43) */
static void xi_to_i_di(real X, int* i, float* di) {
  *i  = (int)(X + (real)1) - 1;
  *di = (float)X - (float)(*i);
}

void orc_gr_push(const orc_grid* g, const orc_qks* q, orc_species* sp, const void* em,
                 const void* em0, double dt_d, double omegaB0, int niter, int order,
                 const int absorb[2], const int axis[2], int island_lo, int island_hi) {
  real*      u[3] = { (real*)sp->ux1, (real*)sp->ux2, (real*)sp->ux3 };
  const int  massive = sp->pusher != ORC_PUSHER_PHOTON;
  const real dt      = (real)dt_d;
  /* normalized_dt_half (gr.hpp:98-99) in real_t, with the float q/m */
  const real ndth = (real)0.5 * (real)(sp->charge / sp->mass) * (real)omegaB0 * dt;
  const qks_f mf = qks_make_f(q);
  const qks_d md = qks_make_d(q);
  if (sp->pusher == ORC_PUSHER_NONE) return;
  for (int64_t p = 0; p < sp->npart; ++p) {
    if (sp->tag[p] != ORC_TAG_ALIVE) continue;
    sp->i1_prev[p]  = sp->i1[p];
    sp->i2_prev[p]  = sp->i2[p];
    sp->dx1_prev[p] = sp->dx1[p];
    sp->dx2_prev[p] = sp->dx2[p];
    double Dc[3] = { 0, 0, 0 }, Bc[3] = { 0, 0, 0 };
    if (massive) orc_interp2(g, em, em0, order, sp->i1[p], sp->i2[p], sp->dx1[p], sp->dx2[p], Dc, Bc);
    real xo[2], uo[3];
#ifdef ORC_SINGLE
    const int dbl = sp->i1[p] >= island_lo && sp->i1[p] < island_hi;
#else
    const int dbl = 1;
    (void)island_lo;
    (void)island_hi;
#endif
    if (dbl) {
      /* i_di_to_Xi in real_t, then the island's double arithmetic */
      const double xp[2] = { (double)((real)sp->i1[p] + (real)sp->dx1[p]),
                             (double)((real)sp->i2[p] + (real)sp->dx2[p]) };
      const double ui[3] = { (double)u[0][p], (double)u[1][p], (double)u[2][p] };
      double       xd[2], ud[3];
      gr_push_one_d(&md, massive, (double)ndth, (double)dt, niter, xp, Dc, Bc, ui, xd, ud);
      xo[0] = (real)xd[0];
      xo[1] = (real)xd[1];
      for (int c = 0; c < 3; ++c) uo[c] = (real)ud[c];
    } else {
      const float xp[2] = { (float)((real)sp->i1[p] + (real)sp->dx1[p]),
                            (float)((real)sp->i2[p] + (real)sp->dx2[p]) };
      const float Df[3] = { (float)Dc[0], (float)Dc[1], (float)Dc[2] };
      const float Bf[3] = { (float)Bc[0], (float)Bc[1], (float)Bc[2] };
      const float ui[3] = { (float)u[0][p], (float)u[1][p], (float)u[2][p] };
      float       xf[2], uf[3];
      gr_push_one_f(&mf, massive, (float)ndth, (float)dt, niter, xp, Df, Bf, ui, xf, uf);
      xo[0] = (real)xf[0];
      xo[1] = (real)xf[1];
      for (int c = 0; c < 3; ++c) uo[c] = (real)uf[c];
    }
    int   i1, i2;
    float d1, d2;
    xi_to_i_di(xo[0], &i1, &d1);
    xi_to_i_di(xo[1], &i2, &d2);
    sp->i1[p]  = i1;
    sp->dx1[p] = d1;
    sp->i2[p]  = i2;
    sp->dx2[p] = d2;
    u[0][p] = uo[0];
    u[1][p] = uo[1];
    u[2][p] = uo[2];
    /* boundaryConditions (gr.hpp:818-865) */
    if ((sp->i1[p] < 0 && absorb[0]) || (sp->i1[p] >= g->n1 && absorb[1])) sp->tag[p] = ORC_TAG_DEAD;
    if (sp->i2[p] < 0) {
      if (axis[0]) {
        sp->i2[p]  = 0;
        sp->dx2[p] = 1.0f - sp->dx2[p];
        u[1][p]    = -u[1][p];
      }
    } else if (sp->i2[p] >= g->n2) {
      if (axis[1]) {
        sp->i2[p]  = g->n2 - 1;
        sp->dx2[p] = 1.0f - sp->dx2[p];
        u[1][p]    = -u[1][p];
      }
    }
  }
}

void orc_gr_deposit(const orc_grid* g, const orc_qks* q, const orc_species* sp, void* J,
                    double dt, int island_lo, int island_hi) {
  if (sp->pusher == ORC_PUSHER_NONE || sp->npart == 0 || sp->charge == 0.0f) return;
  const real* u[3] = { (const real*)sp->ux1, (const real*)sp->ux2, (const real*)sp->ux3 };
  real*       vz   = (real*)calloc((size_t)sp->npart, sizeof(real));
  const qks_f mf   = qks_make_f(q);
  const qks_d md   = qks_make_d(q);
  for (int64_t p = 0; p < sp->npart; ++p) {
    if (sp->tag[p] == ORC_TAG_DEAD) continue;
#ifdef ORC_SINGLE
    const int dbl = sp->i1[p] >= island_lo && sp->i1[p] < island_hi;
#else
    const int dbl = 1;
    (void)island_lo;
    (void)island_hi;
#endif
    if (dbl) {
      const double xp[2] = { (double)((real)sp->i1[p] + (real)sp->dx1[p]),
                             (double)((real)sp->i2[p] + (real)sp->dx2[p]) };
      const double ui[3] = { (double)u[0][p], (double)u[1][p], (double)u[2][p] };
      vz[p]              = (real)gr_vz_d(&md, xp, ui);
    } else {
      const float xp[2] = { (float)((real)sp->i1[p] + (real)sp->dx1[p]),
                            (float)((real)sp->i2[p] + (real)sp->dx2[p]) };
      const float ui[3] = { (float)u[0][p], (float)u[1][p], (float)u[2][p] };
      vz[p]             = (real)gr_vz_f(&mf, xp, ui);
    }
  }
  /* the GR deposit is hard-wired to shape order 1 (currents_deposit.hpp:33) */
  orc_deposit_vz(g, sp, J, 1, dt, vz);
  free(vz);
}

/* ------------------------------------------------------------------------ */
/* field kernels (2D). Metric values in real_t at the staggered points.      */
/* ------------------------------------------------------------------------ */
#define PT(a, b)  ((const real[2]){ (real)(a), (real)(b) })

void orc_gr_faraday(const orc_grid* g, const orc_qks* q, const void* Bin_, void* Bout_,
                    const void* E_, double coeff_d, int axis_min) {
  /* Faraday_kernel::operator() (faraday_gr.hpp:62-90) */
  const real* Bin  = (const real*)Bin_;
  real*       Bout = (real*)Bout_;
  const real* E    = (const real*)E_;
  const MT    m    = MK(q);
  const real  coeff = (real)coeff_d;
  const int   ng = g->ng, i2min = ng;
  for (int i2 = ng; i2 < g->n2 + ng; ++i2)
    for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
      const real i1_ = (real)(i1 - ng), i2_ = (real)(i2 - ng);
      const real inv_0pH  = (real)1 / M_(sqrt_det_h)(&m, PT(i1_, i2_ + (real)0.5));
      const real inv_pHpH = (real)1 / M_(sqrt_det_h)(&m, PT(i1_ + (real)0.5, i2_ + (real)0.5));
      Bout[EBI(g, i1, i2, 3)] = Bin[EBI(g, i1, i2, 3)] +
                                coeff * inv_0pH * (E[EBI(g, i1, i2, 2)] - E[EBI(g, i1, i2 + 1, 2)]);
      if (i2 == i2min && axis_min) {
        Bout[EBI(g, i1, i2, 4)] = 0;
      } else {
        const real inv_pH0 = (real)1 / M_(sqrt_det_h)(&m, PT(i1_ + (real)0.5, i2_));
        Bout[EBI(g, i1, i2, 4)] = Bin[EBI(g, i1, i2, 4)] +
                                  coeff * inv_pH0 * (E[EBI(g, i1 + 1, i2, 2)] - E[EBI(g, i1, i2, 2)]);
      }
      Bout[EBI(g, i1, i2, 5)] =
        Bin[EBI(g, i1, i2, 5)] +
        coeff * inv_pHpH *
          (E[EBI(g, i1, i2 + 1, 0)] - E[EBI(g, i1, i2, 0)] + E[EBI(g, i1, i2, 1)] -
           E[EBI(g, i1 + 1, i2, 1)]);
    }
}

void orc_gr_ampere(const orc_grid* g, const orc_qks* q, const void* Din_, void* Dout_,
                   const void* H_, double coeff_d, int axis_min, int axis_max) {
  /* Ampere_kernel::operator() (ampere_gr.hpp:66-98) */
  const real* Din  = (const real*)Din_;
  real*       Dout = (real*)Dout_;
  const real* H    = (const real*)H_;
  const MT    m    = MK(q);
  const real  coeff = (real)coeff_d;
  const int   ng = g->ng, i2min = ng, i2max = g->n2 + ng;
  for (int i2 = ng; i2 < i2max + 1; ++i2)
    for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
      const real i1_ = (real)(i1 - ng), i2_ = (real)(i2 - ng);
      if (i2 == i2min && axis_min) {
        const real inv = (real)1 / M_(sqrt_det_h)(&m, PT(i1_, (real)0.5));
        Dout[EBI(g, i1, i2, 1)] = Din[EBI(g, i1, i2, 1)] +
                                  coeff * inv * (H[EBI(g, i1 - 1, i2, 5)] - H[EBI(g, i1, i2, 5)]);
      } else if (i2 == i2max && axis_max) {
      } else {
        const real inv_0pH = (real)1 / M_(sqrt_det_h)(&m, PT(i1_, i2_ + (real)0.5));
        const real inv_00  = (real)1 / M_(sqrt_det_h)(&m, PT(i1_, i2_));
        const real inv_pH0 = (real)1 / M_(sqrt_det_h)(&m, PT(i1_ + (real)0.5, i2_));
        Dout[EBI(g, i1, i2, 0)] = Din[EBI(g, i1, i2, 0)] +
                                  coeff * inv_pH0 * (H[EBI(g, i1, i2, 5)] - H[EBI(g, i1, i2 - 1, 5)]);
        Dout[EBI(g, i1, i2, 1)] = Din[EBI(g, i1, i2, 1)] +
                                  coeff * inv_0pH * (H[EBI(g, i1 - 1, i2, 5)] - H[EBI(g, i1, i2, 5)]);
        Dout[EBI(g, i1, i2, 2)] =
          Din[EBI(g, i1, i2, 2)] +
          coeff * inv_00 *
            ((H[EBI(g, i1, i2 - 1, 3)] - H[EBI(g, i1, i2, 3)]) +
             (H[EBI(g, i1, i2, 4)] - H[EBI(g, i1 - 1, i2, 4)]));
      }
    }
  /* the axis cells copy dx1 from their neighbour row; that row is read
   * after its own update (the reference reads it unordered) */
  for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
    if (axis_min) Dout[EBI(g, i1, i2min, 0)] = Din == Dout ? Dout[EBI(g, i1, i2min + 1, 0)]
                                                           : Din[EBI(g, i1, i2min + 1, 0)];
    if (axis_max) Dout[EBI(g, i1, i2max, 0)] = Din == Dout ? Dout[EBI(g, i1, i2max - 1, 0)]
                                                           : Din[EBI(g, i1, i2max - 1, 0)];
  }
}

void orc_gr_currents_ampere(const orc_grid* g, const orc_qks* q, void* D_, const void* J_,
                            double coeff_d, int axis_min, int axis_max) {
  /* CurrentsAmpere_kernel::operator() (ampere_gr.hpp:143-172) */
  real*       D = (real*)D_;
  const real* J = (const real*)J_;
  const MT    m = MK(q);
  const real  coeff = (real)coeff_d;
  const int   ng = g->ng, i2min = ng, i2max = g->n2 + ng;
  for (int i2 = ng; i2 < i2max + 1; ++i2)
    for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
      const real i1_ = (real)(i1 - ng), i2_ = (real)(i2 - ng);
      const real inv_0pH = (real)1 / M_(sqrt_det_h)(&m, PT(i1_, i2_ + (real)0.5));
      if (i2 == i2min && axis_min) {
        D[EBI(g, i1, i2, 0)] += J[JI(g, i1, i2, 0)] * (real)0.5 * coeff /
                                M_(polar_area)(&m, i1_ + (real)0.5);
        D[EBI(g, i1, i2, 1)] += J[JI(g, i1, i2, 1)] * coeff * inv_0pH;
      } else if (i2 == i2max && axis_max) {
        D[EBI(g, i1, i2, 0)] += J[JI(g, i1, i2, 0)] * (real)0.5 * coeff /
                                M_(polar_area)(&m, i1_ + (real)0.5);
      } else {
        const real inv_00  = (real)1 / M_(sqrt_det_h)(&m, PT(i1_, i2_));
        const real inv_pH0 = (real)1 / M_(sqrt_det_h)(&m, PT(i1_ + (real)0.5, i2_));
        D[EBI(g, i1, i2, 0)] += J[JI(g, i1, i2, 0)] * coeff * inv_pH0;
        D[EBI(g, i1, i2, 1)] += J[JI(g, i1, i2, 1)] * coeff * inv_0pH;
        D[EBI(g, i1, i2, 2)] += J[JI(g, i1, i2, 2)] * coeff * inv_00;
      }
    }
}

void orc_gr_aux_e(const orc_grid* g, const orc_qks* q, const void* D_, const void* B_, void* E_,
                  int axis_max) {
  /* ComputeAuxE_kernel::operator() (aux_fields_gr.hpp:47-109) */
  const real* Df = (const real*)D_;
  const real* Bf = (const real*)B_;
  real*       Ef = (real*)E_;
  const MT    m  = MK(q);
  const real  H_ = (real)0.5;
  const int   ng = g->ng;
  const int   j1 = g->n2 + ng + (axis_max ? 1 : 0);
  for (int i2 = ng; i2 < j1; ++i2)
    for (int i1 = ng - 1; i1 < g->n1 + ng; ++i1) {
      const real i1_ = (real)(i1 - ng), i2_ = (real)(i2 - ng);
      const real h_11_pH0  = M_(h_11)(&m, PT(i1_ + H_, i2_));
      const real h_22_0pH  = M_(h_22)(&m, PT(i1_, i2_ + H_));
      const real h_33_00   = M_(h_33)(&m, PT(i1_, i2_));
      const real alpha_00  = M_(alpha)(&m, PT(i1_, i2_));
      const real alpha_pH0 = M_(alpha)(&m, PT(i1_ + H_, i2_));
      const real alpha_0pH = M_(alpha)(&m, PT(i1_, i2_ + H_));
      real w1, w2, ww, h1, h2, s1, s2, b1, b2;
      w1 = M_(sqrt_det_h_tilde)(&m, PT(i1_ - H_, i2_));
      w2 = M_(sqrt_det_h_tilde)(&m, PT(i1_ + H_, i2_));
      ww = (real)2 * M_(sqrt_det_h_tilde)(&m, PT(i1_, i2_));
      h1 = M_(h_13)(&m, PT(i1_ - H_, i2_));
      h2 = M_(h_13)(&m, PT(i1_ + H_, i2_));
      const real D1_half = (w1 * h1 * Df[EBI(g, i1 - 1, i2, 0)] + w2 * h2 * Df[EBI(g, i1, i2, 0)]) / ww;
      s1 = M_(sqrt_det_h)(&m, PT(i1_ - H_, i2_));
      s2 = M_(sqrt_det_h)(&m, PT(i1_ + H_, i2_));
      b1 = M_(beta1)(&m, PT(i1_ - H_, i2_));
      b2 = M_(beta1)(&m, PT(i1_ + H_, i2_));
      const real B2_half =
        (w1 * s1 * b1 * Bf[EBI(g, i1 - 1, i2, 4)] + w2 * s2 * b2 * Bf[EBI(g, i1, i2, 4)]) / ww;
      w1 = M_(sqrt_det_h_tilde)(&m, PT(i1_ - H_, i2_ + H_));
      w2 = M_(sqrt_det_h_tilde)(&m, PT(i1_ + H_, i2_ + H_));
      ww = (real)2 * M_(sqrt_det_h_tilde)(&m, PT(i1_, i2_ + H_));
      s1 = M_(sqrt_det_h)(&m, PT(i1_ - H_, i2_ + H_));
      s2 = M_(sqrt_det_h)(&m, PT(i1_ + H_, i2_ + H_));
      b1 = M_(beta1)(&m, PT(i1_ - H_, i2_ + H_));
      b2 = M_(beta1)(&m, PT(i1_ + H_, i2_ + H_));
      const real B3_half =
        (w1 * s1 * b1 * Bf[EBI(g, i1 - 1, i2, 5)] + w2 * s2 * b2 * Bf[EBI(g, i1, i2, 5)]) / ww;
      w1 = M_(sqrt_det_h_tilde)(&m, PT(i1_, i2_));
      w2 = M_(sqrt_det_h_tilde)(&m, PT(i1_ + (real)1, i2_));
      ww = (real)2 * M_(sqrt_det_h_tilde)(&m, PT(i1_ + H_, i2_));
      h1 = M_(h_13)(&m, PT(i1_, i2_));
      h2 = M_(h_13)(&m, PT(i1_ + (real)1, i2_));
      const real D3_half = (w1 * h1 * Df[EBI(g, i1, i2, 2)] + w2 * h2 * Df[EBI(g, i1 + 1, i2, 2)]) / ww;
      const real D1_cov = h_11_pH0 * Df[EBI(g, i1, i2, 0)] + D3_half;
      const real D2_cov = h_22_0pH * Df[EBI(g, i1, i2, 1)];
      const real D3_cov = h_33_00 * Df[EBI(g, i1, i2, 2)] + D1_half;
      Ef[EBI(g, i1, i2, 0)] = alpha_pH0 * D1_cov;
      Ef[EBI(g, i1, i2, 1)] = alpha_0pH * D2_cov - B3_half;
      Ef[EBI(g, i1, i2, 2)] = alpha_00 * D3_cov + B2_half;
    }
}

void orc_gr_aux_h(const orc_grid* g, const orc_qks* q, const void* D_, const void* B_, void* H_f,
                  int axis_max) {
  /* ComputeAuxH_kernel::operator() (aux_fields_gr.hpp:131-193) */
  const real* Df = (const real*)D_;
  const real* Bf = (const real*)B_;
  real*       Hf = (real*)H_f;
  const MT    m  = MK(q);
  const real  H_ = (real)0.5;
  const int   ng = g->ng;
  const int   j1 = g->n2 + ng + (axis_max ? 1 : 0);
  for (int i2 = ng; i2 < j1; ++i2)
    for (int i1 = ng - 1; i1 < g->n1 + ng; ++i1) {
      const real i1_ = (real)(i1 - ng), i2_ = (real)(i2 - ng);
      const real h_11_0pH   = M_(h_11)(&m, PT(i1_, i2_ + H_));
      const real h_22_pH0   = M_(h_22)(&m, PT(i1_ + H_, i2_));
      const real h_33_pHpH  = M_(h_33)(&m, PT(i1_ + H_, i2_ + H_));
      const real alpha_0pH  = M_(alpha)(&m, PT(i1_, i2_ + H_));
      const real alpha_pH0  = M_(alpha)(&m, PT(i1_ + H_, i2_));
      const real alpha_pHpH = M_(alpha)(&m, PT(i1_ + H_, i2_ + H_));
      real w1, w2, ww, h1, h2, s1, s2, b1, b2;
      w1 = M_(sqrt_det_h_tilde)(&m, PT(i1_, i2_ + H_));
      w2 = M_(sqrt_det_h_tilde)(&m, PT(i1_ + (real)1, i2_ + H_));
      ww = (real)2 * M_(sqrt_det_h_tilde)(&m, PT(i1_ + H_, i2_ + H_));
      h1 = M_(h_13)(&m, PT(i1_, i2_ + H_));
      h2 = M_(h_13)(&m, PT(i1_ + (real)1, i2_ + H_));
      const real B1_half = (w1 * h1 * Bf[EBI(g, i1, i2, 3)] + w2 * h2 * Bf[EBI(g, i1 + 1, i2, 3)]) / ww;
      s1 = M_(sqrt_det_h)(&m, PT(i1_, i2_ + H_));
      s2 = M_(sqrt_det_h)(&m, PT(i1_ + (real)1, i2_ + H_));
      b1 = M_(beta1)(&m, PT(i1_, i2_ + H_));
      b2 = M_(beta1)(&m, PT(i1_ + (real)1, i2_ + H_));
      const real D2_half =
        (w1 * s1 * b1 * Df[EBI(g, i1, i2, 1)] + w2 * s2 * b2 * Df[EBI(g, i1 + 1, i2, 1)]) / ww;
      w1 = M_(sqrt_det_h_tilde)(&m, PT(i1_, i2_));
      w2 = M_(sqrt_det_h_tilde)(&m, PT(i1_ + (real)1, i2_));
      ww = (real)2 * M_(sqrt_det_h_tilde)(&m, PT(i1_ + H_, i2_));
      s1 = M_(sqrt_det_h)(&m, PT(i1_, i2_));
      s2 = M_(sqrt_det_h)(&m, PT(i1_ + (real)1, i2_));
      b1 = M_(beta1)(&m, PT(i1_, i2_));
      b2 = M_(beta1)(&m, PT(i1_ + (real)1, i2_));
      const real D3_half =
        (w1 * s1 * b1 * Df[EBI(g, i1, i2, 2)] + w2 * s2 * b2 * Df[EBI(g, i1 + 1, i2, 2)]) / ww;
      w1 = M_(sqrt_det_h_tilde)(&m, PT(i1_ - H_, i2_ + H_));
      w2 = M_(sqrt_det_h_tilde)(&m, PT(i1_ + H_, i2_ + H_));
      ww = (real)2 * M_(sqrt_det_h_tilde)(&m, PT(i1_, i2_ + H_));
      h1 = M_(h_13)(&m, PT(i1_ - H_, i2_ + H_));
      h2 = M_(h_13)(&m, PT(i1_ + H_, i2_ + H_));
      const real B3_half = (w1 * h1 * Bf[EBI(g, i1 - 1, i2, 5)] + w2 * h2 * Bf[EBI(g, i1, i2, 5)]) / ww;
      const real B1_cov = h_11_0pH * Bf[EBI(g, i1, i2, 3)] + B3_half;
      const real B2_cov = h_22_pH0 * Bf[EBI(g, i1, i2, 4)];
      const real B3_cov = h_33_pHpH * Bf[EBI(g, i1, i2, 5)] + B1_half;
      Hf[EBI(g, i1, i2, 3)] = alpha_0pH * B1_cov;
      Hf[EBI(g, i1, i2, 4)] = alpha_pH0 * B2_cov + D3_half;
      Hf[EBI(g, i1, i2, 5)] = alpha_pHpH * B3_cov - D2_half;
    }
}

void orc_gr_average_db(const orc_grid* g, const void* f_, void* f0_) {
  /* TimeAverageDB_kernel (aux_fields_gr.hpp:222-250) */
  const real* f  = (const real*)f_;
  real*       f0 = (real*)f0_;
  const int   ng = g->ng;
  for (int i2 = ng; i2 < g->n2 + ng; ++i2)
    for (int i1 = ng; i1 < g->n1 + ng; ++i1)
      for (int c = 0; c < 6; ++c)
        f0[EBI(g, i1, i2, c)] = (real)0.5 * (f0[EBI(g, i1, i2, c)] + f[EBI(g, i1, i2, c)]);
}

void orc_gr_average_j(const orc_grid* g, void* J_, const void* J0_) {
  /* TimeAverageJ_kernel (aux_fields_gr.hpp:260-280) */
  real*       J  = (real*)J_;
  const real* J0 = (const real*)J0_;
  const int   ng = g->ng;
  for (int i2 = ng; i2 < g->n2 + ng; ++i2)
    for (int i1 = ng; i1 < g->n1 + ng; ++i1)
      for (int c = 0; c < 3; ++c)
        J[JI(g, i1, i2, c)] = (real)0.5 * (J0[JI(g, i1, i2, c)] + J[JI(g, i1, i2, c)]);
}

void orc_gr_filter_pass(const orc_grid* g, void* J_, void* buff_, int axis_min, int axis_max) {
  /* grpic::CurrentsFilter (src/engines/grpic/currents.h:74-101), one pass:
   * buff <- cur0 (the whole array), then DigitalFilter_kernel's 2D
   * non-Cartesian branch (src/kernels/digital_filter.hpp:196-276) over
   * i1 in [i1min, i1max), i2 in [i2min, i2max] with the axis rows */
  /* src/global/utils/numeric.h: ZERO, INV_2, INV_4, INV_8, INV_16 */
  const real  ZERO = 0, INV_2 = 0.5, INV_4 = 0.25, INV_8 = 0.125, INV_16 = 0.0625;
  real*       J  = (real*)J_;
  real*       B  = (real*)buff_;
  const int   ng = g->ng;
  const int   N1 = g->n1 + 2 * ng, N2 = g->n2 + 2 * ng;
  for (int i2 = 0; i2 < N2; ++i2)
    for (int i1 = 0; i1 < N1; ++i1)
      for (int c = 0; c < 3; ++c) B[JI(g, i1, i2, c)] = J[JI(g, i1, i2, c)];
  const int   i2min = ng, i2max = g->n2 + ng;
#define F1(c, a, b) (INV_2 * B[JI(g, a, b, c)] + INV_4 * (B[JI(g, (a) - 1, b, c)] + B[JI(g, (a) + 1, b, c)]))
  for (int i2 = i2min; i2 <= i2max; ++i2) {
    for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
      real c00, c0p1, c0m1;
      if (axis_min && i2 == i2min) {
        c00  = F1(0, i1, i2);
        c0p1 = F1(0, i1, i2 + 1);
        J[JI(g, i1, i2, 0)] = INV_2 * c00 + INV_2 * c0p1;
        J[JI(g, i1, i2, 2)] = ZERO;
        c00  = F1(1, i1, i2);
        c0p1 = F1(1, i1, i2 + 1);
        J[JI(g, i1, i2, 1)] = INV_4 * (c00 + c0p1);
      } else if (axis_min && i2 == i2min + 1) {
        c00  = F1(0, i1, i2);
        c0p1 = F1(0, i1, i2 + 1);
        c0m1 = F1(0, i1, i2 - 1);
        J[JI(g, i1, i2, 0)] = INV_2 * c00 + INV_4 * (c0p1 + c0m1);
        c00  = F1(2, i1, i2);
        c0p1 = F1(2, i1, i2 + 1);
        J[JI(g, i1, i2, 2)] = INV_2 * c00 + INV_4 * c0p1;
        c00  = F1(1, i1, i2);
        c0p1 = F1(1, i1, i2 + 1);
        c0m1 = F1(1, i1, i2 - 1);
        J[JI(g, i1, i2, 1)] = INV_2 * c00 + INV_4 * (c0m1 + c0p1);
      } else if (axis_max && i2 == i2max - 1) {
        c00  = F1(0, i1, i2);
        c0p1 = F1(0, i1, i2 + 1);
        c0m1 = F1(0, i1, i2 - 1);
        J[JI(g, i1, i2, 0)] = INV_2 * c00 + INV_4 * (c0m1 + c0p1);
        c00  = F1(2, i1, i2);
        c0m1 = F1(2, i1, i2 - 1);
        J[JI(g, i1, i2, 2)] = INV_2 * c00 + INV_4 * c0m1;
        c00  = F1(1, i1, i2);
        c0m1 = F1(1, i1, i2 - 1);
        J[JI(g, i1, i2, 1)] = INV_4 * (c00 + c0m1);
      } else if (axis_max && i2 == i2max) {
        c00  = F1(0, i1, i2);
        c0m1 = F1(0, i1, i2 - 1);
        J[JI(g, i1, i2, 0)] = INV_2 * c00 + INV_2 * c0m1;
        J[JI(g, i1, i2, 2)] = ZERO;
      } else {
        for (int c = 0; c < 3; ++c) {
          J[JI(g, i1, i2, c)] =
            INV_4 * B[JI(g, i1, i2, c)] +
            INV_8 * (B[JI(g, i1 - 1, i2, c)] + B[JI(g, i1 + 1, i2, c)] +
                     B[JI(g, i1, i2 - 1, c)] + B[JI(g, i1, i2 + 1, c)]) +
            INV_16 * (B[JI(g, i1 - 1, i2 - 1, c)] + B[JI(g, i1 + 1, i2 + 1, c)] +
                      B[JI(g, i1 - 1, i2 + 1, c)] + B[JI(g, i1 + 1, i2 - 1, c)]);
        }
      }
    }
  }
#undef F1
}

void orc_gr_field_bcs(const orc_grid* g, void* fld_, int set_e, int set_b, int axis_min,
                      int axis_max, int horizon, int nfilter) {
  real*     F  = (real*)fld_;
  const int ng = g->ng;
  const int N1 = g->n1 + 2 * ng;
  /* the sides in Directions<2>::orth order (grpic/fields_bcs.h:242-252):
   * the horizon (-x1) first, then the axes (-x2, +x2) */
  /* HorizonBoundaries_kernel (fields_bcs.hpp:1188-1240) over i2 in
   * [i2min, i2max + 1) */
  if (horizon) {
    const int i1min = ng;
    for (int i2 = ng; i2 < g->n2 + ng + 1; ++i2) {
      if (set_e)
        for (int i = 0; i <= 2 + nfilter; ++i)
          for (int c = 0; c < 3; ++c)
            F[EBI(g, i1min - ng + i, i2, c)] = F[EBI(g, i1min + 1 + nfilter, i2, c)];
      if (set_b)
        for (int i = 0; i <= 2 + nfilter; ++i)
          for (int c = 3; c < 6; ++c)
            F[EBI(g, i1min - ng + i, i2, c)] = F[EBI(g, i1min + 1 + nfilter, i2, c)];
    }
  }
  /* AxisBoundaries_kernel (fields_bcs.hpp:825-868) */
  if (axis_min) {
    const int e = ng;
    for (int i1 = 0; i1 < N1; ++i1) {
      if (set_e) {
        F[EBI(g, i1, e - 1, 1)] = -F[EBI(g, i1, e, 1)];
        F[EBI(g, i1, e, 2)]     = 0;
        F[EBI(g, i1, e - 1, 2)] = F[EBI(g, i1, e + 1, 2)];
      }
      if (set_b) {
        F[EBI(g, i1, e - 1, 3)] = F[EBI(g, i1, e, 3)];
        F[EBI(g, i1, e, 4)]     = 0;
        F[EBI(g, i1, e - 1, 4)] = -F[EBI(g, i1, e + 1, 4)];
        F[EBI(g, i1, e - 1, 5)] = F[EBI(g, i1, e, 5)];
      }
    }
  }
  if (axis_max) {
    const int e = g->n2 + ng;
    for (int i1 = 0; i1 < N1; ++i1) {
      if (set_e) {
        F[EBI(g, i1, e, 1)]     = -F[EBI(g, i1, e - 1, 1)];
        F[EBI(g, i1, e, 2)]     = 0;
        F[EBI(g, i1, e + 1, 2)] = F[EBI(g, i1, e - 1, 2)];
      }
      if (set_b) {
        F[EBI(g, i1, e, 3)]     = F[EBI(g, i1, e - 1, 3)];
        F[EBI(g, i1, e, 4)]     = 0;
        F[EBI(g, i1, e + 1, 4)] = -F[EBI(g, i1, e - 1, 4)];
        F[EBI(g, i1, e, 5)]     = F[EBI(g, i1, e - 1, 5)];
      }
    }
  }
}

/* the +x1 match layer's cells (MatchFieldsIn, grpic/fields_bcs.h:53-92, and
 * Mesh::ExtentToRange, mesh.h:133-202), x1 end clamped to the array */
static void match_range(const orc_grid* g, const orc_qks* q, double ds, double r_lo, double r_hi,
                        int* i0, int* i1) {
  const real r0 = (real)q->r0, chi_min = (real)q->chi_min, dchi_inv = (real)q->dchi_inv;
  const real hi = (real)r_hi, lo_raw = (real)r_hi - (real)ds;
  const real lo = lo_raw < (real)r_lo ? (real)r_lo : (lo_raw > hi ? hi : lo_raw);
#ifdef ORC_SINGLE
  const real xlo = (logf(lo - r0) - chi_min) * dchi_inv, xhi = (logf(hi - r0) - chi_min) * dchi_inv;
  int        a = (int)floorf(xlo) + g->ng, b = (int)ceilf(xhi) + 2 * g->ng;
#else
  const real xlo = (log(lo - r0) - chi_min) * dchi_inv, xhi = (log(hi - r0) - chi_min) * dchi_inv;
  int        a = (int)floor(xlo) + g->ng, b = (int)ceil(xhi) + 2 * g->ng;
#endif
  if (a < g->ng) a = g->ng;
  if (b > g->n1 + 2 * g->ng) b = g->n1 + 2 * g->ng;
  *i0 = a;
  *i1 = b < a ? a : b;
}

/* the radius at code coordinate x1 (QKerrSchild::convert<1, Cd, Ph>) */
static real r_of(const orc_qks* q, real x1) {
#ifdef ORC_SINGLE
  return (real)q->r0 + expf(x1 * (real)q->dchi + (real)q->chi_min);
#else
  return (real)q->r0 + exp(x1 * (real)q->dchi + (real)q->chi_min);
#endif
}

/* MatchBoundaries_kernel, GRPIC branch, 2D, o = x1 (fields_bcs.hpp:181-340) */
void orc_gr_match(const orc_grid* g, const orc_qks* q, void* fld_, const void* tgt_, double ds,
                  double r_lo, double r_hi, int set_e, int set_b, int axis_min, int axis_max) {
  real*       F = (real*)fld_;
  const real* T = (const real*)tgt_;
  int         i0, i1e;
  match_range(g, q, ds, r_lo, r_hi, &i0, &i1e);
  const real H = 0.5, ONE = 1, FOUR = 4, edge = (real)r_hi, dsr = (real)ds;
  const int  N2 = g->n2 + 2 * g->ng;
  for (int i1 = i0; i1 < i1e; ++i1) {
    const real i1_ = (real)(i1 - g->ng);
#ifdef ORC_SINGLE
    const real sH = tanhf(fabsf(r_of(q, i1_ + H) - edge) * FOUR / dsr);
    const real s0 = tanhf(fabsf(r_of(q, i1_) - edge) * FOUR / dsr);
#else
    const real sH = tanh(fabs(r_of(q, i1_ + H) - edge) * FOUR / dsr);
    const real s0 = tanh(fabs(r_of(q, i1_) - edge) * FOUR / dsr);
#endif
    for (int i2 = 0; i2 < N2; ++i2) {
      if (set_e) {
        F[EBI(g, i1, i2, 0)] = sH * F[EBI(g, i1, i2, 0)] + (ONE - sH) * T[EBI(g, i1, i2, 0)];
        F[EBI(g, i1, i2, 1)] = s0 * F[EBI(g, i1, i2, 1)] + (ONE - s0) * T[EBI(g, i1, i2, 1)];
        F[EBI(g, i1, i2, 2)] = s0 * F[EBI(g, i1, i2, 2)];
        if ((!axis_min || i2 > g->ng) && (!axis_max || i2 < N2 - g->ng))
          F[EBI(g, i1, i2, 2)] += (ONE - s0) * T[EBI(g, i1, i2, 2)];
      }
      if (set_b) {
        F[EBI(g, i1, i2, 3)] = s0 * F[EBI(g, i1, i2, 3)] + (ONE - s0) * T[EBI(g, i1, i2, 3)];
        F[EBI(g, i1, i2, 4)] = sH * F[EBI(g, i1, i2, 4)] + (ONE - sH) * T[EBI(g, i1, i2, 4)];
        F[EBI(g, i1, i2, 5)] = sH * F[EBI(g, i1, i2, 5)] + (ONE - sH) * T[EBI(g, i1, i2, 5)];
      }
    }
  }
}

/* gr::AbsorbCurrents_kernel<M, 1> (fields_bcs.hpp:1243-1280) */
void orc_gr_absorb_currents(const orc_grid* g, const orc_qks* q, void* J_, double ds,
                            double r_lo, double r_hi) {
  real* J = (real*)J_;
  int   i0, i1e;
  match_range(g, q, ds, r_lo, r_hi, &i0, &i1e);
  const real INV_4 = 0.25, edge = (real)r_hi, dsr = (real)ds;
  const int  N2 = g->n2 + 2 * g->ng;
  for (int i1 = i0; i1 < i1e; ++i1) {
    const real i1_ = (real)(i1 - g->ng);
#ifdef ORC_SINGLE
    const real t = tanhf(fabsf(r_of(q, i1_) - edge) / (INV_4 * dsr));
#else
    const real t = tanh(fabs(r_of(q, i1_) - edge) / (INV_4 * dsr));
#endif
    for (int i2 = 0; i2 < N2; ++i2)
      for (int c = 0; c < 3; ++c) J[JI(g, i1, i2, c)] *= t;
  }
}

/* the GRPIC branch of UniformInjector_kernel (injectors.hpp:230-239): the
 * tetrad-frame sample transformed to covariant components at the particle
 * (transform<Idx::T, Idx::D>), weight sqrt(det h) / V0 there */
int64_t orc_gr_inject_uniform(const orc_grid* g, const orc_qks* q, orc_species* sp1,
                              orc_species* sp2, const orc_inject_params* ip, double V0,
                              int64_t* failures) {
  const MT      m       = MK(q);
  const int64_t n       = orc_inject_count(2, ip);
  const float   mass[2] = { sp1->mass, sp2->mass };
  orc_species*  sps[2]  = { sp1, sp2 };
  const mreal   inv_V0  = (mreal)1 / (mreal)V0;
  int64_t       bad     = 0;
  (void)g;
  for (int64_t p = 0; p < n; ++p) {
    real x[3] = { 0, 0, 0 }, v[6];
    if (!orc_inject_sample_pair(2, ip, mass, (uint64_t)p, x, v)) ++bad;
    const mreal xp[2] = { (mreal)x[0], (mreal)x[1] };
    const mreal w     = M_(sqrt_det_h)(&m, xp) * inv_V0;
    for (int s = 0; s < 2; ++s) {
      orc_species*  S = sps[s];
      const int64_t k = S->npart + p;
      const mreal   vt[3] = { (mreal)v[3 * s], (mreal)v[3 * s + 1], (mreal)v[3 * s + 2] };
      mreal         vd[3];
      M_(t_to_d)(&m, xp, vt, vd);
      const int i1 = (int)x[0], i2 = (int)x[1];
      S->i1[k]  = i1;
      S->i2[k]  = i2;
      S->dx1[k] = (float)(x[0] - (real)i1);
      S->dx2[k] = (float)(x[1] - (real)i2);
      ((real*)S->ux1)[k]    = (real)vd[0];
      ((real*)S->ux2)[k]    = (real)vd[1];
      ((real*)S->ux3)[k]    = (real)vd[2];
      ((real*)S->weight)[k] = (real)w;
      S->tag[k]             = ORC_TAG_ALIVE;
    }
  }
  sp1->npart += n;
  sp2->npart += n;
  if (failures) *failures = bad;
  return n;
}
