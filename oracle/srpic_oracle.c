/*
 * CPU oracle for the SR particle-in-cell hot path (TEST INFRASTRUCTURE ONLY).
 * See srpic_oracle.h for the contract. Each function restates the cited
 * reference kernel; operation order follows the reference's source.
 */
#include "srpic_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORC_SINGLE
typedef float real;
#define RSQRT sqrtf
#define RFABS fabsf
/* src/global/utils/numeric.h:31-48 (SINGLE_PRECISION) */
static const real THIRD = 0.333333f;
#else
typedef double real;
#define RSQRT sqrt
#define RFABS fabs
/* src/global/utils/numeric.h:50-67 */
static const real THIRD = 0.3333333333333333;
#endif

/* one term of the shape-order interpolation sums (sr.hpp:1118-1369,
 * gr.hpp:594-662): `c += a * b`, product and sum rounded separately */
#define IACC(a, b, c) ((c) + (a) * (b))

static const real ZERO = 0, ONE = 1, TWO = 2, HALF = 0.5, INV_2 = 0.5;
static const real INV_4 = 0.25, INV_8 = 0.125, INV_16 = 0.0625;
static const real INV_32 = 0.03125, INV_64 = 0.015625;
static const real THREE_FOURTHS = 0.75, THREE_HALFS = 1.5;

#define SQR(x) ((x) * (x))

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int orc_real_size(void) { return (int)sizeof(real); }

/* ------------------------------------------------------------------------ */
/* field accessors                                                          */
/* ------------------------------------------------------------------------ */
#define EBI(g, i, j, k, c)                                                     \
  ((int64_t)(i) * (g)->em_s[0] + (int64_t)(j) * (g)->em_s[1] +                 \
   (int64_t)(k) * (g)->em_s[2] + (int64_t)(c) * (g)->em_s[3])
#define JI(g, i, j, k, c)                                                      \
  ((int64_t)(i) * (g)->cur_s[0] + (int64_t)(j) * (g)->cur_s[1] +               \
   (int64_t)(k) * (g)->cur_s[2] + (int64_t)(c) * (g)->cur_s[3])

/* EB index of the cell at `i` along `axis` and (pa, pb) along the two other
 * axes (oa < ob) */
static int64_t cond_idx(const orc_grid* g, int axis, int oa, int ob, int i, int pa, int pb,
                        int c) {
  int x[3] = { 0, 0, 0 };
  x[axis] = i;
  x[oa]   = pa;
  if (g->dim == 3) x[ob] = pb;
  return EBI(g, x[0], x[1], x[2], c);
}

static int ext(const orc_grid* g, int d) {
  const int n = d == 0 ? g->n1 : (d == 1 ? g->n2 : g->n3);
  return (d < g->dim) ? n + 2 * g->ng : 1;
}

/* ------------------------------------------------------------------------ */
/* shape functions: src/kernels/particle_shapes.hpp:25-63, 544-614           */
/* ------------------------------------------------------------------------ */
static real S3f(real x) { /* particle_shapes.hpp:56-63 */
  if (x < ONE) {
    return (real)(2.0 / 3.0) - SQR(x) + HALF * (x * x * x);
  } else if (x < TWO) {
    return (real)(4.0 / 3.0) - TWO * x + SQR(x) - (real)(1.0 / 6.0) * (x * x * x);
  }
  return ZERO;
}

static void shape(int stag, int O, int i, real di, int* imin, real* S) {
  if (O == 1) { /* particle_shapes.hpp:547-566 */
    if (!stag) {
      *imin = i;
      S[0]  = ONE - di;
      S[1]  = di;
    } else if (di < HALF) {
      *imin = i - 1;
      S[0]  = HALF - di;
      S[1]  = ONE - S[0];
    } else {
      *imin = i;
      S[0]  = THREE_HALFS - di;
      S[1]  = ONE - S[0];
    }
  } else if (O == 2) { /* particle_shapes.hpp:567-590 */
    if (!stag) {
      if (di < HALF) {
        *imin = i - 1;
        S[0]  = HALF * SQR(HALF - di);
        S[1]  = THREE_FOURTHS - SQR(di);
        S[2]  = ONE - S[0] - S[1];
      } else {
        *imin = i;
        S[0]  = HALF * SQR(THREE_HALFS - di);
        S[1]  = THREE_FOURTHS - SQR(ONE - di);
        S[2]  = ONE - S[0] - S[1];
      }
    } else {
      *imin = i - 1;
      S[0]  = HALF * SQR(ONE - di);
      S[2]  = HALF * SQR(di);
      S[1]  = ONE - S[0] - S[2];
    }
  } else { /* O == 3, particle_shapes.hpp:591-614 */
    if (!stag) {
      *imin = i - 1;
      for (int n = 0; n < 4; n++) S[n] = S3f(RFABS(ONE + di - (real)n));
    } else if (di < HALF) {
      *imin = i - 2;
      for (int n = 0; n < 4; n++) S[n] = S3f(RFABS((real)1.5 + di - (real)n));
    } else {
      *imin = i - 1;
      for (int n = 0; n < 4; n++) S[n] = S3f(RFABS(HALF + di - (real)n));
    }
  }
}

/* prtl_shape::for_deposit (particle_shapes.hpp:934-1024) */
static void for_deposit(int O, int i_init, real di_init, int i_fin, real di_fin,
                        int* i_min, int* i_max, real* iS, real* fS) {
  int  i_init_min, i_fin_min;
  real iS_[4], fS_[4];
  shape(0, O, i_init, di_init, &i_init_min, iS_);
  shape(0, O, i_fin, di_fin, &i_fin_min, fS_);
  if (i_init_min < i_fin_min) {
    *i_min = i_init_min;
    *i_max = *i_min + O + 1;
    for (int j = 0; j < O + 1; j++) iS[j] = iS_[j];
    iS[O + 1] = ZERO;
    fS[0]     = ZERO;
    for (int j = 0; j < O + 1; j++) fS[j + 1] = fS_[j];
  } else if (i_init_min > i_fin_min) {
    *i_min = i_fin_min;
    *i_max = *i_min + O + 1;
    iS[0]  = ZERO;
    for (int j = 0; j < O + 1; j++) iS[j + 1] = iS_[j];
    for (int j = 0; j < O + 1; j++) fS[j] = fS_[j];
    fS[O + 1] = ZERO;
  } else {
    *i_min = i_init_min;
    *i_max = *i_min + O;
    for (int j = 0; j < O + 1; j++) iS[j] = iS_[j];
    iS[O + 1] = ZERO;
    for (int j = 0; j < O + 1; j++) fS[j] = fS_[j];
    fS[O + 1] = ZERO;
  }
}

/* ------------------------------------------------------------------------ */
/* field interpolation: src/kernels/pushers/sr.hpp:851-1369                  */
/* ------------------------------------------------------------------------ */
/* staggering pattern of the six components: 1 = dual (staggered) along the
 * axis, 0 = primal (sr.hpp:1210-1266 for 2D, 1290-1366 for 3D) */
static const int STAG3[6][3] = {
  { 1, 0, 0 }, /* ex1 */
  { 0, 1, 0 }, /* ex2 */
  { 0, 0, 1 }, /* ex3 */
  { 0, 1, 1 }, /* bx1 */
  { 1, 0, 1 }, /* bx2 */
  { 1, 1, 0 }  /* bx3 */
};

static void interp_zigzag_2d(const orc_grid* g, const real* EB, int i1, int i2,
                             real dx1_, real dx2_, real* e0, real* b0) {
  /* sr.hpp:905-977 */
  const int i = i1 + g->ng, j = i2 + g->ng;
  int       indx = (int)(dx1_ + HALF);
  int       indy = (int)(dx2_ + HALF);
  real      c000, c100, c010, c110, c00, c10;
  real      ponpmx = ONE - dx1_, ponppx = dx1_;
  real      ponpmy = ONE - dx2_, ponppy = dx2_;
  real      pondmx = (real)(indx + 1) - (dx1_ + HALF);
  real      pondpx = ONE - pondmx;
  real      pondmy = (real)(indy + 1) - (dx2_ + HALF);
  real      pondpy = ONE - pondmy;
#define E2(a, b, c) EB[EBI(g, a, b, 0, c)]
  c000  = E2(i - 1 + indx, j, 0);
  c100  = E2(i + indx, j, 0);
  c010  = E2(i - 1 + indx, j + 1, 0);
  c110  = E2(i + indx, j + 1, 0);
  c00   = c000 * pondmx + c100 * pondpx;
  c10   = c010 * pondmx + c110 * pondpx;
  e0[0] = c00 * ponpmy + c10 * ponppy;
  c000  = E2(i, j - 1 + indy, 1);
  c100  = E2(i + 1, j - 1 + indy, 1);
  c010  = E2(i, j + indy, 1);
  c110  = E2(i + 1, j + indy, 1);
  c00   = c000 * ponpmx + c100 * ponppx;
  c10   = c010 * ponpmx + c110 * ponppx;
  e0[1] = c00 * pondmy + c10 * pondpy;
  c000  = E2(i, j, 2);
  c100  = E2(i + 1, j, 2);
  c010  = E2(i, j + 1, 2);
  c110  = E2(i + 1, j + 1, 2);
  c00   = c000 * ponpmx + c100 * ponppx;
  c10   = c010 * ponpmx + c110 * ponppx;
  e0[2] = c00 * ponpmy + c10 * ponppy;
  c000  = E2(i, j - 1 + indy, 3);
  c100  = E2(i + 1, j - 1 + indy, 3);
  c010  = E2(i, j + indy, 3);
  c110  = E2(i + 1, j + indy, 3);
  c00   = c000 * ponpmx + c100 * ponppx;
  c10   = c010 * ponpmx + c110 * ponppx;
  b0[0] = c00 * pondmy + c10 * pondpy;
  c000  = E2(i - 1 + indx, j, 4);
  c100  = E2(i + indx, j, 4);
  c010  = E2(i - 1 + indx, j + 1, 4);
  c110  = E2(i + indx, j + 1, 4);
  c00   = c000 * pondmx + c100 * pondpx;
  c10   = c010 * pondmx + c110 * pondpx;
  b0[1] = c00 * ponpmy + c10 * ponppy;
  c000  = E2(i - 1 + indx, j - 1 + indy, 5);
  c100  = E2(i + indx, j - 1 + indy, 5);
  c010  = E2(i - 1 + indx, j + indy, 5);
  c110  = E2(i + indx, j + indy, 5);
  c00   = c000 * pondmx + c100 * pondpx;
  c10   = c010 * pondmx + c110 * pondpx;
  b0[2] = c00 * pondmy + c10 * pondpy;
#undef E2
}

/* sr.hpp:978-1117: trilinear with primal (p) or dual (d) weights per axis */
static void interp_zigzag_3d(const orc_grid* g, const real* EB, int i1, int i2,
                             int i3, real dx1_, real dx2_, real dx3_, real* e0,
                             real* b0) {
  const int i = i1 + g->ng, j = i2 + g->ng, k = i3 + g->ng;
  int       ind[3] = { (int)(dx1_ + HALF), (int)(dx2_ + HALF), (int)(dx3_ + HALF) };
  const real d_[3] = { dx1_, dx2_, dx3_ };
  real      wpm[3], wpp[3], wdm[3], wdp[3];
  for (int a = 0; a < 3; ++a) {
    wpm[a] = ONE - d_[a];
    wpp[a] = d_[a];
    wdm[a] = (real)(ind[a] + 1) - (d_[a] + HALF);
    wdp[a] = ONE - wdm[a];
  }
  const int base[3] = { i, j, k };
  for (int c = 0; c < 6; ++c) {
    int  lo[3];
    real wm[3], wp[3];
    for (int a = 0; a < 3; ++a) {
      if (STAG3[c][a]) {
        lo[a] = base[a] - 1 + ind[a];
        wm[a] = wdm[a];
        wp[a] = wdp[a];
      } else {
        lo[a] = base[a];
        wm[a] = wpm[a];
        wp[a] = wpp[a];
      }
    }
    /* reference quirk (sr.hpp:1100-1116): Bx3 reads the dual x2 stencil
     * (j - 1 + indy, j + indy) but weights it with the primal ponpmy/ponppy */
    if (c == 5) {
      wm[1] = wpm[1];
      wp[1] = wpp[1];
    }
    const real c000 = EB[EBI(g, lo[0], lo[1], lo[2], c)];
    const real c100 = EB[EBI(g, lo[0] + 1, lo[1], lo[2], c)];
    const real c010 = EB[EBI(g, lo[0], lo[1] + 1, lo[2], c)];
    const real c110 = EB[EBI(g, lo[0] + 1, lo[1] + 1, lo[2], c)];
    const real c001 = EB[EBI(g, lo[0], lo[1], lo[2] + 1, c)];
    const real c101 = EB[EBI(g, lo[0] + 1, lo[1], lo[2] + 1, c)];
    const real c011 = EB[EBI(g, lo[0], lo[1] + 1, lo[2] + 1, c)];
    const real c111 = EB[EBI(g, lo[0] + 1, lo[1] + 1, lo[2] + 1, c)];
    const real c00  = c000 * wm[0] + c100 * wp[0];
    const real c10  = c010 * wm[0] + c110 * wp[0];
    const real c0   = c00 * wm[1] + c10 * wp[1];
    const real c01  = c001 * wm[0] + c101 * wp[0];
    const real c11  = c011 * wm[0] + c111 * wp[0];
    const real c1   = c01 * wm[1] + c11 * wp[1];
    const real v    = c0 * wm[2] + c1 * wp[2];
    if (c < 3) e0[c] = v; else b0[c - 3] = v;
  }
}

static void interp_shape(const orc_grid* g, const real* EB, int O, const int* ic,
                         const real* dc, real* e0, real* b0) {
  /* sr.hpp:1151-1369 */
  int  pmin[3] = { 0, 0, 0 }, dmin[3] = { 0, 0, 0 };
  real Sp[3][4], Sd[3][4];
  for (int a = 0; a < g->dim; ++a) {
    shape(0, O, ic[a] + g->ng, dc[a], &pmin[a], Sp[a]);
    shape(1, O, ic[a] + g->ng, dc[a], &dmin[a], Sd[a]);
  }
  for (int c = 0; c < 6; ++c) {
    const real* S[3];
    int         mn[3];
    for (int a = 0; a < 3; ++a) {
      const int st = STAG3[c][a];
      S[a]         = st ? Sd[a] : Sp[a];
      mn[a]        = st ? dmin[a] : pmin[a];
    }
    real v = ZERO;
    if (g->dim == 2) {
      for (int b = 0; b < O + 1; b++) {
        real c0 = ZERO;
        for (int a = 0; a < O + 1; a++) {
          c0 = IACC(S[0][a], EB[EBI(g, mn[0] + a, mn[1] + b, 0, c)], c0);
        }
        v = IACC(c0, S[1][b], v);
      }
    } else {
      for (int cc = 0; cc < O + 1; cc++) {
        real c0 = ZERO;
        for (int b = 0; b < O + 1; b++) {
          real c00 = ZERO;
          for (int a = 0; a < O + 1; a++) {
            c00 = IACC(S[0][a], EB[EBI(g, mn[0] + a, mn[1] + b, mn[2] + cc, c)], c00);
          }
          c0 = IACC(c00, S[1][b], c0);
        }
        v = IACC(c0, S[2][cc], v);
      }
    }
    if (c < 3) e0[c] = v; else b0[c - 3] = v;
  }
}

/* ------------------------------------------------------------------------ */
/* velocity pushers: sr.hpp:337-437                                         */
/* ------------------------------------------------------------------------ */
static void boris(real ndth, real* u, real* e0, real* b0) {
  real COEFF = ndth;
  e0[0] *= COEFF;
  e0[1] *= COEFF;
  e0[2] *= COEFF;
  real u0[3] = { u[0] + e0[0], u[1] + e0[1], u[2] + e0[2] };
  COEFF *= ONE / RSQRT(ONE + (u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]));
  b0[0] *= COEFF;
  b0[1] *= COEFF;
  b0[2] *= COEFF;
  COEFF = TWO / (ONE + (b0[0] * b0[0] + b0[1] * b0[1] + b0[2] * b0[2]));
  const real u1[3] = { (u0[0] + (u0[1] * b0[2] - u0[2] * b0[1])) * COEFF,
                       (u0[1] + (u0[2] * b0[0] - u0[0] * b0[2])) * COEFF,
                       (u0[2] + (u0[0] * b0[1] - u0[1] * b0[0])) * COEFF };
  u0[0] += (u1[1] * b0[2] - u1[2] * b0[1]) + e0[0];
  u0[1] += (u1[2] * b0[0] - u1[0] * b0[2]) + e0[1];
  u0[2] += (u1[0] * b0[1] - u1[1] * b0[0]) + e0[2];
  u[0] = u0[0];
  u[1] = u0[1];
  u[2] = u0[2];
}

static void vay(real ndth, real* u, real* e0, real* b0) {
  real COEFF = ndth;
  e0[0] *= COEFF;
  e0[1] *= COEFF;
  e0[2] *= COEFF;
  b0[0] *= COEFF;
  b0[1] *= COEFF;
  b0[2] *= COEFF;
  COEFF = ONE / RSQRT(ONE + (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
  real u1[3] = { (u[0] + TWO * e0[0] + (u[1] * b0[2] - u[2] * b0[1]) * COEFF),
                 (u[1] + TWO * e0[1] + (u[2] * b0[0] - u[0] * b0[2]) * COEFF),
                 (u[2] + TWO * e0[2] + (u[0] * b0[1] - u[1] * b0[0]) * COEFF) };
  COEFF       = (u1[0] * b0[0] + u1[1] * b0[1] + u1[2] * b0[2]);
  real COEFF2 = ONE + (u1[0] * u1[0] + u1[1] * u1[1] + u1[2] * u1[2]) -
                (b0[0] * b0[0] + b0[1] * b0[1] + b0[2] * b0[2]);
  COEFF = ONE / RSQRT(INV_2 * (COEFF2 + RSQRT(SQR(COEFF2) +
                                              (real)4 * (SQR(b0[0]) + SQR(b0[1]) +
                                                         SQR(b0[2]) + SQR(COEFF)))));
  COEFF2 = ONE / (ONE + SQR(b0[0] * COEFF) + SQR(b0[1] * COEFF) + SQR(b0[2] * COEFF));
  const real dotub = (u1[0] * b0[0] + u1[1] * b0[1] + u1[2] * b0[2]);
  u[0] = COEFF2 * (u1[0] + COEFF * dotub * (b0[0] * COEFF) + u1[1] * b0[2] * COEFF -
                   u1[2] * b0[1] * COEFF);
  u[1] = COEFF2 * (u1[1] + COEFF * dotub * (b0[1] * COEFF) + u1[2] * b0[0] * COEFF -
                   u1[0] * b0[2] * COEFF);
  u[2] = COEFF2 * (u1[2] + COEFF * dotub * (b0[2] * COEFF) + u1[0] * b0[1] * COEFF -
                   u1[1] * b0[0] * COEFF);
}

/* ------------------------------------------------------------------------ */
/* the pusher: sr.hpp:117-332 (massive & photon, no policies)               */
/* ------------------------------------------------------------------------ */
static int bc_of(const orc_grid* g, int d, int side) { return g->prtl_bc[d][side]; }

int64_t orc_push(const orc_grid* g, orc_species* sp, const void* EBv, int order,
                 double dt_d, double omegaB0_d, double dx_d) {
  const real* EB      = (const real*)EBv;
  real*       ux1     = (real*)sp->ux1;
  real*       ux2     = (real*)sp->ux2;
  real*       ux3     = (real*)sp->ux3;
  const real  dt      = (real)dt_d;
  const real  omegaB0 = (real)omegaB0_d;
  const real  dx      = (real)dx_d;
  /* sr.hpp:111: HALF * (charge / mass) * omegaB0 * dt, charge/mass as float */
  const float qm   = (sp->pusher == ORC_PUSHER_PHOTON) ? 0.0f : sp->charge / sp->mass;
  const real  ndth = HALF * (real)qm * omegaB0 * dt;
  const int   D    = g->dim;
  const int   ni[3] = { g->n1, g->n2, g->n3 };
  int64_t     nbad  = 0;
  if (sp->pusher == ORC_PUSHER_NONE) return 0;
#pragma omp parallel for reduction(+ : nbad) schedule(static)
  for (int64_t p = 0; p < sp->npart; ++p) {
    if (sp->tag[p] != ORC_TAG_ALIVE) {
      if (sp->tag[p] != ORC_TAG_DEAD) nbad++;
      continue;
    }
    int32_t* ic[3]  = { sp->i1, sp->i2, sp->i3 };
    int32_t* icp[3] = { sp->i1_prev, sp->i2_prev, sp->i3_prev };
    float*   dc[3]  = { sp->dx1, sp->dx2, sp->dx3 };
    float*   dcp[3] = { sp->dx1_prev, sp->dx2_prev, sp->dx3_prev };
    real     u[3]   = { ux1[p], ux2[p], ux3[p] };
    if (sp->pusher != ORC_PUSHER_PHOTON) {
      real e0[3], b0[3];
      if (order == 0) {
        if (D == 2) {
          interp_zigzag_2d(g, EB, sp->i1[p], sp->i2[p], (real)sp->dx1[p],
                           (real)sp->dx2[p], e0, b0);
        } else {
          interp_zigzag_3d(g, EB, sp->i1[p], sp->i2[p], sp->i3[p], (real)sp->dx1[p],
                           (real)sp->dx2[p], (real)sp->dx3[p], e0, b0);
        }
      } else {
        int  ii[3] = { sp->i1[p], sp->i2[p], D == 3 ? sp->i3[p] : 0 };
        real dd[3] = { (real)sp->dx1[p], (real)sp->dx2[p],
                       D == 3 ? (real)sp->dx3[p] : ZERO };
        interp_shape(g, EB, order, ii, dd, e0, b0);
      }
      /* transform_xyz<U, XYZ> for Minkowski (minkowski.h:264-296) */
      for (int a = 0; a < D; ++a) {
        e0[a] = e0[a] * dx;
        b0[a] = b0[a] * dx;
      }
      if (sp->pusher == ORC_PUSHER_BORIS) {
        boris(ndth, u, e0, b0);
      } else {
        vay(ndth, u, e0, b0);
      }
    }
    /* positionPush, Cartesian branch (sr.hpp:526-572) */
    const real dt_inv_energy =
      (sp->pusher != ORC_PUSHER_PHOTON)
        ? (dt / RSQRT(ONE + SQR(u[0]) + SQR(u[1]) + SQR(u[2])))
        : (dt / RSQRT(SQR(u[0]) + SQR(u[1]) + SQR(u[2])));
    for (int a = 0; a < D; ++a) {
      icp[a][p] = ic[a][p];
      dcp[a][p] = dc[a][p];
      dc[a][p] += (u[a] / dx) * dt_inv_energy;
      ic[a][p] += (int)(dc[a][p] >= ONE) - (int)(dc[a][p] < ZERO);
      dc[a][p] -= (dc[a][p] >= ONE);
      dc[a][p] += (dc[a][p] < ZERO);
    }
    /* boundaryConditions (sr.hpp:659-814) */
    for (int a = 0; a < D; ++a) {
      int invert = 0;
      if (ic[a][p] < 0) {
        const int bc = bc_of(g, a, 0);
        if (bc == 0) {
          ic[a][p] += ni[a];
          icp[a][p] += ni[a];
        } else if (bc == 1) {
          sp->tag[p] = ORC_TAG_DEAD;
        } else if (bc == 2) {
          ic[a][p] = 0;
          dc[a][p] = ONE - dc[a][p];
          invert   = 1;
        } else if (bc == 3 && a == 1) {
          ic[a][p] = 0;
          dc[a][p] = ONE - dc[a][p];
        }
      } else if (ic[a][p] >= ni[a]) {
        const int bc = bc_of(g, a, 1);
        if (bc == 0) {
          ic[a][p] -= ni[a];
          icp[a][p] -= ni[a];
        } else if (bc == 1) {
          sp->tag[p] = ORC_TAG_DEAD;
        } else if (bc == 2) {
          ic[a][p] = ni[a] - 1;
          dc[a][p] = ONE - dc[a][p];
          invert   = 1;
        } else if (bc == 3 && a == 1) {
          ic[a][p] = ni[a] - 1;
          dc[a][p] = ONE - dc[a][p];
        }
      }
      if (invert) u[a] = -u[a];
    }
    ux1[p] = u[0];
    ux2[p] = u[1];
    ux3[p] = u[2];
  }
  return nbad;
}

/* ------------------------------------------------------------------------ */
/* current deposition: src/kernels/currents_deposit.hpp:108-761              */
/* ------------------------------------------------------------------------ */
static void deposit_one(const orc_grid* g, const orc_species* sp, real* J,
                        int O, real inv_dt, real dx, int64_t p, const real* vz) {
  const real* ux1 = (const real*)sp->ux1;
  const real* ux2 = (const real*)sp->ux2;
  const real* ux3 = (const real*)sp->ux3;
  const real* w   = (const real*)sp->weight;
  const int   D   = g->dim;
  const int   ng  = g->ng;
  /* velocity for the unsimulated direction (currents_deposit.hpp:109-165) */
  real        vp[3];
  vp[0] = ux1[p] / dx;
  vp[1] = ux2[p] / dx;
  vp[2] = (D == 3) ? ux3[p] / dx : ux3[p];
  const real inv_energy =
    ONE / RSQRT(ONE + (ux1[p] * ux1[p] + ux2[p] * ux2[p] + ux3[p] * ux3[p]));
  if (isnan(vp[2]) || isinf(vp[2])) vp[2] = ZERO;
  vp[0] *= inv_energy;
  vp[1] *= inv_energy;
  vp[2] *= inv_energy;
  /* a caller-supplied out-of-plane velocity (the GR deposit's metric one) */
  if (vz) vp[2] = vz[p];
  const real coeff = w[p] * (real)sp->charge;
  const int  ip[3] = { sp->i1_prev[p], sp->i2_prev[p], D == 3 ? sp->i3_prev[p] : 0 };
  const int  ic[3] = { sp->i1[p], sp->i2[p], D == 3 ? sp->i3[p] : 0 };
  const float dp[3] = { sp->dx1_prev[p], sp->dx2_prev[p], D == 3 ? sp->dx3_prev[p] : 0.f };
  const float dc[3] = { sp->dx1[p], sp->dx2[p], D == 3 ? sp->dx3[p] : 0.f };

  if (O == 0) {
    /* zigzag (currents_deposit.hpp:167-405) */
    real W_1[3], W_2[3], F_1[3], F_2[3];
    for (int a = 0; a < D; ++a) {
      const float dxp_r = (float)(ic[a] == ip[a]) * (dc[a] + dp[a]) * (float)INV_2;
      W_1[a] = INV_2 * ((real)(dxp_r + dp[a]) + (real)(ic[a] > ip[a]));
      W_2[a] = INV_2 * ((real)(dc[a] + dxp_r) +
                        (real)((int)(ic[a] > ip[a]) + ip[a] - ic[a]));
      F_1[a] = ((real)(ic[a] > ip[a]) + (real)dxp_r - (real)dp[a]) * coeff * inv_dt;
      F_2[a] = ((real)(ic[a] - ip[a] - (int)(ic[a] > ip[a])) + (real)dc[a] -
                (real)dxp_r) *
               coeff * inv_dt;
    }
    if (D == 2) {
      const real Fx3_1 = HALF * vp[2] * coeff;
      const real Fx3_2 = HALF * vp[2] * coeff;
      const int  a = ip[0] + ng, b = ip[1] + ng, c = ic[0] + ng, d = ic[1] + ng;
      J[JI(g, a, b, 0, 0)] += F_1[0] * (ONE - W_1[1]);
      J[JI(g, a, b + 1, 0, 0)] += F_1[0] * W_1[1];
      J[JI(g, c, d, 0, 0)] += F_2[0] * (ONE - W_2[1]);
      J[JI(g, c, d + 1, 0, 0)] += F_2[0] * W_2[1];

      J[JI(g, a, b, 0, 1)] += F_1[1] * (ONE - W_1[0]);
      J[JI(g, a + 1, b, 0, 1)] += F_1[1] * W_1[0];
      J[JI(g, c, d, 0, 1)] += F_2[1] * (ONE - W_2[0]);
      J[JI(g, c + 1, d, 0, 1)] += F_2[1] * W_2[0];

      J[JI(g, a, b, 0, 2)] += Fx3_1 * (ONE - W_1[0]) * (ONE - W_1[1]);
      J[JI(g, a + 1, b, 0, 2)] += Fx3_1 * W_1[0] * (ONE - W_1[1]);
      J[JI(g, a, b + 1, 0, 2)] += Fx3_1 * (ONE - W_1[0]) * W_1[1];
      J[JI(g, a + 1, b + 1, 0, 2)] += Fx3_1 * W_1[0] * W_1[1];
      J[JI(g, c, d, 0, 2)] += Fx3_2 * (ONE - W_2[0]) * (ONE - W_2[1]);
      J[JI(g, c + 1, d, 0, 2)] += Fx3_2 * W_2[0] * (ONE - W_2[1]);
      J[JI(g, c, d + 1, 0, 2)] += Fx3_2 * (ONE - W_2[0]) * W_2[1];
      J[JI(g, c + 1, d + 1, 0, 2)] += Fx3_2 * W_2[0] * W_2[1];
    } else {
      /* for component a, the two transverse axes t1 < t2 get (1-W) / W;
       * order: component, then the previous then the current half-segment,
       * then (t1, t2) in {(0,0), (1,0), (0,1), (1,1)} (lines 295-403) */
      for (int a = 0; a < 3; ++a) {
        for (int half = 0; half < 2; ++half) {
          const int*  o = half == 0 ? ip : ic;
          const real* W = half == 0 ? W_1 : W_2;
          const real* F = half == 0 ? F_1 : F_2;
          const int t1 = a == 0 ? 1 : 0;
          const int t2 = a == 2 ? 1 : 2;
          for (int s2 = 0; s2 < 2; ++s2) {
            for (int s1 = 0; s1 < 2; ++s1) {
              int idx[3] = { o[0] + ng, o[1] + ng, o[2] + ng };
              idx[t1] += s1;
              idx[t2] += s2;
              const real w1 = s1 ? W[t1] : (ONE - W[t1]);
              const real w2 = s2 ? W[t2] : (ONE - W[t2]);
              J[JI(g, idx[0], idx[1], idx[2], a)] += F[a] * w1 * w2;
            }
          }
        }
      }
    }
    return;
  }

  /* Esirkepov, orders 1..3 (currents_deposit.hpp:406-754) */
  real iS[3][5], fS[3][5];
  int  imin[3] = { 0, 0, 0 }, imax[3] = { 0, 0, 0 };
  for (int a = 0; a < D; ++a) {
    for_deposit(O, ip[a], (real)dp[a], ic[a], (real)dc[a], &imin[a], &imax[a], iS[a],
                fS[a]);
  }
  const real Q = coeff * inv_dt;
  if (D == 2) {
    real Wx1[5][5], Wx2[5][5], Wx3[5][5], jx1[5][5], jx2[5][5];
    for (int i = 0; i < O + 2; ++i) {
      for (int j = 0; j < O + 2; ++j) {
        Wx1[i][j] = HALF * (fS[0][i] - iS[0][i]) * (fS[1][j] + iS[1][j]);
        Wx2[i][j] = HALF * (fS[0][i] + iS[0][i]) * (fS[1][j] - iS[1][j]);
        Wx3[i][j] = THIRD * (fS[1][j] * (HALF * iS[0][i] + fS[0][i]) +
                             iS[1][j] * (HALF * fS[0][i] + iS[0][i]));
      }
    }
    const real QVx3 = coeff * vp[2];
    for (int j = 0; j < O + 2; ++j) jx1[0][j] = -Q * Wx1[0][j];
    for (int i = 1; i < O + 2; ++i)
      for (int j = 0; j < O + 2; ++j) jx1[i][j] = jx1[i - 1][j] - Q * Wx1[i][j];
    for (int i = 0; i < O + 2; ++i) jx2[i][0] = -Q * Wx2[i][0];
    for (int j = 1; j < O + 2; ++j)
      for (int i = 0; i < O + 2; ++i) jx2[i][j] = jx2[i][j - 1] - Q * Wx2[i][j];
    const int i0 = imin[0] + ng, j0 = imin[1] + ng;
    const int d1 = imax[0] - imin[0], d2 = imax[1] - imin[1];
    for (int i = 0; i < d1; ++i)
      for (int j = 0; j <= d2; ++j) J[JI(g, i0 + i, j0 + j, 0, 0)] += jx1[i][j];
    for (int i = 0; i <= d1; ++i)
      for (int j = 0; j < d2; ++j) J[JI(g, i0 + i, j0 + j, 0, 1)] += jx2[i][j];
    for (int i = 0; i <= d1; ++i)
      for (int j = 0; j <= d2; ++j) J[JI(g, i0 + i, j0 + j, 0, 2)] += QVx3 * Wx3[i][j];
  } else {
    real Wx1[5][5][5], Wx2[5][5][5], Wx3[5][5][5];
    real jx1[5][5][5], jx2[5][5][5], jx3[5][5][5];
    for (int i = 0; i < O + 2; ++i) {
      for (int j = 0; j < O + 2; ++j) {
        for (int k = 0; k < O + 2; ++k) {
          Wx1[i][j][k] = THIRD * (fS[0][i] - iS[0][i]) *
                         ((iS[1][j] * iS[2][k] + fS[1][j] * fS[2][k]) +
                          HALF * (iS[2][k] * fS[1][j] + iS[1][j] * fS[2][k]));
          Wx2[i][j][k] = THIRD * (fS[1][j] - iS[1][j]) *
                         (iS[0][i] * iS[2][k] + fS[0][i] * fS[2][k] +
                          HALF * (iS[2][k] * fS[0][i] + iS[0][i] * fS[2][k]));
          Wx3[i][j][k] = THIRD * (fS[2][k] - iS[2][k]) *
                         (iS[0][i] * iS[1][j] + fS[0][i] * fS[1][j] +
                          HALF * (iS[0][i] * fS[1][j] + iS[1][j] * fS[0][i]));
        }
      }
    }
    for (int j = 0; j < O + 2; ++j)
      for (int k = 0; k < O + 2; ++k) jx1[0][j][k] = -Q * Wx1[0][j][k];
    for (int i = 1; i < O + 2; ++i)
      for (int j = 0; j < O + 2; ++j)
        for (int k = 0; k < O + 2; ++k) jx1[i][j][k] = jx1[i - 1][j][k] - Q * Wx1[i][j][k];
    for (int i = 0; i < O + 2; ++i)
      for (int k = 0; k < O + 2; ++k) jx2[i][0][k] = -Q * Wx2[i][0][k];
    for (int i = 0; i < O + 2; ++i)
      for (int j = 1; j < O + 2; ++j)
        for (int k = 0; k < O + 2; ++k) jx2[i][j][k] = jx2[i][j - 1][k] - Q * Wx2[i][j][k];
    for (int i = 0; i < O + 2; ++i)
      for (int j = 0; j < O + 2; ++j) jx3[i][j][0] = -Q * Wx3[i][j][0];
    for (int i = 0; i < O + 2; ++i)
      for (int j = 0; j < O + 2; ++j)
        for (int k = 1; k < O + 2; ++k) jx3[i][j][k] = jx3[i][j][k - 1] - Q * Wx3[i][j][k];
    const int i0 = imin[0] + ng, j0 = imin[1] + ng, k0 = imin[2] + ng;
    const int d1 = imax[0] - imin[0], d2 = imax[1] - imin[1], d3 = imax[2] - imin[2];
    for (int i = 0; i < d1; ++i)
      for (int j = 0; j <= d2; ++j)
        for (int k = 0; k <= d3; ++k) J[JI(g, i0 + i, j0 + j, k0 + k, 0)] += jx1[i][j][k];
    for (int i = 0; i <= d1; ++i)
      for (int j = 0; j < d2; ++j)
        for (int k = 0; k <= d3; ++k) J[JI(g, i0 + i, j0 + j, k0 + k, 1)] += jx2[i][j][k];
    for (int i = 0; i <= d1; ++i)
      for (int j = 0; j <= d2; ++j)
        for (int k = 0; k < d3; ++k) J[JI(g, i0 + i, j0 + j, k0 + k, 2)] += jx3[i][j][k];
  }
}

static void deposit_all(const orc_grid* g, const orc_species* sp, void* Jv, int order,
                        double dt_d, double dx_d, const real* vz);

void orc_deposit(const orc_grid* g, const orc_species* sp, void* Jv, int order,
                 double dt_d, double dx_d) {
  deposit_all(g, sp, Jv, order, dt_d, dx_d, NULL);
}

void orc_deposit_vz(const orc_grid* g, const orc_species* sp, void* Jv, int order, double dt_d,
                    const void* vz) {
  deposit_all(g, sp, Jv, order, dt_d, 1.0, (const real*)vz);
}

void orc_interp2(const orc_grid* g, const void* emD, const void* emB, int order, int i1, int i2,
                 float dx1, float dx2, double* e, double* b) {
  const int  ic[3] = { i1, i2, 0 };
  const real dc[3] = { (real)dx1, (real)dx2, ZERO };
  real       e0[3], b0[3], e1[3], b1[3];
  interp_shape(g, (const real*)emD, order, ic, dc, e0, b0);
  interp_shape(g, (const real*)emB, order, ic, dc, e1, b1);
  for (int c = 0; c < 3; ++c) {
    e[c] = (double)e0[c];
    b[c] = (double)b1[c];
  }
}

static void deposit_all(const orc_grid* g, const orc_species* sp, void* Jv, int order,
                        double dt_d, double dx_d, const real* vz) {
  real*      J      = (real*)Jv;
  const real inv_dt = ONE / (real)dt_d;
  const real dx     = (real)dx_d;
  if (sp->pusher == ORC_PUSHER_NONE || sp->npart == 0 || sp->charge == 0.0f) return;
#ifdef _OPENMP
  /* per-thread copies reduced in thread order (deterministic), the OpenMP
   * analogue of the reference's duplicated ScatterView */
  const int64_t nJ = (int64_t)ext(g, 0) * ext(g, 1) * ext(g, 2) * 3;
  const int     nt = omp_get_max_threads();
  if (nt > 1 && g->cur_s[3] == (int64_t)ext(g, 0) * ext(g, 1) * ext(g, 2)) {
    real* part = (real*)calloc((size_t)nJ * (size_t)nt, sizeof(real));
#pragma omp parallel
    {
      const int t  = omp_get_thread_num();
      real*     Jt = part + (int64_t)t * nJ;
#pragma omp for schedule(static)
      for (int64_t p = 0; p < sp->npart; ++p) {
        if (sp->tag[p] == ORC_TAG_DEAD) continue;
        deposit_one(g, sp, Jt, order, inv_dt, dx, p, vz);
      }
#pragma omp for schedule(static)
      for (int64_t q = 0; q < nJ; ++q) {
        real acc = J[q];
        for (int tt = 0; tt < nt; ++tt) acc += part[(int64_t)tt * nJ + q];
        J[q] = acc;
      }
    }
    free(part);
    return;
  }
#endif
  for (int64_t p = 0; p < sp->npart; ++p) {
    if (sp->tag[p] == ORC_TAG_DEAD) continue;
    deposit_one(g, sp, J, order, inv_dt, dx, p, vz);
  }
}

/* ------------------------------------------------------------------------ */
/* field solvers                                                            */
/* ------------------------------------------------------------------------ */
void orc_faraday(const orc_grid* g, void* EBv, double c1d, double c2d,
                 const double* st) {
  real*      EB     = (real*)EBv;
  const real coeff1 = (real)c1d, coeff2 = (real)c2d;
  real       deltax = 0, deltay = 0, betaxy = 0, betayx = 0, deltaz = 0, betaxz = 0,
       betazx = 0, betayz = 0, betazy = 0;
  if (st) {
    deltax = (real)st[0];
    deltay = (real)st[1];
    betaxy = (real)st[2];
    betayx = (real)st[3];
    deltaz = (real)st[4];
    betaxz = (real)st[5];
    betazx = (real)st[6];
    betayz = (real)st[7];
    betazy = (real)st[8];
  }
  const int ng = g->ng;
  if (g->dim == 2) {
    /* faraday_mink.hpp:92-119 */
    const real alphax = ONE - TWO * betaxy - (real)3 * deltax;
    const real alphay = ONE - TWO * betayx - (real)3 * deltay;
#pragma omp parallel for schedule(static)
    for (int i2 = ng; i2 < g->n2 + ng; ++i2) {
      for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
#define F(a, b, c) EB[EBI(g, a, b, 0, c)]
        F(i1, i2, 3) += coeff1 * (-alphay * (F(i1, i2 + 1, 2) - F(i1, i2, 2)) -
                                  deltay * (F(i1, i2 + 2, 2) - F(i1, i2 - 1, 2)) -
                                  betayx * (F(i1 + 1, i2 + 1, 2) - F(i1 + 1, i2, 2)) -
                                  betayx * (F(i1 - 1, i2 + 1, 2) - F(i1 - 1, i2, 2)));
        F(i1, i2, 4) += coeff1 * (+alphax * (F(i1 + 1, i2, 2) - F(i1, i2, 2)) +
                                  deltax * (F(i1 + 2, i2, 2) - F(i1 - 1, i2, 2)) +
                                  betaxy * (F(i1 + 1, i2 + 1, 2) - F(i1, i2 + 1, 2)) +
                                  betaxy * (F(i1 + 1, i2 - 1, 2) - F(i1, i2 - 1, 2)));
        F(i1, i2, 5) += coeff2 * (+alphay * (F(i1, i2 + 1, 0) - F(i1, i2, 0)) +
                                  deltay * (F(i1, i2 + 2, 0) - F(i1, i2 - 1, 0)) +
                                  betayx * (F(i1 + 1, i2 + 1, 0) - F(i1 + 1, i2, 0)) +
                                  betayx * (F(i1 - 1, i2 + 1, 0) - F(i1 - 1, i2, 0)) -
                                  alphax * (F(i1 + 1, i2, 1) - F(i1, i2, 1)) -
                                  deltax * (F(i1 + 2, i2, 1) - F(i1 - 1, i2, 1)) -
                                  betaxy * (F(i1 + 1, i2 + 1, 1) - F(i1, i2 + 1, 1)) -
                                  betaxy * (F(i1 + 1, i2 - 1, 1) - F(i1, i2 - 1, 1)));
#undef F
      }
    }
  } else {
    /* faraday_mink.hpp:121-162 */
    const real alphax = ONE - TWO * betaxy - TWO * betaxz - (real)3 * deltax;
    const real alphay = ONE - TWO * betayx - TWO * betayz - (real)3 * deltay;
    const real alphaz = ONE - TWO * betazx - TWO * betazy - (real)3 * deltaz;
#pragma omp parallel for schedule(static) collapse(2)
    for (int i3 = ng; i3 < g->n3 + ng; ++i3) {
      for (int i2 = ng; i2 < g->n2 + ng; ++i2) {
        for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
#define F(a, b, c, d) EB[EBI(g, a, b, c, d)]
          F(i1, i2, i3, 3) +=
            coeff1 * (+alphaz * (F(i1, i2, i3 + 1, 1) - F(i1, i2, i3, 1)) +
                      deltaz * (F(i1, i2, i3 + 2, 1) - F(i1, i2, i3 - 1, 1)) +
                      betazx * (F(i1 + 1, i2, i3 + 1, 1) - F(i1 + 1, i2, i3, 1)) +
                      betazx * (F(i1 - 1, i2, i3 + 1, 1) - F(i1 - 1, i2, i3, 1)) +
                      betazy * (F(i1, i2 + 1, i3 + 1, 1) - F(i1, i2 + 1, i3, 1)) +
                      betazy * (F(i1, i2 - 1, i3 + 1, 1) - F(i1, i2 - 1, i3, 1)) -
                      alphay * (F(i1, i2 + 1, i3, 2) - F(i1, i2, i3, 2)) -
                      deltay * (F(i1, i2 + 2, i3, 2) - F(i1, i2 - 1, i3, 2)) -
                      betayx * (F(i1 + 1, i2 + 1, i3, 2) - F(i1 + 1, i2, i3, 2)) -
                      betayx * (F(i1 - 1, i2 + 1, i3, 2) - F(i1 - 1, i2, i3, 2)) -
                      betayz * (F(i1, i2 + 1, i3 + 1, 2) - F(i1, i2, i3 + 1, 2)) -
                      betayz * (F(i1, i2 + 1, i3 - 1, 2) - F(i1, i2, i3 - 1, 2)));
          F(i1, i2, i3, 4) +=
            coeff1 * (+alphax * (F(i1 + 1, i2, i3, 2) - F(i1, i2, i3, 2)) +
                      deltax * (F(i1 + 2, i2, i3, 2) - F(i1 - 1, i2, i3, 2)) +
                      betaxy * (F(i1 + 1, i2 + 1, i3, 2) - F(i1, i2 + 1, i3, 2)) +
                      betaxy * (F(i1 + 1, i2 - 1, i3, 2) - F(i1, i2 - 1, i3, 2)) +
                      betaxz * (F(i1 + 1, i2, i3 + 1, 2) - F(i1, i2, i3 + 1, 2)) +
                      betaxz * (F(i1 + 1, i2, i3 - 1, 2) - F(i1, i2, i3 - 1, 2)) -
                      alphaz * (F(i1, i2, i3 + 1, 0) - F(i1, i2, i3, 0)) -
                      deltaz * (F(i1, i2, i3 + 2, 0) - F(i1, i2, i3 - 1, 0)) -
                      betazx * (F(i1 + 1, i2, i3 + 1, 0) - F(i1 + 1, i2, i3, 0)) -
                      betazx * (F(i1 - 1, i2, i3 + 1, 0) - F(i1 - 1, i2, i3, 0)) -
                      betazy * (F(i1, i2 + 1, i3 + 1, 0) - F(i1, i2 + 1, i3, 0)) -
                      betazy * (F(i1, i2 - 1, i3 + 1, 0) - F(i1, i2 - 1, i3, 0)));
          F(i1, i2, i3, 5) +=
            coeff1 * (+alphay * (F(i1, i2 + 1, i3, 0) - F(i1, i2, i3, 0)) +
                      deltay * (F(i1, i2 + 2, i3, 0) - F(i1, i2 - 1, i3, 0)) +
                      betayx * (F(i1 + 1, i2 + 1, i3, 0) - F(i1 + 1, i2, i3, 0)) +
                      betayx * (F(i1 - 1, i2 + 1, i3, 0) - F(i1 - 1, i2, i3, 0)) +
                      betayz * (F(i1, i2 + 1, i3 + 1, 0) - F(i1, i2, i3 + 1, 0)) +
                      betayz * (F(i1, i2 + 1, i3 - 1, 0) - F(i1, i2, i3 - 1, 0)) -
                      alphax * (F(i1 + 1, i2, i3, 1) - F(i1, i2, i3, 1)) -
                      deltax * (F(i1 + 2, i2, i3, 1) - F(i1 - 1, i2, i3, 1)) -
                      betaxy * (F(i1 + 1, i2 + 1, i3, 1) - F(i1, i2 + 1, i3, 1)) -
                      betaxy * (F(i1 + 1, i2 - 1, i3, 1) - F(i1, i2 - 1, i3, 1)) -
                      betaxz * (F(i1 + 1, i2, i3 + 1, 1) - F(i1, i2, i3 + 1, 1)) -
                      betaxz * (F(i1 + 1, i2, i3 - 1, 1) - F(i1, i2, i3 - 1, 1)));
#undef F
        }
      }
    }
  }
}

void orc_ampere(const orc_grid* g, void* EBv, double c1d, double c2d) {
  real*      EB     = (real*)EBv;
  const real coeff1 = (real)c1d, coeff2 = (real)c2d;
  const int  ng     = g->ng;
  if (g->dim == 2) {
    /* ampere_mink.hpp:58-69 */
#pragma omp parallel for schedule(static)
    for (int i2 = ng; i2 < g->n2 + ng; ++i2) {
      for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
#define F(a, b, c) EB[EBI(g, a, b, 0, c)]
        F(i1, i2, 0) += coeff1 * (F(i1, i2, 5) - F(i1, i2 - 1, 5));
        F(i1, i2, 1) += coeff1 * (F(i1 - 1, i2, 5) - F(i1, i2, 5));
        F(i1, i2, 2) +=
          coeff2 * (F(i1, i2 - 1, 3) - F(i1, i2, 3) + F(i1, i2, 4) - F(i1 - 1, i2, 4));
#undef F
      }
    }
  } else {
    /* ampere_mink.hpp:71-87 */
#pragma omp parallel for schedule(static) collapse(2)
    for (int i3 = ng; i3 < g->n3 + ng; ++i3) {
      for (int i2 = ng; i2 < g->n2 + ng; ++i2) {
        for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
#define F(a, b, c, d) EB[EBI(g, a, b, c, d)]
          F(i1, i2, i3, 0) += coeff1 * (F(i1, i2, i3 - 1, 4) - F(i1, i2, i3, 4) +
                                        F(i1, i2, i3, 5) - F(i1, i2 - 1, i3, 5));
          F(i1, i2, i3, 1) += coeff1 * (F(i1 - 1, i2, i3, 5) - F(i1, i2, i3, 5) +
                                        F(i1, i2, i3, 3) - F(i1, i2, i3 - 1, 3));
          F(i1, i2, i3, 2) += coeff1 * (F(i1, i2 - 1, i3, 3) - F(i1, i2, i3, 3) +
                                        F(i1, i2, i3, 4) - F(i1 - 1, i2, i3, 4));
#undef F
        }
      }
    }
  }
}

void orc_currents_ampere(const orc_grid* g, void* EBv, void* Jv, double coeff_d,
                         double ppc0_d) {
  real*      EB    = (real*)EBv;
  real*      J     = (real*)Jv;
  const real coeff = (real)coeff_d, ppc0 = (real)ppc0_d;
  const int  ng    = g->ng;
  const int  k0 = g->dim == 3 ? ng : 0, k1 = g->dim == 3 ? g->n3 + ng : 1;
  /* ampere_mink.hpp:155-166, 183-210 */
#pragma omp parallel for schedule(static) collapse(2)
  for (int i3 = k0; i3 < k1; ++i3) {
    for (int i2 = ng; i2 < g->n2 + ng; ++i2) {
      for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
        for (int c = 0; c < 3; ++c) EB[EBI(g, i1, i2, i3, c)] += J[JI(g, i1, i2, i3, c)] * coeff;
        for (int c = 0; c < 3; ++c) J[JI(g, i1, i2, i3, c)] /= ppc0;
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* digital filter: src/kernels/digital_filter.hpp:183-195, 352-379           */
/* ------------------------------------------------------------------------ */
/* DigitalFilter_kernel with conductor walls (digital_filter.hpp:99-379) for
 * one active cell: the first matching wall case in the order x1, x2, x3
 * writes the components the reference writes; other cells take the full
 * stencil. The wall's inner neighbour index is i + 1 whenever the lower side
 * is a conductor, as the reference picks it. Returns 0 when no wall case
 * applies. */
static int filter_cond_cell(const orc_grid* g, real* J, const real* B, int i1, int i2, int i3) {
  const int c1l = g->fbc[0][0] == 2, c1h = g->fbc[0][1] == 2;
  const int c2l = g->fbc[1][0] == 2, c2h = g->fbc[1][1] == 2;
  const int c3l = g->dim == 3 && g->fbc[2][0] == 2, c3h = g->dim == 3 && g->fbc[2][1] == 2;
  const int i1min = g->ng, i1max = g->n1 + g->ng, i2min = g->ng, i2max = g->n2 + g->ng;
  const int i3min = g->ng, i3max = g->n3 + g->ng;
  const real THREE = 3;
#define bb(x, y, z, c) B[JI(g, x, y, z, c)]
#define aa(c)          J[JI(g, i1, i2, i3, c)]
  if (g->dim == 2) {
#define FI1(c, I, Jj) (INV_2 * bb((I), (Jj), 0, c) + INV_4 * (bb((I) - 1, (Jj), 0, c) + bb((I) + 1, (Jj), 0, c)))
#define FI2(c, I, Jj) (INV_2 * bb((I), (Jj), 0, c) + INV_4 * (bb((I), (Jj) - 1, 0, c) + bb((I), (Jj) + 1, 0, c)))
    if ((c1l && i1 == i1min) || (c1h && i1 == i1max - 1)) {
      const int s = c1l ? i1 + 1 : i1 - 1;
      aa(0) = (THREE * INV_4) * (FI2(0, i1, i2)) + (INV_4) * (FI2(0, s, i2));
    } else if ((c1l && i1 == i1min + 1) || (c1h && i1 == i1max - 2)) {
      const int s = c1l ? i1 + 1 : i1 - 1;
      aa(0) = INV_2 * (FI2(0, i1, i2)) + INV_4 * ((FI2(0, i1 - 1, i2)) + (FI2(0, i1 + 1, i2)));
      aa(1) = (INV_2) * (FI2(1, i1, i2)) + (INV_4) * (FI2(1, s, i2));
      aa(2) = (INV_2) * (FI2(2, i1, i2)) + (INV_4) * (FI2(2, s, i2));
    } else if ((c2l && i2 == i2min) || (c2h && i2 == i2max - 1)) {
      const int s = c2l ? i2 + 1 : i2 - 1;
      aa(1) = (THREE * INV_4) * (FI1(1, i1, i2)) + (INV_4) * (FI1(1, i1, s));
    } else if ((c2l && i2 == i2min + 1) || (c2h && i2 == i2max - 2)) {
      const int s = c2l ? i2 + 1 : i2 - 1;
      aa(0) = INV_2 * (FI1(0, i1, i2)) + INV_4 * (FI1(0, i1, s));
      aa(1) = INV_2 * (FI1(1, i1, i2)) + INV_4 * ((FI1(1, i1, i2 - 1)) + (FI1(1, i1, i2 + 1)));
      aa(2) = INV_2 * (FI1(2, i1, i2)) + INV_4 * (FI1(2, i1, s));
    } else {
      return 0;
    }
#undef FI1
#undef FI2
    return 1;
  }
#define P23(c, I, Jj, K)                                                                       \
  (INV_4 * bb(I, Jj, K, c) +                                                                   \
   INV_8 * (bb((I), (Jj) - 1, (K), c) + bb((I), (Jj) + 1, (K), c) + bb((I), (Jj), (K) - 1, c) + \
            bb((I), (Jj), (K) + 1, c)) +                                                       \
   INV_16 * (bb((I), (Jj) - 1, (K) - 1, c) + bb((I), (Jj) + 1, (K) + 1, c) +                   \
             bb((I), (Jj) - 1, (K) + 1, c) + bb((I), (Jj) + 1, (K) - 1, c)))
#define P13(c, I, Jj, K)                                                                       \
  (INV_4 * bb(I, Jj, K, c) +                                                                   \
   INV_8 * (bb((I) - 1, (Jj), (K), c) + bb((I) + 1, (Jj), (K), c) + bb((I), (Jj), (K) - 1, c) + \
            bb((I), (Jj), (K) + 1, c)) +                                                       \
   INV_16 * (bb((I) - 1, (Jj), (K) - 1, c) + bb((I) + 1, (Jj), (K) + 1, c) +                   \
             bb((I) - 1, (Jj), (K) + 1, c) + bb((I) + 1, (Jj), (K) - 1, c)))
#define P12(c, I, Jj, K)                                                                       \
  (INV_4 * bb(I, Jj, K, c) +                                                                   \
   INV_8 * (bb((I) - 1, (Jj), (K), c) + bb((I) + 1, (Jj), (K), c) + bb((I), (Jj) - 1, (K), c) + \
            bb((I), (Jj) + 1, (K), c)) +                                                       \
   INV_16 * (bb((I) - 1, (Jj) - 1, (K), c) + bb((I) + 1, (Jj) + 1, (K), c) +                   \
             bb((I) - 1, (Jj) + 1, (K), c) + bb((I) + 1, (Jj) - 1, (K), c)))
  if ((c1l && i1 == i1min) || (c1h && i1 == i1max - 1)) {
    const int s = c1l ? i1 + 1 : i1 - 1;
    aa(0) = (THREE * INV_4) * (P23(0, i1, i2, i3)) + (INV_4) * (P23(0, s, i2, i3));
  } else if ((c1l && i1 == i1min + 1) || (c1h && i1 == i1max - 2)) {
    const int s = c1l ? i1 + 1 : i1 - 1;
    aa(0) = INV_2 * (P23(0, i1, i2, i3)) + INV_4 * ((P23(0, i1 - 1, i2, i3)) + (P23(0, i1 + 1, i2, i3)));
    aa(1) = INV_2 * (P23(1, i1, i2, i3)) + INV_4 * (P23(1, s, i2, i3));
    aa(2) = INV_2 * (P23(2, i1, i2, i3)) + INV_4 * (P23(2, s, i2, i3));
  } else if ((c2l && i2 == i2min) || (c2h && i2 == i2max - 1)) {
    const int s = c2l ? i2 + 1 : i2 - 1;
    aa(1) = (THREE * INV_4) * (P13(1, i1, i2, i3)) + (INV_4) * (P13(1, i1, s, i3));
  } else if ((c2l && i2 == i2min + 1) || (c2h && i2 == i2max - 2)) {
    const int s = c2l ? i2 + 1 : i2 - 1;
    aa(0) = INV_2 * (P13(0, i1, i2, i3)) + INV_4 * (P13(0, i1, s, i3));
    aa(1) = INV_2 * (P13(1, i1, i2, i3)) + INV_4 * ((P13(1, i1, i2 - 1, i3)) + (P13(1, i1, i2 + 1, i3)));
    aa(2) = INV_2 * (P13(2, i1, i2, i3)) + INV_4 * (P13(2, i1, s, i3));
  } else if ((c3l && i3 == i3min) || (c3h && i3 == i3max - 1)) {
    const int s = c3l ? i3 + 1 : i3 - 1;
    aa(2) = (THREE * INV_4) * (P12(2, i1, i2, i3)) + (INV_4) * (P12(2, i1, i2, s));
  } else if ((c3l && i3 == i3min + 1) || (c3h && i3 == i3max - 2)) {
    const int s = c3l ? i3 + 1 : i3 - 1;
    aa(0) = INV_2 * (P12(0, i1, i2, i3)) + INV_4 * (P12(0, i1, i2, s));
    aa(1) = INV_2 * (P12(1, i1, i2, i3)) + INV_4 * (P12(1, i1, i2, s));
    aa(2) = INV_2 * (P12(2, i1, i2, i3)) + INV_4 * ((P12(2, i1, i2, i3 - 1)) + (P12(2, i1, i2, i3 + 1)));
  } else {
    return 0;
  }
#undef P23
#undef P13
#undef P12
#undef aa
#undef bb
  return 1;
}

void orc_filter_pass(const orc_grid* g, void* Jv, void* buffv) {
  real*         J  = (real*)Jv;
  real*         B  = (real*)buffv;
  const int     ng = g->ng;
  const int64_t n  = (int64_t)ext(g, 0) * ext(g, 1) * ext(g, 2);
  /* currents.h:109: deep_copy(buff, cur) (all cells incl. ghosts) */
  for (int c = 0; c < 3; ++c)
    for (int k = 0; k < ext(g, 2); ++k)
      for (int j = 0; j < ext(g, 1); ++j)
        for (int i = 0; i < ext(g, 0); ++i) B[JI(g, i, j, k, c)] = J[JI(g, i, j, k, c)];
  (void)n;
  if (g->dim == 2) {
#pragma omp parallel for schedule(static)
    for (int i2 = ng; i2 < g->n2 + ng; ++i2) {
      for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
        if (filter_cond_cell(g, J, B, i1, i2, 0)) continue;
        for (int c = 0; c < 3; ++c) {
#define b(a, bb) B[JI(g, a, bb, 0, c)]
          J[JI(g, i1, i2, 0, c)] =
            INV_4 * b(i1, i2) +
            INV_8 * (b(i1 - 1, i2) + b(i1 + 1, i2) + b(i1, i2 - 1) + b(i1, i2 + 1)) +
            INV_16 * (b(i1 - 1, i2 - 1) + b(i1 + 1, i2 + 1) + b(i1 - 1, i2 + 1) +
                      b(i1 + 1, i2 - 1));
#undef b
        }
      }
    }
  } else {
#pragma omp parallel for schedule(static) collapse(2)
    for (int i3 = ng; i3 < g->n3 + ng; ++i3) {
      for (int i2 = ng; i2 < g->n2 + ng; ++i2) {
        for (int i1 = ng; i1 < g->n1 + ng; ++i1) {
          if (filter_cond_cell(g, J, B, i1, i2, i3)) continue;
          for (int c = 0; c < 3; ++c) {
#define b(x, y, z) B[JI(g, x, y, z, c)]
            /* the (i, j, k +- 1) pair appears twice in the 1/32 group, as in
             * digital_filter.hpp:365 */
            J[JI(g, i1, i2, i3, c)] =
              INV_8 * b(i1, i2, i3) +
              INV_16 * (b(i1 - 1, i2, i3) + b(i1 + 1, i2, i3) + b(i1, i2 - 1, i3) +
                        b(i1, i2 + 1, i3) + b(i1, i2, i3 - 1) + b(i1, i2, i3 + 1)) +
              INV_32 * (b(i1 - 1, i2 - 1, i3) + b(i1 + 1, i2 + 1, i3) +
                        b(i1 - 1, i2 + 1, i3) + b(i1 + 1, i2 - 1, i3) +
                        b(i1, i2 - 1, i3 - 1) + b(i1, i2 + 1, i3 + 1) +
                        b(i1, i2, i3 - 1) + b(i1, i2, i3 + 1) +
                        b(i1 - 1, i2, i3 - 1) + b(i1 + 1, i2, i3 + 1) +
                        b(i1 - 1, i2, i3 + 1) + b(i1 + 1, i2, i3 - 1)) +
              INV_64 * (b(i1 - 1, i2 - 1, i3 - 1) + b(i1 + 1, i2 + 1, i3 + 1) +
                        b(i1 - 1, i2 + 1, i3 + 1) + b(i1 + 1, i2 - 1, i3 - 1) +
                        b(i1 - 1, i2 - 1, i3 + 1) + b(i1 + 1, i2 + 1, i3 - 1) +
                        b(i1 - 1, i2 + 1, i3 - 1) + b(i1 + 1, i2 - 1, i3 + 1));
#undef b
          }
        }
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* periodic self-exchange                                                   */
/* ------------------------------------------------------------------------ */
/* direction list of dir::Directions<D>::all (src/global/arch/directions.h:
 * 173-232): lexicographic over {-1, 0, 1}^D without the zero vector */
static int directions(int D, int out[26][3]) {
  int n = 0;
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b)
      for (int c = -1; c <= (D == 3 ? 1 : -1); ++c) {
        const int cc = D == 3 ? c : 0;
        if (a == 0 && b == 0 && cc == 0) continue;
        out[n][0] = a;
        out[n][1] = b;
        out[n][2] = cc;
        n++;
        if (D == 2) break;
      }
  return n;
}

void orc_fill_ghosts(const orc_grid* g, void* fv, int is_em, int c0, int c1) {
  real*          f  = (real*)fv;
  const int64_t* s  = is_em ? g->em_s : g->cur_s;
  const int      ng = g->ng;
  const int      n[3] = { g->n1, g->n2, g->n3 };
  int            dirs[26][3];
  const int      nd = directions(g->dim, dirs);
  for (int q = 0; q < nd; ++q) {
    int ok = 1, slo[3] = { 0, 0, 0 }, shi[3] = { 1, 1, 1 }, off[3] = { 0, 0, 0 };
    for (int d = 0; d < g->dim; ++d) {
      const int dir = dirs[q][d];
      if (dir != 0 && !g->periodic[d]) ok = 0;
      /* metadomain_comm.cpp:142-165: send from active, recv into ghosts */
      if (dir == 0) {
        slo[d] = ng;
        shi[d] = ng + n[d];
        off[d] = 0;
      } else if (dir == 1) {
        slo[d] = ng + n[d] - ng;
        shi[d] = ng + n[d];
        off[d] = -n[d]; /* recv index = send index - n */
      } else {
        slo[d] = ng;
        shi[d] = ng + ng;
        off[d] = n[d];
      }
    }
    if (!ok) continue;
    for (int c = c0; c < c1; ++c)
      for (int k = slo[2]; k < shi[2]; ++k)
        for (int j = slo[1]; j < shi[1]; ++j)
          for (int i = slo[0]; i < shi[0]; ++i) {
            const int64_t src = i * s[0] + j * s[1] + k * s[2] + c * s[3];
            const int64_t dst = (i + off[0]) * s[0] + (j + off[1]) * s[1] +
                                (k + off[2]) * s[2] + c * s[3];
            f[dst] = f[src];
          }
  }
}

void orc_sync_currents(const orc_grid* g, void* Jv, void* buffv) {
  real*          J  = (real*)Jv;
  real*          B  = (real*)buffv;
  const int64_t* s  = g->cur_s;
  const int      ng = g->ng;
  const int      n[3] = { g->n1, g->n2, g->n3 };
  int            dirs[26][3];
  const int      nd = directions(g->dim, dirs);
  for (int c = 0; c < 3; ++c)
    for (int k = 0; k < ext(g, 2); ++k)
      for (int j = 0; j < ext(g, 1); ++j)
        for (int i = 0; i < ext(g, 0); ++i) B[JI(g, i, j, k, c)] = ZERO;
  for (int q = 0; q < nd; ++q) {
    int ok = 1, rlo[3] = { 0, 0, 0 }, rhi[3] = { 1, 1, 1 }, off[3] = { 0, 0, 0 };
    for (int d = 0; d < g->dim; ++d) {
      const int dir = dirs[q][d];
      if (dir != 0 && !g->periodic[d]) ok = 0;
      /* metadomain_comm.cpp:166-191: recv slice for -dir, send slice for dir */
      if (dir == 0) {
        rlo[d] = 0;
        rhi[d] = n[d] + 2 * ng;
        off[d] = 0;
      } else if (dir == 1) {
        rlo[d] = 0; /* recv [imin - ng, imin + ng) */
        rhi[d] = 2 * ng;
        off[d] = n[d]; /* send index = recv index + n */
      } else {
        rlo[d] = n[d]; /* recv [imax - ng, imax + ng) */
        rhi[d] = n[d] + 2 * ng;
        off[d] = -n[d];
      }
    }
    if (!ok) continue;
    for (int c = 0; c < 3; ++c)
      for (int k = rlo[2]; k < rhi[2]; ++k)
        for (int j = rlo[1]; j < rhi[1]; ++j)
          for (int i = rlo[0]; i < rhi[0]; ++i) {
            const int64_t dst = i * s[0] + j * s[1] + k * s[2] + c * s[3];
            const int64_t src = (i + off[0]) * s[0] + (j + off[1]) * s[1] +
                                (k + off[2]) * s[2] + c * s[3];
            B[dst] += J[src];
          }
  }
  /* AddBufferedFields over the active cells (metadomain_comm.cpp:374-406) */
  const int k0 = g->dim == 3 ? ng : 0, k1 = g->dim == 3 ? g->n3 + ng : 1;
  for (int c = 0; c < 3; ++c)
    for (int k = k0; k < k1; ++k)
      for (int j = ng; j < g->n2 + ng; ++j)
        for (int i = ng; i < g->n1 + ng; ++i) J[JI(g, i, j, k, c)] += B[JI(g, i, j, k, c)];
}

/* ------------------------------------------------------------------------ */
/* sorting                                                                  */
/* ------------------------------------------------------------------------ */
#define PERMUTE(T, arr)                                                        \
  do {                                                                         \
    if (arr) {                                                                 \
      T* tmp = (T*)malloc(sizeof(T) * (size_t)np);                             \
      for (int64_t q = 0; q < np; ++q) tmp[q] = (arr)[perm[q]];                \
      memcpy((arr), tmp, sizeof(T) * (size_t)np);                              \
      free(tmp);                                                               \
    }                                                                          \
  } while (0)

static void permute_all(const orc_grid* g, orc_species* sp, const int64_t* perm) {
  const int64_t np = sp->npart;
  PERMUTE(int32_t, sp->i1);
  PERMUTE(int32_t, sp->i1_prev);
  PERMUTE(float, sp->dx1);
  PERMUTE(float, sp->dx1_prev);
  PERMUTE(int32_t, sp->i2);
  PERMUTE(int32_t, sp->i2_prev);
  PERMUTE(float, sp->dx2);
  PERMUTE(float, sp->dx2_prev);
  if (g->dim == 3) {
    PERMUTE(int32_t, sp->i3);
    PERMUTE(int32_t, sp->i3_prev);
    PERMUTE(float, sp->dx3);
    PERMUTE(float, sp->dx3_prev);
  }
  PERMUTE(real, (real*)sp->ux1);
  PERMUTE(real, (real*)sp->ux2);
  PERMUTE(real, (real*)sp->ux3);
  PERMUTE(real, (real*)sp->weight);
  PERMUTE(int16_t, sp->tag);
}

/* tile: NULL for the reference's cell key, else the tile shape of the
 * tile-major key (tile index i1-fastest over tiles, then the cell inside the
 * tile i1-fastest, a row's even cells before its odd ones) that the GPU's
 * tiled sort uses */
static void sort_keyed(const orc_grid* g, orc_species* sp, const int* tile, int64_t* perm) {
  const int64_t np    = sp->npart;
  int           nt[3] = { 1, 1, 1 }, ts[3] = { 1, 1, 1 };
  const int     nn[3] = { g->n1, g->n2, g->dim == 3 ? g->n3 : 1 };
  if (tile) {
    for (int d = 0; d < 3; ++d) {
      ts[d] = d < g->dim ? tile[d] : 1;
      nt[d] = (nn[d] + ts[d] - 1) / ts[d];
    }
  }
  const int64_t total = tile ? (int64_t)nt[0] * nt[1] * nt[2] * ts[0] * ts[1] * ts[2]
                             : (int64_t)g->n1 * g->n2 * (g->dim == 3 ? g->n3 : 1);
  int64_t*      key   = (int64_t*)malloc(sizeof(int64_t) * (size_t)(np > 0 ? np : 1));
  int64_t*      cnt   = (int64_t*)calloc((size_t)(total + 3), sizeof(int64_t));
  for (int64_t p = 0; p < np; ++p) {
    if (sp->tag[p] != ORC_TAG_ALIVE) {
      key[p] = total + 1; /* sorting.h:114-116 */
    } else if (tile) {
      const int     c[3] = { sp->i1[p], sp->i2[p], g->dim == 3 ? sp->i3[p] : 0 };
      const int64_t t    = ((int64_t)(c[2] / ts[2]) * nt[1] + c[1] / ts[1]) * nt[0] + c[0] / ts[0];
      /* within a tile row the even cells come first, then the odd ones */
      const int lx = c[0] % ts[0], slot = (lx & 1) ? (ts[0] + 1) / 2 + lx / 2 : lx / 2;
      key[p] = ((t * ts[2] + c[2] % ts[2]) * ts[1] + c[1] % ts[1]) * ts[0] + slot;
    } else if (g->dim == 2) {
      key[p] = (int64_t)sp->i1[p] * g->n2 + sp->i2[p];
    } else {
      key[p] = ((int64_t)sp->i1[p] * g->n2 + sp->i2[p]) * g->n3 + sp->i3[p];
    }
    cnt[key[p] + 1]++;
  }
  for (int64_t b = 0; b < total + 2; ++b) cnt[b + 1] += cnt[b];
  for (int64_t p = 0; p < np; ++p) perm[cnt[key[p]]++] = p;
  permute_all(g, sp, perm);
  free(key);
  free(cnt);
}

void orc_sort(const orc_grid* g, orc_species* sp, int64_t* perm) { sort_keyed(g, sp, NULL, perm); }

void orc_sort_tiled(const orc_grid* g, orc_species* sp, const int* tile, int64_t* perm) {
  sort_keyed(g, sp, tile, perm);
}

int64_t orc_remove_dead(const orc_grid* g, orc_species* sp) {
  const int64_t np = sp->npart;
  int64_t*      perm = (int64_t*)calloc((size_t)(np > 0 ? np : 1), sizeof(int64_t));
  int64_t       na   = 0;
  if (!perm) return np;
  for (int64_t p = 0; p < np; ++p)
    if (sp->tag[p] == ORC_TAG_ALIVE) perm[na++] = p;
  int64_t nd = na;
  for (int64_t p = 0; p < np; ++p)
    if (sp->tag[p] != ORC_TAG_ALIVE) perm[nd++] = p;
  permute_all(g, sp, perm);
  for (int64_t p = 0; p < np; ++p) sp->tag[p] = p < na ? ORC_TAG_ALIVE : ORC_TAG_DEAD;
  free(perm);
  sp->npart = na;
  return na;
}

/* ------------------------------------------------------------------------ */
/* diagnostics (FP64)                                                       */
/* ------------------------------------------------------------------------ */
void orc_field_energy(const orc_grid* g, const void* EBv, double dx, double* out) {
  const real* EB = (const real*)EBv;
  const int   ng = g->ng, D = g->dim;
  const int   k0 = D == 3 ? ng : 0, k1 = D == 3 ? g->n3 + ng : 1;
  double      dV = D == 3 ? dx * dx * dx : dx * dx;
  double      e2 = 0, b2 = 0;
  for (int k = k0; k < k1; ++k)
    for (int j = ng; j < g->n2 + ng; ++j)
      for (int i = ng; i < g->n1 + ng; ++i)
        for (int c = 0; c < 3; ++c) {
          const double h  = (c < D) ? dx * dx : 1.0;
          const double ev = (double)EB[EBI(g, i, j, k, c)];
          const double bv = (double)EB[EBI(g, i, j, k, c + 3)];
          e2 += ev * ev * h * dV;
          b2 += bv * bv * h * dV;
        }
  out[0] = e2;
  out[1] = b2;
}

double orc_kinetic_energy(const orc_species* sp) {
  const real* u1 = (const real*)sp->ux1;
  const real* u2 = (const real*)sp->ux2;
  const real* u3 = (const real*)sp->ux3;
  const real* w  = (const real*)sp->weight;
  double      s  = 0;
  for (int64_t p = 0; p < sp->npart; ++p) {
    if (sp->tag[p] != ORC_TAG_ALIVE) continue;
    const double a = u1[p], b = u2[p], c = u3[p];
    s += (double)w[p] * (sqrt(1.0 + a * a + b * b + c * c) - 1.0) * (double)sp->mass;
  }
  return s;
}

void orc_charge_density(const orc_grid* g, const orc_species* sp, void* rho_, int order) {
  real*       rho = (real*)rho_;
  const real* w   = (const real*)sp->weight;
  const int   O   = order == 0 ? 1 : order;
  const int   ng  = g->ng;
  const real  charge = (real)sp->charge;
  for (int64_t p = 0; p < sp->npart; ++p) {
    if (sp->tag[p] != ORC_TAG_ALIVE) continue;
    int  imin[3] = { 0, 0, 0 };
    real S[3][4];
    shape(0, O, sp->i1[p], (real)sp->dx1[p], &imin[0], S[0]);
    shape(0, O, sp->i2[p], (real)sp->dx2[p], &imin[1], S[1]);
    if (g->dim == 3) shape(0, O, sp->i3[p], (real)sp->dx3[p], &imin[2], S[2]);
    const real q = charge * w[p];
    if (g->dim == 2) {
      for (int j = 0; j <= O; ++j) {
        const real qj = q * S[1][j];
        for (int i = 0; i <= O; ++i)
          rho[JI(g, imin[0] + ng + i, imin[1] + ng + j, 0, 0)] += qj * S[0][i];
      }
    } else {
      for (int k = 0; k <= O; ++k)
        for (int j = 0; j <= O; ++j) {
          const real qjk = q * S[2][k] * S[1][j];
          for (int i = 0; i <= O; ++i)
            rho[JI(g, imin[0] + ng + i, imin[1] + ng + j, imin[2] + ng + k, 0)] +=
              qjk * S[0][i];
        }
    }
  }
}

void orc_particle_moments(const orc_species* sp, double* out) {
  const real*  u1 = (const real*)sp->ux1;
  const real*  u2 = (const real*)sp->ux2;
  const real*  u3 = (const real*)sp->ux3;
  const real*  w  = (const real*)sp->weight;
  const double m  = (double)sp->mass;
  for (int64_t p = 0; p < sp->npart; ++p) {
    if (sp->tag[p] != ORC_TAG_ALIVE) continue;
    const double a = u1[p], b = u2[p], c = u3[p];
    const double u2s = a * a + b * b + c * c;
    const double gm  = sqrt(1.0 + u2s);
    out[0] += m == 0.0 ? sqrt(u2s) : m * gm;
    out[1] += a;
    out[2] += b;
    out[3] += c;
    out[4] += (double)w[p] * (m == 0.0 ? sqrt(u2s) : m * (u2s / (gm + 1.0)));
    out[5] += (double)w[p];
  }
}

/* ------------------------------------------------------------------------ */
/* SR field boundaries                                                      */
/* ------------------------------------------------------------------------ */
/* ConductorBoundaries_kernel (fields_bcs.hpp:522-800) on one side: offsets
 * k from the wall cell, over [0, ng + 1) below and [0, ng) above */
static void conductor_side(const orc_grid* g, real* F, int axis, int hi, int set_e, int set_b) {
  const int ng = g->ng, n = axis == 0 ? g->n1 : (axis == 1 ? g->n2 : g->n3);
  const int edge = hi ? n + ng : ng, K = hi ? ng : ng + 1;
  const int oa = axis == 0 ? 1 : 0, ob = axis == 2 ? 1 : 2;
  const int t1 = oa, t2 = g->dim == 3 ? ob : 2;
  const int ea = ext(g, oa), eb = g->dim == 3 ? ext(g, ob) : 1;
  for (int pb = 0; pb < eb; ++pb)
    for (int pa = 0; pa < ea; ++pa)
      for (int k = 0; k < K; ++k) {
#define AT(i, c) F[cond_idx(g, axis, oa, ob, i, pa, pb, c)]
        if (set_e) {
          if (k == 0) {
            AT(edge, t1) = 0;
            AT(edge, t2) = 0;
          } else if (!hi) {
            AT(edge - k, axis) = AT(edge + k - 1, axis);
            AT(edge - k, t1)   = -AT(edge + k, t1);
            AT(edge - k, t2)   = -AT(edge + k, t2);
          } else {
            AT(edge + k - 1, axis) = AT(edge - k, axis);
            AT(edge + k, t1)       = -AT(edge - k, t1);
            AT(edge + k, t2)       = -AT(edge - k, t2);
          }
        }
        if (set_b) {
          if (k == 0) {
            AT(edge, 3 + axis) = 0;
          } else if (!hi) {
            AT(edge - k, 3 + axis) = -AT(edge + k, 3 + axis);
            AT(edge - k, 3 + t1)   = AT(edge + k - 1, 3 + t1);
            AT(edge - k, 3 + t2)   = AT(edge + k - 1, 3 + t2);
          } else {
            AT(edge + k, 3 + axis)   = -AT(edge - k, 3 + axis);
            AT(edge + k - 1, 3 + t1) = AT(edge - k, 3 + t1);
            AT(edge + k - 1, 3 + t2) = AT(edge - k, 3 + t2);
          }
        }
#undef AT
      }
}

/* MatchBoundaries_kernel, SRPIC branch, on one side over the cells that
 * MatchFieldsIn / ExtentToRange select (srpic/fields_bcs.h:60-202, mesh.h:
 * 133-202) */
static void match_side(const orc_grid* g, real* F, const real* T, int axis, int hi, int set_e,
                       int set_b, const double x_min[3], double dx_d, double ds_d) {
  const int  ng = g->ng, n = axis == 0 ? g->n1 : (axis == 1 ? g->n2 : g->n3);
  const real dx = (real)dx_d, x0 = (real)x_min[axis], x1 = x0 + (real)n * dx, ds = (real)ds_d;
  real       lo_x = hi ? x1 - ds : x0, hi_x = hi ? x1 : x0 + ds;
  lo_x = lo_x < x0 ? x0 : (lo_x > x1 ? x1 : lo_x);
  hi_x = hi_x > x1 ? x1 : (hi_x < x0 ? x0 : hi_x);
#ifdef ORC_SINGLE
  real a = floorf((lo_x - x0) / dx), e = ceilf((hi_x - x0) / dx);
#else
  real a = floor((lo_x - x0) / dx), e = ceil((hi_x - x0) / dx);
#endif
  int i0, i1;
  if (hi) {
    if (a < 0) a = 0;
    i0 = (int)a + ng;
    i1 = (int)e + 2 * ng;
  } else {
    if (e > (real)n) e = (real)n;
    i0 = (int)a;
    i1 = (int)e + ng;
  }
  if (i0 < 0) i0 = 0;
  if (i1 > n + 2 * ng) i1 = n + 2 * ng;
  const real x_edge = hi ? x1 : x0, ONE = 1, FOUR = 4, H = 0.5;
  const int  oa = axis == 0 ? 1 : 0, ob = axis == 2 ? 1 : 2;
  const int  ea = ext(g, oa), eb = g->dim == 3 ? ext(g, ob) : 1;
  for (int i = i0; i < i1; ++i) {
    const real i_ = (real)(i - ng);
#ifdef ORC_SINGLE
    const real s0 = tanhf(fabsf((x0 + i_ * dx) - x_edge) * FOUR / ds);
    const real sH = tanhf(fabsf((x0 + (i_ + H) * dx) - x_edge) * FOUR / ds);
#else
    const real s0 = tanh(fabs((x0 + i_ * dx) - x_edge) * FOUR / ds);
    const real sH = tanh(fabs((x0 + (i_ + H) * dx) - x_edge) * FOUR / ds);
#endif
    for (int pb = 0; pb < eb; ++pb)
      for (int pa = 0; pa < ea; ++pa)
        for (int c = 0; c < 6; ++c) {
          if (c < 3 ? !set_e : !set_b) continue;
          const int  half = c < 3 ? (c == axis) : (c - 3 != axis);
          const real s    = half ? sH : s0;
          const int64_t q = cond_idx(g, axis, oa, ob, i, pa, pb, c);
          F[q] = s * F[q] + (ONE - s) * T[q];
        }
  }
}

void orc_field_boundaries(const orc_grid* g, void* EB, int set_e, int set_b, const void* target,
                          const double x_min[3], double dx, const double ds[3][2]) {
  real* F = (real*)EB;
  int   order[6][2], m = 0;
  for (int d = 0; d < g->dim; ++d) order[m][0] = d, order[m++][1] = 0;
  for (int d = g->dim - 1; d >= 0; --d) order[m][0] = d, order[m++][1] = 1;
  for (int k = 0; k < m; ++k) {
    const int axis = order[k][0], hi = order[k][1], kind = g->fbc[axis][hi];
    if (kind == 2) conductor_side(g, F, axis, hi, set_e, set_b);
    else if (kind == 3)
      match_side(g, F, (const real*)target, axis, hi, set_e, set_b, x_min, dx, ds[axis][hi]);
  }
}
