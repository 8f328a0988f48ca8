/*
 * CPU oracle: output preparation (TEST INFRASTRUCTURE ONLY).
 * See output_oracle.h for what each function restates.
 */
#include "output_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef ORC_SINGLE
typedef float real;
#define RSQRT sqrtf
#define RFABS fabsf
static const real EPS = 1.1920928955078125e-07f;
#else
typedef double real;
#define RSQRT sqrt
#define RFABS fabs
static const real EPS = 2.220446049250313e-16;
#endif

#define SQR(x)  ((x) * (x))
#define CUBE(x) ((x) * (x) * (x))

static const real ZERO = 0, ONE = 1, TWO = 2, THREE = 3, HALF = 0.5, THREE_HALFS = 1.5;
static const real INV_2 = 0.5, INV_4 = 0.25, INV_8 = 0.125, THREE_FOURTHS = 0.75;

/* prtl_shape::S1..S6 (src/kernels/particle_shapes.hpp:25-166) */
static real spline(int order, real x) {
  switch (order) {
    case 0: return ONE;
    case 1: return x < ONE ? ONE - x : ZERO;
    case 2:
      if (x < HALF) return (real)0.75 - SQR(x);
      if (x < THREE_HALFS) return HALF * SQR(THREE_HALFS - x);
      return ZERO;
    case 3:
      if (x < ONE) return (real)(2.0 / 3.0) - SQR(x) + HALF * CUBE(x);
      if (x < TWO) return (real)(4.0 / 3.0) - TWO * x + SQR(x) - (real)(1.0 / 6.0) * CUBE(x);
      return ZERO;
    case 4:
      if (x < HALF)
        return (real)(115.0 / 192.0) - (real)(5.0 / 8.0) * SQR(x) + INV_4 * SQR(SQR(x));
      if (x < THREE_HALFS)
        return (real)(55.0 / 96.0) + (real)(5.0 / 24.0) * x - (real)(5.0 / 4.0) * SQR(x) +
               (real)(5.0 / 6.0) * CUBE(x) - (real)(1.0 / 6.0) * SQR(SQR(x));
      if (x < (real)2.5)
        return (real)(625.0 / 384.0) - (real)(125.0 / 48.0) * x + (real)(25.0 / 16.0) * SQR(x) -
               (real)(5.0 / 12.0) * CUBE(x) + (real)(1.0 / 24.0) * SQR(SQR(x));
      return ZERO;
    case 5:
      if (x <= ONE)
        return (real)(11.0 / 20.0) - HALF * SQR(x) + INV_4 * SQR(SQR(x)) -
               (real)(1.0 / 12.0) * CUBE(x) * SQR(x);
      if (x < TWO)
        return (real)(17.0 / 40.0) + (real)(5.0 / 8.0) * x - (real)(7.0 / 4.0) * SQR(x) +
               (real)(5.0 / 4.0) * CUBE(x) - (real)(3.0 / 8.0) * SQR(SQR(x)) +
               (real)(1.0 / 24.0) * CUBE(x) * SQR(x);
      if (x < THREE)
        return (real)(81.0 / 40.0) - (real)(27.0 / 8.0) * x + (real)(9.0 / 4.0) * SQR(x) -
               THREE_FOURTHS * CUBE(x) + INV_8 * SQR(SQR(x)) -
               (real)(1.0 / 120.0) * CUBE(x) * SQR(x);
      return ZERO;
    case 6:
      if (x <= HALF)
        return (real)(5887.0 / 11520.0) - (real)(77.0 / 192.0) * SQR(x) +
               (real)(7.0 / 48.0) * SQR(SQR(x)) - (real)(1.0 / 36.0) * SQR(CUBE(x));
      if (x < THREE_HALFS)
        return (real)(7861.0 / 15360.0) - (real)(7.0 / 768.0) * x -
               (real)(91.0 / 256.0) * SQR(x) - (real)(35.0 / 288.0) * CUBE(x) +
               (real)(21.0 / 64.0) * SQR(SQR(x)) - (real)(7.0 / 48.0) * CUBE(x) * SQR(x) +
               (real)(1.0 / 48.0) * SQR(CUBE(x));
      if (x < (real)2.5)
        return (real)(1379.0 / 7680.0) + (real)(1267.0 / 960.0) * x -
               (real)(329.0 / 128.0) * SQR(x) + (real)(133.0 / 72.0) * CUBE(x) -
               (real)(21.0 / 32.0) * SQR(SQR(x)) + (real)(7.0 / 60.0) * CUBE(x) * SQR(x) -
               (real)(1.0 / 120.0) * SQR(CUBE(x));
      if (x < (real)3.5)
        return (real)(117649.0 / 46080.0) - (real)(16807.0 / 3840.0) * x +
               (real)(2401.0 / 768.0) * SQR(x) - (real)(343.0 / 288.0) * CUBE(x) +
               (real)(49.0 / 192.0) * SQR(SQR(x)) - (real)(7.0 / 240.0) * CUBE(x) * SQR(x) +
               (real)(1.0 / 720.0) * SQR(CUBE(x));
      return ZERO;
  }
  return ZERO;
}

double orc_spline(int order, double x) { return (double)spline(order, (real)x); }

static int64_t eidx(const orc_grid* g, int i, int j, int k, int c) {
  return (int64_t)i * g->em_s[0] + (int64_t)j * g->em_s[1] + (int64_t)k * g->em_s[2] +
         (int64_t)c * g->em_s[3];
}

/* ParticleMoments_kernel::operator() (particle_moments.hpp:291-404) for
 * every particle in index order; computeStressEnergyComponent (146-222) and
 * computeBulk3VelocityTimesMass (224-254) on a Cartesian grid */
void orc_output_moment(const orc_grid* g, const orc_species* sp, int id, int c1, int c2,
                       int order, int smoothing, int use_weights, double inv_n0_d, double dx_d,
                       void* bckpv, int comp) {
  real*          buf = (real*)bckpv;
  const int      D = g->dim, W = (order + 1) / 2, n[3] = { g->n1, g->n2, g->n3 };
  const int32_t* ia[3] = { sp->i1, sp->i2, sp->i3 };
  const float*   da[3] = { sp->dx1, sp->dx2, sp->dx3 };
  const real*    ux[3] = { (const real*)sp->ux1, (const real*)sp->ux2, (const real*)sp->ux3 };
  const real*    w     = (const real*)sp->weight;
  const real     mass = (real)sp->mass, m_or_1 = sp->mass == 0.0f ? ONE : mass;
  const real     inv_n0 = (real)inv_n0_d, dx = (real)dx_d;
  const real     h = D == 2 ? SQR(dx) : CUBE(dx); /* Minkowski sqrt_det_h */
  for (int64_t p = 0; p < sp->npart; ++p) {
    if (sp->tag[p] != ORC_TAG_ALIVE) continue;
    int cell[3] = { 0, 0, 0 }, ok = 1;
    for (int d = 0; d < D; ++d) {
      cell[d] = ia[d][p];
      if (cell[d] < 0 || cell[d] >= n[d]) ok = 0;
    }
    if (!ok) continue;
    real coeff;
    if (id == 4 || id == 5) {
      const real u[3] = { ux[0][p], ux[1][p], ux[2][p] };
      const real u0   = sp->mass == 0.0f ? RSQRT(u[0] * u[0] + u[1] * u[1] + u[2] * u[2])
                                         : RSQRT(ONE + (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
      if (id == 4) {
        coeff = m_or_1 / u0;
        const int cs[2] = { c1, c2 };
        for (int q = 0; q < 2; ++q) coeff *= cs[q] > 0 ? u[cs[q] - 1] : u0;
      } else {
        coeff = m_or_1 * u[c1 - 1] / u0;
      }
    } else {
      coeff = id == 0 ? mass : id == 1 ? (real)sp->charge : ONE;
    }
    if (id != 3) {
      coeff *= inv_n0 / h;
      if (use_weights) coeff *= w[p];
    }
    const int kmin = D == 3 ? -W : 0, kmax = D == 3 ? W : 0;
    for (int dk = kmin; dk <= kmax; ++dk)
      for (int dj = -W; dj <= W; ++dj)
        for (int di = -W; di <= W; ++di) {
          const int  dd[3] = { di, dj, dk };
          real       S[3] = { ONE, ONE, ONE };
          for (int d = 0; d < D; ++d) {
            const real dl = RFABS((real)da[d][p] - ((real)dd[d] + HALF));
            S[d] = smoothing == 2 ? spline(order, dl) : ONE / (TWO * (real)W + ONE);
          }
          real sh = S[0] * S[1];
          if (D == 3) sh = sh * S[2];
          const int k = D == 3 ? cell[2] + dk + g->ng : 0;
          buf[eidx(g, cell[0] + di + g->ng, cell[1] + dj + g->ng, k, comp)] += coeff * sh;
        }
  }
}

static int directions(int D, int out[26][3]) {
  int m = 0;
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b)
      for (int c = (D == 3 ? -1 : 0); c <= (D == 3 ? 1 : 0); ++c) {
        if (a == 0 && b == 0 && c == 0) continue;
        out[m][0] = a, out[m][1] = b, out[m][2] = c;
        ++m;
      }
  return m;
}

static int ext(const orc_grid* g, int d) {
  const int n[3] = { g->n1, g->n2, g->n3 };
  return d < g->dim ? n[d] + 2 * g->ng : 1;
}

/* SynchronizeFields(Comm::Bckp) on one domain: every direction adds the
 * sender's slice into a zeroed receive buffer (comm_nompi.hpp:28-119 with
 * synchronize = true), then AddBufferedFields over the active cells
 * (metadomain_comm.cpp:374-406) */
void orc_sync_moments(const orc_grid* g, void* bckpv, int c0, int c1) {
  real*         f  = (real*)bckpv;
  const int     ng = g->ng, n[3] = { g->n1, g->n2, g->n3 };
  const int64_t total = (int64_t)ext(g, 0) * ext(g, 1) * ext(g, 2) * 6;
  real*         recv  = (real*)calloc((size_t)total, sizeof(real));
  /* the receive buffer uses a compact layout: i fastest, then j, k, c */
  const int64_t rs[4] = { 1, ext(g, 0), (int64_t)ext(g, 0) * ext(g, 1),
                          (int64_t)ext(g, 0) * ext(g, 1) * ext(g, 2) };
  int           dirs[26][3];
  const int     nd = directions(g->dim, dirs);
  for (int q = 0; q < nd; ++q) {
    int ok = 1, lo[3] = { 0, 0, 0 }, hi[3] = { 1, 1, 1 }, off[3] = { 0, 0, 0 };
    for (int d = 0; d < g->dim; ++d) {
      const int dir = dirs[q][d];
      if (dir != 0 && !g->periodic[d]) ok = 0;
      if (dir == 0) {
        lo[d] = 0, hi[d] = n[d] + 2 * ng, off[d] = 0;
      } else if (dir == 1) {
        lo[d] = 0, hi[d] = 2 * ng, off[d] = n[d];
      } else {
        lo[d] = n[d], hi[d] = n[d] + 2 * ng, off[d] = -n[d];
      }
    }
    if (!ok) continue;
    for (int c = c0; c < c1; ++c)
      for (int k = lo[2]; k < hi[2]; ++k)
        for (int j = lo[1]; j < hi[1]; ++j)
          for (int i = lo[0]; i < hi[0]; ++i)
            recv[i * rs[0] + j * rs[1] + k * rs[2] + c * rs[3]] +=
              f[eidx(g, i + off[0], j + off[1], k + off[2], c)];
  }
  const int k0 = g->dim == 3 ? ng : 0, k1 = g->dim == 3 ? g->n3 + ng : 1;
  for (int c = c0; c < c1; ++c)
    for (int k = k0; k < k1; ++k)
      for (int j = ng; j < g->n2 + ng; ++j)
        for (int i = ng; i < g->n1 + ng; ++i)
          f[eidx(g, i, j, k, c)] += recv[i * rs[0] + j * rs[1] + k * rs[2] + c * rs[3]];
  free(recv);
}

/* NormalizeVectorByRho_kernel (particle_moments.hpp:440-478) */
void orc_normalize_by_rho(const orc_grid* g, void* bckpv, int c_rho, int c_v1, int c_v2, int c_v3) {
  real*     f  = (real*)bckpv;
  const int ng = g->ng;
  const int k0 = g->dim == 3 ? ng : 0, k1 = g->dim == 3 ? g->n3 + ng : 1;
  for (int k = k0; k < k1; ++k)
    for (int j = ng; j < g->n2 + ng; ++j)
      for (int i = ng; i < g->n1 + ng; ++i) {
        const real rho = f[eidx(g, i, j, k, c_rho)];
        if (RFABS(rho) <= EPS) continue;
        f[eidx(g, i, j, k, c_v1)] /= rho;
        f[eidx(g, i, j, k, c_v2)] /= rho;
        f[eidx(g, i, j, k, c_v3)] /= rho;
      }
}

/* FieldsToPhys_kernel<Minkowski>::operator() (fields_to_phys.hpp:125-236) at
 * the downsampled cells of the writer (writer.cpp:199-300) */
void orc_output_field(const orc_grid* g, const void* srcv, int is_em, int c0, int ncomp,
                      unsigned flags, double dx_d, const int dwn[3], void* outv) {
  const real*    F  = (const real*)srcv;
  real*          out = (real*)outv;
  const int64_t* s  = is_em ? g->em_s : g->cur_s;
  const int      D = g->dim, ng = g->ng, n[3] = { g->n1, g->n2, g->n3 };
  const real     dx = (real)dx_d;
  int            o[3] = { 1, 1, 1 }, dd[3] = { 1, 1, 1 };
  for (int d = 0; d < D; ++d) {
    dd[d] = dwn[d];
    o[d]  = (n[d] + dwn[d] - 1) / dwn[d];
  }
  const int64_t count = (int64_t)o[0] * o[1] * o[2];
#define AT(ii, jj, kk, cc) \
  F[(int64_t)(ii) * s[0] + (int64_t)(jj) * s[1] + (int64_t)(kk) * s[2] + (int64_t)(c0 + (cc)) * s[3]]
  for (int e = 0; e < o[2]; ++e)
    for (int b = 0; b < o[1]; ++b)
      for (int a = 0; a < o[0]; ++a) {
        const int64_t t = a + (int64_t)o[0] * (b + (int64_t)o[1] * e);
        const int     i = a * dd[0] + ng, j = b * dd[1] + ng, k = D == 3 ? e * dd[2] + ng : 0;
        real          v[3];
        if (ncomp == 1) {
          out[t] = AT(i, j, k, 0);
          continue;
        }
        if (flags & 1u) {
          if (D == 2) {
            v[0] = INV_2 * (AT(i, j, k, 0) + AT(i, j + 1, k, 0));
            v[1] = INV_2 * (AT(i, j, k, 1) + AT(i + 1, j, k, 1));
            v[2] = INV_4 * (AT(i, j, k, 2) + AT(i + 1, j, k, 2) + AT(i, j + 1, k, 2) +
                            AT(i + 1, j + 1, k, 2));
          } else {
            v[0] = INV_4 * (AT(i, j, k, 0) + AT(i, j + 1, k, 0) + AT(i, j, k + 1, 0) +
                            AT(i, j + 1, k + 1, 0));
            v[1] = INV_4 * (AT(i, j, k, 1) + AT(i + 1, j, k, 1) + AT(i, j, k + 1, 1) +
                            AT(i + 1, j, k + 1, 1));
            v[2] = INV_4 * (AT(i, j, k, 2) + AT(i + 1, j, k, 2) + AT(i, j + 1, k, 2) +
                            AT(i + 1, j + 1, k, 2));
          }
        } else if (flags & 2u) {
          v[0] = INV_2 * (AT(i, j, k, 0) + AT(i + 1, j, k, 0));
          v[1] = INV_2 * (AT(i, j, k, 1) + AT(i, j + 1, k, 1));
          v[2] = D == 3 ? INV_2 * (AT(i, j, k, 2) + AT(i, j, k + 1, 2)) : AT(i, j, k, 2);
        } else {
          v[0] = AT(i, j, k, 0);
          v[1] = AT(i, j, k, 1);
          v[2] = AT(i, j, k, 2);
        }
        if (flags & 4u) {
          /* transform<i, Idx::U, Idx::T>: v * sqrt(h_ii) = v * dx for i <= D */
          for (int c = 0; c < D; ++c) v[c] = v[c] * dx;
        }
        for (int c = 0; c < 3; ++c) out[t + c * count] = v[c];
      }
#undef AT
}

/* PrtlToPhys_kernel<SRPIC, Minkowski, false> (prtls_to_phys.hpp:121-200) */
int64_t orc_output_particles(const orc_grid* g, const orc_species* sp, int64_t stride, double dx_d,
                             const double xmin[3], void* x1, void* x2, void* x3, void* u1,
                             void* u2, void* u3, void* w) {
  const int64_t  nout = sp->npart / stride;
  const real     dx   = (real)dx_d;
  const int32_t* ia[3] = { sp->i1, sp->i2, sp->i3 };
  const float*   da[3] = { sp->dx1, sp->dx2, sp->dx3 };
  real*          xo[3] = { (real*)x1, (real*)x2, (real*)x3 };
  const real*    ui[3] = { (const real*)sp->ux1, (const real*)sp->ux2, (const real*)sp->ux3 };
  real*          uo[3] = { (real*)u1, (real*)u2, (real*)u3 };
  for (int64_t p = 0; p < nout; ++p) {
    const int64_t q = p * stride;
    for (int d = 0; d < g->dim; ++d) {
      const real xc = (real)ia[d][q] + (real)da[d][q];
      xo[d][p]      = xc * dx + (real)xmin[d];
    }
    for (int d = 0; d < 3; ++d) uo[d][p] = ui[d][q];
    ((real*)w)[p] = ((const real*)sp->weight)[q];
  }
  return nout;
}

/* ComputeDivergence_kernel<Minkowski> (divergences.hpp:23-135), Cartesian */
void orc_output_divergence(const orc_grid* g, const void* EBv, void* bckpv, int comp) {
  const real* E  = (const real*)EBv;
  real*       f  = (real*)bckpv;
  const int   ng = g->ng;
  const int   k0 = g->dim == 3 ? ng : 0, k1 = g->dim == 3 ? g->n3 + ng : 1;
  for (int k = k0; k < k1; ++k)
    for (int j = ng; j < g->n2 + ng; ++j)
      for (int i = ng; i < g->n1 + ng; ++i) {
        real v = E[eidx(g, i, j, k, 0)] - E[eidx(g, i - 1, j, k, 0)] + E[eidx(g, i, j, k, 1)] -
                 E[eidx(g, i, j - 1, k, 1)];
        if (g->dim == 3) v = v + E[eidx(g, i, j, k, 2)] - E[eidx(g, i, j, k - 1, 2)];
        f[eidx(g, i, j, k, comp)] = v;
      }
}
