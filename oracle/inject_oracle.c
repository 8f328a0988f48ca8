/*
 * CPU oracle: uniform Maxwellian pair injection (TEST INFRASTRUCTURE ONLY).
 * See inject_oracle.h for the random-number contract.
 */
#include "inject_oracle.h"

#include <math.h>
#include <stdlib.h>

#ifdef ORC_SINGLE
typedef float real;
#define RSQRT sqrtf
#define RLOG  logf
#define RCOS  cosf
#define RSIN  sinf
#define RFABS fabsf
static const real EPS = 1.1920929e-07f;
#else
typedef double real;
#define RSQRT sqrt
#define RLOG  log
#define RCOS  cos
#define RSIN  sin
#define RFABS fabs
static const real EPS = 2.220446049250313e-16;
#endif

/* Philox4x32-10: ten rounds of two 32x32 -> 64 multiplications, the key
 * bumped by the Weyl constants between rounds */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t k0 = key_in[0], k1 = key_in[1];
  uint32_t x0 = ctr[0], x1 = ctr[1], x2 = ctr[2], x3 = ctr[3];
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * x0, p1 = (uint64_t)0xCD9E8D57u * x2;
    const uint32_t y0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0;
    const uint32_t y2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1;
    x1 = (uint32_t)p1;
    x3 = (uint32_t)p0;
    x0 = y0;
    x2 = y2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = x0, out[1] = x1, out[2] = x2, out[3] = x3;
}

typedef struct {
  uint32_t key[2], ctr[4], buf[4];
  int      used;
} rng_t;

static void rng_init(rng_t* g, uint64_t seed, uint64_t stream) {
  g->key[0] = (uint32_t)seed;
  g->key[1] = (uint32_t)(seed >> 32);
  g->ctr[0] = g->ctr[1] = 0u;
  g->ctr[2] = (uint32_t)stream;
  g->ctr[3] = (uint32_t)(stream >> 32);
  g->used   = 4;
}

static uint32_t rng_next(rng_t* g) {
  if (g->used == 4) {
    orc_philox4x32_10(g->ctr, g->key, g->buf);
    if (++g->ctr[0] == 0u) ++g->ctr[1];
    g->used = 0;
  }
  return g->buf[g->used++];
}

static real uniform(rng_t* g) {
#ifdef ORC_SINGLE
  return (real)(rng_next(g) >> 8) * 5.9604644775390625e-8f;
#else
  const uint32_t a = rng_next(g) >> 5, b = rng_next(g) >> 6;
  return ((double)a * 67108864.0 + (double)b) * 1.1102230246251565e-16;
#endif
}

static int almost_zero(real x) { return RFABS(x) <= EPS; }

enum { MAX_ZERO_REDRAWS = 64, MAX_SOBOL_PASSES = 4096 };

typedef struct {
  real temp, d3, d4, dir[3];
  int  ddir;
} maxwell_t;

/* Maxwellian's constructor (energy_dist.h:184-222) */
static void maxwell_init(maxwell_t* m, double temperature, float mass, const double* drift) {
  m->temp = (real)temperature / (real)mass;
  const real u[3] = { (real)drift[0], (real)drift[1], (real)drift[2] };
  const real d4   = RSQRT(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  m->d4 = d4;
  m->d3 = 0;
  m->dir[0] = m->dir[1] = m->dir[2] = 0;
  m->ddir = 0;
  if (almost_zero(d4)) return;
  m->d3     = d4 / RSQRT((real)1 + d4 * d4);
  m->dir[0] = u[0] / d4;
  m->dir[1] = u[1] / d4;
  m->dir[2] = u[2] / d4;
  m->ddir   = 4;
  for (int d = 0; d < 3; ++d) {
    if (almost_zero(u[(d + 2) % 3]) && almost_zero(u[(d + 1) % 3])) {
      m->ddir = (u[d] < (real)0 ? -1 : 1) * (d + 1);
      break;
    }
  }
}

static real product3(rng_t* g) {
  const real a = uniform(g);
  const real b = uniform(g);
  const real c = uniform(g);
  return a * b * c;
}

/* JuttnerSinge (energy_dist.h:79-134) */
static int juttner_synge(real* v, real temp, rng_t* g) {
  const real ONE = 1, TWO = 2, TWO_PI = (real)6.28318530717958647692;
  int        ok = 1;
  if (temp < (real)0.5) {
    for (int c = 0; c < 3; ++c) {
      real x1 = uniform(g);
      int  k  = 0;
      while (almost_zero(x1) && k++ < MAX_ZERO_REDRAWS) x1 = uniform(g);
      ok = ok && k <= MAX_ZERO_REDRAWS;
      x1 = RSQRT(-TWO * RLOG(x1));
      const real x2 = TWO_PI * uniform(g);
      v[c] = x1 * RCOS(x2) * RSQRT(temp);
    }
  } else {
    real u = ONE, eta = uniform(g), x1 = 0, x2 = 0;
    int  pass = 0;
    while (eta * eta <= u * u + ONE && pass++ < MAX_SOBOL_PASSES) {
      x1    = product3(g);
      int k = 0;
      while (almost_zero(x1) && k++ < MAX_ZERO_REDRAWS) x1 = product3(g);
      ok = ok && k <= MAX_ZERO_REDRAWS;
      u  = -temp * RLOG(x1);
      x2 = uniform(g);
      k  = 0;
      while (almost_zero(x2) && k++ < MAX_ZERO_REDRAWS) x2 = uniform(g);
      ok  = ok && k <= MAX_ZERO_REDRAWS;
      eta = -temp * RLOG(x1 * x2);
    }
    ok   = ok && pass <= MAX_SOBOL_PASSES;
    x1   = uniform(g);
    x2   = uniform(g);
    v[0] = u * (TWO * x1 - ONE);
    v[2] = TWO * u * RSQRT(x1 * (ONE - x1));
    v[1] = v[2] * RCOS(TWO_PI * x2);
    v[2] = v[2] * RSIN(TWO_PI * x2);
  }
  return ok;
}

/* Maxwellian::operator() (energy_dist.h:224-273) */
static int maxwellian(const maxwell_t* m, rng_t* g, real* v) {
  const real ONE = 1;
  int        ok  = 1;
  if (almost_zero(m->temp)) {
    v[0] = v[1] = v[2] = 0;
  } else {
    ok = juttner_synge(v, m->temp, g);
  }
  if (m->ddir != 0) {
    const real gamma = RSQRT(ONE + (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
    if (-m->d3 * v[0] > gamma * uniform(g)) v[0] = -v[0];
    v[0] = RSQRT(ONE + m->d4 * m->d4) * (v[0] + m->d3 * gamma);
    if (m->ddir == -1) {
      v[0] = -v[0];
    } else if (m->ddir == 2 || m->ddir == -2) {
      const real t = v[1];
      v[1] = m->ddir > 0 ? v[0] : -v[0];
      v[0] = t;
    } else if (m->ddir == 3 || m->ddir == -3) {
      const real t = v[2];
      v[2] = m->ddir > 0 ? v[0] : -v[0];
      v[0] = t;
    } else if (m->ddir == 4) {
      const real o0 = v[0], o1 = v[1], o2 = v[2];
      const real a = m->dir[0], b = m->dir[1], c = m->dir[2];
      v[0] = o0 * a - o1 * b - o2 * c;
      v[1] = (o0 * b * (a + ONE) + o1 * (a * a + a + c * c) - o2 * b * c) / (a + ONE);
      v[2] = (o0 * c * (a + ONE) - o1 * b * c - o2 * (-a + c * c - ONE)) / (a + ONE);
    }
  }
  return ok;
}

int64_t orc_inject_count(int dim, const orc_inject_params* ip) {
  long double cells = 1.0L;
  for (int d = 0; d < dim; ++d)
    cells *= (long double)(real)ip->xi_max[d] - (long double)(real)ip->xi_min[d];
  const real dens = (real)ip->ppc0 * (real)ip->number_density * (real)0.5;
  return (int64_t)((long double)dens * cells);
}

int orc_inject_sample_pair(int dim, const orc_inject_params* ip, const float mass[2], uint64_t p,
                           void* x_out, void* v_out) {
  real*     x = (real*)x_out;
  real*     v = (real*)v_out;
  maxwell_t m[2];
  for (int s = 0; s < 2; ++s) maxwell_init(&m[s], ip->temperature[s], mass[s], ip->drift[s]);
  rng_t g;
  rng_init(&g, ip->seed, ip->first_pair + p);
  for (int d = 0; d < dim; ++d)
    x[d] = (real)ip->xi_min[d] + uniform(&g) * ((real)ip->xi_max[d] - (real)ip->xi_min[d]);
  int ok = maxwellian(&m[0], &g, v);
  ok     = maxwellian(&m[1], &g, v + 3) && ok;
  return ok;
}

int64_t orc_inject_uniform(const orc_grid* gr, orc_species* sp1, orc_species* sp2,
                           const orc_inject_params* ip, int64_t* failures) {
  const int     D = gr->dim;
  const int64_t n = orc_inject_count(D, ip);
  const float   mass[2] = { sp1->mass, sp2->mass };
  orc_species*  sps[2]  = { sp1, sp2 };
  int64_t       bad     = 0;
  for (int64_t p = 0; p < n; ++p) {
    real x[3] = { 0, 0, 0 }, v[6];
    if (!orc_inject_sample_pair(D, ip, mass, (uint64_t)p, x, v)) ++bad;
    for (int s = 0; s < 2; ++s) {
      orc_species*  S = sps[s];
      const int64_t q = S->npart + p;
      int32_t*      ia[3] = { S->i1, S->i2, S->i3 };
      float*        da[3] = { S->dx1, S->dx2, S->dx3 };
      for (int d = 0; d < D; ++d) {
        const int i = (int)x[d];
        ia[d][q]    = i;
        da[d][q]    = (float)(x[d] - (real)i);
      }
      ((real*)S->ux1)[q]    = v[3 * s + 0];
      ((real*)S->ux2)[q]    = v[3 * s + 1];
      ((real*)S->ux3)[q]    = v[3 * s + 2];
      ((real*)S->weight)[q] = (real)1;
      S->tag[q]             = ORC_TAG_ALIVE;
    }
  }
  sp1->npart += n;
  sp2->npart += n;
  if (failures) *failures = bad;
  return n;
}
