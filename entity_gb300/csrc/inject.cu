// Uniform Maxwellian pair injection on the device and its C ABI.
//
// The reference's arch::InjectUniformMaxwellians (src/archetypes/utils.h:
// 46-107) builds two arch::energy_dist::Maxwellian samplers
// (src/archetypes/energy_dist.h:79-279) and runs
// kernel::UniformInjector_kernel (src/kernels/injectors.hpp:83-289) once per
// pair: a uniform position in the injection box shared by both species, a
// velocity per species, weight 1 (Cartesian) or sqrt(det h) / V0 (GR), tag
// alive, appended after each species' live particles. The pair count is
// ComputeNumInject's (src/archetypes/particle_injector.h:112-139).
//
// Random numbers: Kokkos' XorShift pool streams are not reproducible outside
// Kokkos, so each pair draws from its own Philox4x32-10 stream (Salmon et
// al., "Parallel random numbers: as easy as 1, 2, 3", SC11): key = seed,
// counter = (block, pair index). A pair's numbers do not depend on the launch
// shape, and the oracle draws the same ones.
#include <cmath>
#include <cstdint>

#include "ctx_internal.cuh"
#include "gr_host.cuh"
#include "gr_metric.cuh"

using namespace pic_internal;

namespace pic {

// ---------------------------------------------------------------------------
// Philox4x32-10
// ---------------------------------------------------------------------------
struct Philox4x32 {
  uint32_t key[2];
  uint32_t ctr[4];
  uint32_t buf[4];
  int      used;

  __device__ void init(uint64_t seed, uint64_t stream) {
    key[0] = (uint32_t)seed;
    key[1] = (uint32_t)(seed >> 32);
    ctr[0] = 0u;
    ctr[1] = 0u;
    ctr[2] = (uint32_t)stream;
    ctr[3] = (uint32_t)(stream >> 32);
    used   = 4;
  }
  __device__ void block() {
    uint32_t k0 = key[0], k1 = key[1];
    uint32_t x0 = ctr[0], x1 = ctr[1], x2 = ctr[2], x3 = ctr[3];
#pragma unroll
    for (int r = 0; r < 10; ++r) {
      const uint32_t hi0 = __umulhi(0xD2511F53u, x0), lo0 = 0xD2511F53u * x0;
      const uint32_t hi1 = __umulhi(0xCD9E8D57u, x2), lo1 = 0xCD9E8D57u * x2;
      x0 = hi1 ^ x1 ^ k0;
      x1 = lo1;
      x2 = hi0 ^ x3 ^ k1;
      x3 = lo0;
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    buf[0] = x0, buf[1] = x1, buf[2] = x2, buf[3] = x3;
    if (++ctr[0] == 0u) ++ctr[1];
    used = 0;
  }
  __device__ uint32_t next() {
    if (used == 4) block();
    return buf[used++];
  }
};

// uniform in [0, 1): 24 bits (float) or 53 bits from two draws (double)
__device__ __forceinline__ float uniform(Philox4x32& g, float) {
  return (float)(g.next() >> 8) * 5.9604644775390625e-8f;
}
__device__ __forceinline__ double uniform(Philox4x32& g, double) {
  const uint32_t a = g.next() >> 5, b = g.next() >> 6;
  return ((double)a * 67108864.0 + (double)b) * 1.1102230246251565e-16;
}

__device__ __forceinline__ float  mlog(float x) { return logf(x); }
__device__ __forceinline__ double mlog(double x) { return log(x); }
__device__ __forceinline__ float  msin(float x) { return sinf(x); }
__device__ __forceinline__ double msin(double x) { return sin(x); }

template <typename real>
__device__ __forceinline__ bool almost_zero(real x) {
  return fabs(x) <= (sizeof(real) == 4 ? (real)1.1920929e-07 : (real)2.220446049250313e-16);
}

// one species' sampler: Maxwellian's constructor (energy_dist.h:184-222)
// evaluated on the host in real_t
template <typename real>
struct MaxwellParams {
  real temp;    // temperature / mass
  real d3, d4;  // drift 3- and 4-velocity
  real dir[3];  // unit drift direction (ddir = 4)
  int  ddir;    // 0 none, +-1..+-3 along x1..x3, 4 arbitrary
};

// bounds on the samplers' rejection loops: each pass accepts with
// probability close to one, so hitting a bound means a broken input
constexpr int kMaxZeroRedraws = 64;
constexpr int kMaxSobolPasses = 4096;

// three uniforms drawn in turn and multiplied left to right (the
// reference's Random() * Random() * Random() leaves the order to the compiler)
template <typename real>
__device__ __forceinline__ real product3(Philox4x32& g) {
  const real a = uniform(g, (real)0);
  const real b = uniform(g, (real)0);
  const real c = uniform(g, (real)0);
  return a * b * c;
}

// JuttnerSinge (energy_dist.h:79-134): Box-Muller below temp 0.5, the Sobol
// rejection method above; false if a loop bound was hit
template <typename real>
__device__ bool juttner_synge(real* v, real temp, Philox4x32& g) {
  const real ONE = 1, TWO = 2, TWO_PI = (real)6.28318530717958647692;
  const real z   = 0;
  bool       ok  = true;
  if (temp < (real)0.5) {
#pragma unroll 1
    for (int c = 0; c < 3; ++c) {
      real x1 = uniform(g, z);
      int  k  = 0;
      while (almost_zero(x1) && k++ < kMaxZeroRedraws) x1 = uniform(g, z);
      ok       = ok && k <= kMaxZeroRedraws;
      x1       = sqrt(-TWO * mlog(x1));
      const real x2 = TWO_PI * uniform(g, z);
      v[c]     = x1 * mcos(x2) * sqrt(temp);
    }
  } else {
    real u = ONE, eta = uniform(g, z), x1 = 0, x2 = 0;
    int  pass = 0;
    while (eta * eta <= u * u + ONE && pass++ < kMaxSobolPasses) {
      x1    = product3<real>(g);
      int k = 0;
      while (almost_zero(x1) && k++ < kMaxZeroRedraws) x1 = product3<real>(g);
      ok = ok && k <= kMaxZeroRedraws;
      u  = -temp * mlog(x1);
      x2 = uniform(g, z);
      k  = 0;
      while (almost_zero(x2) && k++ < kMaxZeroRedraws) x2 = uniform(g, z);
      ok  = ok && k <= kMaxZeroRedraws;
      eta = -temp * mlog(x1 * x2);
    }
    ok = ok && pass <= kMaxSobolPasses;
    x1   = uniform(g, z);
    x2   = uniform(g, z);
    v[0] = u * (TWO * x1 - ONE);
    v[2] = TWO * u * sqrt(x1 * (ONE - x1));
    v[1] = v[2] * mcos(TWO_PI * x2);
    v[2] = v[2] * msin(TWO_PI * x2);
  }
  return ok;
}

// Maxwellian::operator() (energy_dist.h:224-273): the isotropic sample,
// then the flipping boost along x1 (arXiv:1504.03910) and the rotation to
// the drift direction
template <typename real>
__device__ bool maxwellian(const MaxwellParams<real>& m, Philox4x32& g, real* v) {
  const real ONE = 1;
  bool       ok  = true;
  if (almost_zero(m.temp)) {
    v[0] = v[1] = v[2] = 0;
  } else {
    ok = juttner_synge(v, m.temp, g);
  }
  if (m.ddir != 0) {
    const real gamma = sqrt(ONE + (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
    if (-m.d3 * v[0] > gamma * uniform(g, (real)0)) v[0] = -v[0];
    v[0] = sqrt(ONE + m.d4 * m.d4) * (v[0] + m.d3 * gamma);
    if (m.ddir == -1) {
      v[0] = -v[0];
    } else if (m.ddir == 2 || m.ddir == -2) {
      const real t = v[1];
      v[1]         = m.ddir > 0 ? v[0] : -v[0];
      v[0]         = t;
    } else if (m.ddir == 3 || m.ddir == -3) {
      const real t = v[2];
      v[2]         = m.ddir > 0 ? v[0] : -v[0];
      v[0]         = t;
    } else if (m.ddir == 4) {
      const real o0 = v[0], o1 = v[1], o2 = v[2];
      const real a = m.dir[0], b = m.dir[1], c = m.dir[2];
      v[0] = o0 * a - o1 * b - o2 * c;
      v[1] = (o0 * b * (a + ONE) + o1 * (a * a + a + c * c) - o2 * b * c) / (a + ONE);
      v[2] = (o0 * c * (a + ONE) - o1 * b * c - o2 * (-a + c * c - ONE)) / (a + ONE);
    }
  }
  return ok;
}

template <typename real>
struct InjArgs {
  SpeciesPtrs         sp[2];
  int64_t             off[2];
  int64_t             npairs;
  real                xmin[3], xmax[3];
  MaxwellParams<real> md[2];
  uint64_t            seed, first_pair;
  QKS<double>         m;  // GR only
  real                inv_V0;
  unsigned long long* err;
};

template <int D, bool GR, typename real>
__global__ void __launch_bounds__(256) k_inject_uniform(InjArgs<real> a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.npairs; p += stride) {
    Philox4x32 g;
    g.init(a.seed, a.first_pair + (uint64_t)p);
    real  x[3]  = { 0, 0, 0 };
    int   xi[3] = { 0, 0, 0 };
    float dx[3] = { 0.f, 0.f, 0.f };
#pragma unroll
    for (int d = 0; d < D; ++d) {
      x[d]  = a.xmin[d] + uniform(g, (real)0) * (a.xmax[d] - a.xmin[d]);
      xi[d] = (int)x[d];
      dx[d] = (float)(x[d] - (real)xi[d]);
    }
    real v[2][3];
    bool ok = maxwellian(a.md[0], g, v[0]);
    ok      = maxwellian(a.md[1], g, v[1]) && ok;
    real weight = 1;
    if constexpr (GR) {
      // tetrad -> covariant (transform<Idx::T, Idx::D>), weight sqrt(det h) / V0
      const QKS<real> m  = a.m.template as<real>();
      const QPt<real> pt = qpt(m, x[0], x[1]);
      const QMet<real> gm = qmet(m, pt);
      for (int s = 0; s < 2; ++s) {
        real o[3];
        t_to_d(gm, v[s], o);
        v[s][0] = o[0], v[s][1] = o[1], v[s][2] = o[2];
      }
      weight = sqrt_det_h(m, pt) * a.inv_V0;
    }
    if (!ok) atomicAdd(a.err + ERR_SAMPLER, 1ull);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const SpeciesPtrs& S = a.sp[s];
      const int64_t      q = a.off[s] + p;
      S.i1[q]  = xi[0];
      S.dx1[q] = dx[0];
      if (D >= 2) {
        S.i2[q]  = xi[1];
        S.dx2[q] = dx[1];
      }
      if (D == 3) {
        S.i3[q]  = xi[2];
        S.dx3[q] = dx[2];
      }
      ((real*)S.ux1)[q] = v[s][0];
      ((real*)S.ux2)[q] = v[s][1];
      ((real*)S.ux3)[q] = v[s][2];
      ((real*)S.w)[q]   = weight;
      S.tag[q]          = PIC_TAG_ALIVE;
    }
  }
}

}  // namespace pic

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
namespace {

template <typename real>
bool almost_zero_host(real x) {
  return std::fabs(x) <= (sizeof(real) == 4 ? (real)1.1920929e-07 : (real)2.220446049250313e-16);
}

// Maxwellian's constructor (energy_dist.h:184-222), in real_t
template <typename real>
int maxwell_params(double temperature, float mass, const double* drift,
                   pic::MaxwellParams<real>& m) {
  if (!(temperature >= 0.0) || !(mass > 0.0f)) return PIC_ERR_ARG;
  m.temp = (real)temperature / (real)mass;
  const real u[3] = { (real)drift[0], (real)drift[1], (real)drift[2] };
  const real d4   = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  m.d4 = d4, m.d3 = 0, m.dir[0] = m.dir[1] = m.dir[2] = 0;
  m.ddir = 0;
  if (almost_zero_host(d4)) return PIC_OK;
  m.d3     = d4 / std::sqrt((real)1 + d4 * d4);
  m.dir[0] = u[0] / d4, m.dir[1] = u[1] / d4, m.dir[2] = u[2] / d4;
  m.ddir   = 4;
  for (int d = 0; d < 3; ++d) {
    if (almost_zero_host(u[(d + 2) % 3]) && almost_zero_host(u[(d + 1) % 3])) {
      m.ddir = (u[d] < (real)0 ? -1 : 1) * (d + 1);
      break;
    }
  }
  return PIC_OK;
}

template <typename real>
int inject(pic_ctx* c, const pic_gr_metric* gm, pic_species* sp1, pic_species* sp2,
           const pic_inject_params* ip, double V0, int64_t* n_pairs, cudaStream_t s) {
  const int D = c->grid.dim;
  pic::InjArgs<real> a;
  // ComputeNumInject (particle_injector.h:128-136)
  long double cells = 1.0L;
  for (int d = 0; d < D; ++d) {
    a.xmin[d] = (real)ip->xi_min[d];
    a.xmax[d] = (real)ip->xi_max[d];
    if (!(ip->xi_max[d] > ip->xi_min[d]) || ip->xi_min[d] < 0.0 || ip->xi_max[d] > c->grid.n[d])
      return PIC_ERR_ARG;
    cells *= (long double)a.xmax[d] - (long double)a.xmin[d];
  }
  const real    dens = (real)ip->ppc0 * (real)ip->number_density * (real)0.5;
  const int64_t n    = (int64_t)((long double)dens * cells);
  if (n < 0) return PIC_ERR_ARG;
  pic_species* sps[2] = { sp1, sp2 };
  for (int k = 0; k < 2; ++k) {
    if (sps[k]->npart + n > sps[k]->maxnpart) return PIC_ERR_ARG;
    int st = maxwell_params<real>(ip->temperature[k], sps[k]->mass, ip->drift[k], a.md[k]);
    if (st != PIC_OK) return st;
    // the reference boosts in Cartesian coordinates only (energy_dist.h:214-218)
    if (gm && a.md[k].ddir != 0) return PIC_ERR_UNSUPPORTED;
    a.sp[k]  = sptrs(sps[k]);
    a.off[k] = sps[k]->npart;
  }
  a.npairs     = n;
  a.seed       = ip->seed;
  a.first_pair = ip->first_pair;
  a.inv_V0     = gm ? (real)1 / (real)V0 : (real)1;
  a.err        = c->d_err;
  if (gm) a.m = make_qks<real>(c, gm);
  *n_pairs = n;
  if (n == 0) return PIC_OK;
  int64_t b = (n + 255) / 256;
  if (b > pic::sm_count() * 32) b = pic::sm_count() * 32;
  if (gm) {
    PIC_KL(pic::k_inject_uniform<2, true, real><<<(unsigned)b, 256, 0, s>>>(a));
  } else if (D == 2) {
    PIC_KL(pic::k_inject_uniform<2, false, real><<<(unsigned)b, 256, 0, s>>>(a));
  } else {
    PIC_KL(pic::k_inject_uniform<3, false, real><<<(unsigned)b, 256, 0, s>>>(a));
  }
  if (cudaGetLastError() != cudaSuccess) return PIC_ERR_CUDA;
  sp1->npart += n;
  sp2->npart += n;
  return PIC_OK;
}

int inject_entry(pic_ctx* c, const pic_gr_metric* gm, pic_species* sp1, pic_species* sp2,
                 const pic_inject_params* ip, double V0, int64_t* n_pairs, void* stream) {
  if (!c || !sp1 || !sp2 || !ip || !n_pairs || sp1 == sp2) return PIC_ERR_ARG;
  *n_pairs = 0;
  for (pic_species* sp : { sp1, sp2 }) {
    const int st = validate_species(c, sp, false);
    if (st != PIC_OK) return st;
    // the arrays are written even when the species is empty so far
    if (!sp->i1 || !sp->i2 || !sp->dx1 || !sp->dx2 || !sp->ux1 || !sp->ux2 || !sp->ux3 ||
        !sp->weight || !sp->tag || (c->grid.dim == 3 && (!sp->i3 || !sp->dx3)))
      return PIC_ERR_ARG;
  }
  if (gm && !(V0 > 0.0)) return PIC_ERR_ARG;
  const cudaStream_t s = strm(stream);
  return is_f64(c) ? inject<double>(c, gm, sp1, sp2, ip, V0, n_pairs, s)
                   : inject<float>(c, gm, sp1, sp2, ip, V0, n_pairs, s);
}

}  // namespace

extern "C" {

int pic_inject_uniform_maxwellians(pic_ctx* c, pic_species* sp1, pic_species* sp2,
                                   const pic_inject_params* ip, int64_t* n_pairs, void* stream) {
  return inject_entry(c, nullptr, sp1, sp2, ip, 0.0, n_pairs, stream);
}

int pic_gr_inject_uniform_maxwellians(pic_ctx* c, const pic_gr_metric* m, pic_species* sp1,
                                      pic_species* sp2, const pic_inject_params* ip, double V0,
                                      int64_t* n_pairs, void* stream) {
  const int st = gr_check(c, m);
  if (st != PIC_OK) return st;
  return inject_entry(c, m, sp1, sp2, ip, V0, n_pairs, stream);
}

}  // extern "C"
