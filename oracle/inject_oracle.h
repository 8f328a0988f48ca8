/*
 * CPU oracle for the uniform Maxwellian pair injection (TEST INFRASTRUCTURE
 * ONLY: used by tests/ as the checker, never linked into the product).
 *
 * Restates arch::InjectUniformMaxwellians (src/archetypes/utils.h:46-107),
 * ComputeNumInject (src/archetypes/particle_injector.h:112-139),
 * kernel::UniformInjector_kernel (src/kernels/injectors.hpp:83-289) and the
 * Maxwellian sampler (src/archetypes/energy_dist.h:79-273), with the random
 * numbers of the product: one Philox4x32-10 stream per pair (Salmon et al.,
 * SC11), key = seed, counter = (block low, block high, pair low, pair high).
 * Uniforms: float = (x >> 8) * 2^-24; double = ((a >> 5) * 2^26 + (b >> 6))
 * * 2^-53 from two draws. Draw order per pair: the D position uniforms, then
 * species 1's velocity, then species 2's; three-factor products are drawn
 * left to right.
 */
#ifndef ENTITY_INJECT_ORACLE_H
#define ENTITY_INJECT_ORACLE_H

#include <stdint.h>

#include "srpic_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double   number_density;
  double   ppc0;
  double   xi_min[3], xi_max[3];
  double   temperature[2];
  double   drift[2][3];
  uint64_t seed, first_pair;
} orc_inject_params;

/* one Philox4x32-10 block */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ComputeNumInject: (long)(ppc0 * number_density * 0.5 * box cells) */
int64_t orc_inject_count(int dim, const orc_inject_params* ip);

/* pair p's position x[0..dim) (real_t, code units) and the two species'
 * velocities in the sampler's frame (Cartesian: with the boost); returns 0
 * when a sampler loop ran out of its bound */
int orc_inject_sample_pair(int dim, const orc_inject_params* ip, const float mass[2],
                           uint64_t p, void* x, void* v);

/* the Cartesian injection: n pairs appended at each species' npart (which is
 * advanced); returns n; *failures counts sampler bound hits */
int64_t orc_inject_uniform(const orc_grid* g, orc_species* sp1, orc_species* sp2,
                           const orc_inject_params* ip, int64_t* failures);

#ifdef __cplusplus
}
#endif

#endif /* ENTITY_INJECT_ORACLE_H */
