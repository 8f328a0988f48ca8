/*
 * CPU oracle: output preparation on a Cartesian SR grid (TEST INFRASTRUCTURE
 * ONLY; never linked into the product library).
 *
 * Restates, particle by particle and cell by cell in a fixed order:
 *  - ParticleMoments_kernel<SRPIC, Minkowski, F> (src/kernels/particle_moments.hpp:44-405);
 *  - SynchronizeFields(Comm::Bckp) for one domain (src/framework/domain/
 *    metadomain_comm.cpp:408-562): the direction-by-direction additive fold;
 *  - NormalizeVectorByRho_kernel (particle_moments.hpp:407-478);
 *  - ComputeDivergence_kernel<Minkowski> (src/kernels/divergences.hpp:23-135);
 *  - FieldsToPhys_kernel<Minkowski> (src/kernels/fields_to_phys.hpp:33-241)
 *    with the writer's downsampling (src/output/writer.cpp:199-300);
 *  - PrtlToPhys_kernel<SRPIC, Minkowski, false> (src/kernels/prtls_to_phys.hpp:28-218).
 */
#ifndef ENTITY_OUTPUT_ORACLE_H
#define ENTITY_OUTPUT_ORACLE_H

#include "srpic_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

/* moment ids: 0 Rho, 1 Charge, 2 N, 3 Nppc, 4 T, 5 V; smoothing 1 const, 2 spline */
void orc_output_moment(const orc_grid* g, const orc_species* sp, int id, int c1, int c2,
                       int order, int smoothing, int use_weights, double inv_n0, double dx,
                       void* bckp, int comp);

/* prtl_shape::S0..S6 at x >= 0 */
double orc_spline(int order, double x);

void orc_sync_moments(const orc_grid* g, void* bckp, int c0, int c1);

void orc_normalize_by_rho(const orc_grid* g, void* bckp, int c_rho, int c_v1, int c_v2, int c_v3);

void orc_output_divergence(const orc_grid* g, const void* EB, void* bckp, int comp);

/* flags: 1 edges, 2 faces, 4 to hat; out[c][o3][o2][o1] */
void orc_output_field(const orc_grid* g, const void* src, int is_em, int c0, int ncomp,
                      unsigned flags, double dx, const int dwn[3], void* out);

/* returns npart / stride */
int64_t orc_output_particles(const orc_grid* g, const orc_species* sp, int64_t stride, double dx,
                             const double xmin[3], void* x1, void* x2, void* x3, void* u1,
                             void* u2, void* u3, void* w);

#ifdef __cplusplus
}
#endif

#endif
