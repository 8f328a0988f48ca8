/*
 * CPU oracle for the SR particle-in-cell hot path (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain-C restatement of the reference's kernels, used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker. It
 * is never linked into, or called by, the product library.
 *
 * Compiled twice: with -DORC_SINGLE (real = float, the reference's
 * SINGLE_PRECISION build) and without (real = double). Every function cites the
 * reference file:line it restates (paths relative to the entity repository).
 *
 * Arithmetic contract (shared with the CUDA kernels so results are bit-exact):
 *  - every operation is rounded separately in the reference's source order
 *    (the oracle is built with -ffp-contract=off, the CUDA code with
 *    -fmad=false), including the running sums of the field interpolation
 *    (`c += S * EB`, src/kernels/pushers/sr.hpp:1118-1369). This is the
 *    arithmetic of the reference's own kernels compiled without contraction,
 *    which tests/test_ref_pin.py checks against oracle/_ref;
 *  - current deposition differs from the GPU only in summation order.
 */
#ifndef ENTITY_SRPIC_ORACLE_H
#define ENTITY_SRPIC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* grid: active cells n1 x n2 x n3 (n3 = 1 in 2D), ng ghost layers on every
 * side of every simulated dimension. Field element (i1, i2, i3, c) with
 * ghost-inclusive indices lives at i1*s[0] + i2*s[1] + i3*s[2] + c*s[3]. */
typedef struct {
  int     dim;
  int     n1, n2, n3;
  int     ng;
  int64_t em_s[4];  /* strides of the 6-component EB field */
  int64_t cur_s[4]; /* strides of the 3-component J / buff fields */
  int     periodic[3];
  /* particle boundary per side: 0 periodic, 1 absorb, 2 reflect, 3 axis */
  int     prtl_bc[3][2];
  /* field boundary per side: 0 periodic, 1 none, 2 conductor, 3 match */
  int     fbc[3][2];
} orc_grid;

/* one species, structure of arrays (src/framework/containers/particles.h:47-71) */
typedef struct {
  int32_t *i1, *i2, *i3;
  int32_t *i1_prev, *i2_prev, *i3_prev;
  float   *dx1, *dx2, *dx3;
  float   *dx1_prev, *dx2_prev, *dx3_prev;
  void    *ux1, *ux2, *ux3; /* real */
  void    *weight;          /* real */
  int16_t *tag;
  int64_t  npart;
  float    mass, charge;
  int      pusher; /* 0 none, 1 Boris, 2 Vay, 3 photon */
} orc_species;

/* ParticleTag (src/global/global.h:168-171) */
enum { ORC_TAG_DEAD = 0, ORC_TAG_ALIVE = 1 };
enum { ORC_PUSHER_NONE = 0, ORC_PUSHER_BORIS = 1, ORC_PUSHER_VAY = 2, ORC_PUSHER_PHOTON = 3 };

/* number of OpenMP threads the oracle uses (1 when built without OpenMP) */
int orc_max_threads(void);
int orc_real_size(void);

/* kernel::sr::Pusher_kernel (src/kernels/pushers/sr.hpp:117-332), Minkowski,
 * shape order `order` for the field interpolation. Returns the number of
 * particles whose tag was neither alive nor dead (the reference's KernelError). */
int64_t orc_push(const orc_grid* g, orc_species* sp, const void* EB, int order,
                 double dt, double omegaB0, double dx);

/* kernel::DepositCurrents_kernel (src/kernels/currents_deposit.hpp:108-761)
 * accumulating into J (does not zero it). */
void orc_deposit(const orc_grid* g, const orc_species* sp, void* J, int order,
                 double dt, double dx);

/* srpic::FieldBoundaries (src/engines/srpic/fields_bcs.h:622-672) for the
 * conductor and match sides of g->fbc, in Directions<D>::orth order:
 * ConductorBoundaries_kernel (src/kernels/fields_bcs.hpp:522-800) and the
 * SRPIC branch of MatchBoundaries_kernel (fields_bcs.hpp:42-520) relaxing
 * toward `target` with s = tanh(4 |x - x_edge| / ds), x = x_min + x_Cd dx. */
void orc_field_boundaries(const orc_grid* g, void* EB, int set_e, int set_b, const void* target,
                          const double x_min[3], double dx, const double ds[3][2]);

/* kernel::mink::Faraday_kernel (src/kernels/faraday_mink.hpp:71-166) over the
 * active cells. stencil = {deltax, deltay, betaxy, betayx, deltaz, betaxz,
 * betazx, betayz, betazy} (NULL = Yee). */
void orc_faraday(const orc_grid* g, void* EB, double coeff1, double coeff2,
                 const double* stencil);

/* kernel::mink::Ampere_kernel (src/kernels/ampere_mink.hpp:48-88) */
void orc_ampere(const orc_grid* g, void* EB, double coeff1, double coeff2);

/* kernel::mink::CurrentsAmpere_kernel (src/kernels/ampere_mink.hpp:134-214) */
void orc_currents_ampere(const orc_grid* g, void* EB, void* J, double coeff,
                         double ppc0);

/* one pass of kernel::DigitalFilter_kernel, Cartesian, no conductors
 * (src/kernels/digital_filter.hpp:129-195, 289-379): array <- filter(buffer).
 * The reference's buff <- J copy (src/engines/srpic/currents.h:108-118) is
 * done here too. */
void orc_filter_pass(const orc_grid* g, void* J, void* buff);

/* Metadomain::CommunicateFields for one field with periodic self-exchange
 * (src/framework/domain/metadomain_comm.cpp:204-367,
 * src/framework/domain/comm_nompi.hpp:44-63): ghost <- active images for
 * components [c0, c1). `is_em` selects EB (6 comps) vs J (3 comps) strides. */
void orc_fill_ghosts(const orc_grid* g, void* fld, int is_em, int c0, int c1);

/* Metadomain::SynchronizeFields(J) (src/framework/domain/metadomain_comm.cpp:
 * 408-562): buff <- 0; buff(recv) += J(send) over all directions; J(active) +=
 * buff(active). */
void orc_sync_currents(const orc_grid* g, void* J, void* buff);

/* Particles::SortSpatially (src/framework/containers/particles_sort.cpp:196-253)
 * with a stable counting sort on the PositionToTileIndex key
 * (src/global/utils/sorting.h:119-135). Fills perm[new] = old and permutes
 * every array of the species in place. */
void orc_sort(const orc_grid* g, orc_species* sp, int64_t* perm);

/* The same stable counting sort on the GPU path's tile-major key (tile
 * index i1-fastest over tiles of shape tile[0..2], then the cell inside the
 * tile i1-fastest); checks PIC_SORT_TILED, which has no reference
 * counterpart. */
void orc_sort_tiled(const orc_grid* g, orc_species* sp, const int* tile, int64_t* perm);

/* Particles::RemoveDead (src/framework/containers/particles_sort.cpp:103-194):
 * stable compaction of alive particles, tags reset, returns new npart. */
int64_t orc_remove_dead(const orc_grid* g, orc_species* sp);

/* FP64 diagnostics (definitions of src/kernels/reduced_stats.hpp:145-187 for
 * Minkowski): out[0] = sum E^2 dV-weighted, out[1] = sum B^2. */
void orc_field_energy(const orc_grid* g, const void* EB, double dx, double* out);

/* the deposit with a caller-supplied out-of-plane velocity vz[p] (real) in
 * place of the SR one (the GR deposit, currents_deposit.hpp:138-165) */
void orc_deposit_vz(const orc_grid* g, const orc_species* sp, void* J, int order, double dt,
                    const void* vz);

/* shape-order interpolation (sr.hpp:1151-1369) at a 2D particle position of
 * the E part of emD and the B part of emB (gr.hpp:594-662 reads D from em and
 * B from em0) */
void orc_interp2(const orc_grid* g, const void* emD, const void* emB, int order, int i1, int i2,
                 float dx1, float dx2, double* e, double* b);

/* sum over particles of w * (gamma - 1) * mass (in FP64) */
double orc_kinetic_energy(const orc_species* sp);

/* node charge density conserved by the deposit, added into component 0 of a
 * current-layout array: rho(n) += charge * w * prod_d S(n_d - x_d) with the
 * unstaggered shape of the given order (order 0: the linear shape); the
 * discrete form of the continuity equation that Esirkepov's weights
 * (currents_deposit.hpp:406-754) and the zigzag fluxes satisfy */
void orc_charge_density(const orc_grid* g, const orc_species* sp, void* rho, int order);

/* FP64 particle moments over alive particles (reduced_stats.hpp:403-538,
 * SR Cartesian T components, unweighted): out[0] += sum m gamma,
 * out[1..3] += sum u_i, out[4] += sum w m (gamma - 1), out[5] += sum w */
void orc_particle_moments(const orc_species* sp, double* out);

#ifdef __cplusplus
}
#endif

#endif
