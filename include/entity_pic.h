/*
 * entity_pic.h — C ABI of the GB300 particle-in-cell hot path.
 *
 * One entry point per phase of the reference's SR step
 * (SRPICEngine::step_forward, src/engines/srpic/srpic.hpp:65-188), taking
 * plain device pointers, element strides and scalars. The caller owns every
 * array (the reference's Kokkos Views pass `.data()`); the library never
 * frees caller memory and allocates only inside pic_create and lazily in
 * pic_sort (scratch that lives in the context).
 *
 * Errors: every entry point returns int (PIC_OK = 0, negative on failure) and
 * never throws or traps. Device-side faults that the reference reports with
 * Kokkos::abort (invalid particle tag, particle outside the grid after the
 * boundary step) are counted in a device error word, read with
 * pic_get_device_errors after the stream is synchronised.
 *
 * Threading: one host thread drives a context; calls are asynchronous on the
 * given stream (NULL = legacy default stream).
 *
 * Paths in citations are relative to the entity repository.
 */
#ifndef ENTITY_PIC_H
#define ENTITY_PIC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PIC_ABI_VERSION 1

/* status codes */
#define PIC_OK 0
#define PIC_ERR_ARG -1         /* invalid argument (null pointer, bad size) */
#define PIC_ERR_CUDA -2        /* a CUDA runtime call failed */
#define PIC_ERR_UNSUPPORTED -3 /* configuration outside what is built */
#define PIC_ERR_NOMEM -4       /* device allocation failed */
#define PIC_ERR_DEVICE -5      /* a device-side check failed (see error word) */

/* particle tags: ParticleTag, src/global/global.h:168-171 */
#define PIC_TAG_DEAD 0
#define PIC_TAG_ALIVE 1

/* pusher kinds: ParticlePusher flags, src/global/enums.h */
#define PIC_PUSHER_NONE 0
#define PIC_PUSHER_BORIS 1
#define PIC_PUSHER_VAY 2
#define PIC_PUSHER_PHOTON 3

/* particle boundary kinds: PusherBoundaries, src/kernels/pushers/context.h:124-178 */
#define PIC_BC_PERIODIC 0
#define PIC_BC_ABSORB 1
#define PIC_BC_REFLECT 2
#define PIC_BC_AXIS 3

/* push/deposit flags */
#define PIC_PD_WRITE_PREV 1u    /* store i*_prev / dx*_prev like the reference pusher */
#define PIC_PD_NO_ZERO 2u       /* do not zero J before depositing */
#define PIC_PD_FLOAT_ATOMICS 4u /* FP32: add contributions to J with float atomics in
                                   arrival order instead of the exact accumulation */

/* sort flags */
#define PIC_SORT_REMOVE_DEAD 1u /* Particles::RemoveDead before the spatial sort */
#define PIC_SORT_SKIP_PREV 2u   /* leave i*_prev / dx*_prev arrays unpermuted */
#define PIC_SORT_SPATIAL 4u     /* Particles::SortSpatially */
/* With PIC_SORT_SPATIAL: order by tile of cells first, then by cell inside
 * the tile (cells inside a tile i1-fastest, each row's even cells before its
 * odd ones), instead of the reference's
 * i1-major cell key. The context then remembers each species' tile offsets
 * and pic_push_deposit runs the tiled kernel for it until the species' npart
 * changes or it is sorted again with another key. No reference counterpart:
 * the reference's key only sets a traversal order, and this one lets a tile's
 * particles be read as one contiguous range. */
#define PIC_SORT_TILED 8u
/* Without PIC_SORT_REMOVE_DEAD: return without waiting for the sort (npart
 * cannot change). Out-of-grid particles are then only counted in the error
 * word (out[1]) instead of also failing the call with PIC_ERR_DEVICE. With
 * PIC_SORT_REMOVE_DEAD it is PIC_ERR_ARG: the new count needs the wait. No
 * reference counterpart. */
#define PIC_SORT_NO_SYNC 16u

/* Grid and build choices of a domain (Grid/Mesh, src/framework/domain/grid.h;
 * N_GHOSTS and SHAPE_ORDER, src/global/global.h:130-136). Field element
 * (i1, i2, i3, comp) with ghost-inclusive indices is at
 * i1*s[0] + i2*s[1] + i3*s[2] + comp*s[3] (elements of real_bytes each);
 * Kokkos LayoutLeft and LayoutRight are both expressible. */
typedef struct {
  int32_t dim;           /* 2 or 3 */
  int32_t n[3];          /* active cells per dimension (n[2] = 1 in 2D) */
  int32_t ng;            /* ghost layers */
  int32_t order;         /* shape order 0 (zigzag) .. 3 */
  int32_t real_bytes;    /* sizeof(real_t): 4 or 8 */
  int32_t fld_periodic[3];
  int32_t prtl_bc[3][2]; /* PIC_BC_* for (min, max) of each dimension */
  int64_t em_stride[4];  /* strides of the 6-component EB (E at 0..2, B at 3..5) */
  int64_t cur_stride[4]; /* strides of the 3-component J and buff */
} pic_grid;

/* One species as structure of arrays, field for field the reference's
 * ParticleArrays (src/framework/containers/particles.h:47-71). ux*, weight are
 * real_t; i*_prev / dx*_prev may be NULL when PIC_PD_WRITE_PREV is not set
 * and the sort is asked to skip them. i3-arrays are unused in 2D.
 * The trailing fields are optional (zero them when unused): phi (real_t, the
 * reference keeps it for 2D non-Cartesian grids) and the payloads pld_r
 * (real_t) and pld_i (npart_t: 32-bit unsigned, global.h:385), npld_r /
 * npld_i columns each, element
 * (p, k) at pld[p * pld_stride[0] + k * pld_stride[1]] (elements; a Kokkos
 * LayoutLeft View on the device has strides {1, maxnpart}). Only the sort and
 * dead removal touch them: particles carry their phi and payloads along. */
typedef struct {
  int32_t *i1, *i2, *i3;
  int32_t *i1_prev, *i2_prev, *i3_prev;
  float   *dx1, *dx2, *dx3;
  float   *dx1_prev, *dx2_prev, *dx3_prev;
  void    *ux1, *ux2, *ux3;
  void    *weight;
  int16_t *tag;
  int64_t  npart;
  int64_t  maxnpart;
  float    mass;
  float    charge;
  int32_t  pusher; /* PIC_PUSHER_* */
  int32_t  index;  /* species index (1-based as in the reference) */
  void*    phi;
  void*    pld_r;
  void*    pld_i;
  int64_t  pld_r_stride[2];
  int64_t  pld_i_stride[2];
  int32_t  npld_r;
  int32_t  npld_i;
} pic_species;

typedef struct pic_ctx pic_ctx;

/* Library version and the build's compute capability (e.g. 103). */
int pic_version(int32_t* abi_version, int32_t* built_sm);

/* Human-readable status. */
const char* pic_status_string(int status);

/* Number of CUDA kernels this library has launched in the process so far
 * (host-side counter; no device synchronisation). No reference counterpart:
 * it lets a caller attribute launches to this library. */
int64_t pic_kernel_launches(void);

/* Creates a context for one domain: validates the grid, allocates the device
 * error word. Replaces nothing in the reference (its Domain owns the Views). */
int pic_create(const pic_grid* grid, pic_ctx** out);
int pic_destroy(pic_ctx* ctx);

/* Copy of the grid the context was created with. */
int pic_get_grid(const pic_ctx* ctx, pic_grid* out);

/* Cells per tile along each axis used by PIC_SORT_TILED and the tiled
 * push/deposit of this context (no reference counterpart). */
int pic_tile_shape(const pic_ctx* ctx, int32_t out[3]);

/* srpic::Faraday (src/engines/srpic/fieldsolvers.h:36-99) with
 * Faraday_kernel (src/kernels/faraday_mink.hpp:71-166), fused with
 * Metadomain::CommunicateFields(Comm::B) (metadomain_comm.cpp:204-367) for
 * periodic dimensions. coeff1/coeff2 as the reference computes them in
 * real_t; stencil = {deltax, deltay, betaxy, betayx, deltaz, betaxz, betazx,
 * betayz, betazy} or NULL for Yee. */
int pic_faraday(pic_ctx* ctx, void* EB, double coeff1, double coeff2,
                const double* stencil, void* stream);

/* srpic::Ampere (fieldsolvers.h:101-140), Ampere_kernel
 * (src/kernels/ampere_mink.hpp:48-88); no ghost exchange (the reference
 * exchanges E after CurrentsAmpere). */
int pic_ampere(pic_ctx* ctx, void* EB, double coeff1, double coeff2, void* stream);

/* srpic::CurrentsAmpere (fieldsolvers.h:142-200), CurrentsAmpere_kernel
 * (ampere_mink.hpp:96-214): E += coeff*J, J /= ppc0, then
 * CommunicateFields(Comm::E | Comm::J). */
int pic_currents_ampere(pic_ctx* ctx, void* EB, void* J, double coeff, double ppc0,
                        void* stream);

/* Ampere + CurrentsAmpere + CommunicateFields(E|J) in one pass over the grid
 * (srpic.hpp:155-166); with J == NULL only Ampere + CommunicateFields(E). */
int pic_ampere_currents(pic_ctx* ctx, void* EB, void* J, double coeff1, double coeff2,
                        double jcoeff, double ppc0, void* stream);

/* srpic::ParticlePush (src/engines/srpic/particle_pusher.h:35-185) for one
 * species: Pusher_kernel (src/kernels/pushers/sr.hpp:117-332), Minkowski,
 * Boris / Vay / photon, with the particle boundaries of the grid. Always
 * writes i*_prev / dx*_prev. */
int pic_push(pic_ctx* ctx, const pic_species* sp, const void* EB, double dt,
             double omegaB0, double dx, void* stream);

/* srpic::CurrentsDeposit (src/engines/srpic/currents.h:64-87): zeroes J and
 * deposits every species with DepositCurrents_kernel
 * (src/kernels/currents_deposit.hpp:108-761) from the prev arrays. */
int pic_deposit(pic_ctx* ctx, const pic_species* sp, int32_t nspecies, void* J, double dt,
                double dx, void* stream);

/* Fused ParticlePush + CurrentsDeposit for nspecies species: one pass reads
 * each particle once, moves it and deposits its current; the previous
 * position stays in registers (written out only with PIC_PD_WRITE_PREV).
 * J is zeroed first unless PIC_PD_NO_ZERO.
 * FP32 grids accumulate the call's contributions exactly: each is a multiple
 * of 2^(e - b) (2^e bounds |q w| max(1/dt, 1) over the call's particles,
 * b = min(34, 62 - ceil(log2(N + 1))) for N particles), summed as 64-bit
 * integers in a context-owned buffer and converted to float once per entry,
 * so J does not depend on the order of the additions and repeats bit for bit
 * from run to run. The reference's device build adds floats atomically in
 * arrival order (ScatterView); PIC_PD_FLOAT_ATOMICS does the same here. */
int pic_push_deposit(pic_ctx* ctx, const pic_species* sp, int32_t nspecies, const void* EB,
                     void* J, double dt, double omegaB0, double dx, uint32_t flags,
                     void* stream);

/* The tile offsets of a species binned by PIC_SORT_TILED: out[t] is the first
 * particle of tile t (tiles in the sort's linear order, out[ntiles] = the
 * alive count; dead particles follow). *ntiles is always set; with
 * out == NULL only the count is returned. PIC_ERR_UNSUPPORTED when the
 * species has no valid binning (not sorted with PIC_SORT_TILED since its
 * npart last changed). Synchronises the stream. No reference counterpart. */
int pic_tile_offsets(pic_ctx* ctx, const pic_species* sp, int32_t* out, int64_t cap,
                     int64_t* ntiles, void* stream);

/* pic_push_deposit for the particles of tiles [tile_lo, tile_hi) of one
 * binned species (Boris or Vay): the tiled kernel over those tiles, then the
 * per-particle kernel over the ones it deferred. J is zeroed first unless
 * PIC_PD_NO_ZERO. Covering every tile once, in any number of calls, gives the
 * same particles and the same J (up to the order of the J additions: these
 * calls add to J with float atomics) as one pic_push_deposit call. Dead particles after the alive prefix are not
 * visited. PIC_ERR_UNSUPPORTED without a valid binning. No reference
 * counterpart: it lets a caller push part of a species while the rest is
 * still being copied in. */
int pic_push_deposit_tiles(pic_ctx* ctx, const pic_species* sp, const void* EB, void* J,
                           double dt, double omegaB0, double dx, int64_t tile_lo,
                           int64_t tile_hi, uint32_t flags, void* stream);

/* Metadomain::SynchronizeFields(Comm::J) + CommunicateFields(Comm::J)
 * (metadomain_comm.cpp:408-562, 204-367): periodic ghost currents are added
 * to their active images, then ghosts are refilled. buff is unused (kept for
 * signature parity with the reference, which stages through it). */
int pic_sync_currents(pic_ctx* ctx, void* J, void* buff, void* stream);

/* srpic::CurrentsFilter (src/engines/srpic/currents.h:89-119):
 * npasses x (buff <- J; DigitalFilter_kernel; CommunicateFields(J)),
 * src/kernels/digital_filter.hpp:129-389, Cartesian. */
int pic_filter_currents(pic_ctx* ctx, void* J, void* buff, int32_t npasses, void* stream);

/* Metadomain::CommunicateFields for one field (periodic self-exchange,
 * src/framework/domain/comm_nompi.hpp:44-63): ghosts of components [c0, c1)
 * are filled from their active images. is_em selects em_stride vs cur_stride. */
int pic_fill_ghosts(pic_ctx* ctx, void* field, int32_t is_em, int32_t c0, int32_t c1,
                    void* stream);

/* Metadomain::SortParticles (src/framework/domain/metadomain_sort.cpp:15-34)
 * for one species: PIC_SORT_REMOVE_DEAD = Particles::RemoveDead
 * (particles_sort.cpp:103-194), PIC_SORT_SPATIAL = Particles::SortSpatially
 * (particles_sort.cpp:196-253) as a stable counting sort on the
 * PositionToTileIndex key (src/global/utils/sorting.h:119-135). Synchronises
 * the stream; writes the new npart (dead removed) to *npart_out. */
int pic_sort(pic_ctx* ctx, pic_species* sp, uint32_t flags, int64_t* npart_out, void* stream);

/* FP64 field energy: out[0] = sum E^2, out[1] = sum B^2 with the Minkowski
 * weights of ReducedFields_kernel (src/kernels/reduced_stats.hpp:145-187).
 * Synchronises the stream. */
int pic_field_energy(pic_ctx* ctx, const void* EB, double dx, double* out, void* stream);

/* The field energy of pic_field_energy for callers that cannot allocate
 * device memory (a framework that reserves all device memory for its own
 * pool, a between-steps hook where cudaMalloc could synchronise the device,
 * a fixed device-memory budget). No counterpart in the reference. Needs no
 * context: it takes the grid description directly and allocates nothing; its
 * scratch is a fixed 1 MiB array inside the library, one slot pair per grid
 * row, so grids with more than 65536 rows (n2 * n3 in 3D, n2 in 2D) are
 * rejected with PIC_ERR_UNSUPPORTED. The first call on a device resolves the
 * array's device address, so make it before any stream capture; later calls
 * outside capture look it up again (a reset device gets the new address).
 * Calls share the array: calls that overlap on the GPU race and must be
 * serialised. An error already pending from the caller's earlier work is
 * returned as PIC_ERR_CUDA without being cleared. The result is computed in a
 * fixed order (bitwise reproducible). Synchronises the stream. */
int pic_field_energy_noalloc(const pic_grid* grid, const void* EB, double dx, double* out,
                             void* stream);

/* FP64 particle moments over the alive particles of nspecies species, the
 * SR Cartesian stress-energy sums of ReducedParticleMoments_kernel<SRPIC,
 * Minkowski, T> (src/kernels/reduced_stats.hpp:403-538, unweighted as there):
 * out[0] = sum m * gamma (sum |u| for massless), out[1..3] = sum u1, u2, u3;
 * and out[4] = sum w * m * (gamma - 1), the weighted kinetic energy (|u| for
 * massless), out[5] = sum w. The reference's normalisation (dV / (total
 * volume * ppc0), metadomain_stats.cpp:113-116) is the caller's.
 * Synchronises the stream. */
#define PIC_NMOMENTS 6
int pic_particle_moments(pic_ctx* ctx, const pic_species* sp, int32_t nspecies,
                         double out[PIC_NMOMENTS], void* stream);

/* Node charge density conserved by the current deposit: adds
 * rho(n) += charge * w * prod_d S(n_d - x_d) for every alive particle into
 * component 0 of `rho`, an array with the current layout (cur_stride), where
 * S is the unstaggered shape of the grid's order (order 0, the zigzag
 * deposit: the linear shape). Ghost nodes receive contributions like J and
 * are folded by pic_sync_currents. With it the discrete continuity equation
 * (rho_after - rho_before) / dt + D^- J = 0 holds node by node for one
 * pic_deposit (D^- the backward difference of J's staggered components).
 * The caller zeroes `rho`. No counterpart in the reference, whose Rho moment
 * (particle_moments.hpp) smooths with its own window. */
int pic_charge_density(pic_ctx* ctx, const pic_species* sp, int32_t nspecies, void* rho,
                       void* stream);

/* Device error word: out[0] = particles with an invalid tag seen by the
 * pusher, out[1] = alive particles whose cell lies outside the grid (skipped
 * by the pusher, reported by the sort), out[2] = particles whose deposit
 * stencil would leave the ghost layers (a step beyond the CFL limit; their
 * current is not deposited), out[3] = injected pairs whose velocity sampler
 * ran out of its rejection-loop bound.
 * Synchronises the stream. reset != 0 clears the counters. */
int pic_get_device_errors(pic_ctx* ctx, int64_t out[4], int32_t reset, void* stream);

/* Waits inside kernels that ran out of their iteration limit (the tiled
 * push/deposit's wait for its TMA field-window load); a tile whose wait ran
 * out is abandoned and counted here. No counterpart in the reference.
 * Synchronises the stream. reset != 0 clears the counter. */
int pic_get_wait_timeouts(pic_ctx* ctx, int64_t* out, int32_t reset, void* stream);

/* Phase timers, the counterpart of timer::Timers with blocking timers
 * (src/global/utils/timer.h:51-148, phases of srpic.hpp:85-187): when enabled,
 * pic_srpic_step records a CUDA event pair on its stream around every phase;
 * pic_timers_read synchronises on the recorded events and returns the summed
 * milliseconds and the number of intervals per phase. */
#define PIC_PHASE_FIELDSOLVER 0    /* Faraday halves + Ampere + J->E (+ fused exchanges) */
#define PIC_PHASE_PUSH_DEPOSIT 1   /* ParticlePusher + CurrentDeposit (fused) */
#define PIC_PHASE_COMMUNICATIONS 2 /* J fold and ghost fill */
#define PIC_PHASE_FILTERING 3      /* CurrentFiltering */
#define PIC_PHASE_SORT 4           /* ParticleSort */
#define PIC_PHASE_STEP 5           /* the whole step */
#define PIC_NPHASES 6

int pic_timers_enable(pic_ctx* ctx, int32_t on);
int pic_timers_reset(pic_ctx* ctx);
int pic_timers_read(pic_ctx* ctx, double ms[PIC_NPHASES], int64_t count[PIC_NPHASES]);
/* record the start / end of one interval of `phase` on `stream` (no-ops when
 * timers are disabled); used by the host engine */
int pic_timer_mark(pic_ctx* ctx, int32_t phase, int32_t is_end, void* stream);

/* The whole SR step of SRPICEngine::step_forward (srpic.hpp:65-188) for a
 * periodic Cartesian domain, driven by the C++ host engine in this library:
 * Faraday(1/2) + comm B, push + deposit of every species, J sync + comm,
 * nfilter passes, Faraday(1/2) + comm B, Ampere + CurrentsAmpere + comm E,J,
 * and a spatial sort of every species when sort_interval > 0 and
 * step % sort_interval == 0. */
typedef struct {
  double  dt;
  double  dx;
  double  omegaB0;   /* scales.omegaB0 */
  double  correction;/* algorithms.timestep.correction */
  double  q0, B0, V0, ppc0;
  int32_t nfilter;
  int32_t sort_interval;
  int32_t clear_interval;
  int32_t fieldsolver_enabled;
  int32_t deposit_enabled;
  int32_t write_prev;
  int32_t sort_tiled; /* spatial sorts use PIC_SORT_TILED */
  int32_t deposit_flags; /* extra pic_push_deposit flags: PIC_PD_FLOAT_ATOMICS or 0 */
} pic_step_params;

int pic_srpic_step(pic_ctx* ctx, pic_species* sp, int32_t nspecies, void* EB, void* J,
                   void* buff, const pic_step_params* prm, int64_t step, void* stream);

/* A domain whose state lives in pinned host memory, as the reference's OpenMP
 * build keeps its Views on the host (the caller of this path then passes host
 * buffers). The pipe holds two copy streams and per-array events; create one
 * per domain. No reference counterpart. */
typedef struct pic_host_pipe pic_host_pipe;
int pic_host_pipe_create(pic_host_pipe** out);
int pic_host_pipe_destroy(pic_host_pipe* pipe);
/* Waits for every copy the pipe has queued; the host arrays then hold the
 * last step's result. */
int pic_host_pipe_sync(pic_host_pipe* pipe);
/* How binned species are cut into tile groups: at most max_groups groups
 * (default 8) of at least min_group_bytes of particle state each (default
 * 256 MiB). Fewer, larger groups suit small species; more groups overlap the
 * copies and the push more finely. */
int pic_host_pipe_set_groups(pic_host_pipe* pipe, int32_t max_groups, int64_t min_group_bytes);
/* Bytes the last pic_srpic_step_host call copied host to device and back
 * (steps that sort copy the weights out as well). */
int pic_host_pipe_bytes(const pic_host_pipe* pipe, int64_t* bytes_in, int64_t* bytes_out);

/* One pic_srpic_step with host arrays as source and sink: hsp[k] (pinned host)
 * and dsp[k] (device) describe the same species, with equal npart; hEB / dEB
 * and hJ / dJ likewise, buff is device scratch. Copied in: EB and each
 * species' i, dx, u, weight and tag (the prev arrays stay on the device, as
 * the step rewrites them before reading). Copied out: J, EB and the same
 * species arrays, with npart updated in both descriptions; the weights only
 * on steps that sort (or clear), since no other phase changes them and the
 * host copy is otherwise current. Each array's
 * input copy waits only for the previous call's output copy of that array,
 * so one step's device-to-host copies overlap the next step's host-to-device
 * copies. Asynchronous: the host arrays hold the result after
 * pic_host_pipe_sync, and the device mirrors belong to the pipe until then. */
int pic_srpic_step_host(pic_ctx* ctx, pic_host_pipe* pipe, pic_species* hsp, pic_species* dsp,
                        int32_t nspecies, void* hEB, void* dEB, void* hJ, void* dJ, void* buff,
                        const pic_step_params* prm, int64_t step, void* stream);

/* ------------------------------------------------------------------------
 * Adjoint (reverse mode) of the SR step. No counterpart in the reference.
 *
 * Scope: 2D Cartesian grids, periodic fields and particles, Boris pusher
 * (pusher NONE species are carried along untouched), shape orders 1-3, Yee
 * solver, any number of filter passes. Positions are differentiated as
 * continuous coordinates X = i + dx, so orders >= 2 give an almost
 * everywhere smooth gradient.
 * ------------------------------------------------------------------------ */

/* Adjoint arrays of one species, real_t, at least npart long: the gradient
 * with respect to the position along each simulated axis (lx3 unused in 2D),
 * to the three momentum components, and to the weight. */
typedef struct {
  void* lx1;
  void* lx2;
  void* lx3;
  void* lu1;
  void* lu2;
  void* lu3;
  void* lw;
} pic_species_adjoint;

/* Checkpoint store inside the context. A slot holds EB and, per species, the
 * arrays a step changes (cells, offsets, momenta, tags); weights are not
 * copied. Slots are allocated on first use and kept until
 * pic_checkpoint_release or pic_destroy. Stream-ordered. */
int pic_checkpoint_save(pic_ctx* ctx, int32_t slot, const pic_species* sp, int32_t nspecies,
                        const void* EB, void* stream);
/* Restores a slot into the given arrays and npart (same species count). */
int pic_checkpoint_restore(pic_ctx* ctx, int32_t slot, pic_species* sp, int32_t nspecies,
                           void* EB, void* stream);
/* Species descriptors (copies of `like` with their state arrays pointing
 * into the slot) and the slot's EB, for reading a saved state in place. */
int pic_checkpoint_view(pic_ctx* ctx, int32_t slot, const pic_species* like, int32_t nspecies,
                        pic_species* out, void** EB);
int pic_checkpoint_release(pic_ctx* ctx);

/* lamEB = d/dEB of the E part of pic_field_energy (out[0]): 2 h dV E on the
 * active cells, zero elsewhere (ghosts included). */
int pic_field_energy_adjoint_seed(pic_ctx* ctx, const void* EB, void* lamEB, double dx,
                                  void* stream);

/* One step backwards. Given the state at the start of step n (species
 * arrays and EB, ghosts need not be filled) and the adjoint of the state at
 * the start of step n + 1 (adj arrays and lamEB, an EB-shaped array whose
 * ghosts are zero), overwrites them with the adjoint of the state at the
 * start of step n; adj.lw accumulates. The step is the one pic_srpic_step
 * takes with `prm` (sort and dead removal are not differentiated: the
 * caller runs the forward with both off). */
int pic_srpic_step_adjoint(pic_ctx* ctx, const pic_species* sp, pic_species_adjoint* adj,
                           int32_t nspecies, const void* EB, void* lamEB,
                           const pic_step_params* prm, void* stream);

/* Gradient of the final E-field energy (pic_field_energy out[0]) after
 * `nsteps` forward steps with respect to the initial state: runs the
 * forward from the given state with a checkpoint every `checkpoint_every`
 * steps (sort and dead removal off), then each segment backwards,
 * recomputing its steps from its checkpoint. On return *loss holds the
 * energy, adj the gradients with respect to the initial positions, momenta
 * and weights, lamEB the gradient with respect to the initial E and B, and
 * the species and EB arrays hold the initial state again. Memory: about
 * (nsteps / checkpoint_every + checkpoint_every) copies of the particle
 * state. Synchronises the stream. */
int pic_srpic_gradient(pic_ctx* ctx, pic_species* sp, pic_species_adjoint* adj,
                       int32_t nspecies, void* EB, void* J, void* buff,
                       const pic_step_params* prm, int64_t nsteps, int64_t checkpoint_every,
                       void* lamEB, double* loss, void* stream);

/* ------------------------------------------------------------------------
 * GR: 2D quasi-spherical Kerr-Schild grids (metric::QKerrSchild<Dim::_2D>,
 * src/metrics/qkerr_schild.h). The grid's axis 1 is the radial code
 * coordinate (log-spaced r), axis 2 the polar one (theta). Fields are
 * 6-component arrays with the em layout: D (or the auxiliary E) in 0..2, B
 * (or the auxiliary H) in 3..5; currents use the cur layout. Particle
 * boundaries come from pic_grid.prtl_bc: PIC_BC_ABSORB in r, PIC_BC_AXIS in
 * theta. The polar code coordinate is eta, with theta = eta + 2 h eta
 * (pi - 2 eta)(pi - eta) / pi^2 (qsph_h = h, 0 <= h < 1; h = 0 gives
 * theta = eta); x2min and x2max are theta extents.
 * ------------------------------------------------------------------------ */
typedef struct {
  double  a;              /* spin, 0 <= a < 1 */
  double  r0, h;          /* qsph_r0, qsph_h (0 <= h < 1) */
  double  x1min, x1max;   /* r extent (r_g) */
  double  x2min, x2max;   /* theta extent */
  int32_t axis_min;       /* field AXIS boundary at theta = x2min */
  int32_t axis_max;       /* field AXIS boundary at theta = x2max */
  int32_t horizon;        /* field HORIZON boundary at r = x1min */
} pic_gr_metric;

/* metric functions at n code-coordinate points x (device, n x 2 doubles);
 * out (device, n x PIC_GR_NQ doubles): h_11 h_22 h_33 h_13 h11 h22 h33 h13
 * alpha beta1 sqrt_det_h sqrt_det_h_tilde dr_alpha dt_alpha dr_beta1
 * dt_beta1 dr_h11 dr_h22 dr_h33 dr_h13 dt_h11 dt_h22 dt_h33 dt_h13, in the
 * grid's real_t */
#define PIC_GR_NQ 24
int pic_gr_metric_eval(pic_ctx* ctx, const pic_gr_metric* m, const double* x, int64_t n,
                       double* out, void* stream);

/* kernel::gr::Pusher_kernel (src/kernels/pushers/gr.hpp:664-865) for one
 * species: D interpolated from em, B from em0 at the grid's shape order
 * (1-3); Boris (massive) or photon; `niter` implicit iterations; prev arrays
 * written. In a single-precision build, particles with island_lo <= i1 <
 * island_hi (the FP64 island: a band of cells around the horizon) run the
 * metric and both implicit iterations in double; an empty band (island_hi <=
 * island_lo) pushes every particle in single precision. The reference's
 * UpdatePhi takes phi by value (gr.hpp:459-480), so phi is never changed
 * there; it is not written here either. */
int pic_gr_push(pic_ctx* ctx, const pic_gr_metric* m, pic_species* sp, const void* em,
                const void* em0, double dt, double omegaB0, int32_t niter, int32_t island_lo,
                int32_t island_hi, void* stream);

/* grpic::ParticlePush (src/engines/grpic/particle_pusher.h:26-94): the push
 * of pic_gr_push for every species with particles and a pusher. The FP64
 * islands of all species run at once, each on its own stream beside the
 * single-precision bulk. */
int pic_gr_particle_push(pic_ctx* ctx, const pic_gr_metric* m, pic_species* sp,
                         int32_t nspecies, const void* em, const void* em0, double dt,
                         double omegaB0, int32_t niter, int32_t island_lo, int32_t island_hi,
                         void* stream);

/* grpic::CurrentsDeposit (src/engines/grpic/currents.h:29-73): the current
 * of the last push at shape order 1 (hard-wired in the reference) with the
 * metric out-of-plane velocity (currents_deposit.hpp:138-159), evaluated
 * in double inside the FP64 island [island_lo, island_hi); J is zeroed
 * first unless flags has PIC_PD_NO_ZERO. */
int pic_gr_deposit(pic_ctx* ctx, const pic_gr_metric* m, const pic_species* sp,
                   int32_t nspecies, void* J, double dt, int32_t island_lo, int32_t island_hi,
                   uint32_t flags, void* stream);

/* gr::Faraday_kernel (faraday_gr.hpp:31-102) over the active cells:
 * Bout = Bin + coeff * curl E (coeff = fraction * correction * dt; Bin may
 * alias Bout) */
int pic_gr_faraday(pic_ctx* ctx, const pic_gr_metric* m, const void* Bin, void* Bout,
                   const void* E, double coeff, void* stream);
/* gr::Ampere_kernel (ampere_gr.hpp:32-101) over i2 in [i2min, i2max + 1):
 * Dout = Din + coeff * curl H. The axis cells copy dx1 from the neighbouring
 * row after that row is updated (when Din aliases Dout the reference reads it
 * unordered). */
int pic_gr_ampere(pic_ctx* ctx, const pic_gr_metric* m, const void* Din, void* Dout,
                  const void* H, double coeff, void* stream);
/* gr::CurrentsAmpere_kernel (ampere_gr.hpp:106-176): D += coeff * J with
 * the metric factors (coeff = -dt q0 / B0, fieldsolvers.h:216-221) */
int pic_gr_currents_ampere(pic_ctx* ctx, const pic_gr_metric* m, void* D, const void* J,
                           double coeff, void* stream);
/* ComputeAuxE (which = 0) / ComputeAuxH (which = 1) (aux_fields_gr.hpp:27-
 * 210) over range_with_axis_BCs (fieldsolvers.h:58-81): out's E (or H) from
 * the D of D and the B of B */
int pic_gr_aux(pic_ctx* ctx, const pic_gr_metric* m, int32_t which, const void* D, const void* B,
               void* out, void* stream);
/* TimeAverageDB (which = 0: b = (b + a) / 2 over the 6 EM components) and
 * TimeAverageJ (which = 1: a = (b + a) / 2 over the 3 current components),
 * active cells (aux_fields_gr.hpp:214-280) */
int pic_gr_average(pic_ctx* ctx, int32_t which, void* a, void* b, void* stream);
/* grpic::CurrentsFilter (src/engines/grpic/currents.h:74-101): npasses times
 * buff <- J, then DigitalFilter_kernel's 2D non-Cartesian stencil
 * (src/kernels/digital_filter.hpp:196-276) from buff into J over the active
 * cells and the row above them, with the reference's one-sided theta weights
 * on the rows next to an axis (m's axis flags). The exchange that follows
 * each pass in the reference is a no-op on one non-periodic domain. */
int pic_gr_filter_currents(pic_ctx* ctx, const pic_gr_metric* m, void* J, void* buff,
                           int32_t npasses, void* stream);
/* AxisBoundaries_kernel and HorizonBoundaries_kernel (fields_bcs.hpp:825-868,
 * 1188-1240) on one field, per m's axis/horizon flags; set_e / set_b select
 * the D (E) and B (H) components */
int pic_gr_field_bcs(pic_ctx* ctx, const pic_gr_metric* m, void* fld, int32_t set_e,
                     int32_t set_b, int32_t nfilter, void* stream);
/* MatchFieldsIn at +x1 (src/engines/grpic/fields_bcs.h:42-137) with
 * MatchBoundaries_kernel's GRPIC branch (src/kernels/fields_bcs.hpp:181-340):
 * over the cells of the layer r in [r_max - ds, r_max] (upper ghosts and all
 * theta cells included), each component relaxes toward `target`:
 * F = s F + (1 - s) target, s = tanh(4 |r - r_max| / ds) at the component's
 * radius. The reference evaluates the problem generator's field setter
 * there; the caller stores that field in `target` (em layout). set_e / set_b
 * select the D and B components. */
int pic_gr_match_fields(pic_ctx* ctx, const pic_gr_metric* m, void* fld, const void* target,
                        double ds, int32_t set_e, int32_t set_b, void* stream);
/* gr::AbsorbCurrents_kernel (src/kernels/fields_bcs.hpp:1243-1280) over the
 * same layer: J *= tanh(|r - r_max| / (ds / 4)) at the cell's radius. */
int pic_gr_absorb_currents(pic_ctx* ctx, const pic_gr_metric* m, void* J, double ds,
                           void* stream);
/* the vertical seed field of pgens/wald (InitFields, init_field = vertical)
 * on every cell, ghosts included; D = 0 */
int pic_gr_init_vertical(pic_ctx* ctx, const pic_gr_metric* m, void* EB, void* stream);
/* QKerrSchild::find_dxMin (qkerr_schild.h:112-129): min over cell centres of
 * 1 / (alpha sqrt(h^11 + h^22) + beta^1); dt = CFL * this. Synchronises. */
int pic_gr_min_cell_size(pic_ctx* ctx, const pic_gr_metric* m, double* out, void* stream);

/* GR step parameters beyond pic_step_params */
typedef struct {
  int32_t     niter;        /* pusher iterations (algorithms.gr.pusher_niter, default 10) */
  int32_t     island_lo;    /* particles with island_lo <= i1 < island_hi run the */
  int32_t     island_hi;    /* pusher in FP64 (single-precision builds) */
  double      match_ds;     /* > 0: MATCH fields at r max (grid.boundaries.match.ds) */
  const void* match_target; /* the field MATCH relaxes toward (6 components, em layout) */
} pic_gr_params;

/* GRPICEngine::step_forward (src/engines/grpic/grpic.hpp:66-634) on one
 * domain: fields[0..5] = em, em0, aux, cur, cur0, buff (device pointers);
 * the step swaps em <-> em0 and cur <-> cur0 in the array as the reference
 * swaps its views. Step 0 runs the reference's initialisation block.
 * prm->nfilter passes of pic_gr_filter_currents follow the deposit and the
 * current absorption (fields[5] is the filter's buffer). With gprm->match_ds > 0
 * the MATCH boundary at r max follows the axis and horizon boundaries on em
 * and em0 (FieldBoundaries, gr_bc::main), and, when particles are absorbed
 * at r max, the currents are absorbed there after the deposit (gr_bc::curr). */
int pic_grpic_step(pic_ctx* ctx, const pic_gr_metric* m, pic_species* sp, int32_t nspecies,
                   void* fields[6], const pic_step_params* prm, const pic_gr_params* gprm,
                   int64_t step, void* stream);

/* ---- SR field boundaries ---------------------------------------------- */

/* grid.boundaries.fields, per side; PERIODIC exactly on the axes the grid
 * was created periodic on. NONE leaves the ghost cells as they are (the
 * default of a non-periodic axis). */
#define PIC_FBC_PERIODIC 0
#define PIC_FBC_NONE 1
#define PIC_FBC_CONDUCTOR 2
#define PIC_FBC_MATCH 3

typedef struct {
  int32_t     kind[3][2];     /* PIC_FBC_* for (min, max) of each axis */
  double      x_min[3];       /* physical lower edge per axis (MATCH's coordinate) */
  double      dx;             /* cell size (MATCH) */
  double      match_ds[3][2]; /* grid.boundaries.match.ds per side (MATCH) */
  const void* match_target;   /* field MATCH relaxes toward, em layout (the
                                 problem generator's MatchFields, kept current
                                 by the caller) */
} pic_field_bcs;

/* Sets the context's field boundaries. PERIODIC must sit on the grid's
 * periodic axes. A context starts with PERIODIC there and NONE elsewhere. */
int pic_set_field_bcs(pic_ctx* ctx, const pic_field_bcs* bcs);

/* srpic::FieldBoundaries (src/engines/srpic/fields_bcs.h:622-672) on EB for
 * the E (set_e) and/or B (set_b) components, sides in Directions<D>::orth
 * order:
 *  - CONDUCTOR: ConductorBoundaries_kernel (src/kernels/fields_bcs.hpp:
 *    522-800): tangential E and normal B vanish on the wall, ghosts mirror
 *    the active cells;
 *  - MATCH: MatchBoundaries_kernel, SRPIC branch (fields_bcs.hpp:42-520):
 *    F = s F + (1 - s) target over the match layer, s = tanh(4 |x - x_edge|
 *    / ds) at each component's position.
 * pic_srpic_step calls it after each Faraday half (B) and after Ampere (E).
 * With conductor walls the current filter also takes the reference's wall
 * stencils (digital_filter.hpp:129-379). */
int pic_field_boundaries(pic_ctx* ctx, void* EB, int32_t set_e, int32_t set_b, void* stream);

/* ---- particle injection ------------------------------------------------ */

/* Parameters of arch::InjectUniformMaxwellians (src/archetypes/utils.h:46-107)
 * for one species pair. The box is in code units (cells from the first
 * active cell) per simulated axis; the reference takes it in physical
 * coordinates and maps it with DeduceRegion. */
typedef struct {
  double   number_density; /* total over the pair, in units of n0 */
  double   ppc0;           /* particles.ppc0 */
  double   xi_min[3];      /* injection box [xi_min, xi_max), code units */
  double   xi_max[3];
  double   temperature[2]; /* per species, m0 c^2 units (divided by the species' mass) */
  double   drift[2][3];    /* drift four-velocities (Cartesian only) */
  uint64_t seed;           /* Philox4x32-10 key */
  uint64_t first_pair;     /* pair p draws from the stream first_pair + p */
} pic_inject_params;

/* arch::InjectUniform (src/archetypes/particle_injector.h:203-261) with
 * kernel::UniformInjector_kernel (src/kernels/injectors.hpp:83-289) on a
 * Cartesian SR grid: n = (long)(ppc0 number_density / 2 * box cells) pairs
 * (ComputeNumInject, particle_injector.h:112-139). Each pair gets one uniform
 * position shared by both species and a Maxwell-Juttner velocity per species
 * (energy_dist.h:79-273: Box-Muller below temperature 0.5, the Sobol method
 * above, then the flipping boost toward the drift), weight 1, tag alive. The
 * particles are appended at each species' npart, which is advanced by n on
 * return (*n_pairs = n). Random numbers come from a Philox4x32-10 stream per
 * pair (counter-based, so independent of the launch shape); the reference's
 * Kokkos XorShift streams have no portable counterpart. The prev arrays are
 * not written. PIC_ERR_ARG if a species would exceed maxnpart, a mass is not
 * positive or the box leaves the grid. A sampler loop that runs out of its
 * iteration bound is counted in the error word's out[3]. */
int pic_inject_uniform_maxwellians(pic_ctx* ctx, pic_species* sp1, pic_species* sp2,
                                   const pic_inject_params* prm, int64_t* n_pairs, void* stream);

/* The same on the 2D QKerrSchild grid (the GRPIC branch of
 * UniformInjector_kernel): the tetrad-frame sample is transformed to
 * covariant components (transform<Idx::T, Idx::D>) at the particle, and the
 * weight is sqrt(det h) / V0 there. The reference ignores a drift outside
 * Cartesian coordinates; here a nonzero drift returns PIC_ERR_UNSUPPORTED. */
int pic_gr_inject_uniform_maxwellians(pic_ctx* ctx, const pic_gr_metric* m, pic_species* sp1,
                                      pic_species* sp2, const pic_inject_params* prm, double V0,
                                      int64_t* n_pairs, void* stream);

/* ---- output preparation (SR, Cartesian) -------------------------------- */

/* moments (FldsID, src/global/enums.h) */
#define PIC_MOM_RHO 0    /* mass density: contribution m */
#define PIC_MOM_CHARGE 1 /* charge density: contribution q */
#define PIC_MOM_N 2      /* number density: contribution 1 */
#define PIC_MOM_NPPC 3   /* particles per cell: no volume or weight factor */
#define PIC_MOM_T 4      /* stress-energy component T^{c1 c2} (0 = time) */
#define PIC_MOM_V 5      /* m u_c1 / u^0, to be divided by Rho (pic_normalize_by_rho) */

/* OutputSmoothingType (src/global/enums.h:405-435) */
#define PIC_SMOOTH_CONST 1u
#define PIC_SMOOTH_SPLINE 2u

typedef struct {
  int32_t id;          /* PIC_MOM_* */
  int32_t c1, c2;      /* components: T uses both (0..3), V uses c1 (1..3) */
  int32_t order;       /* output.fields.smoothing.order: window = ceil(order / 2) cells */
  int32_t smoothing;   /* PIC_SMOOTH_* (output.fields.smoothing.method) */
  int32_t use_weights; /* particles.use_weights */
  double  inv_n0;      /* 1 / scales.n0 */
  double  dx;          /* cell size; Minkowski sqrt(det h) = dx^D */
} pic_moment_params;

/* ComputeMoments (src/framework/domain/metadomain_io.cpp:123-170) with
 * ParticleMoments_kernel<SRPIC, Minkowski, F> (src/kernels/particle_moments.hpp:
 * 44-405): every alive particle of the nspecies species adds
 *   coeff * prod_d S(|dx_d - (di_d + 1/2)|),  |di_d| <= window,
 * to component `comp` of `bckp` at the cell i + di (ghosts included), where S
 * is the spline of the given order (prtl_shape::S1..S6) or the constant
 * 1 / (2 window + 1), and coeff is the moment's contribution times
 * inv_n0 / dx^D (and the weight with use_weights; neither for Nppc). bckp
 * has the EB layout (em_stride, 6 components); the caller zeroes it and folds
 * the ghosts with pic_sync_moments. Sums run in no fixed order (atomics), like
 * the reference's ScatterView. Particles whose cell lies outside the grid are
 * skipped and counted in the error word's out[1]. PIC_ERR_ARG: Rho or Charge
 * of a massless species, window > ng, an unknown smoothing; orders above 6
 * return PIC_ERR_UNSUPPORTED. */
int pic_output_moment(pic_ctx* ctx, const pic_species* sp, int32_t nspecies,
                      const pic_moment_params* prm, void* bckp, int32_t comp, void* stream);

/* Metadomain::SynchronizeFields(domain, Comm::Bckp, {c0, c1})
 * (src/framework/domain/metadomain_comm.cpp:408-562) along periodic axes:
 * the active cells add their ghost images of components [c0, c1). The
 * ghosts are zero afterwards (the reference leaves them as they were; output
 * reads active cells only). */
int pic_sync_moments(pic_ctx* ctx, void* bckp, int32_t c0, int32_t c1, void* stream);

/* NormalizeVectorByRho_kernel (src/kernels/particle_moments.hpp:407-478) on
 * the active cells: components c_v1..c_v3 are divided by c_rho where
 * |rho| > the real type's epsilon. */
int pic_normalize_by_rho(pic_ctx* ctx, void* bckp, int32_t c_rho, int32_t c_v1, int32_t c_v2,
                         int32_t c_v3, void* stream);

/* The divE output: ComputeDivergence_kernel<Minkowski> (src/kernels/
 * divergences.hpp:23-135) writes E1(i) - E1(i-1) + E2(j) - E2(j-1)
 * [+ E3(k) - E3(k-1)] into component `comp` of bckp (EB layout) at the
 * active cells; EB's lower ghosts must be filled. */
int pic_output_divergence(pic_ctx* ctx, const void* EB, void* bckp, int32_t comp, void* stream);

/* PrepareOutput flags (src/global/enums.h) */
#define PIC_OUT_INTERP_EDGES 1u /* E, J: cell centre from the edges */
#define PIC_OUT_INTERP_FACES 2u /* B: cell centre from the faces */
#define PIC_OUT_TO_HAT 4u       /* ConvertToHat: times dx along the simulated axes */

/* The field output of Metadomain::Write (src/framework/domain/
 * metadomain_io.cpp:380-700) for one quantity, in one pass:
 * DeepCopyFields, FieldsToPhys_kernel<Minkowski> (src/kernels/
 * fields_to_phys.hpp:33-241) and the writer's downsampling
 * (src/output/writer.cpp:199-300, first cell 0). Reads components
 * c0 .. c0 + ncomp - 1 (ncomp 1 or 3) of `src` (EB layout if is_em, else the
 * current layout) and writes out[c][o3][o2][o1] (o1 fastest), o_d over
 * ceil(n_d / dwn[d]) output cells taking cell o_d * dwn[d]. With ncomp = 1
 * (a moment) the values are copied as they are (flags must be 0). The
 * interpolation reads the first ghost layer above the active range: fill the
 * ghosts first. */
int pic_output_field(pic_ctx* ctx, const void* src, int32_t is_em, int32_t c0, int32_t ncomp,
                     uint32_t flags, double dx, const int32_t dwn[3], void* out, void* stream);

/* Particles::OutputWrite without tracking (src/framework/containers/
 * particles_io.cpp:93-235) with PrtlToPhys_kernel<SRPIC, Minkowski, false>
 * (src/kernels/prtls_to_phys.hpp:28-218): *nout = npart / stride records, the
 * p-th from particle p * stride, dead ones included as there:
 * x_d = (i_d + dx_d) * dx + xmin[d] for the simulated axes, u and the weight
 * copied. Output arrays are real_t, device-resident, caller-allocated with
 * room for npart / stride records. */
int pic_output_particles(pic_ctx* ctx, const pic_species* sp, int64_t stride, double dx,
                         const double xmin[3], void* const x_out[3], void* const u_out[3],
                         void* w_out, int64_t* nout, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ENTITY_PIC_H */
