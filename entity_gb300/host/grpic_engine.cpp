// GRPICEngine::step_forward (src/engines/grpic/grpic.hpp:66-634) over the C
// ABI: the leapfrog of D, B (em at the newer time, em0 at the older one),
// the auxiliary E and H, the GR push and deposit, and the field swap, with
// the axis, horizon and (optionally) MATCH field boundaries and the current
// absorption at r max, and the current filter. CommunicateFields and
// SynchronizeFields are no-ops on one non-periodic (r, theta) domain.
#include <cstdint>
#include <cuda_runtime.h>
#include <utility>

#include "../../include/entity_pic.h"
#include "srpic_engine.hpp"

namespace {

template <typename real>
int gr_step(pic_ctx* ctx, const pic_gr_metric* m, pic_species* sp, int32_t nsp, void** f,
            const pic_step_params& p, const pic_gr_params& gp, int64_t step, void* stream,
            size_t em_bytes) {
  int st;
#define PIC_TRY(x)            \
  do {                        \
    if ((st = (x)) != PIC_OK) \
      return st;              \
  } while (0)
  auto mark = [&](int phase, int end) { return pic_timer_mark(ctx, phase, end, stream); };
  // gr_bc::main boundaries act on both em and em0 (grpic/fields_bcs.h:220-262)
  // the directions in Directions<2>::orth order: horizon (-x1), axis (-x2,
  // +x2), match (+x1)
  const bool match  = gp.match_ds > 0.0;
  auto       bc_main = [&](int set_e, int set_b) {
    for (int k = 0; k < 2; ++k) {
      int s = pic_gr_field_bcs(ctx, m, f[k], set_e, set_b, p.nfilter, stream);
      if (s == PIC_OK && match)
        s = pic_gr_match_fields(ctx, m, f[k], gp.match_target, gp.match_ds, set_e, set_b,
                                stream);
      if (s != PIC_OK) return s;
    }
    return (int)PIC_OK;
  };
  auto swap = [&]() {
    std::swap(f[0], f[1]);
    std::swap(f[3], f[4]);
  };
  // coefficients in real_t (grpic/fieldsolvers.h:120-221)
  const real dt     = (real)p.dt;
  const real dT1    = (real)1 * (real)p.correction * dt;
  const real dThalf = (real)0.5 * (real)p.correction * dt;
  const real jcoeff = -dt * (real)p.q0 / (real)p.B0;
  const bool fs = p.fieldsolver_enabled != 0, dep = p.deposit_enabled != 0;
  pic_grid   g;
  PIC_TRY(pic_get_grid(ctx, &g));
  const bool absorb_max = g.prtl_bc[0][1] == PIC_BC_ABSORB;
  void*      aux = f[2];

  PIC_TRY(mark(PIC_PHASE_STEP, 0));
  if (step == 0) {
    if (fs) {
      PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 0));
      PIC_TRY(bc_main(1, 1));
      if (cudaMemcpyAsync(f[1], f[0], em_bytes, cudaMemcpyDeviceToDevice,
                          (cudaStream_t)stream) != cudaSuccess)
        return PIC_ERR_CUDA;
      PIC_TRY(pic_gr_aux(ctx, m, 0, f[0], f[1], aux, stream));
      PIC_TRY(pic_gr_aux(ctx, m, 1, f[0], f[1], aux, stream));
      PIC_TRY(pic_gr_faraday(ctx, m, f[1], f[1], aux, (double)dThalf, stream));
      PIC_TRY(bc_main(0, 1));
      PIC_TRY(pic_gr_ampere(ctx, m, f[0], f[0], aux, (double)dThalf, stream));
      PIC_TRY(bc_main(1, 0));
      PIC_TRY(pic_gr_aux(ctx, m, 0, f[0], f[1], aux, stream));
      PIC_TRY(pic_gr_aux(ctx, m, 1, f[0], f[1], aux, stream));
      PIC_TRY(pic_gr_faraday(ctx, m, f[0], f[1], aux, (double)dT1, stream));
      PIC_TRY(bc_main(0, 1));
      PIC_TRY(pic_gr_ampere(ctx, m, f[1], f[1], aux, (double)dT1, stream));
      PIC_TRY(bc_main(1, 0));
      PIC_TRY(pic_gr_aux(ctx, m, 1, f[1], f[1], aux, stream));
      PIC_TRY(pic_gr_ampere(ctx, m, f[0], f[1], aux, (double)dT1, stream));
      PIC_TRY(bc_main(1, 0));
      swap();
      PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 1));
    } else {
      if (cudaMemcpyAsync(f[1], f[0], em_bytes, cudaMemcpyDeviceToDevice,
                          (cudaStream_t)stream) != cudaSuccess)
        return PIC_ERR_CUDA;
    }
  }
  if (fs) {
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 0));
    PIC_TRY(pic_gr_average(ctx, 0, f[0], f[1], stream));            // em0 = (em0 + em) / 2
    PIC_TRY(pic_gr_aux(ctx, m, 0, f[1], f[0], aux, stream));         // E(D0, B)
    PIC_TRY(pic_gr_faraday(ctx, m, f[1], f[1], aux, (double)dT1, stream));
    PIC_TRY(bc_main(0, 1));
    PIC_TRY(pic_gr_aux(ctx, m, 1, f[0], f[1], aux, stream));         // H(D, B0)
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 1));
  }
  PIC_TRY(mark(PIC_PHASE_PUSH_DEPOSIT, 0));
  PIC_TRY(pic_gr_particle_push(ctx, m, sp, nsp, f[0], f[1], (double)dt, (double)(real)p.omegaB0,
                               gp.niter, gp.island_lo, gp.island_hi, stream));
  if (dep) {
    PIC_TRY(pic_gr_deposit(ctx, m, sp, nsp, f[4], (double)dt, gp.island_lo, gp.island_hi, 0u,
                           stream));
    // FieldBoundaries(gr_bc::curr): absorbing particles at r max (fields_bcs.h:262-268)
    if (match && absorb_max) PIC_TRY(pic_gr_absorb_currents(ctx, m, f[4], gp.match_ds, stream));
    // CurrentsFilter on cur0 (grpic.hpp:437-439)
    if (p.nfilter > 0) PIC_TRY(pic_gr_filter_currents(ctx, m, f[4], f[5], p.nfilter, stream));
  }
  PIC_TRY(mark(PIC_PHASE_PUSH_DEPOSIT, 1));
  if (fs) {
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 0));
    if (dep) PIC_TRY(pic_gr_average(ctx, 1, f[3], f[4], stream));  // J = (J0 + J) / 2
    PIC_TRY(pic_gr_aux(ctx, m, 0, f[0], f[1], aux, stream));         // E(D, B0)
    PIC_TRY(pic_gr_faraday(ctx, m, f[0], f[1], aux, (double)dT1, stream));
    PIC_TRY(bc_main(0, 1));
    PIC_TRY(pic_gr_ampere(ctx, m, f[1], f[1], aux, (double)dT1, stream));
    if (dep) PIC_TRY(pic_gr_currents_ampere(ctx, m, f[1], f[3], (double)jcoeff, stream));
    PIC_TRY(bc_main(1, 0));
    PIC_TRY(pic_gr_aux(ctx, m, 1, f[1], f[1], aux, stream));         // H(D0, B0)
    PIC_TRY(pic_gr_ampere(ctx, m, f[0], f[1], aux, (double)dT1, stream));
    if (dep) PIC_TRY(pic_gr_currents_ampere(ctx, m, f[1], f[4], (double)jcoeff, stream));
    swap();
    PIC_TRY(bc_main(1, 0));
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 1));
  }
  PIC_TRY(mark(PIC_PHASE_SORT, 0));
  entity_gb300::Domain dom;
  dom.ctx = ctx;
  dom.dim = 2;
  dom.species.assign(sp, sp + nsp);
  PIC_TRY(entity_gb300::srpic::SortParticles(dom, p, step, stream));
  for (int32_t k = 0; k < nsp; ++k) sp[k].npart = dom.species[k].npart;
  PIC_TRY(mark(PIC_PHASE_SORT, 1));
  PIC_TRY(mark(PIC_PHASE_STEP, 1));
#undef PIC_TRY
  return PIC_OK;
}

}  // namespace

extern "C" int pic_grpic_step(pic_ctx* ctx, const pic_gr_metric* m, pic_species* sp,
                              int32_t nspecies, void* fields[6], const pic_step_params* prm,
                              const pic_gr_params* gprm, int64_t step, void* stream) {
  if (!ctx || !m || !fields || !prm || !gprm || nspecies < 0 || (nspecies > 0 && !sp))
    return PIC_ERR_ARG;
  for (int k = 0; k < 5; ++k)
    if (!fields[k]) return PIC_ERR_ARG;
  if (prm->nfilter < 0 || (prm->nfilter > 0 && !fields[5])) return PIC_ERR_ARG;
  if (gprm->niter < 1) return PIC_ERR_UNSUPPORTED;
  if (gprm->match_ds < 0.0 || (gprm->match_ds > 0.0 && !gprm->match_target)) return PIC_ERR_ARG;
  pic_grid g;
  int      st = pic_get_grid(ctx, &g);
  if (st != PIC_OK) return st;
  if (g.dim != 2) return PIC_ERR_UNSUPPORTED;
  // bytes spanned by a 6-component field with the em strides
  int64_t span = 5 * g.em_stride[3];
  for (int d = 0; d < 2; ++d) span += (int64_t)(g.n[d] + 2 * g.ng - 1) * g.em_stride[d];
  const size_t em_bytes = (size_t)(span + 1) * (size_t)g.real_bytes;
  return g.real_bytes == 8
           ? gr_step<double>(ctx, m, sp, nspecies, fields, *prm, *gprm, step, stream, em_bytes)
           : gr_step<float>(ctx, m, sp, nspecies, fields, *prm, *gprm, step, stream, em_bytes);
}
