// C++ host engine above the C ABI: the phase functions of the reference's SR
// engine (src/engines/srpic/{fieldsolvers,particle_pusher,currents}.h) and
// its step_forward (src/engines/srpic/srpic.hpp:65-188), on a Domain that
// holds device pointers. Coefficients are derived in real_t with the
// reference's operation order so that a float build reproduces its values.
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/entity_pic.h"

namespace entity_gb300 {

struct Domain {
  pic_ctx*                 ctx  = nullptr;
  void*                    EB   = nullptr;  // ndfield_t<D, 6>
  void*                    J    = nullptr;  // ndfield_t<D, 3> (fields.cur)
  void*                    buff = nullptr;  // ndfield_t<D, 3> (fields.buff)
  std::vector<pic_species> species;
  int                      dim  = 3;
};

namespace srpic {

// srpic::Faraday (fieldsolvers.h:36-99): dT = fraction * correction * dt;
// dx = sqrt(h_11); 2D: coeff1 = dT / dx^2, coeff2 = dT; 3D: coeff1 = dT / dx
template <typename real>
int Faraday(Domain& dom, const pic_step_params& p, real fraction, void* stream) {
  const real dT = fraction * (real)p.correction * (real)p.dt;
  const real h  = (real)p.dx * (real)p.dx;
  const real dx = std::sqrt(h);
  real       coeff1, coeff2;
  if (dom.dim == 2) {
    coeff1 = dT / (dx * dx);
    coeff2 = dT;
  } else {
    coeff1 = dT / dx;
    coeff2 = (real)0;
  }
  return pic_faraday(dom.ctx, dom.EB, (double)coeff1, (double)coeff2, nullptr, stream);
}

// srpic::Ampere (fieldsolvers.h:101-140) fused with srpic::CurrentsAmpere
// (fieldsolvers.h:142-200): coeff = -dt * q0 / (B0 * V0)
template <typename real>
int AmpereWithCurrents(Domain& dom, const pic_step_params& p, real fraction, bool deposit,
                       void* stream) {
  const real dT = fraction * (real)p.correction * (real)p.dt;
  const real h  = (real)p.dx * (real)p.dx;
  const real dx = std::sqrt(h);
  real       coeff1, coeff2;
  if (dom.dim == 2) {
    coeff1 = dT / (dx * dx);
    coeff2 = dT;
  } else {
    coeff1 = dT / dx;
    coeff2 = (real)0;
  }
  const real jcoeff = -(real)p.dt * (real)p.q0 / ((real)p.B0 * (real)p.V0);
  return pic_ampere_currents(dom.ctx, dom.EB, deposit ? dom.J : nullptr, (double)coeff1,
                             (double)coeff2, (double)jcoeff, (double)(real)p.ppc0, stream);
}

// srpic::ParticlePush + srpic::CurrentsDeposit, fused
template <typename real>
int PushDeposit(Domain& dom, const pic_step_params& p, bool deposit, void* stream) {
  const uint32_t flags = (p.write_prev ? PIC_PD_WRITE_PREV : 0u) |
                         ((uint32_t)p.deposit_flags & PIC_PD_FLOAT_ATOMICS);
  if (deposit) {
    return pic_push_deposit(dom.ctx, dom.species.data(), (int32_t)dom.species.size(), dom.EB, dom.J,
                            (double)(real)p.dt, (double)(real)p.omegaB0, (double)(real)p.dx,
                            flags, stream);
  }
  for (auto& s : dom.species) {
    const int st = pic_push(dom.ctx, &s, dom.EB, (double)(real)p.dt, (double)(real)p.omegaB0,
                            (double)(real)p.dx, stream);
    if (st != PIC_OK) return st;
  }
  return PIC_OK;
}

// Metadomain::SortParticles (metadomain_sort.cpp:15-34)
inline int SortParticles(Domain& dom, const pic_step_params& p, int64_t step, void* stream) {
  for (auto& s : dom.species) {
    uint32_t flags = 0;
    if (p.clear_interval > 0 && step % p.clear_interval == 0 && step > 0) flags |= PIC_SORT_REMOVE_DEAD;
    if (p.sort_interval > 0 && step % p.sort_interval == 0) {
      flags |= PIC_SORT_SPATIAL;
      if (p.sort_tiled) flags |= PIC_SORT_TILED;
    }
    if (!flags) continue;
    if (!p.write_prev) flags |= PIC_SORT_SKIP_PREV;
    // a spatial sort leaves npart as it is: no need to wait for it
    if (!(flags & PIC_SORT_REMOVE_DEAD)) flags |= PIC_SORT_NO_SYNC;
    int64_t    n  = s.npart;
    const int  st = pic_sort(dom.ctx, &s, flags, &n, stream);
    if (st != PIC_OK) return st;
    s.npart = n;
  }
  return PIC_OK;
}

// SRPICEngine::step_forward (srpic.hpp:65-188), Cartesian domain
template <typename real>
int StepForward(Domain& dom, const pic_step_params& p, int64_t step, void* stream) {
  int st;
#define PIC_TRY(x)            \
  do {                        \
    if ((st = (x)) != PIC_OK) \
      return st;              \
  } while (0)
  // timer::Timers phases (srpic.hpp:85-187); no-ops unless timers are enabled
  auto mark = [&](int phase, int end) { return pic_timer_mark(dom.ctx, phase, end, stream); };
  PIC_TRY(mark(PIC_PHASE_STEP, 0));
  if (step == 0) {
    // srpic.hpp:71-73: CommunicateFields(B | E) on the first step
    PIC_TRY(pic_fill_ghosts(dom.ctx, dom.EB, 1, 0, 6, stream));
  }
  const bool fs  = p.fieldsolver_enabled != 0;
  const bool dep = p.deposit_enabled != 0;
  if (fs) {
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 0));
    PIC_TRY(Faraday<real>(dom, p, (real)0.5, stream));
    // FieldBoundaries(BC::B) (srpic.hpp:94-101); no launch on periodic sides
    PIC_TRY(pic_field_boundaries(dom.ctx, dom.EB, 0, 1, stream));
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 1));
  }
  PIC_TRY(mark(PIC_PHASE_PUSH_DEPOSIT, 0));
  PIC_TRY(PushDeposit<real>(dom, p, dep, stream));
  PIC_TRY(mark(PIC_PHASE_PUSH_DEPOSIT, 1));
  if (dep) {
    PIC_TRY(mark(PIC_PHASE_COMMUNICATIONS, 0));
    PIC_TRY(pic_sync_currents(dom.ctx, dom.J, dom.buff, stream));
    PIC_TRY(mark(PIC_PHASE_COMMUNICATIONS, 1));
    PIC_TRY(mark(PIC_PHASE_FILTERING, 0));
    PIC_TRY(pic_filter_currents(dom.ctx, dom.J, dom.buff, p.nfilter, stream));
    PIC_TRY(mark(PIC_PHASE_FILTERING, 1));
  }
  if (fs) {
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 0));
    PIC_TRY(Faraday<real>(dom, p, (real)0.5, stream));
    PIC_TRY(pic_field_boundaries(dom.ctx, dom.EB, 0, 1, stream));
    PIC_TRY(AmpereWithCurrents<real>(dom, p, (real)1, dep, stream));
    // FieldBoundaries(BC::E) (srpic.hpp:169-176)
    PIC_TRY(pic_field_boundaries(dom.ctx, dom.EB, 1, 0, stream));
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 1));
  }
  PIC_TRY(mark(PIC_PHASE_SORT, 0));
  PIC_TRY(SortParticles(dom, p, step, stream));
  PIC_TRY(mark(PIC_PHASE_SORT, 1));
  PIC_TRY(mark(PIC_PHASE_STEP, 1));
#undef PIC_TRY
  return PIC_OK;
}

}  // namespace srpic
}  // namespace entity_gb300
