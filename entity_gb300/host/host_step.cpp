// pic_srpic_step_host: one SR step of a domain whose state lives in pinned
// host memory, as the reference's OpenMP build keeps its Views on the host.
//
// Every call copies the step's inputs in (EB and each species' i, dx, u,
// weight, tag), runs pic_srpic_step on the device mirrors, and copies the
// results out (EB, J and the species' arrays). The copies go through two
// streams of the pipe per direction (fields and particles apart). Each array's input copy waits only
// for the previous call's output copy of the same array. So the previous
// step's device-to-host traffic overlaps this step's host-to-device traffic,
// and the host link runs in both directions at once. The call returns once
// the copies and the step are queued: the host arrays hold the result after
// pic_host_pipe_sync, and the device mirrors belong to the pipe until then.
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/entity_pic.h"
#include "srpic_engine.hpp"

struct pic_host_pipe {
  cudaStream_t             up = nullptr, down = nullptr;
  cudaStream_t             up_f = nullptr, down_f = nullptr;  // the fields' copies
  cudaEvent_t              entry = nullptr, eb_in = nullptr, step_done = nullptr;
  std::vector<cudaEvent_t> out_done;        // per array slot
  std::vector<cudaEvent_t> sp_in, sp_done;  // per species
  std::vector<char>        pending;   // slot has an output copy from an earlier call
  int64_t                  bytes_in = 0, bytes_out = 0;
};

namespace {

struct Slot {
  void*  host;
  void*  dev;
  size_t bytes;
};

// elements spanned by a field of `ncomp` components with the grid's strides
size_t field_span(const pic_grid& g, const int64_t s[4], int ncomp) {
  int64_t last = (int64_t)(ncomp - 1) * s[3];
  for (int d = 0; d < 3; ++d) {
    const int64_t ext = d < g.dim ? g.n[d] + 2 * g.ng : 1;
    last += (ext - 1) * s[d];
  }
  return (size_t)(last + 1);
}

// the arrays of one species that carry state from one step to the next
void species_slots(const pic_grid& g, const pic_species& h, const pic_species& d,
                   std::vector<Slot>& out) {
  const size_t n = (size_t)d.npart, rb = (size_t)g.real_bytes;
  void* const  hs[] = { h.i1, h.i2, h.i3, h.dx1, h.dx2, h.dx3, h.ux1, h.ux2, h.ux3, h.weight,
                        h.tag };
  void* const  ds[] = { d.i1, d.i2, d.i3, d.dx1, d.dx2, d.dx3, d.ux1, d.ux2, d.ux3, d.weight,
                        d.tag };
  const size_t es[] = { 4, 4, 4, 4, 4, 4, rb, rb, rb, rb, 2 };
  for (int a = 0; a < 11; ++a) {
    if ((a == 2 || a == 5) && g.dim != 3) continue;
    out.push_back({ hs[a], ds[a], n * es[a] });
  }
}

bool species_ok(const pic_grid& g, const pic_species& h, const pic_species& d) {
  if (h.npart != d.npart || h.npart < 0) return false;
  if (d.maxnpart > 0 && d.npart > d.maxnpart) return false;
  if (h.npart == 0) return true;
  const void* need[] = { h.i1, h.i2, h.dx1, h.dx2, h.ux1, h.ux2, h.ux3, h.weight, h.tag,
                         d.i1, d.i2, d.dx1, d.dx2, d.ux1, d.ux2, d.ux3, d.weight, d.tag };
  for (const void* p : need)
    if (!p) return false;
  if (g.dim == 3 && (!h.i3 || !h.dx3 || !d.i3 || !d.dx3)) return false;
  return true;
}

int resize(pic_host_pipe* p, size_t nslots, int nspecies) {
  if (p->out_done.size() == nslots && p->sp_in.size() == (size_t)nspecies) return PIC_OK;
  // a different array set: finish earlier copies, then rebuild the events
  for (cudaStream_t q : { p->up, p->down, p->up_f, p->down_f })
    if (cudaStreamSynchronize(q) != cudaSuccess) return PIC_ERR_CUDA;
  for (auto* v : { &p->out_done, &p->sp_in, &p->sp_done }) {
    for (cudaEvent_t e : *v) cudaEventDestroy(e);
    v->clear();
  }
  p->out_done.assign(nslots, nullptr);
  p->pending.assign(nslots, 0);
  p->sp_in.assign(nspecies, nullptr);
  p->sp_done.assign(nspecies, nullptr);
  for (auto* v : { &p->out_done, &p->sp_in, &p->sp_done })
    for (auto& e : *v)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return PIC_ERR_CUDA;
  return PIC_OK;
}

}  // namespace

extern "C" {

int pic_host_pipe_create(pic_host_pipe** out) {
  if (!out) return PIC_ERR_ARG;
  *out = nullptr;
  auto* p = new pic_host_pipe();
  bool  ok = true;
  for (cudaStream_t* q : { &p->up, &p->down, &p->up_f, &p->down_f })
    ok = ok && cudaStreamCreateWithFlags(q, cudaStreamNonBlocking) == cudaSuccess;
  for (cudaEvent_t* e : { &p->entry, &p->eb_in, &p->step_done })
    ok = ok && cudaEventCreateWithFlags(e, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    pic_host_pipe_destroy(p);
    return PIC_ERR_CUDA;
  }
  *out = p;
  return PIC_OK;
}

int pic_host_pipe_destroy(pic_host_pipe* p) {
  if (!p) return PIC_ERR_ARG;
  for (cudaStream_t q : { p->up, p->down, p->up_f, p->down_f })
    if (q) cudaStreamSynchronize(q);
  for (cudaEvent_t e : p->out_done) cudaEventDestroy(e);
  for (cudaEvent_t e : p->sp_in) cudaEventDestroy(e);
  for (cudaEvent_t e : p->sp_done) cudaEventDestroy(e);
  for (cudaEvent_t e : { p->entry, p->eb_in, p->step_done })
    if (e) cudaEventDestroy(e);
  for (cudaStream_t q : { p->up, p->down, p->up_f, p->down_f })
    if (q) cudaStreamDestroy(q);
  delete p;
  return PIC_OK;
}

int pic_host_pipe_sync(pic_host_pipe* p) {
  if (!p) return PIC_ERR_ARG;
  for (cudaStream_t q : { p->up, p->down, p->up_f, p->down_f })
    if (cudaStreamSynchronize(q) != cudaSuccess) return PIC_ERR_CUDA;
  return PIC_OK;
}

int pic_host_pipe_bytes(const pic_host_pipe* p, int64_t* bytes_in, int64_t* bytes_out) {
  if (!p || !bytes_in || !bytes_out) return PIC_ERR_ARG;
  *bytes_in  = p->bytes_in;
  *bytes_out = p->bytes_out;
  return PIC_OK;
}

int pic_srpic_step_host(pic_ctx* ctx, pic_host_pipe* p, pic_species* hsp, pic_species* dsp,
                        int32_t nspecies, void* hEB, void* dEB, void* hJ, void* dJ, void* buff,
                        const pic_step_params* prm, int64_t step, void* stream) {
  if (!ctx || !p || !hEB || !dEB || !prm || nspecies < 0) return PIC_ERR_ARG;
  if (nspecies > 0 && (!hsp || !dsp)) return PIC_ERR_ARG;
  if (prm->deposit_enabled && (!hJ || !dJ || !buff)) return PIC_ERR_ARG;
  pic_grid g;
  int      st = pic_get_grid(ctx, &g);
  if (st != PIC_OK) return st;
  for (int k = 0; k < nspecies; ++k)
    if (!species_ok(g, hsp[k], dsp[k])) return PIC_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t rb = (size_t)g.real_bytes;
  const bool   dep = prm->deposit_enabled != 0, fs = prm->fieldsolver_enabled != 0;

  // slot 0: J (output only); slot 1: EB; then every species' state arrays
  std::vector<Slot>   slots;
  std::vector<size_t> first(nspecies + 1);
  slots.push_back({ hJ, dJ, dep ? field_span(g, g.cur_stride, 3) * rb : 0 });
  slots.push_back({ hEB, dEB, field_span(g, g.em_stride, 6) * rb });
  for (int k = 0; k < nspecies; ++k) {
    first[k] = slots.size();
    species_slots(g, hsp[k], dsp[k], slots);
  }
  first[nspecies] = slots.size();
  if ((st = resize(p, slots.size(), nspecies)) != PIC_OK) return st;

  auto wait_out = [&](cudaStream_t on, size_t a) {
    return !p->pending[a] || cudaStreamWaitEvent(on, p->out_done[a], 0) == cudaSuccess;
  };
  // fields (slots 0, 1) and particles copy on separate streams, so that a
  // species' input copy never queues behind the fields' and vice versa
  auto copy_out = [&](size_t a0, size_t a1, int64_t& bytes) {
    for (size_t a = a0; a < a1; ++a) {
      cudaStream_t q = a < 2 ? p->down_f : p->down;
      if (slots[a].bytes > 0 && cudaMemcpyAsync(slots[a].host, slots[a].dev, slots[a].bytes,
                                                cudaMemcpyDeviceToHost, q) != cudaSuccess)
        return false;
      bytes += (int64_t)slots[a].bytes;
      if (cudaEventRecord(p->out_done[a], q) != cudaSuccess) return false;
      p->pending[a] = 1;
    }
    return true;
  };

  // inputs, EB first, then species by species; a fresh pipe first waits for
  // the caller's earlier work on `stream`
  bool fresh = true;
  for (char c : p->pending) fresh = fresh && !c;
  if (fresh) {
    if (cudaEventRecord(p->entry, s) != cudaSuccess) return PIC_ERR_CUDA;
    if (cudaStreamWaitEvent(p->up, p->entry, 0) != cudaSuccess) return PIC_ERR_CUDA;
    if (cudaStreamWaitEvent(p->up_f, p->entry, 0) != cudaSuccess) return PIC_ERR_CUDA;
  }
  int64_t bin = 0;
  for (size_t a = 1; a < slots.size(); ++a) {
    cudaStream_t q = a < 2 ? p->up_f : p->up;
    if (!wait_out(q, a)) return PIC_ERR_CUDA;
    if (slots[a].bytes > 0 && cudaMemcpyAsync(slots[a].dev, slots[a].host, slots[a].bytes,
                                              cudaMemcpyHostToDevice, q) != cudaSuccess)
      return PIC_ERR_CUDA;
    bin += (int64_t)slots[a].bytes;
    if (a == 1 && cudaEventRecord(p->eb_in, q) != cudaSuccess) return PIC_ERR_CUDA;
    for (int k = 0; k < nspecies; ++k)
      if (a + 1 == first[k + 1] && cudaEventRecord(p->sp_in[k], p->up) != cudaSuccess)
        return PIC_ERR_CUDA;
  }

  // the step (SRPICEngine::step_forward, as pic_srpic_step runs it), with
  // each species pushed as soon as its arrays are in
  entity_gb300::Domain dom;
  dom.ctx  = ctx;
  dom.EB   = dEB;
  dom.J    = dJ;
  dom.buff = buff;
  dom.dim  = g.dim;
  dom.species.assign(dsp, dsp + nspecies);
  const bool f64 = g.real_bytes == 8;
  bool       sorts = false;  // particle arrays change after the push this step
  for (int k = 0; k < nspecies; ++k)
    sorts = sorts || (prm->clear_interval > 0 && step % prm->clear_interval == 0 && step > 0) ||
            (prm->sort_interval > 0 && step % prm->sort_interval == 0);
#define PIC_TRY(x)                \
  do {                            \
    if ((st = (x)) != PIC_OK)     \
      return st;                  \
  } while (0)
  auto mark = [&](int phase, int end) { return pic_timer_mark(ctx, phase, end, stream); };
  if (cudaStreamWaitEvent(s, p->eb_in, 0) != cudaSuccess) return PIC_ERR_CUDA;
  PIC_TRY(mark(PIC_PHASE_STEP, 0));
  if (step == 0) {
    PIC_TRY(pic_fill_ghosts(ctx, dEB, 1, 0, 6, stream));
  }
  if (fs) {
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 0));
    PIC_TRY(f64 ? entity_gb300::srpic::Faraday<double>(dom, *prm, 0.5, stream)
                : entity_gb300::srpic::Faraday<float>(dom, *prm, 0.5f, stream));
    PIC_TRY(pic_field_boundaries(ctx, dEB, 0, 1, stream));
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 1));
  }
  // J is written from here on: its previous output copy must be done
  if (!wait_out(s, 0)) return PIC_ERR_CUDA;
  int64_t bout = 0;
  PIC_TRY(mark(PIC_PHASE_PUSH_DEPOSIT, 0));
  const double dt  = f64 ? prm->dt : (double)(float)prm->dt;
  const double wB  = f64 ? prm->omegaB0 : (double)(float)prm->omegaB0;
  const double dxc = f64 ? prm->dx : (double)(float)prm->dx;
  const uint32_t fl = prm->write_prev ? PIC_PD_WRITE_PREV : 0u;
  if (dep && nspecies == 0) {
    PIC_TRY(pic_push_deposit(ctx, nullptr, 0, dEB, dJ, dt, wB, dxc, fl, stream));
  }
  for (int k = 0; k < nspecies; ++k) {
    if (cudaStreamWaitEvent(s, p->sp_in[k], 0) != cudaSuccess) return PIC_ERR_CUDA;
    if (dep) {
      PIC_TRY(pic_push_deposit(ctx, &dom.species[k], 1, dEB, dJ, dt, wB, dxc,
                               fl | (k > 0 ? PIC_PD_NO_ZERO : 0u), stream));
    } else {
      PIC_TRY(pic_push(ctx, &dom.species[k], dEB, dt, wB, dxc, stream));
    }
    if (!sorts) {
      // nothing later in the step touches this species' state arrays
      if (cudaEventRecord(p->sp_done[k], s) != cudaSuccess) return PIC_ERR_CUDA;
      if (cudaStreamWaitEvent(p->down, p->sp_done[k], 0) != cudaSuccess) return PIC_ERR_CUDA;
      if (!copy_out(first[k], first[k + 1], bout)) return PIC_ERR_CUDA;
    }
  }
  PIC_TRY(mark(PIC_PHASE_PUSH_DEPOSIT, 1));
  if (dep) {
    PIC_TRY(mark(PIC_PHASE_COMMUNICATIONS, 0));
    PIC_TRY(pic_sync_currents(ctx, dJ, buff, stream));
    PIC_TRY(mark(PIC_PHASE_COMMUNICATIONS, 1));
    PIC_TRY(mark(PIC_PHASE_FILTERING, 0));
    PIC_TRY(pic_filter_currents(ctx, dJ, buff, prm->nfilter, stream));
    PIC_TRY(mark(PIC_PHASE_FILTERING, 1));
  }
  if (fs) {
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 0));
    PIC_TRY(f64 ? entity_gb300::srpic::Faraday<double>(dom, *prm, 0.5, stream)
                : entity_gb300::srpic::Faraday<float>(dom, *prm, 0.5f, stream));
    PIC_TRY(pic_field_boundaries(ctx, dEB, 0, 1, stream));
    PIC_TRY(f64 ? entity_gb300::srpic::AmpereWithCurrents<double>(dom, *prm, 1.0, dep, stream)
                : entity_gb300::srpic::AmpereWithCurrents<float>(dom, *prm, 1.0f, dep, stream));
    PIC_TRY(pic_field_boundaries(ctx, dEB, 1, 0, stream));
    PIC_TRY(mark(PIC_PHASE_FIELDSOLVER, 1));
  }
  PIC_TRY(mark(PIC_PHASE_SORT, 0));
  PIC_TRY(entity_gb300::srpic::SortParticles(dom, *prm, step, stream));
  PIC_TRY(mark(PIC_PHASE_SORT, 1));
  PIC_TRY(mark(PIC_PHASE_STEP, 1));
#undef PIC_TRY
  for (int k = 0; k < nspecies; ++k) dsp[k].npart = hsp[k].npart = dom.species[k].npart;

  // outputs after the step: J, EB, and the species when the sort moved them
  if (cudaEventRecord(p->step_done, s) != cudaSuccess) return PIC_ERR_CUDA;
  if (cudaStreamWaitEvent(p->down, p->step_done, 0) != cudaSuccess) return PIC_ERR_CUDA;
  if (cudaStreamWaitEvent(p->down_f, p->step_done, 0) != cudaSuccess) return PIC_ERR_CUDA;
  if (sorts) {
    // counts may have changed in the dead removal
    slots.resize(2);
    for (int k = 0; k < nspecies; ++k) species_slots(g, hsp[k], dsp[k], slots);
  }
  if (!copy_out(dep ? 0 : 1, 2, bout)) return PIC_ERR_CUDA;
  if (sorts && !copy_out(2, slots.size(), bout)) return PIC_ERR_CUDA;
  p->bytes_in  = bin;
  p->bytes_out = bout;
  return PIC_OK;
}

}  // extern "C"
