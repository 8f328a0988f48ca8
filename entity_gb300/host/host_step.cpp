// pic_srpic_step_host: one SR step of a domain whose state lives in pinned
// host memory, as the reference's OpenMP build keeps its Views on the host.
//
// Every call copies the step's inputs in (EB and each species' i, dx, u,
// weight, tag), steps the device mirrors exactly as pic_srpic_step does, and
// copies the results out (J, EB and the species' arrays; the weights only on
// steps that sort, the one phase that changes them).
//
// The copies are pipelined against the compute and against each other:
//   - A species binned by the tiled sort is cut into up to kChunks groups of
//     tiles with about equal particle counts (at least kMinGroupBytes of
//     state each). Each group is a contiguous range
//     of the particle arrays. It is copied in, pushed with
//     pic_push_deposit_tiles as soon as it has arrived, and (on steps without
//     a sort) copied out as soon as its push ends.
//   - Every array range has its own event. Its input copy in the next call
//     waits only for its own output copy. So one step's outgoing traffic
//     overlaps the next step's incoming traffic, and the host link runs in
//     both directions at once.
//   - Fields and particles use separate streams in each direction, and the
//     fields are copied by a kernel through the mapped host pointer, so that
//     they never queue behind the particle groups on the copy engines.
// The call returns once everything is queued: the host arrays hold the result
// after pic_host_pipe_sync, and the device mirrors belong to the pipe until
// then.
#include <algorithm>
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/entity_pic.h"
#include "srpic_engine.hpp"

namespace pic {
void note_launch();  // the library's kernel launch counter
}

namespace {
constexpr int     kChunks        = 8;             // most tile groups per binned species
constexpr int64_t kMinGroupBytes = 256ll << 20;  // least state per group: fewer, larger
                                                 // copies for small species

// one species' split: tile ranges and the particle ranges they cover
struct Split {
  bool                 tiled = false;  // pushed by tile groups
  int64_t              npart = -1;     // npart the split was made for
  std::vector<int64_t> tile;           // group c: tiles [tile[c], tile[c + 1])
  std::vector<int64_t> part;           // group c: particles [part[c], part[c + 1])
};

struct Slot {
  void*  host;
  void*  dev;
  size_t bytes;
  bool   sort_only = false;  // changed only by a sort (the weights): copied
                             // out only on steps that sort
};
}  // namespace

struct pic_host_pipe {
  cudaStream_t             up = nullptr, down = nullptr;      // particles
  cudaStream_t             up_f = nullptr, down_f = nullptr;  // fields
  cudaEvent_t              entry = nullptr, eb_in = nullptr, step_done = nullptr;
  cudaEvent_t              down_all = nullptr, down_f_all = nullptr;
  std::vector<cudaEvent_t> out_done;        // per array range
  std::vector<char>        pending;         // the range has an earlier output copy
  std::vector<cudaEvent_t> ch_in, ch_done;  // per species group
  std::vector<Split>       split;           // per species
  std::vector<int64_t>     layout;          // range sizes of the previous call
  bool                     any_out = false;
  int64_t                  bytes_in = 0, bytes_out = 0;
  int                      max_groups      = kChunks;
  int64_t                  min_group_bytes = kMinGroupBytes;
};

namespace {

// elements spanned by a field of `ncomp` components with the grid's strides
size_t field_span(const pic_grid& g, const int64_t s[4], int ncomp) {
  int64_t last = (int64_t)(ncomp - 1) * s[3];
  for (int d = 0; d < 3; ++d) {
    const int64_t ext = d < g.dim ? g.n[d] + 2 * g.ng : 1;
    last += (ext - 1) * s[d];
  }
  return (size_t)(last + 1);
}

// the arrays of particles [p0, p1) of one species that carry state from one
// step to the next
void species_slots(const pic_grid& g, const pic_species& h, const pic_species& d, int64_t p0,
                   int64_t p1, std::vector<Slot>& out) {
  const size_t n = (size_t)(p1 - p0), rb = (size_t)g.real_bytes;
  void* const  hs[] = { h.i1, h.i2, h.i3, h.dx1, h.dx2, h.dx3, h.ux1, h.ux2, h.ux3, h.weight,
                        h.tag };
  void* const  ds[] = { d.i1, d.i2, d.i3, d.dx1, d.dx2, d.dx3, d.ux1, d.ux2, d.ux3, d.weight,
                        d.tag };
  const size_t es[] = { 4, 4, 4, 4, 4, 4, rb, rb, rb, rb, 2 };
  for (int a = 0; a < 11; ++a) {
    if ((a == 2 || a == 5) && g.dim != 3) continue;
    const size_t off = (size_t)p0 * es[a];
    out.push_back({ hs[a] ? (char*)hs[a] + off : nullptr, ds[a] ? (char*)ds[a] + off : nullptr,
                    n * es[a], a == 9 });
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

// tile groups of a binned species (reading its tile offsets synchronises
// the stream once), or one group over the whole species
int make_split(pic_ctx* ctx, const pic_grid& g, const pic_species& sp, int max_groups,
               int64_t min_bytes, cudaStream_t s, Split& out) {
  out        = Split();
  out.npart  = sp.npart;
  int64_t nt = 0;
  const bool pushable = (sp.pusher == PIC_PUSHER_BORIS || sp.pusher == PIC_PUSHER_VAY) &&
                        sp.mass != 0.0f && sp.npart > 0;
  if (pushable && pic_tile_offsets(ctx, &sp, nullptr, 0, &nt, s) == PIC_OK && nt > 0) {
    std::vector<int32_t> off((size_t)nt + 1);
    const int            st = pic_tile_offsets(ctx, &sp, off.data(), nt + 1, &nt, s);
    if (st != PIC_OK) return st;
    out.tiled = true;
    out.tile.push_back(0);
    out.part.push_back(0);
    const int64_t alive = off[(size_t)nt];
    const int64_t per   = (int64_t)g.dim * 8 + 4 * (int64_t)g.real_bytes + 2;  // state bytes
    const int64_t ngrp  = std::max<int64_t>(1, std::min<int64_t>(max_groups,
                                                               sp.npart * per / min_bytes));
    for (int64_t c = 1; c < ngrp; ++c) {
      // the first tile that starts at or after c / ngrp of the particles
      const int64_t target = alive * c / ngrp;
      const int64_t t = std::lower_bound(off.begin(), off.end(), (int32_t)target) - off.begin();
      if (t > out.tile.back() && t < nt) {
        out.tile.push_back(t);
        out.part.push_back(off[(size_t)t]);
      }
    }
    out.tile.push_back(nt);
    out.part.push_back(sp.npart);  // the last group also carries the dead tail
    return PIC_OK;
  }
  out.tile = { 0, 0 };
  out.part = { 0, sp.npart };
  return PIC_OK;
}

// SM-driven copy between device memory and mapped pinned host memory. The
// fields travel this way: the copy engines serve their queue in submission
// order, so the fields' copies at the end of a step would otherwise wait
// behind every particle group queued earlier in the step.
__global__ void k_copy_bytes(const unsigned char* __restrict__ src,
                             unsigned char* __restrict__ dst, size_t bytes) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t0     = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const bool   vec    = ((((uintptr_t)src) | ((uintptr_t)dst)) & 15u) == 0;
  size_t       head   = 0;
  if (vec) {
    const size_t n16 = bytes / 16;
    const uint4* s4  = (const uint4*)src;
    uint4*       d4  = (uint4*)dst;
    for (size_t i = t0; i < n16; i += stride) d4[i] = s4[i];
    head = n16 * 16;
  }
  for (size_t i = head + t0; i < bytes; i += stride) dst[i] = src[i];
}

// the device address of a pinned host buffer, or nullptr when the device
// cannot address it directly
void* mapped(void* host) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

cudaError_t copy_field(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind,
                       cudaStream_t q) {
  void* hd = mapped(kind == cudaMemcpyHostToDevice ? const_cast<void*>(src) : dst);
  if (!hd || bytes == 0) return bytes ? cudaMemcpyAsync(dst, src, bytes, kind, q) : cudaSuccess;
  const unsigned char* s = (const unsigned char*)(kind == cudaMemcpyHostToDevice ? hd : src);
  unsigned char*       d = (unsigned char*)(kind == cudaMemcpyHostToDevice ? dst : hd);
  int dev = 0, sms = 0;  // four blocks per SM stream the link at full rate
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
    return cudaMemcpyAsync(dst, src, bytes, kind, q);
  k_copy_bytes<<<sms * 4, 256, 0, q>>>(s, d, bytes);
  pic::note_launch();
  return cudaGetLastError();
}

int remake_events(std::vector<cudaEvent_t>& v, size_t n) {
  for (cudaEvent_t e : v) cudaEventDestroy(e);
  v.assign(n, nullptr);
  for (auto& e : v)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return PIC_ERR_CUDA;
  return PIC_OK;
}

// new event sets for a new range count, after every earlier copy ended
int reset_events(pic_host_pipe* p, size_t nslots, size_t ngroups) {
  for (cudaStream_t q : { p->up, p->down, p->up_f, p->down_f })
    if (cudaStreamSynchronize(q) != cudaSuccess) return PIC_ERR_CUDA;
  int st;
  if ((st = remake_events(p->out_done, nslots)) != PIC_OK) return st;
  if ((st = remake_events(p->ch_in, ngroups)) != PIC_OK) return st;
  if ((st = remake_events(p->ch_done, ngroups)) != PIC_OK) return st;
  p->pending.assign(nslots, 0);
  p->any_out = false;
  return PIC_OK;
}

}  // namespace

extern "C" {

int pic_host_pipe_create(pic_host_pipe** out) {
  if (!out) return PIC_ERR_ARG;
  *out    = nullptr;
  auto* p = new pic_host_pipe();
  bool  ok = true;
  for (cudaStream_t* q : { &p->up, &p->down, &p->up_f, &p->down_f })
    ok = ok && cudaStreamCreateWithFlags(q, cudaStreamNonBlocking) == cudaSuccess;
  for (cudaEvent_t* e : { &p->entry, &p->eb_in, &p->step_done, &p->down_all, &p->down_f_all })
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
  for (auto* v : { &p->out_done, &p->ch_in, &p->ch_done })
    for (cudaEvent_t e : *v) cudaEventDestroy(e);
  for (cudaEvent_t e : { p->entry, p->eb_in, p->step_done, p->down_all, p->down_f_all })
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

int pic_host_pipe_set_groups(pic_host_pipe* p, int32_t max_groups, int64_t min_group_bytes) {
  if (!p || max_groups < 1 || min_group_bytes < 1) return PIC_ERR_ARG;
  p->max_groups      = max_groups;
  p->min_group_bytes = min_group_bytes;
  for (Split& sp : p->split) sp.npart = -1;  // split anew at the next call
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
  cudaStream_t s   = (cudaStream_t)stream;
  const size_t rb  = (size_t)g.real_bytes;
  const bool   dep = prm->deposit_enabled != 0, fs = prm->fieldsolver_enabled != 0;
  const bool   sorts = nspecies > 0 &&
                     ((prm->clear_interval > 0 && step % prm->clear_interval == 0 && step > 0) ||
                      (prm->sort_interval > 0 && step % prm->sort_interval == 0));
#define PIC_TRY(x)            \
  do {                        \
    if ((st = (x)) != PIC_OK) \
      return st;              \
  } while (0)
#define PIC_CU(x)           \
  do {                      \
    if ((x) != cudaSuccess) \
      return PIC_ERR_CUDA;  \
  } while (0)

  // the species' groups: kept from the previous call unless npart changed
  p->split.resize((size_t)nspecies);
  for (int k = 0; k < nspecies; ++k)
    if (p->split[k].npart != dsp[k].npart || p->split[k].part.empty())
      PIC_TRY(make_split(ctx, g, dsp[k], p->max_groups, p->min_group_bytes, s, p->split[k]));

  // array ranges: 0 = J (output only), 1 = EB, then the species group by group
  std::vector<Slot>    slots;
  std::vector<size_t>  first;   // first range of each group, and the end
  std::vector<int64_t> layout;  // every range's size
  auto build = [&]() {
    slots.clear();
    first.clear();
    slots.push_back({ hJ, dJ, dep ? field_span(g, g.cur_stride, 3) * rb : 0 });
    slots.push_back({ hEB, dEB, field_span(g, g.em_stride, 6) * rb });
    for (int k = 0; k < nspecies; ++k) {
      const Split& sp = p->split[k];
      for (size_t c = 0; c + 1 < sp.part.size(); ++c) {
        first.push_back(slots.size());
        species_slots(g, hsp[k], dsp[k], sp.part[c], sp.part[c + 1], slots);
      }
    }
    first.push_back(slots.size());
    layout.clear();
    for (const Slot& x : slots) layout.push_back((int64_t)x.bytes);
  };
  build();
  const size_t ngroups = first.size() - 1;

  // a new range count needs new events; when only the range bounds moved,
  // the input copies wait for every earlier output copy instead of their own
  bool all_wait = false;
  if (p->out_done.size() != slots.size() || p->ch_in.size() != ngroups) {
    PIC_TRY(reset_events(p, slots.size(), ngroups));
  } else if (p->layout != layout) {
    all_wait = p->any_out;
  }
  bool fresh = true;
  for (char c : p->pending) fresh = fresh && !c;

  auto copy_out = [&](size_t a0, size_t a1, int64_t& bytes) {
    for (size_t a = a0; a < a1; ++a) {
      cudaStream_t q = a < 2 ? p->down_f : p->down;
      if (slots[a].sort_only && !sorts) {
        // a step without a sort leaves the range as it came in, so the host
        // copy is current; the event still marks the end of the step's use
        // of the device range for the next call's input copy
        if (cudaEventRecord(p->out_done[a], q) != cudaSuccess) return false;
        p->pending[a] = 1;
        continue;
      }
      const cudaError_t e =
        a < 2 ? copy_field(slots[a].host, slots[a].dev, slots[a].bytes, cudaMemcpyDeviceToHost, q)
        : slots[a].bytes > 0
          ? cudaMemcpyAsync(slots[a].host, slots[a].dev, slots[a].bytes, cudaMemcpyDeviceToHost, q)
          : cudaSuccess;
      if (e != cudaSuccess) return false;
      bytes += (int64_t)slots[a].bytes;
      if (cudaEventRecord(p->out_done[a], q) != cudaSuccess) return false;
      p->pending[a] = 1;
    }
    return true;
  };
  auto wait_out = [&](cudaStream_t on, size_t a) {
    return !p->pending[a] || cudaStreamWaitEvent(on, p->out_done[a], 0) == cudaSuccess;
  };

  // inputs: EB on the field stream, the groups in order on the particle
  // stream; a fresh pipe first waits for the caller's earlier work
  if (fresh) {
    PIC_CU(cudaEventRecord(p->entry, s));
    PIC_CU(cudaStreamWaitEvent(p->up, p->entry, 0));
    PIC_CU(cudaStreamWaitEvent(p->up_f, p->entry, 0));
  }
  if (all_wait) {
    for (cudaStream_t q : { p->up, p->up_f }) {
      PIC_CU(cudaStreamWaitEvent(q, p->down_all, 0));
      PIC_CU(cudaStreamWaitEvent(q, p->down_f_all, 0));
    }
  }
  int64_t bin = 0;
  for (size_t a = 1; a < slots.size(); ++a) {
    cudaStream_t q = a < 2 ? p->up_f : p->up;
    if (!wait_out(q, a)) return PIC_ERR_CUDA;
    if (a < 2)
      PIC_CU(copy_field(slots[a].dev, slots[a].host, slots[a].bytes, cudaMemcpyHostToDevice, q));
    else if (slots[a].bytes > 0)
      PIC_CU(cudaMemcpyAsync(slots[a].dev, slots[a].host, slots[a].bytes, cudaMemcpyHostToDevice,
                             q));
    bin += (int64_t)slots[a].bytes;
    if (a == 1) PIC_CU(cudaEventRecord(p->eb_in, q));
    for (size_t c = 0; c < ngroups; ++c)
      if (a + 1 == first[c + 1]) PIC_CU(cudaEventRecord(p->ch_in[c], q));
  }

  // the step (SRPICEngine::step_forward, as pic_srpic_step runs it)
  entity_gb300::Domain dom;
  dom.ctx  = ctx;
  dom.EB   = dEB;
  dom.J    = dJ;
  dom.buff = buff;
  dom.dim  = g.dim;
  dom.species.assign(dsp, dsp + nspecies);
  const bool f64   = g.real_bytes == 8;
  // a group leaves as soon as its push ends unless the sort moves it later
  const bool early = dep && !sorts;
  auto mark = [&](int phase, int end) { return pic_timer_mark(ctx, phase, end, stream); };
  PIC_CU(cudaStreamWaitEvent(s, p->eb_in, 0));
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
  // the coefficients in real_t, as srpic::PushDeposit passes them
  const double   dt     = f64 ? prm->dt : (double)(float)prm->dt;
  const double   wB     = f64 ? prm->omegaB0 : (double)(float)prm->omegaB0;
  const double   dxc    = f64 ? prm->dx : (double)(float)prm->dx;
  const uint32_t fl     = (prm->write_prev ? PIC_PD_WRITE_PREV : 0u) |
                          ((uint32_t)prm->deposit_flags & PIC_PD_FLOAT_ATOMICS);
  bool           zeroed = false;
  if (dep && nspecies == 0) {
    PIC_TRY(pic_push_deposit(ctx, nullptr, 0, dEB, dJ, dt, wB, dxc, fl, stream));
  }
  size_t grp = 0;
  for (int k = 0; k < nspecies; ++k) {
    const Split& sp = p->split[k];
    const size_t ng = sp.part.size() - 1;
    for (size_t c = 0; c < ng; ++c, ++grp) {
      PIC_CU(cudaStreamWaitEvent(s, p->ch_in[grp], 0));
      const uint32_t f = fl | (zeroed ? PIC_PD_NO_ZERO : 0u);
      if (!dep) {
        // push only: the whole species once all its groups are in
        if (c + 1 == ng) PIC_TRY(pic_push(ctx, &dom.species[k], dEB, dt, wB, dxc, stream));
      } else if (sp.tiled) {
        PIC_TRY(pic_push_deposit_tiles(ctx, &dom.species[k], dEB, dJ, dt, wB, dxc, sp.tile[c],
                                       sp.tile[c + 1], f, stream));
        zeroed = true;
      } else {
        PIC_TRY(pic_push_deposit(ctx, &dom.species[k], 1, dEB, dJ, dt, wB, dxc, f, stream));
        zeroed = true;
      }
      if (early) {
        // nothing later in the step touches these particles
        PIC_CU(cudaEventRecord(p->ch_done[grp], s));
        PIC_CU(cudaStreamWaitEvent(p->down, p->ch_done[grp], 0));
        if (!copy_out(first[grp], first[grp + 1], bout)) return PIC_ERR_CUDA;
      }
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
  for (int k = 0; k < nspecies; ++k) dsp[k].npart = hsp[k].npart = dom.species[k].npart;
  PIC_CU(cudaEventRecord(p->step_done, s));

  if (!early && nspecies > 0) {
    if (sorts) {
      // the sort moved the particles (and may have removed the dead): split
      // anew and copy out by the new ranges, which the next call reads by.
      // Every input copy of this call has ended (the sort synchronised the
      // stream after the pushes that waited for them).
      for (int k = 0; k < nspecies; ++k)
        PIC_TRY(make_split(ctx, g, dsp[k], p->max_groups, p->min_group_bytes, s, p->split[k]));
      build();
      if (p->out_done.size() != slots.size() || p->ch_in.size() != first.size() - 1)
        PIC_TRY(reset_events(p, slots.size(), first.size() - 1));
    }
    PIC_CU(cudaStreamWaitEvent(p->down, p->step_done, 0));
    if (!copy_out(2, slots.size(), bout)) return PIC_ERR_CUDA;
  }
  PIC_CU(cudaStreamWaitEvent(p->down_f, p->step_done, 0));
  if (!copy_out(dep ? 0 : 1, 2, bout)) return PIC_ERR_CUDA;
  PIC_CU(cudaEventRecord(p->down_all, p->down));
  PIC_CU(cudaEventRecord(p->down_f_all, p->down_f));
  p->layout    = layout;
  p->any_out   = true;
  p->bytes_in  = bin;
  p->bytes_out = bout;
#undef PIC_TRY
#undef PIC_CU
  return PIC_OK;
}

}  // extern "C"
