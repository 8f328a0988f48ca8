// C ABI of the particle-in-cell hot path: argument validation, dispatch to
// the templated kernels by (dimension, shape order, precision), the device
// error word, and the context's persistent scratch.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <type_traits>
#include <utility>
#include <vector>
#include <cstring>
#include <cuda_runtime.h>

#include "../../include/entity_pic.h"
#include "ctx_internal.cuh"
#include "deposit_fixed.cuh"
#include "fields.cuh"
#include "moments.cuh"
#include "push_deposit_tiled.cuh"
#include "sort.cuh"

namespace pic {
namespace {
template <int D, typename real, int O>
void shape_of(int out[3]) {
  out[0] = TileShape<D, real, O>::X;
  out[1] = TileShape<D, real, O>::Y;
  out[2] = D == 3 ? TileShape<D, real, O>::Z : 1;
}
template <int D, typename real>
void shape_by_order(int order, int out[3]) {
  switch (order) {
    case 0: shape_of<D, real, 0>(out); break;
    case 1: shape_of<D, real, 1>(out); break;
    case 2: shape_of<D, real, 2>(out); break;
    default: shape_of<D, real, 3>(out); break;
  }
}
}  // namespace
void tile_shape(int dim, int real_bytes, int order, int out[3]) {
  if (dim == 3 && real_bytes == 4) shape_by_order<3, float>(order, out);
  else if (dim == 3)               shape_by_order<3, double>(order, out);
  else if (real_bytes == 4)        shape_by_order<2, float>(order, out);
  else                             shape_by_order<2, double>(order, out);
}
}  // namespace pic


using namespace pic_internal;

namespace {

using pic::FieldView;
using pic::GridInfo;


int min_ghosts(int order) { return order == 0 ? 1 : (order + 1) / 2 + 1; }

int validate_grid(const pic_grid* g) {
  if (!g) return PIC_ERR_ARG;
  if (g->dim != 2 && g->dim != 3) return PIC_ERR_UNSUPPORTED;
  if (g->order < 0 || g->order > 3) return PIC_ERR_UNSUPPORTED;
  if (g->real_bytes != 4 && g->real_bytes != 8) return PIC_ERR_UNSUPPORTED;
  if (g->ng < min_ghosts(g->order)) return PIC_ERR_ARG;
  for (int d = 0; d < g->dim; ++d) {
    if (g->n[d] < 2 * g->ng) return PIC_ERR_ARG;
    for (int s = 0; s < 2; ++s)
      if (g->prtl_bc[d][s] < PIC_BC_PERIODIC || g->prtl_bc[d][s] > PIC_BC_AXIS) return PIC_ERR_ARG;
  }
  if (g->dim == 2 && g->n[2] != 1) return PIC_ERR_ARG;
  for (int k = 0; k < 4; ++k) {
    if (g->em_stride[k] <= 0 || g->cur_stride[k] <= 0) return PIC_ERR_ARG;
  }
  // cell and key indices are 32-bit
  const int64_t cells = (int64_t)g->n[0] * g->n[1] * (g->dim == 3 ? g->n[2] : 1);
  if (cells >= (int64_t)1 << 30) return PIC_ERR_UNSUPPORTED;
  return PIC_OK;
}






template <typename real>
cudaError_t pd_dispatch(const pic_ctx* c, const pic::PDArgs<real>& a, int mode, bool photon,
                        cudaStream_t s) {
  const int D = c->grid.dim, O = c->grid.order;
#define PIC_PD_CASE(DD, OO) \
  if (D == DD && O == OO) return pic::launch_push_deposit<DD, OO, real>(a, mode, photon, s);
  PIC_PD_CASE(2, 0)
  PIC_PD_CASE(2, 1)
  PIC_PD_CASE(2, 2)
  PIC_PD_CASE(2, 3)
  PIC_PD_CASE(3, 0)
  PIC_PD_CASE(3, 1)
  PIC_PD_CASE(3, 2)
  PIC_PD_CASE(3, 3)
#undef PIC_PD_CASE
  return cudaErrorInvalidValue;
}

template <typename real>
int run_pd(pic_ctx* c, const pic_species* sp, const void* EB, void* J, double dt, double omegaB0,
           double dx, int mode, bool write_prev, cudaStream_t s,
           const pic::FixedJ* fj = nullptr) {
  pic::PDArgs<real> a;
  if (fj) a.fj = *fj;
  a.sp = sptrs(sp);
  for (int d = 0; d < 3; ++d) {
    a.pc.n[d]     = c->grid.n[d];
    a.pc.bc[d][0] = c->grid.prtl_bc[d][0];
    a.pc.bc[d][1] = c->grid.prtl_bc[d][1];
  }
  a.pc.ng = c->grid.ng;
  for (int d = 0; d < 3; ++d)
    a.pc.ext[d] = d < c->grid.dim ? c->grid.n[d] + 2 * c->grid.ng : 1;
  a.EB    = em_view<real>(c, EB);
  a.J     = cur_view<real>(c, J);
  a.dt    = (real)dt;
  a.dx    = (real)dx;
  // normalized_dt_half = HALF * (charge / mass) * omegaB0 * dt with the float
  // charge/mass of the species (src/kernels/pushers/sr.hpp:111)
  const bool  photon = sp->pusher == PIC_PUSHER_PHOTON;
  const float qm     = photon ? 0.0f : sp->charge / sp->mass;
  a.ndth             = (real)0.5 * (real)qm * (real)omegaB0 * (real)dt;
  a.inv_dt           = (real)1 / (real)dt;
  a.charge           = (real)sp->charge;
  a.vay              = sp->pusher == PIC_PUSHER_VAY;
  a.write_prev       = write_prev ? 1 : 0;
  a.err              = c->d_err;
  return cuda_status(pd_dispatch<real>(c, a, mode, photon, s));
}

SpeciesBins* find_bins(pic_ctx* c, int index, bool create) {
  for (auto& b : c->bins)
    if (b.index == index) return &b;
  if (!create) return nullptr;
  c->bins.emplace_back();
  c->bins.back().index = index;
  return &c->bins.back();
}

void ntiles_of(const pic_ctx* c, int nt[3], int ts[3]) {
  pic::tile_shape(c->grid.dim, c->grid.real_bytes, c->grid.order, ts);
  for (int d = 0; d < 3; ++d) {
    const int n = d < c->grid.dim ? c->grid.n[d] : 1;
    nt[d]       = (n + ts[d] - 1) / ts[d];
  }
}

// a copy of `sp` whose arrays start at particle `first`
pic_species species_tail(const pic_species& sp, int64_t first, int real_bytes) {
  pic_species t = sp;
  auto adv      = [&](auto*& p, size_t esz) {
    using P = std::remove_reference_t<decltype(p)>;
    if (p) p = (P)((char*)p + esz * first);
  };
  adv(t.i1, 4);
  adv(t.i2, 4);
  adv(t.i3, 4);
  adv(t.i1_prev, 4);
  adv(t.i2_prev, 4);
  adv(t.i3_prev, 4);
  adv(t.dx1, 4);
  adv(t.dx2, 4);
  adv(t.dx3, 4);
  adv(t.dx1_prev, 4);
  adv(t.dx2_prev, 4);
  adv(t.dx3_prev, 4);
  adv(t.ux1, real_bytes);
  adv(t.ux2, real_bytes);
  adv(t.ux3, real_bytes);
  adv(t.weight, real_bytes);
  adv(t.tag, 2);
  t.npart    = sp.npart - first;
  t.maxnpart = 0;
  return t;
}

template <typename real>
int run_tiled(pic_ctx* c, const std::vector<const pic_species*>& sps, const void* EB, void* J,
              double dt, double omegaB0, double dx, bool write_prev, cudaStream_t s,
              int64_t tile0 = 0, int64_t tile1 = -1, const pic::FixedJ* fj = nullptr) {
  pic::TiledArgs<real> a;
  if (fj) a.fj = *fj;
  a.nsp = (int)sps.size();
  for (int k = 0; k < a.nsp; ++k) {
    const pic_species* sp = sps[k];
    a.s[k].sp             = sptrs(sp);
    a.s[k].tile_start     = find_bins(c, sp->index, false)->tile_start;
    const float qm        = sp->charge / sp->mass;
    a.s[k].ndth           = (real)0.5 * (real)qm * (real)omegaB0 * (real)dt;
    a.s[k].charge         = (real)sp->charge;
    a.s[k].vay            = sp->pusher == PIC_PUSHER_VAY;
    SpeciesBins* b        = find_bins(c, sp->index, false);
    a.s[k].ovf            = b->ovf;
    a.s[k].ovf_count      = b->ovf_count;
    if (cudaMemsetAsync(b->ovf_count, 0, sizeof(unsigned), s) != cudaSuccess) return PIC_ERR_CUDA;
  }
  int ts[3];
  ntiles_of(c, a.ntiles, ts);
  const int64_t nt_all = (int64_t)a.ntiles[0] * a.ntiles[1] * a.ntiles[2];
  a.tile0 = (int)tile0;
  a.tile1 = (int)(tile1 < 0 ? nt_all : tile1);
  for (int d = 0; d < 3; ++d) {
    a.pc.n[d]     = c->grid.n[d];
    a.pc.bc[d][0] = c->grid.prtl_bc[d][0];
    a.pc.bc[d][1] = c->grid.prtl_bc[d][1];
    a.pc.ext[d]   = d < c->grid.dim ? c->grid.n[d] + 2 * c->grid.ng : 1;
    a.periodic[d] = d < c->grid.dim ? c->grid.fld_periodic[d] : 0;
  }
  a.pc.ng      = c->grid.ng;
  a.EB         = em_view<real>(c, EB);
  a.J          = cur_view<real>(c, J);
  a.dt         = (real)dt;
  a.dx         = (real)dx;
  a.inv_dt     = (real)1 / (real)dt;
  a.write_prev = write_prev ? 1 : 0;
  a.err        = c->d_err;
  const int D = c->grid.dim, O = c->grid.order;
  {
    // lanes of a warp over about four cells: the stride from the species'
    // mean particles per cell
    int64_t np = 0, cells = 1;
    for (int k = 0; k < a.nsp; ++k) np += sps[k]->npart;
    for (int d = 0; d < D; ++d) cells *= c->grid.n[d];
    const int64_t ppc = np / std::max<int64_t>(1, (int64_t)a.nsp * cells);
    a.lane_stride     = ppc >= 24 ? 4 : (ppc >= 12 ? 2 : 1);
  }
  if (sizeof(real) == 4 && O >= 1 && (D == 3 || O <= 2)) {
    // 3D: two buffers per SM (one CTA per SM); 2D: eight smaller ones (up to
    // five CTAs per SM). The launcher checks them against the kernel's
    // occupancy and deposits directly when they do not suffice.
    const int cap = D == 2 ? pic::kStageCap / 4 : (O == 3 ? 2 * pic::kStageCap : pic::kStageCap);
    if (!c->stage_rec) {
      const int n = (D == 2 ? 8 : 2) * pic::sm_count();
      if (cudaMalloc((void**)&c->stage_rec, sizeof(uint4) * 2 * (size_t)cap * n) !=
              cudaSuccess ||
          cudaMalloc((void**)&c->stage_claim, sizeof(unsigned) * (size_t)n) != cudaSuccess ||
          cudaMemsetAsync(c->stage_claim, 0, sizeof(unsigned) * (size_t)n, s) != cudaSuccess) {
        cudaGetLastError();
        if (c->stage_rec) cudaFree(c->stage_rec);
        if (c->stage_claim) cudaFree(c->stage_claim);
        c->stage_rec   = nullptr;
        c->stage_claim = nullptr;
      } else {
        c->stage_slots = n;
      }
    }
    if (c->stage_rec) {
      a.st.rec    = c->stage_rec;
      a.st.claim  = c->stage_claim;
      a.st.nslots = c->stage_slots;
      a.st.cap    = cap;
    }
  }
  cudaError_t e = cudaErrorInvalidValue;
#define PIC_TD(DD, OO) \
  if (D == DD && O == OO) e = pic::launch_push_deposit_tiled<DD, OO, real>(a, s);
  PIC_TD(2, 0)
  PIC_TD(2, 1)
  PIC_TD(2, 2)
  PIC_TD(2, 3)
  PIC_TD(3, 0)
  PIC_TD(3, 1)
  PIC_TD(3, 2)
  PIC_TD(3, 3)
#undef PIC_TD
  if (e != cudaSuccess) return PIC_ERR_CUDA;
  // the particles the tiled kernel deferred: per-particle kernel over the list
  for (int k = 0; k < a.nsp; ++k) {
    const pic_species* sp = sps[k];
    pic::PDArgs<real>  pa;
    pa.sp = sptrs(sp);
    pa.pc = a.pc;
    pa.EB = a.EB;
    pa.J  = a.J;
    pa.dt = a.dt;
    pa.dx = a.dx;
    pa.ndth       = a.s[k].ndth;
    pa.inv_dt     = a.inv_dt;
    pa.charge     = a.s[k].charge;
    pa.vay        = a.s[k].vay;
    pa.write_prev = a.write_prev;
    pa.err        = a.err;
    pa.list       = a.s[k].ovf;
    pa.list_count = a.s[k].ovf_count;
    pa.fj         = a.fj;
    e = pd_dispatch<real>(c, pa, pic::MODE_FUSED, false, s);
    if (e != cudaSuccess) return PIC_ERR_CUDA;
  }
  return PIC_OK;
}

template <typename real>
int zero_J(pic_ctx* c, void* J, cudaStream_t s) {
  return cuda_status(pic::launch_zero3<real>(ginfo(c), cur_view<real>(c, J), s));
}


}  // namespace

namespace pic {
static std::atomic<long long> g_launches{ 0 };
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int sm_count() {
  constexpr int           kMaxDevices = 64;
  static std::atomic<int> cache[kMaxDevices];  // 0 = not yet queried
  int                     dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (dev >= 0 && dev < kMaxDevices) {
    const int v = cache[dev].load(std::memory_order_relaxed);
    if (v > 0) return v;
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
    sms = 1;
  if (dev >= 0 && dev < kMaxDevices) cache[dev].store(sms, std::memory_order_relaxed);
  return sms;
}
}  // namespace pic

namespace {

// srpic::CurrentsFilter (currents.h:89-119) with conductor walls: each pass
// copies J to buff, filters with the wall stencils, refills the periodic
// ghosts (CommunicateFields)
template <typename real>
int filter_cond(pic_ctx* c, void* J, void* buff, int npasses, cudaStream_t s) {
  const auto g = ginfo(c);
  int        lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = d < g.dim && c->fbc.kind[d][0] == PIC_FBC_CONDUCTOR;
    hi[d] = d < g.dim && c->fbc.kind[d][1] == PIC_FBC_CONDUCTOR;
  }
  const auto Jv = cur_view<real>(c, J), Bv = cur_view<real>(c, buff);
  for (int p = 0; p < npasses; ++p) {
    cudaError_t e = pic::launch_copy3<real>(g, Jv, Bv, s);
    if (e == cudaSuccess) e = pic::launch_filter_cond<real>(g, lo, hi, Jv, Bv, s);
    if (e == cudaSuccess) e = pic::launch_fill_ghosts<real>(g, Jv, 0, 3, s);
    if (e != cudaSuccess) return PIC_ERR_CUDA;
  }
  return PIC_OK;
}

bool has_conductor(const pic_ctx* c) {
  for (int d = 0; d < c->grid.dim; ++d)
    if (c->fbc.kind[d][0] == PIC_FBC_CONDUCTOR || c->fbc.kind[d][1] == PIC_FBC_CONDUCTOR)
      return true;
  return false;
}

}  // namespace

extern "C" {

int64_t pic_kernel_launches(void) { return (int64_t)pic::g_launches.load(std::memory_order_relaxed); }

int pic_version(int32_t* abi_version, int32_t* built_sm) {
  if (abi_version) *abi_version = PIC_ABI_VERSION;
  if (built_sm) *built_sm = 103;
  return PIC_OK;
}

const char* pic_status_string(int status) {
  switch (status) {
    case PIC_OK: return "ok";
    case PIC_ERR_ARG: return "invalid argument";
    case PIC_ERR_CUDA: return "CUDA runtime error";
    case PIC_ERR_UNSUPPORTED: return "unsupported configuration";
    case PIC_ERR_NOMEM: return "device allocation failed";
    case PIC_ERR_DEVICE: return "device-side check failed";
    default: return "unknown status";
  }
}

int pic_create(const pic_grid* grid, pic_ctx** out) {
  if (!out) return PIC_ERR_ARG;
  *out    = nullptr;
  int st  = validate_grid(grid);
  if (st != PIC_OK) return st;
  pic_ctx* c = new pic_ctx();
  c->grid    = *grid;
  for (int d = 0; d < 3; ++d)
    for (int h = 0; h < 2; ++h)
      c->fbc.kind[d][h] = (d >= grid->dim || grid->fld_periodic[d]) ? PIC_FBC_PERIODIC : PIC_FBC_NONE;
  if (cudaMalloc((void**)&c->d_err, sizeof(unsigned long long) * pic::ERR_COUNT) != cudaSuccess ||
      cudaMalloc((void**)&c->d_energy, sizeof(double) * (2 + PIC_NMOMENTS)) != cudaSuccess) {
    if (c->d_err) cudaFree(c->d_err);
    delete c;
    return PIC_ERR_NOMEM;
  }
  if (cudaMemset(c->d_err, 0, sizeof(unsigned long long) * pic::ERR_COUNT) != cudaSuccess) {
    cudaFree(c->d_err);
    cudaFree(c->d_energy);
    delete c;
    return PIC_ERR_CUDA;
  }
  *out = c;
  return PIC_OK;
}

int pic_timers_reset(pic_ctx* c) {
  if (!c) return PIC_ERR_ARG;
  for (int p = 0; p < PIC_NPHASES; ++p) {
    for (auto& iv : c->intervals[p]) {
      c->event_pool.push_back(iv.first);
      c->event_pool.push_back(iv.second);
    }
    c->intervals[p].clear();
    if (c->open_start[p]) c->event_pool.push_back(c->open_start[p]);
    c->open_start[p] = nullptr;
  }
  return PIC_OK;
}

int pic_destroy(pic_ctx* c) {
  if (!c) return PIC_ERR_ARG;
  cudaDeviceSynchronize();
  pic_timers_reset(c);
  for (auto e : c->event_pool) cudaEventDestroy(e);
  for (auto& b : c->bins) {
    cudaFree(b.tile_start);
    cudaFree(b.ovf);
    cudaFree(b.ovf_count);
  }
  cudaFree(c->d_err);
  cudaFree(c->d_energy);
  if (c->sort_buf) cudaFree(c->sort_buf);
  cudaFree(c->gr_island);
  cudaFree(c->gr_island_cnt);
  if (c->jfix) cudaFree(c->jfix);
  if (c->jfix_bound) cudaFree(c->jfix_bound);
  if (c->stage_rec) cudaFree(c->stage_rec);
  if (c->stage_claim) cudaFree(c->stage_claim);
  if (c->gr_fork) cudaEventDestroy(c->gr_fork);
  for (auto e : c->gr_join) cudaEventDestroy(e);
  for (auto q : c->gr_side) cudaStreamDestroy(q);
  pic::adjoint_release(c->adjoint);
  delete c;
  return PIC_OK;
}

int pic_timers_enable(pic_ctx* c, int32_t on) {
  if (!c) return PIC_ERR_ARG;
  c->timers_on = on != 0;
  return PIC_OK;
}

int pic_timer_mark(pic_ctx* c, int32_t phase, int32_t is_end, void* stream) {
  if (!c || phase < 0 || phase >= PIC_NPHASES) return PIC_ERR_ARG;
  if (!c->timers_on) return PIC_OK;
  cudaEvent_t ev;
  if (!c->event_pool.empty()) {
    ev = c->event_pool.back();
    c->event_pool.pop_back();
  } else if (cudaEventCreate(&ev) != cudaSuccess) {
    return PIC_ERR_CUDA;
  }
  if (cudaEventRecord(ev, strm(stream)) != cudaSuccess) return PIC_ERR_CUDA;
  if (!is_end) {
    if (c->open_start[phase]) c->event_pool.push_back(c->open_start[phase]);
    c->open_start[phase] = ev;
  } else {
    if (!c->open_start[phase]) {
      c->event_pool.push_back(ev);
      return PIC_ERR_ARG;
    }
    c->intervals[phase].emplace_back(c->open_start[phase], ev);
    c->open_start[phase] = nullptr;
  }
  return PIC_OK;
}

int pic_timers_read(pic_ctx* c, double ms[PIC_NPHASES], int64_t count[PIC_NPHASES]) {
  if (!c || !ms || !count) return PIC_ERR_ARG;
  for (int p = 0; p < PIC_NPHASES; ++p) {
    double tot = 0.0;
    for (auto& iv : c->intervals[p]) {
      if (cudaEventSynchronize(iv.second) != cudaSuccess) return PIC_ERR_CUDA;
      float t = 0.f;
      if (cudaEventElapsedTime(&t, iv.first, iv.second) != cudaSuccess) return PIC_ERR_CUDA;
      tot += t;
    }
    ms[p]    = tot;
    count[p] = (int64_t)c->intervals[p].size();
  }
  return PIC_OK;
}

int pic_get_grid(const pic_ctx* c, pic_grid* out) {
  if (!c || !out) return PIC_ERR_ARG;
  *out = c->grid;
  return PIC_OK;
}

int pic_tile_shape(const pic_ctx* c, int32_t out[3]) {
  if (!c || !out) return PIC_ERR_ARG;
  int ts[3];
  pic::tile_shape(c->grid.dim, c->grid.real_bytes, c->grid.order, ts);
  for (int d = 0; d < 3; ++d) out[d] = ts[d];
  return PIC_OK;
}

int pic_faraday(pic_ctx* c, void* EB, double coeff1, double coeff2, const double* st, void* stream) {
  if (!c || !EB) return PIC_ERR_ARG;
  bool yee = true;
  if (st) {
    for (int k = 0; k < 9; ++k) yee = yee && st[k] == 0.0;
  }
  // the extended stencil reads two cells beyond the active range
  if (!yee && c->grid.ng < 2) return PIC_ERR_ARG;
  if (is_f64(c)) {
    pic::Stencil<double> s{};
    if (st) s = { st[0], st[1], st[2], st[3], st[4], st[5], st[6], st[7], st[8] };
    return cuda_status(pic::launch_faraday<double>(ginfo(c), em_view<double>(c, EB), coeff1, coeff2, s,
                                                   yee, strm(stream)));
  }
  pic::Stencil<float> s{};
  if (st)
    s = { (float)st[0], (float)st[1], (float)st[2], (float)st[3], (float)st[4],
          (float)st[5], (float)st[6], (float)st[7], (float)st[8] };
  return cuda_status(pic::launch_faraday<float>(ginfo(c), em_view<float>(c, EB), (float)coeff1,
                                                (float)coeff2, s, yee, strm(stream)));
}

int pic_ampere(pic_ctx* c, void* EB, double coeff1, double coeff2, void* stream) {
  if (!c || !EB) return PIC_ERR_ARG;
  if (is_f64(c))
    return cuda_status(pic::launch_ampere<double>(ginfo(c), em_view<double>(c, EB), cur_view<double>(c, nullptr),
                                                  coeff1, coeff2, 0.0, 1.0, true, false, false,
                                                  strm(stream)));
  return cuda_status(pic::launch_ampere<float>(ginfo(c), em_view<float>(c, EB), cur_view<float>(c, nullptr),
                                               (float)coeff1, (float)coeff2, 0.f, 1.f, true, false,
                                               false, strm(stream)));
}

int pic_currents_ampere(pic_ctx* c, void* EB, void* J, double coeff, double ppc0, void* stream) {
  if (!c || !EB || !J) return PIC_ERR_ARG;
  if (ppc0 == 0.0) return PIC_ERR_ARG;
  if (is_f64(c))
    return cuda_status(pic::launch_ampere<double>(ginfo(c), em_view<double>(c, EB), cur_view<double>(c, J), 0.0,
                                                  0.0, coeff, ppc0, false, true, true, strm(stream)));
  return cuda_status(pic::launch_ampere<float>(ginfo(c), em_view<float>(c, EB), cur_view<float>(c, J), 0.f, 0.f,
                                               (float)coeff, (float)ppc0, false, true, true,
                                               strm(stream)));
}

int pic_ampere_currents(pic_ctx* c, void* EB, void* J, double coeff1, double coeff2, double jcoeff,
                        double ppc0, void* stream) {
  if (!c || !EB) return PIC_ERR_ARG;
  if (J && ppc0 == 0.0) return PIC_ERR_ARG;
  const bool cur = J != nullptr;
  if (is_f64(c))
    return cuda_status(pic::launch_ampere<double>(ginfo(c), em_view<double>(c, EB), cur_view<double>(c, J),
                                                  coeff1, coeff2, jcoeff, ppc0, true, cur, true,
                                                  strm(stream)));
  return cuda_status(pic::launch_ampere<float>(ginfo(c), em_view<float>(c, EB), cur_view<float>(c, J),
                                               (float)coeff1, (float)coeff2, (float)jcoeff,
                                               (float)ppc0, true, cur, true, strm(stream)));
}

int pic_push(pic_ctx* c, const pic_species* sp, const void* EB, double dt, double omegaB0,
             double dx, void* stream) {
  if (!c || !EB) return PIC_ERR_ARG;
  int st = validate_species(c, sp, true);
  if (st != PIC_OK) return st;
  if (sp->npart == 0 || sp->pusher == PIC_PUSHER_NONE) return PIC_OK;
  if (sp->pusher != PIC_PUSHER_PHOTON && sp->mass == 0.0f) return PIC_ERR_ARG;
  if (is_f64(c))
    return run_pd<double>(c, sp, EB, nullptr, dt, omegaB0, dx, pic::MODE_PUSH, true, strm(stream));
  return run_pd<float>(c, sp, EB, nullptr, dt, omegaB0, dx, pic::MODE_PUSH, true, strm(stream));
}

int pic_deposit(pic_ctx* c, const pic_species* sp, int32_t nspecies, void* J, double dt, double dx,
                void* stream) {
  if (!c || !J || nspecies < 0 || (nspecies > 0 && !sp)) return PIC_ERR_ARG;
  for (int k = 0; k < nspecies; ++k) {
    int st = validate_species(c, sp + k, true);
    if (st != PIC_OK) return st;
  }
  int st = is_f64(c) ? zero_J<double>(c, J, strm(stream)) : zero_J<float>(c, J, strm(stream));
  if (st != PIC_OK) return st;
  for (int k = 0; k < nspecies; ++k) {
    const pic_species* s = sp + k;
    // currents.h:75-78: skip pusher NONE, empty species, zero charge
    if (s->pusher == PIC_PUSHER_NONE || s->npart == 0 || s->charge == 0.0f) continue;
    st = is_f64(c) ? run_pd<double>(c, s, nullptr, J, dt, 0.0, dx, pic::MODE_DEPOSIT, false, strm(stream))
                   : run_pd<float>(c, s, nullptr, J, dt, 0.0, dx, pic::MODE_DEPOSIT, false, strm(stream));
    if (st != PIC_OK) return st;
  }
  return PIC_OK;
}

// Arms the exact current accumulator for one FP32 pic_push_deposit call over
// the species that deposit: clears the totals and the bound, then bounds
// |q w| over their particles. Returns false when the accumulator cannot be
// allocated (the call then deposits with float atomics).
bool arm_fixed_J(pic_ctx* c, const pic_species* sp, int32_t nspecies, double dt, cudaStream_t s,
                 pic::FixedJ* fj) {
  const int    dim = c->grid.dim, ng = c->grid.ng;
  const int    e0 = c->grid.n[0] + 2 * ng, e1 = dim >= 2 ? c->grid.n[1] + 2 * ng : 1;
  const int    e2 = dim >= 3 ? c->grid.n[2] + 2 * ng : 1;
  const size_t elems = (size_t)3 * e0 * e1 * e2;
  if (c->jfix_elems < elems) {
    if (c->jfix) cudaFree(c->jfix);
    c->jfix       = nullptr;
    c->jfix_elems = 0;
    if (cudaMalloc((void**)&c->jfix, sizeof(long long) * elems) != cudaSuccess) {
      cudaGetLastError();
      c->jfix = nullptr;
      return false;
    }
    c->jfix_elems = elems;
  }
  if (!c->jfix_bound && cudaMalloc((void**)&c->jfix_bound, sizeof(unsigned)) != cudaSuccess) {
    cudaGetLastError();
    c->jfix_bound = nullptr;
    return false;
  }
  if (cudaMemsetAsync(c->jfix, 0, sizeof(long long) * elems, s) != cudaSuccess ||
      cudaMemsetAsync(c->jfix_bound, 0, sizeof(unsigned), s) != cudaSuccess)
    return false;
  int64_t         ntot = 0;
  pic::BoundArgs  ba;
  ba.bound = c->jfix_bound;
  for (int k = 0; k < nspecies; ++k) {
    const pic_species* q = sp + k;
    if (q->pusher == PIC_PUSHER_NONE || q->npart == 0 || q->charge == 0.0f) continue;
    ntot += q->npart;
    ba.w[ba.ns] = (const float*)q->weight;
    ba.n[ba.ns] = q->npart;
    ba.q[ba.ns] = std::fabs(q->charge);
    if (++ba.ns == pic::kBoundSpecies) {
      if (pic::launch_weight_bound(ba, s) != cudaSuccess) return false;
      ba.ns = 0;
    }
  }
  if (ba.ns > 0 && pic::launch_weight_bound(ba, s) != cudaSuccess) return false;
  int lg = 0;
  while (lg < 62 && (int64_t(1) << lg) < ntot + 1) ++lg;
  fj->p         = c->jfix;
  fj->s1        = e0;
  fj->s2        = (int64_t)e0 * e1;
  fj->s3        = (int64_t)e0 * e1 * e2;
  fj->bound     = c->jfix_bound;
  fj->dt_factor = std::fmax(1.f / (float)dt, 1.f);  // the kernels' inv_dt
  fj->bits      = std::min(34, 62 - lg);
  return fj->bits >= 8;
}

int pic_push_deposit(pic_ctx* c, const pic_species* sp, int32_t nspecies, const void* EB, void* J,
                     double dt, double omegaB0, double dx, uint32_t flags, void* stream) {
  if (!c || !EB || !J || nspecies < 0 || (nspecies > 0 && !sp)) return PIC_ERR_ARG;
  const bool write_prev = (flags & PIC_PD_WRITE_PREV) != 0;
  for (int k = 0; k < nspecies; ++k) {
    int st = validate_species(c, sp + k, write_prev);
    if (st != PIC_OK) return st;
    if (sp[k].pusher != PIC_PUSHER_NONE && sp[k].pusher != PIC_PUSHER_PHOTON && sp[k].mass == 0.0f)
      return PIC_ERR_ARG;
  }
  int st = PIC_OK;
  // FP32: deposit into the exact accumulator, then J (+)= its totals once
  pic::FixedJ fj;
  const bool  exact = !is_f64(c) && !(flags & PIC_PD_FLOAT_ATOMICS) &&
                     arm_fixed_J(c, sp, nspecies, dt, strm(stream), &fj);
  if (!(flags & PIC_PD_NO_ZERO) && !exact) {
    st = is_f64(c) ? zero_J<double>(c, J, strm(stream)) : zero_J<float>(c, J, strm(stream));
    if (st != PIC_OK) return st;
  }
  const pic::FixedJ* fjp = exact ? &fj : nullptr;
  // species with a valid tile binning (PIC_SORT_TILED) go through the tiled
  // kernel together; the rest, and any particles beyond a binned prefix,
  // through the per-particle kernel
  std::vector<const pic_species*> tiled;
  std::vector<pic_species>        rest;
  for (int k = 0; k < nspecies; ++k) {
    const pic_species* s = sp + k;
    if (s->pusher == PIC_PUSHER_NONE || s->npart == 0) continue;
    const SpeciesBins* b = find_bins(c, s->index, false);
    const bool eligible  = b && b->valid && b->npart == s->npart &&
                          (s->pusher == PIC_PUSHER_BORIS || s->pusher == PIC_PUSHER_VAY) &&
                          (int)tiled.size() < pic::kMaxTiledSpecies;
    if (eligible) {
      tiled.push_back(s);
      if (b->nalive < s->npart) rest.push_back(species_tail(*s, b->nalive, c->grid.real_bytes));
    } else {
      rest.push_back(*s);
    }
  }
  if (!tiled.empty()) {
    st = is_f64(c) ? run_tiled<double>(c, tiled, EB, J, dt, omegaB0, dx, write_prev, strm(stream))
                   : run_tiled<float>(c, tiled, EB, J, dt, omegaB0, dx, write_prev, strm(stream),
                                      0, -1, fjp);
    if (st != PIC_OK) return st;
  }
  for (const pic_species& rs : rest) {
    const pic_species* s = &rs;
    // a species that moves but carries no charge is pushed only
    const int mode = (s->charge == 0.0f) ? pic::MODE_PUSH : pic::MODE_FUSED;
    if (mode == pic::MODE_PUSH && !write_prev) {
      // push-only kernels always store prev; without prev arrays use the
      // fused kernel with zero charge semantics instead
      st = is_f64(c) ? run_pd<double>(c, s, EB, J, dt, omegaB0, dx, pic::MODE_FUSED, false, strm(stream))
                     : run_pd<float>(c, s, EB, J, dt, omegaB0, dx, pic::MODE_FUSED, false, strm(stream), fjp);
    } else {
      st = is_f64(c) ? run_pd<double>(c, s, EB, J, dt, omegaB0, dx, mode, write_prev, strm(stream))
                     : run_pd<float>(c, s, EB, J, dt, omegaB0, dx, mode, write_prev, strm(stream), fjp);
    }
    if (st != PIC_OK) return st;
  }
  if (exact) {
    const int ext[3] = { c->grid.n[0] + 2 * c->grid.ng,
                         c->grid.dim >= 2 ? c->grid.n[1] + 2 * c->grid.ng : 1,
                         c->grid.dim >= 3 ? c->grid.n[2] + 2 * c->grid.ng : 1 };
    st = cuda_status(pic::launch_fixed_to_real(fj, cur_view<float>(c, J), ext,
                                               !(flags & PIC_PD_NO_ZERO), strm(stream)));
  }
  return st;
}

int pic_tile_offsets(pic_ctx* c, const pic_species* sp, int32_t* out, int64_t cap,
                     int64_t* ntiles, void* stream) {
  if (!c || !sp || !ntiles) return PIC_ERR_ARG;
  int nt[3], ts[3];
  ntiles_of(c, nt, ts);
  *ntiles                = (int64_t)nt[0] * nt[1] * nt[2];
  const SpeciesBins* b   = find_bins(c, sp->index, false);
  if (!b || !b->valid || b->npart != sp->npart || !b->tile_start) return PIC_ERR_UNSUPPORTED;
  if (!out) return PIC_OK;
  if (cap < *ntiles + 1) return PIC_ERR_ARG;
  cudaStream_t s = strm(stream);
  if (cudaMemcpyAsync(out, b->tile_start, sizeof(int32_t) * (size_t)(*ntiles + 1),
                      cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return PIC_ERR_CUDA;
  return cuda_status(cudaStreamSynchronize(s));
}

int pic_push_deposit_tiles(pic_ctx* c, const pic_species* sp, const void* EB, void* J, double dt,
                           double omegaB0, double dx, int64_t tile_lo, int64_t tile_hi,
                           uint32_t flags, void* stream) {
  if (!c || !sp || !EB || !J) return PIC_ERR_ARG;
  const bool write_prev = (flags & PIC_PD_WRITE_PREV) != 0;
  int        st         = validate_species(c, sp, write_prev);
  if (st != PIC_OK) return st;
  if (sp->pusher != PIC_PUSHER_BORIS && sp->pusher != PIC_PUSHER_VAY) return PIC_ERR_UNSUPPORTED;
  if (sp->mass == 0.0f) return PIC_ERR_ARG;
  int nt[3], ts[3];
  ntiles_of(c, nt, ts);
  const int64_t      nt_all = (int64_t)nt[0] * nt[1] * nt[2];
  const SpeciesBins* b      = find_bins(c, sp->index, false);
  if (!b || !b->valid || b->npart != sp->npart) return PIC_ERR_UNSUPPORTED;
  if (tile_lo < 0 || tile_hi > nt_all || tile_lo > tile_hi) return PIC_ERR_ARG;
  if (!(flags & PIC_PD_NO_ZERO)) {
    st = is_f64(c) ? zero_J<double>(c, J, strm(stream)) : zero_J<float>(c, J, strm(stream));
    if (st != PIC_OK) return st;
  }
  if (tile_lo == tile_hi || sp->npart == 0) return PIC_OK;
  const std::vector<const pic_species*> one{ sp };
  return is_f64(c) ? run_tiled<double>(c, one, EB, J, dt, omegaB0, dx, write_prev, strm(stream),
                                       tile_lo, tile_hi)
                   : run_tiled<float>(c, one, EB, J, dt, omegaB0, dx, write_prev, strm(stream),
                                      tile_lo, tile_hi);
}

int pic_sync_currents(pic_ctx* c, void* J, void* buff, void* stream) {
  (void)buff;
  if (!c || !J) return PIC_ERR_ARG;
  if (is_f64(c)) return cuda_status(pic::launch_sync_currents<double>(ginfo(c), cur_view<double>(c, J), strm(stream)));
  return cuda_status(pic::launch_sync_currents<float>(ginfo(c), cur_view<float>(c, J), strm(stream)));
}

int pic_filter_currents(pic_ctx* c, void* J, void* buff, int32_t npasses, void* stream) {
  if (!c || !J || npasses < 0) return PIC_ERR_ARG;
  if (npasses == 0) return PIC_OK;
  if (!buff) return PIC_ERR_ARG;
  if (has_conductor(c))
    return is_f64(c) ? filter_cond<double>(c, J, buff, npasses, strm(stream))
                     : filter_cond<float>(c, J, buff, npasses, strm(stream));
  if (is_f64(c))
    return cuda_status(pic::launch_filter<double>(ginfo(c), cur_view<double>(c, J), cur_view<double>(c, buff),
                                                  npasses, strm(stream)));
  return cuda_status(pic::launch_filter<float>(ginfo(c), cur_view<float>(c, J), cur_view<float>(c, buff),
                                               npasses, strm(stream)));
}

int pic_fill_ghosts(pic_ctx* c, void* field, int32_t is_em, int32_t c0, int32_t c1, void* stream) {
  if (!c || !field) return PIC_ERR_ARG;
  const int ncomp = is_em ? 6 : 3;
  if (c0 < 0 || c1 > ncomp || c0 >= c1) return PIC_ERR_ARG;
  if (is_f64(c)) {
    auto v = is_em ? em_view<double>(c, field) : cur_view<double>(c, field);
    return cuda_status(pic::launch_fill_ghosts<double>(ginfo(c), v, c0, c1, strm(stream)));
  }
  auto v = is_em ? em_view<float>(c, field) : cur_view<float>(c, field);
  return cuda_status(pic::launch_fill_ghosts<float>(ginfo(c), v, c0, c1, strm(stream)));
}

int pic_field_energy(pic_ctx* c, const void* EB, double dx, double* out, void* stream) {
  if (!c || !EB || !out) return PIC_ERR_ARG;
  cudaStream_t s = strm(stream);
  if (cudaMemsetAsync(c->d_energy, 0, sizeof(double) * 2, s) != cudaSuccess) return PIC_ERR_CUDA;
  cudaError_t e = is_f64(c) ? pic::launch_energy<double>(ginfo(c), em_view<double>(c, EB), dx, c->d_energy, s)
                            : pic::launch_energy<float>(ginfo(c), em_view<float>(c, EB), dx, c->d_energy, s);
  if (e != cudaSuccess) return PIC_ERR_CUDA;
  if (cudaMemcpyAsync(out, c->d_energy, sizeof(double) * 2, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return PIC_ERR_CUDA;
  return cuda_status(cudaStreamSynchronize(s));
}

int pic_particle_moments(pic_ctx* c, const pic_species* sp, int32_t nspecies,
                         double out[PIC_NMOMENTS], void* stream) {
  if (!c || !out || nspecies < 0 || (nspecies > 0 && !sp)) return PIC_ERR_ARG;
  for (int k = 0; k < nspecies; ++k) {
    int st = validate_species(c, sp + k, false);
    if (st != PIC_OK) return st;
  }
  cudaStream_t s = strm(stream);
  double*      d = c->d_energy + 2;
  if (cudaMemsetAsync(d, 0, sizeof(double) * PIC_NMOMENTS, s) != cudaSuccess) return PIC_ERR_CUDA;
  for (int k = 0; k < nspecies; ++k) {
    const pic::SpeciesPtrs p = sptrs(sp + k);
    cudaError_t e = is_f64(c) ? pic::launch_particle_moments<double>(p, d, s)
                              : pic::launch_particle_moments<float>(p, d, s);
    if (e != cudaSuccess) return PIC_ERR_CUDA;
  }
  if (cudaMemcpyAsync(out, d, sizeof(double) * PIC_NMOMENTS, cudaMemcpyDeviceToHost, s) !=
      cudaSuccess)
    return PIC_ERR_CUDA;
  return cuda_status(cudaStreamSynchronize(s));
}

int pic_charge_density(pic_ctx* c, const pic_species* sp, int32_t nspecies, void* rho,
                       void* stream) {
  if (!c || !rho || nspecies < 0 || (nspecies > 0 && !sp)) return PIC_ERR_ARG;
  for (int k = 0; k < nspecies; ++k) {
    int st = validate_species(c, sp + k, false);
    if (st != PIC_OK) return st;
  }
  pic::PushConsts pc{};
  for (int d = 0; d < 3; ++d) {
    pc.n[d]   = c->grid.n[d];
    pc.ext[d] = d < c->grid.dim ? c->grid.n[d] + 2 * c->grid.ng : 1;
  }
  pc.ng          = c->grid.ng;
  cudaStream_t s = strm(stream);
  for (int k = 0; k < nspecies; ++k) {
    if (sp[k].pusher == PIC_PUSHER_PHOTON || sp[k].charge == 0.0f) continue;
    const pic::SpeciesPtrs p = sptrs(sp + k);
    cudaError_t e =
      is_f64(c) ? pic::launch_charge_density<double>(c->grid.dim, c->grid.order, p,
                                                     cur_view<double>(c, rho), c->grid.ng, pc,
                                                     c->d_err, s)
                : pic::launch_charge_density<float>(c->grid.dim, c->grid.order, p,
                                                    cur_view<float>(c, rho), c->grid.ng, pc,
                                                    c->d_err, s);
    if (e != cudaSuccess) return PIC_ERR_CUDA;
  }
  return PIC_OK;
}

int pic_get_device_errors(pic_ctx* c, int64_t out[4], int32_t reset, void* stream) {
  if (!c || !out) return PIC_ERR_ARG;
  cudaStream_t       s = strm(stream);
  unsigned long long h[4];
  if (cudaMemcpyAsync(h, c->d_err, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return PIC_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return PIC_ERR_CUDA;
  for (int k = 0; k < 4; ++k) out[k] = (int64_t)h[k];
  if (reset) {
    if (cudaMemsetAsync(c->d_err, 0, sizeof(h), s) != cudaSuccess) return PIC_ERR_CUDA;
  }
  return PIC_OK;
}

int pic_get_wait_timeouts(pic_ctx* c, int64_t* out, int32_t reset, void* stream) {
  if (!c || !out) return PIC_ERR_ARG;
  cudaStream_t       s = strm(stream);
  unsigned long long h = 0;
  unsigned long long* d = c->d_err + pic::ERR_WAIT_TIMEOUT;
  if (cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return PIC_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return PIC_ERR_CUDA;
  *out = (int64_t)h;
  if (reset && cudaMemsetAsync(d, 0, sizeof(h), s) != cudaSuccess) return PIC_ERR_CUDA;
  return PIC_OK;
}

int pic_sort(pic_ctx* c, pic_species* sp, uint32_t flags, int64_t* npart_out, void* stream) {
  if (!c) return PIC_ERR_ARG;
  const bool skip_prev = (flags & PIC_SORT_SKIP_PREV) != 0;
  int        st        = validate_species(c, sp, !skip_prev);
  if (st != PIC_OK) return st;
  const bool remove_dead = (flags & PIC_SORT_REMOVE_DEAD) != 0;
  const bool spatial     = (flags & PIC_SORT_SPATIAL) != 0;
  const bool no_sync     = (flags & PIC_SORT_NO_SYNC) != 0;
  if (no_sync && remove_dead) return PIC_ERR_ARG;
  cudaStream_t  s        = strm(stream);
  const int64_t np       = sp->npart;
  if (npart_out) *npart_out = np;
  if (np == 0 || (!remove_dead && !spatial)) return PIC_OK;

  const pic_grid& g     = c->grid;
  const bool      tiled = spatial && (flags & PIC_SORT_TILED) != 0;
  int             nt[3] = { 1, 1, 1 }, ts[3] = { 1, 1, 1 };
  if (tiled) ntiles_of(c, nt, ts);
  const int64_t   ntiles = (int64_t)nt[0] * nt[1] * nt[2];
  const int64_t   tcells = (int64_t)ts[0] * ts[1] * ts[2];
  const int64_t   cells  = !spatial ? 1
                           : tiled  ? ntiles * tcells
                                    : (int64_t)g.n[0] * g.n[1] * (g.dim == 3 ? g.n[2] : 1);
  const int64_t   nbins  = cells + 1;  // + dead bin
  if (cells >= ((int64_t)1 << 31) - 2) return PIC_ERR_UNSUPPORTED;
  // any sort moves particles: the previous tile binning no longer holds
  if (SpeciesBins* b = find_bins(c, sp->index, false)) b->valid = false;
  // scratch layout (8-byte aligned pieces)
  auto          al   = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t  b_key = al(4 * np), b_rank = al(4 * np), b_dead = al(np), b_drank = al(4 * np);
  const size_t  b_cnt = al(4 * (nbins + 1)), b_off = al(8 * (nbins + 1)), b_perm = al(4 * np);
  const size_t  b_ptmp = al(4 * np), b_big = al(4 * nbins), b_nbig = al(4);
  const size_t  rb     = (size_t)g.real_bytes;
  // the arrays a sort moves (Particles::SortSpatially and RemoveDead,
  // particles_sort.cpp:103-253): the state, then phi and every payload
  // column; in batches of up to kMaxSortArrays
  struct Moved {
    void*   arr;
    int     esz;
    int64_t stride;
  };
  std::vector<Moved> mv;
  auto add = [&](void* arr, int esz, int64_t stride = 1) {
    if (arr) mv.push_back({ arr, esz, stride });
  };
  add(sp->i1, 4), add(sp->i2, 4), add(sp->dx1, 4), add(sp->dx2, 4);
  if (g.dim == 3) add(sp->i3, 4), add(sp->dx3, 4);
  if (!skip_prev) {
    add(sp->i1_prev, 4), add(sp->i2_prev, 4), add(sp->dx1_prev, 4), add(sp->dx2_prev, 4);
    if (g.dim == 3) add(sp->i3_prev, 4), add(sp->dx3_prev, 4);
  }
  add(sp->ux1, (int)rb), add(sp->ux2, (int)rb), add(sp->ux3, (int)rb), add(sp->weight, (int)rb);
  add(sp->tag, 2);
  add(sp->phi, (int)rb);
  for (int k = 0; k < sp->npld_r; ++k)
    add((char*)sp->pld_r + (size_t)k * sp->pld_r_stride[1] * rb, (int)rb, sp->pld_r_stride[0]);
  // integer payloads are npart_t, 32-bit (global.h:385)
  for (int k = 0; k < sp->npld_i; ++k)
    add((char*)sp->pld_i + (size_t)k * sp->pld_i_stride[1] * 4, 4, sp->pld_i_stride[0]);
  // every array of a batch gets its own staging area when the context can
  // hold them (one gather, one copy back per batch); otherwise they go in
  // turn through one
  size_t b_all = 0;
  for (size_t k = 0; k < mv.size() && k < (size_t)pic::kMaxSortArrays; ++k)
    b_all += al((size_t)np * mv[k].esz);
  const size_t b_big_elem = al(np * 8);
  const size_t b_one = b_big_elem;
  const size_t  fixed_need = b_key + b_rank + b_dead + b_drank + b_cnt + b_off + b_perm + b_ptmp +
                            b_big + b_nbig;
  bool          apart      = true;
  if (fixed_need + b_all > c->sort_bytes) {
    if (c->sort_buf) cudaFree(c->sort_buf);
    c->sort_buf   = nullptr;
    c->sort_bytes = 0;
    if (cudaMalloc(&c->sort_buf, fixed_need + b_all) == cudaSuccess) {
      c->sort_bytes = fixed_need + b_all;
    } else {
      cudaGetLastError();  // the failed allocation leaves no sticky error
      apart = false;
      if (fixed_need + b_one > c->sort_bytes) {
        if (cudaMalloc(&c->sort_buf, fixed_need + b_one) != cudaSuccess) return PIC_ERR_NOMEM;
        c->sort_bytes = fixed_need + b_one;
      }
    }
  }
  char*         base = (char*)c->sort_buf;
  pic::SortArgs a;
  a.i1 = sp->i1;
  a.i2 = sp->i2;
  a.i3 = sp->i3;
  a.tag = sp->tag;
  a.npart = np;
  a.dim = g.dim;
  a.n[0] = g.n[0];
  a.n[1] = g.n[1];
  a.n[2] = g.n[2];
  a.spatial = spatial ? 1 : 0;
  a.tiled   = tiled ? 1 : 0;
  for (int d = 0; d < 3; ++d) {
    a.tile[d]   = ts[d];
    a.ntiles[d] = nt[d];
  }
  a.dead_bin = (int32_t)cells;
  a.key = (int32_t*)base;
  base += b_key;
  a.rank = (int32_t*)base;
  base += b_rank;
  a.is_dead = (uint8_t*)base;
  base += b_dead;
  a.dead_rank = (int32_t*)base;
  base += b_drank;
  a.count = (int32_t*)base;
  base += b_cnt;
  a.off = (int64_t*)base;
  base += b_off;
  a.perm = (int32_t*)base;
  base += b_perm;
  a.perm_tmp = (int32_t*)base;
  base += b_ptmp;
  a.big = (int32_t*)base;
  base += b_big;
  a.nbig = (int32_t*)base;
  base += b_nbig;
  a.err = c->d_err;

  cudaError_t e = pic::sort_build_perm(a, s);
  if (e != cudaSuccess) return PIC_ERR_CUDA;
  for (size_t k0 = 0; k0 < mv.size(); k0 += pic::kMaxSortArrays) {
    pic::GatherSet gs;
    char*          t = base;
    for (size_t k = k0; k < mv.size() && gs.n < pic::kMaxSortArrays; ++k) {
      gs.arr[gs.n]    = mv[k].arr;
      gs.esz[gs.n]    = mv[k].esz;
      gs.stride[gs.n] = mv[k].stride;
      gs.tmp[gs.n]    = t;
      if (apart) t += al((size_t)np * mv[k].esz);
      ++gs.n;
    }
    if ((e = pic::sort_apply_all(gs, a.perm, np, s)) != cudaSuccess) return PIC_ERR_CUDA;
  }
  if (remove_dead) {
    // particles_sort.cpp:175-191: alive tags on the front, dead on the tail
    if ((e = pic::set_tags_after_removal(sp->tag, np, a.count + a.dead_bin, s)) != cudaSuccess)
      return PIC_ERR_CUDA;
  }
  if (tiled) {
    SpeciesBins* b = find_bins(c, sp->index, true);
    if (b->ntiles != (int)ntiles || !b->tile_start) {
      if (b->tile_start) cudaFree(b->tile_start);
      b->tile_start = nullptr;
      if (cudaMalloc((void**)&b->tile_start, sizeof(int32_t) * (ntiles + 1)) != cudaSuccess)
        return PIC_ERR_NOMEM;
      b->ntiles = (int)ntiles;
    }
    if ((e = pic::tile_offsets(a.off, tcells, (int)ntiles, b->tile_start, s)) != cudaSuccess)
      return PIC_ERR_CUDA;
    const int64_t cap = np;  // every binned particle may end up deferred
    if (b->ovf_cap < cap || !b->ovf_count) {
      cudaFree(b->ovf);
      b->ovf = nullptr;
      b->ovf_cap = 0;
      if (!b->ovf_count && cudaMalloc((void**)&b->ovf_count, sizeof(unsigned)) != cudaSuccess)
        return PIC_ERR_NOMEM;
      if (cudaMalloc((void**)&b->ovf, sizeof(int32_t) * (cap > 0 ? cap : 1)) != cudaSuccess)
        return PIC_ERR_NOMEM;
      b->ovf_cap = cap;
    }
  }
  if (no_sync) {
    // npart is unchanged; the dead sit after tile_start[ntiles] and are never
    // pushed, so the binned range may cover the whole species
    if (tiled) {
      SpeciesBins* b = find_bins(c, sp->index, true);
      b->nalive = np;
      b->npart  = np;
      b->valid  = true;
    }
    if (npart_out) *npart_out = np;
    return PIC_OK;
  }
  // the one synchronisation of a sort: the dead count and the error word
  int32_t            n_dead = 0;
  unsigned long long h_err[4];
  if (cudaMemcpyAsync(&n_dead, a.count + a.dead_bin, sizeof(int32_t), cudaMemcpyDeviceToHost, s) !=
        cudaSuccess ||
      cudaMemcpyAsync(h_err, c->d_err, sizeof(h_err), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return PIC_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return PIC_ERR_CUDA;
  const int64_t newn = remove_dead ? np - n_dead : np;
  if (tiled) {
    SpeciesBins* b = find_bins(c, sp->index, true);
    b->nalive = np - n_dead;
    b->npart  = newn;
    b->valid  = true;
  }
  if (npart_out) *npart_out = newn;
  if (remove_dead) sp->npart = newn;
  return h_err[pic::ERR_OUT_OF_GRID] ? PIC_ERR_DEVICE : PIC_OK;
}

}  // extern "C"
