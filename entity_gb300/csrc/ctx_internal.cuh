// Internal definition of the C ABI's opaque context and the helpers that
// every entry-point translation unit shares.
#pragma once

#include <utility>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/entity_pic.h"
#include "fields.cuh"
#include "pic_common.cuh"

namespace pic {
struct AdjointScratch;
void adjoint_release(AdjointScratch* a);
}  // namespace pic

// tile-major binning of one species, valid from a PIC_SORT_TILED sort until
// the species' particle count changes or it is sorted with another key
struct SpeciesBins {
  int32_t  index      = 0;
  int64_t  nalive     = 0;  // particles [0, nalive) are binned by tile
  int64_t  npart      = 0;  // npart right after the sort
  int32_t* tile_start = nullptr;
  int      ntiles     = 0;
  bool     valid      = false;
  // particles the tiled kernel leaves to the per-particle kernel
  int32_t*  ovf       = nullptr;  // capacity ovf_cap
  unsigned* ovf_count = nullptr;
  int64_t   ovf_cap   = 0;
};

struct pic_ctx {
  std::vector<SpeciesBins> bins;
  pic_grid             grid;
  unsigned long long*  d_err     = nullptr;  // 4 counters
  double*              d_energy  = nullptr;  // 2 field sums, then PIC_NMOMENTS
  // sort scratch (grown on demand)
  void*                sort_buf  = nullptr;
  size_t               sort_bytes = 0;
  // phase timers: recorded event pairs per phase, resolved on read
  bool                                            timers_on = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> intervals[PIC_NPHASES];
  cudaEvent_t                                     open_start[PIC_NPHASES] = {};
  std::vector<cudaEvent_t>                        event_pool;
  // checkpoint and snapshot storage of pic_srpic_gradient (grown on demand)
  pic::AdjointScratch*                            adjoint = nullptr;
  // indices of the GR pusher's FP64-island particles, species by species,
  // followed by their membership bitmasks (grown on demand), and two
  // counters per species: the list length and the island kernel's cursor
  int32_t*                                        gr_island     = nullptr;
  int64_t                                         gr_island_cap = 0;  // 32-bit words
  unsigned*                                       gr_island_cnt = nullptr;
  int                                             gr_island_nsp = 0;  // species of the counters
  // per species, the stream of its island kernel and the event that joins it
  // back to the caller's stream; one fork event for all
  std::vector<cudaStream_t>                       gr_side;
  std::vector<cudaEvent_t>                        gr_join;
  cudaEvent_t                                     gr_fork = nullptr;
  // SR field boundaries (pic_set_field_bcs)
  pic_field_bcs                                   fbc = {};
  // exact current accumulator of pic_push_deposit (FP32; grown on demand):
  // 3 x the ghost-inclusive cells of 64-bit totals, and the call's bound
  long long*                                      jfix       = nullptr;
  size_t                                          jfix_elems = 0;
  unsigned*                                       jfix_bound = nullptr;
  // deposit records of the tiled kernel (FP32; allocated on first use):
  // stage_slots buffers and their claim words (sizes: run_tiled)
  uint4*                                          stage_rec   = nullptr;
  unsigned*                                       stage_claim = nullptr;
  int                                             stage_slots = 0;
};

namespace pic_internal {

using pic::FieldView;
using pic::GridInfo;

inline int cuda_status(cudaError_t e) { return e == cudaSuccess ? PIC_OK : PIC_ERR_CUDA; }

inline GridInfo ginfo(const pic_ctx* c) {
  GridInfo g;
  g.dim = c->grid.dim;
  g.ng  = c->grid.ng;
  for (int d = 0; d < 3; ++d) {
    g.n[d]        = c->grid.n[d];
    g.periodic[d] = d < c->grid.dim ? c->grid.fld_periodic[d] : 0;
  }
  return g;
}

template <typename real>
inline FieldView<real> em_view(const pic_ctx* c, const void* p) {
  return FieldView<real>{ (real*)p, c->grid.em_stride[0], c->grid.em_stride[1], c->grid.em_stride[2],
                          c->grid.em_stride[3] };
}

template <typename real>
inline FieldView<real> cur_view(const pic_ctx* c, const void* p) {
  return FieldView<real>{ (real*)p, c->grid.cur_stride[0], c->grid.cur_stride[1],
                          c->grid.cur_stride[2], c->grid.cur_stride[3] };
}

inline cudaStream_t strm(void* s) { return (cudaStream_t)s; }

inline bool is_f64(const pic_ctx* c) { return c->grid.real_bytes == 8; }

inline int validate_species(const pic_ctx* c, const pic_species* sp, bool need_prev) {
  if (!sp) return PIC_ERR_ARG;
  if (sp->npart < 0) return PIC_ERR_ARG;
  if (sp->maxnpart > 0 && sp->npart > sp->maxnpart) return PIC_ERR_ARG;
  if (sp->npart >= ((int64_t)1 << 31)) return PIC_ERR_UNSUPPORTED;
  if (sp->npart == 0) return PIC_OK;
  if (!sp->i1 || !sp->i2 || !sp->dx1 || !sp->dx2 || !sp->ux1 || !sp->ux2 || !sp->ux3 ||
      !sp->weight || !sp->tag)
    return PIC_ERR_ARG;
  if (c->grid.dim == 3 && (!sp->i3 || !sp->dx3)) return PIC_ERR_ARG;
  if (need_prev) {
    if (!sp->i1_prev || !sp->i2_prev || !sp->dx1_prev || !sp->dx2_prev) return PIC_ERR_ARG;
    if (c->grid.dim == 3 && (!sp->i3_prev || !sp->dx3_prev)) return PIC_ERR_ARG;
  }
  if (sp->pusher < PIC_PUSHER_NONE || sp->pusher > PIC_PUSHER_PHOTON) return PIC_ERR_ARG;
  // payload columns: a base pointer and positive strides when present
  if (sp->npld_r < 0 || sp->npld_i < 0) return PIC_ERR_ARG;
  if (sp->npld_r > 0 && (!sp->pld_r || sp->pld_r_stride[0] < 1 || sp->pld_r_stride[1] < 1))
    return PIC_ERR_ARG;
  if (sp->npld_i > 0 && (!sp->pld_i || sp->pld_i_stride[0] < 1 || sp->pld_i_stride[1] < 1))
    return PIC_ERR_ARG;
  return PIC_OK;
}

inline pic::SpeciesPtrs sptrs(const pic_species* sp) {
  pic::SpeciesPtrs s;
  s.i1 = sp->i1;
  s.i2 = sp->i2;
  s.i3 = sp->i3;
  s.i1p = sp->i1_prev;
  s.i2p = sp->i2_prev;
  s.i3p = sp->i3_prev;
  s.dx1 = sp->dx1;
  s.dx2 = sp->dx2;
  s.dx3 = sp->dx3;
  s.dx1p = sp->dx1_prev;
  s.dx2p = sp->dx2_prev;
  s.dx3p = sp->dx3_prev;
  s.ux1 = sp->ux1;
  s.ux2 = sp->ux2;
  s.ux3 = sp->ux3;
  s.w = sp->weight;
  s.tag = sp->tag;
  s.npart = sp->npart;
  s.mass = sp->mass;
  s.charge = sp->charge;
  s.pusher = sp->pusher;
  return s;
}

}  // namespace pic_internal
