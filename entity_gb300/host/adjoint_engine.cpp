// Checkpointed reverse-mode driver over the C ABI: the gradient of the final
// E-field energy with respect to the initial particle and field state.
//
// Forward: steps 0..N-1 through pic_srpic_step (the product step, sort and
// dead removal off so that particle indices stay fixed), with the full state
// saved every K steps. Backward: for each K-step segment, newest first, the
// segment is recomputed from its checkpoint with every step's starting state
// kept, then walked backwards with pic_srpic_step_adjoint. The last segment
// keeps its steps' states during the forward and is not recomputed. Particle state is
// therefore stored for N/K checkpoints plus K snapshots, never per step of
// the whole run.
#include <algorithm>
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/entity_pic.h"

namespace {

int zero_adjoint(const pic_grid& g, const pic_species* sp, pic_species_adjoint* adj, int nsp,
                 cudaStream_t s) {
  for (int k = 0; k < nsp; ++k) {
    const size_t n = (size_t)std::max<int64_t>(sp[k].npart, 0) * (size_t)g.real_bytes;
    if (n == 0) continue;
    void* arrs[7] = { adj[k].lx1, adj[k].lx2, g.dim == 3 ? adj[k].lx3 : nullptr,
                      adj[k].lu1, adj[k].lu2, adj[k].lu3, adj[k].lw };
    for (void* p : arrs) {
      if (p && cudaMemsetAsync(p, 0, n, s) != cudaSuccess) return PIC_ERR_CUDA;
    }
  }
  return PIC_OK;
}

}  // namespace

extern "C" int pic_srpic_gradient(pic_ctx* ctx, pic_species* sp, pic_species_adjoint* adj,
                                  int32_t nsp, void* EB, void* J, void* buff,
                                  const pic_step_params* prm, int64_t nsteps,
                                  int64_t every, void* lamEB, double* loss, void* stream) {
  if (!ctx || !EB || !J || !buff || !prm || !lamEB || !loss || nsteps < 1 || every < 1 ||
      nsp < 0 || (nsp > 0 && (!sp || !adj)))
    return PIC_ERR_ARG;
  pic_grid g;
  int      st = pic_get_grid(ctx, &g);
  if (st != PIC_OK) return st;
  // the scope of pic_srpic_step_adjoint, checked before any forward work
  if (g.dim != 2 || g.order < 1 || g.order > 3 || !prm->fieldsolver_enabled)
    return PIC_ERR_UNSUPPORTED;
  for (int d = 0; d < 2; ++d) {
    if (!g.fld_periodic[d] || g.prtl_bc[d][0] != PIC_BC_PERIODIC ||
        g.prtl_bc[d][1] != PIC_BC_PERIODIC)
      return PIC_ERR_UNSUPPORTED;
  }
  for (int k = 0; k < nsp; ++k) {
    if (sp[k].pusher != PIC_PUSHER_NONE && sp[k].pusher != PIC_PUSHER_BORIS)
      return PIC_ERR_UNSUPPORTED;
  }
  cudaStream_t    s = (cudaStream_t)stream;
  pic_step_params p = *prm;
  p.sort_interval   = 0;
  p.clear_interval  = 0;
  p.write_prev      = 0;
  const int64_t nseg = (nsteps + every - 1) / every;
  if (nseg + every > (int64_t)1 << 30) return PIC_ERR_UNSUPPORTED;
#define PIC_TRY(x)            \
  do {                        \
    if ((st = (x)) != PIC_OK) \
      return st;              \
  } while (0)
  // forward with checkpoints; the steps of the last segment keep their
  // starting states as they go, so that segment needs no recompute
  const int64_t last0 = (nseg - 1) * every;
  for (int64_t n = 0; n < nsteps; ++n) {
    if (n % every == 0) PIC_TRY(pic_checkpoint_save(ctx, (int32_t)(n / every), sp, nsp, EB, stream));
    PIC_TRY(pic_srpic_step(ctx, sp, nsp, EB, J, buff, &p, n, stream));
    if (n >= last0 && n + 1 < nsteps)
      PIC_TRY(pic_checkpoint_save(ctx, (int32_t)(nseg + (n + 1 - last0)), sp, nsp, EB, stream));
  }
  double en[2];
  PIC_TRY(pic_field_energy(ctx, EB, p.dx, en, stream));
  *loss = en[0];
  PIC_TRY(pic_field_energy_adjoint_seed(ctx, EB, lamEB, p.dx, stream));
  PIC_TRY(zero_adjoint(g, sp, adj, nsp, s));
  // backward, one segment at a time
  std::vector<pic_species> view(nsp > 0 ? nsp : 1);
  for (int64_t seg = nseg - 1; seg >= 0; --seg) {
    const int64_t n0 = seg * every, n1 = std::min(nsteps, n0 + every);
    if (seg < nseg - 1) {
      PIC_TRY(pic_checkpoint_restore(ctx, (int32_t)seg, sp, nsp, EB, stream));
      for (int64_t n = n0; n + 1 < n1; ++n) {
        PIC_TRY(pic_srpic_step(ctx, sp, nsp, EB, J, buff, &p, n, stream));
        PIC_TRY(pic_checkpoint_save(ctx, (int32_t)(nseg + (n + 1 - n0)), sp, nsp, EB, stream));
      }
    }
    for (int64_t n = n1 - 1; n >= n0; --n) {
      // the step's starting state is read in place from its slot
      const int32_t slot = n == n0 ? (int32_t)seg : (int32_t)(nseg + (n - n0));
      void*         EBn  = nullptr;
      PIC_TRY(pic_checkpoint_view(ctx, slot, sp, nsp, view.data(), &EBn));
      PIC_TRY(pic_srpic_step_adjoint(ctx, view.data(), adj, nsp, EBn, lamEB, &p, stream));
    }
  }
  PIC_TRY(pic_checkpoint_restore(ctx, 0, sp, nsp, EB, stream));
#undef PIC_TRY
  return cudaStreamSynchronize(s) == cudaSuccess ? PIC_OK : PIC_ERR_CUDA;
}
