// pic_srpic_step: the C entry point of the host engine (srpic_engine.hpp).
#include "srpic_engine.hpp"

extern "C" int pic_srpic_step(pic_ctx* ctx, pic_species* sp, int32_t nspecies, void* EB, void* J,
                              void* buff, const pic_step_params* prm, int64_t step,
                              void* stream) {
  if (!ctx || !EB || !prm || nspecies < 0 || (nspecies > 0 && !sp)) return PIC_ERR_ARG;
  if (prm->deposit_enabled && (!J || !buff)) return PIC_ERR_ARG;
  pic_grid g;
  int      st = pic_get_grid(ctx, &g);
  if (st != PIC_OK) return st;
  entity_gb300::Domain dom;
  dom.ctx  = ctx;
  dom.EB   = EB;
  dom.J    = J;
  dom.buff = buff;
  dom.dim  = g.dim;
  dom.species.assign(sp, sp + nspecies);
  st = (g.real_bytes == 8) ? entity_gb300::srpic::StepForward<double>(dom, *prm, step, stream)
                           : entity_gb300::srpic::StepForward<float>(dom, *prm, step, stream);
  // species counts may change in the sort (dead removal)
  for (int32_t k = 0; k < nspecies; ++k) sp[k].npart = dom.species[k].npart;
  return st;
}
