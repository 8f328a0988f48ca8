// Push/deposit instantiations: 2D, real = float.
#include "push_deposit_inst.inc"

namespace pic {
PIC_INST_PD(2, float)
}  // namespace pic
