// Push/deposit instantiations: 3D, real = float.
#include "push_deposit_inst.inc"

namespace pic {
PIC_INST_PD(3, float)
}  // namespace pic
