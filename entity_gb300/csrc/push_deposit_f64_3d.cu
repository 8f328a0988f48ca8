// Push/deposit instantiations: 3D, real = double.
#include "push_deposit_inst.inc"

namespace pic {
PIC_INST_PD(3, double)
}  // namespace pic
