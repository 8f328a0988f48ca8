// Push/deposit instantiations: 2D, real = double.
#include "push_deposit_inst.inc"

namespace pic {
PIC_INST_PD(2, double)
}  // namespace pic
