// Internal types shared by the host dispatch layer and the kernels.
#pragma once

#include <cstdint>

#include "../../include/entity_pic.h"

namespace pic {

// constants of one push/deposit launch
struct PushConsts {
  int n[3];
  int bc[3][2];
  int ng;
  int ext[3];  // ghost-inclusive extents (1 along an unsimulated axis)
};

// raw species pointers for a kernel (real arrays typed by the kernel)
struct SpeciesPtrs {
  int32_t *i1, *i2, *i3;
  int32_t *i1p, *i2p, *i3p;
  float   *dx1, *dx2, *dx3;
  float   *dx1p, *dx2p, *dx3p;
  void    *ux1, *ux2, *ux3, *w;
  int16_t *tag;
  int64_t  npart;
  float    mass, charge;
  int      pusher;
};

struct Strides {
  int64_t s[4];
};

// device error counters (index meaning documented in entity_pic.h)
enum ErrIdx {
  ERR_BAD_TAG      = 0,
  ERR_OUT_OF_GRID  = 1,
  ERR_STENCIL_OUT  = 2,
  ERR_SAMPLER      = 3,
  ERR_WAIT_TIMEOUT = 4,  // bounded waits (TMA completion barriers) that ran out
  ERR_COUNT        = 5
};

// process-wide count of kernels this library has launched
void note_launch();

// streaming multiprocessors of the current device (queried once per device;
// 1 when the query fails); grid caps are multiples of it
int sm_count();

}  // namespace pic

// launches a kernel and counts it: PIC_KL(k<<<grid, block, smem, stream>>>(args))
#define PIC_KL(...)          \
  do {                       \
    __VA_ARGS__;             \
    ::pic::note_launch();    \
  } while (0)
