// Exact, order-independent accumulation of the deposited current in global
// memory (FP32 grids).
//
// Every contribution of one pic_push_deposit call is an integer multiple of
// one unit, 2^(ex - bits), where 2^ex bounds |q w| max(1/dt, 1) over all of
// the call's particles (the largest current a particle can deposit into one
// entry: the charge crossing a face within a step, or q w |v| for the
// out-of-plane 2D component). The tiled kernel's exact per-tile integer sums
// are scaled to this unit by a left shift, the per-particle kernel rounds each
// contribution to a multiple of 2^(ex - min(30, bits)) (a 32-bit conversion;
// a 64-bit one runs on the FP64 pipe) and shifts it likewise, and everything
// is added as 64-bit integers, so
// the total of every entry is the same whatever the order of the additions.
// A last pass converts each total to real_t once. With N particles in the
// call, bits = min(34, 62 - ceil(log2(N + 1))) keeps every total below 2^62.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "pic_common.cuh"

namespace pic {

struct FixedJ {
  long long*      p = nullptr;       // 3 components over the ghost-inclusive grid, x fastest
  int64_t         s1 = 0, s2 = 0, s3 = 0;
  const unsigned* bound = nullptr;   // bit pattern of max |q w| over the call's particles
  float           dt_factor = 1.f;   // max(1/dt, 1)
  int             bits = 0;

  __device__ __forceinline__ int64_t idx(int i, int j, int k, int c) const {
    return (int64_t)i + (int64_t)j * s1 + (int64_t)k * s2 + (int64_t)c * s3;
  }
  // ex with bound max(1/dt, 1) < 2^ex, held where 2^(bits - ex) is a normal float
  __device__ __forceinline__ int exponent() const {
    int ex = 0;
    frexpf(__uint_as_float(*bound) * dt_factor * 1.0000002f, &ex);
    return max(ex, bits - 126);
  }
  __device__ __forceinline__ void add_units(int i, int j, int k, int c, long long x) const {
    atomicAdd(reinterpret_cast<unsigned long long*>(p + idx(i, j, k, c)), (unsigned long long)x);
  }
};

// bound = max(bound, max |w| |q|) over the weights of up to kBoundSpecies
// species in one launch
constexpr int kBoundSpecies = 8;
struct BoundArgs {
  const float* w[kBoundSpecies];
  int64_t      n[kBoundSpecies];
  float        q[kBoundSpecies];  // |charge|
  int          ns = 0;
  unsigned*    bound = nullptr;
};
cudaError_t launch_weight_bound(const BoundArgs& a, cudaStream_t s);

// J (+)= the totals in real_t: every element written when overwrite, else
// the non-zero totals added; ext = the ghost-inclusive extents
cudaError_t launch_fixed_to_real(const FixedJ& fj, FieldView<float> J, const int* ext,
                                 bool overwrite, cudaStream_t s);

}  // namespace pic
