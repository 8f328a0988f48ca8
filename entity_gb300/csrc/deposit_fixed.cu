// Kernels of the exact global current accumulation (deposit_fixed.cuh).
#include <climits>

#include "deposit_fixed.cuh"
#include "pic_types.h"

namespace pic {

__global__ void k_weight_bound(const float* w, int64_t n, float q, unsigned* bound) {
  float m = 0.f;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(w[p]) * q);
  // non-negative floats order as their bit patterns
  const unsigned b = __reduce_max_sync(0xffffffffu, __float_as_uint(m));
  if ((threadIdx.x & 31) == 0) atomicMax(bound, b);
}

// one block per row (j, k, c) of the grid at a time, threads along x
__global__ void k_fixed_to_real(FixedJ fj, FieldView<float> J, int e0, int e1, int e2,
                                int overwrite) {
  const int   ex      = fj.exponent();
  const float unscale = ldexpf(1.f, ex - fj.bits);
  const int   rows    = 3 * e1 * e2;
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const int j = r % e1, k = (r / e1) % e2, c = r / (e1 * e2);
    for (int i = threadIdx.x; i < e0; i += blockDim.x) {
      const long long x = fj.p[fj.idx(i, j, k, c)];
      float*          o = J.p + J.idx(i, j, k, c);
      if (overwrite) *o = __ll2float_rn(x) * unscale;
      else if (x != 0) *o = *o + __ll2float_rn(x) * unscale;
    }
  }
}

cudaError_t launch_weight_bound(const float* w, int64_t n, float abs_charge, unsigned* bound,
                                cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > sm_count() * 16) blocks = sm_count() * 16;
  PIC_KL(k_weight_bound<<<(unsigned)blocks, 256, 0, s>>>(w, n, abs_charge, bound));
  return cudaGetLastError();
}

cudaError_t launch_fixed_to_real(const FixedJ& fj, FieldView<float> J, const int* ext,
                                 bool overwrite, cudaStream_t s) {
  const int64_t rows = (int64_t)3 * ext[1] * ext[2];
  if (rows > INT32_MAX) return cudaErrorInvalidValue;
  int64_t blocks = rows;
  if (blocks > sm_count() * 32) blocks = sm_count() * 32;
  const int threads = ext[0] >= 256 ? 256 : (ext[0] >= 128 ? 128 : 64);
  PIC_KL(k_fixed_to_real<<<(unsigned)blocks, threads, 0, s>>>(fj, J, ext[0], ext[1], ext[2],
                                                              overwrite ? 1 : 0));
  return cudaGetLastError();
}

}  // namespace pic
