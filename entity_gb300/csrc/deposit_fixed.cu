// Kernels of the exact global current accumulation (deposit_fixed.cuh).
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

__global__ void k_fixed_to_real(FixedJ fj, FieldView<float> J, int e0, int e1, int e2,
                                int overwrite) {
  const int     ex      = fj.exponent();
  const float   unscale = ldexpf(1.f, ex - fj.bits);
  const int64_t total   = (int64_t)3 * e0 * e1 * e2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int       i = (int)(t % e0);
    const int64_t   r = t / e0;
    const int       j = (int)(r % e1);
    const int64_t   r2 = r / e1;
    const int       k = (int)(r2 % e2);
    const int       c = (int)(r2 / e2);
    const long long x = fj.p[fj.idx(i, j, k, c)];
    float*          o = J.p + J.idx(i, j, k, c);
    if (overwrite) *o = __ll2float_rn(x) * unscale;
    else if (x != 0) *o = *o + __ll2float_rn(x) * unscale;
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
  const int64_t total  = (int64_t)3 * ext[0] * ext[1] * ext[2];
  int64_t       blocks = (total + 255) / 256;
  if (blocks > sm_count() * 16) blocks = sm_count() * 16;
  PIC_KL(k_fixed_to_real<<<(unsigned)blocks, 256, 0, s>>>(fj, J, ext[0], ext[1], ext[2],
                                                          overwrite ? 1 : 0));
  return cudaGetLastError();
}

}  // namespace pic
