// Kernels of the exact global current accumulation (deposit_fixed.cuh).
#include <climits>

#include "deposit_fixed.cuh"
#include "pic_types.h"

namespace pic {

// max |w| |q| over the weights of up to kBoundSpecies species (blockIdx.y);
// 16-byte loads where the array allows, one atomic per block
__global__ void k_weight_bound(BoundArgs a) {
  const int     s      = blockIdx.y;
  const float*  w      = a.w[s];
  const int64_t n      = a.n[s];
  const int64_t tid    = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n4     = (reinterpret_cast<uintptr_t>(w) % 16 == 0) ? n / 4 : 0;
  const float4* w4     = reinterpret_cast<const float4*>(w);
  float         m      = 0.f;
  for (int64_t i = tid; i < n4; i += stride) {
    const float4 v = w4[i];
    m = fmaxf(m, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
  }
  for (int64_t i = 4 * n4 + tid; i < n; i += stride) m = fmaxf(m, fabsf(w[i]));
  // |q| max|w| = max |q||w|: multiplication by |q| >= 0 keeps the order
  m = m * a.q[s];
  // non-negative floats order as their bit patterns
  __shared__ unsigned sm;
  if (threadIdx.x == 0) sm = 0u;
  __syncthreads();
  atomicMax(&sm, __reduce_max_sync(0xffffffffu, __float_as_uint(m)));
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(a.bound, sm);
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

cudaError_t launch_weight_bound(const BoundArgs& a, cudaStream_t s) {
  int64_t nmax = 0;
  for (int k = 0; k < a.ns; ++k) nmax = a.n[k] > nmax ? a.n[k] : nmax;
  if (a.ns <= 0 || nmax <= 0) return cudaSuccess;
  // enough 256-thread blocks for one 16-byte load per thread, at most 4 per SM
  int64_t blocks = (nmax / 4 + 255) / 256;
  if (blocks > sm_count() * 4) blocks = sm_count() * 4;
  if (blocks < 1) blocks = 1;
  PIC_KL(k_weight_bound<<<dim3((unsigned)blocks, (unsigned)a.ns), 256, 0, s>>>(a));
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
