// pic_field_energy_noalloc: the FP64 field-energy reduction of
// pic_field_energy for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: a host framework that reserves all
// device memory for its own pool at start-up and forbids allocations behind
// it, a diagnostics hook that runs between steps where cudaMalloc could
// synchronise the device and stall the simulation's stream, or a process held
// to a fixed device-memory budget. pic_field_energy needs a context, and
// pic_create allocates; this entry point needs neither. Its only scratch is
// the file-scope array below: one pair of partial sums per grid row (i2, i3),
// at most kMaxRows rows (1 MiB of device memory that every GPU loading the
// library keeps until the process exits). Grids with more rows are rejected.
//
// Every call shares that array and overwrites the slots it uses, so nothing
// needs clearing, but two calls whose kernels overlap on the GPU (on
// different streams, or on the same device from different host threads
// without ordering) race on it; serialise them.
//
// The per-row sums and their final combination run in a fixed order, so the
// result is bitwise reproducible (the context version adds block sums with
// atomics, in no fixed order).
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/entity_pic.h"
#include "pic_types.h"

namespace pic {
namespace {

constexpr int kMaxRows = 1 << 16;  // 65536 rows: 256 x 256 in 3D, any 2D grid up to that

// [0, kMaxRows): E^2 row sums, [kMaxRows, 2 kMaxRows): B^2 row sums,
// [2 kMaxRows, 2 kMaxRows + 2): the totals
static __device__ __align__(256) double g_energy_scratch[2 * kMaxRows + 2];

constexpr int kMaxDevices = 64;
std::mutex    g_setup_mutex;
double*       g_scratch_ptr[kMaxDevices] = {};

// one warp per row: fixed lane mapping and shuffle tree, so the row sum is
// the same on every call
template <typename real>
__global__ void k_energy_rows(const real* EB, int64_t s0, int64_t s1, int64_t s2, int64_t s3, int n1,
                              int n2, int rows, int ng, int dim, double dx, double* scratch) {
  const int warps = (blockDim.x >> 5);
  const int row   = blockIdx.x * warps + (threadIdx.x >> 5);
  const int lane  = threadIdx.x & 31;
  if (row >= rows) return;
  const int    j  = row % n2 + ng;
  const int    k  = dim == 3 ? row / n2 + ng : 0;
  const double dV = dim == 3 ? dx * dx * dx : dx * dx;
  double       e2 = 0.0, b2 = 0.0;
  for (int i = ng + lane; i < n1 + ng; i += 32) {
    const int64_t base = (int64_t)i * s0 + (int64_t)j * s1 + (int64_t)k * s2;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double h  = (c < dim) ? dx * dx : 1.0;
      const double ev = (double)EB[base + (int64_t)c * s3];
      const double bv = (double)EB[base + (int64_t)(c + 3) * s3];
      e2 += ev * ev * h * dV;
      b2 += bv * bv * h * dV;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    e2 += __shfl_down_sync(0xffffffffu, e2, o);
    b2 += __shfl_down_sync(0xffffffffu, b2, o);
  }
  if (lane == 0) {
    scratch[row]            = e2;
    scratch[kMaxRows + row] = b2;
  }
}

// one block combines the row sums in a fixed order
__global__ void k_energy_total(int rows, double* scratch) {
  __shared__ double sh[2][32];
  double            e2 = 0.0, b2 = 0.0;
  for (int r = threadIdx.x; r < rows; r += blockDim.x) {
    e2 += scratch[r];
    b2 += scratch[kMaxRows + r];
  }
  for (int o = 16; o > 0; o >>= 1) {
    e2 += __shfl_down_sync(0xffffffffu, e2, o);
    b2 += __shfl_down_sync(0xffffffffu, b2, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sh[0][wid] = e2;
    sh[1][wid] = b2;
  }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    e2 = lane < nw ? sh[0][lane] : 0.0;
    b2 = lane < nw ? sh[1][lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      e2 += __shfl_down_sync(0xffffffffu, e2, o);
      b2 += __shfl_down_sync(0xffffffffu, b2, o);
    }
    if (lane == 0) {
      scratch[2 * kMaxRows]     = e2;
      scratch[2 * kMaxRows + 1] = b2;
    }
  }
}

// device address of the scratch array on the current device (the host-side
// name of a __device__ array is not a device address). It is looked up again
// on every call made outside stream capture, so a context that was destroyed
// and recreated (cudaDeviceReset) gets the array's new address; inside a
// capture the address of the last such call is used.
int scratch_for_current_device(cudaStream_t s, double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PIC_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return PIC_ERR_UNSUPPORTED;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return PIC_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (cap == cudaStreamCaptureStatusNone || !g_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_energy_scratch) != cudaSuccess || !p) return PIC_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return PIC_OK;
}

}  // namespace
}  // namespace pic

extern "C" int pic_field_energy_noalloc(const pic_grid* g, const void* EB, double dx, double* out,
                                        void* stream) {
  if (!g || !EB || !out) return PIC_ERR_ARG;
  if (g->dim != 2 && g->dim != 3) return PIC_ERR_UNSUPPORTED;
  if (g->real_bytes != 4 && g->real_bytes != 8) return PIC_ERR_UNSUPPORTED;
  if (g->ng < 0 || g->n[0] <= 0 || g->n[1] <= 0 || (g->dim == 3 && g->n[2] <= 0)) return PIC_ERR_ARG;
  for (int k = 0; k < 4; ++k)
    if (g->em_stride[k] <= 0) return PIC_ERR_ARG;
  const int64_t rows = (int64_t)g->n[1] * (g->dim == 3 ? g->n[2] : 1);
  if (rows > pic::kMaxRows) return PIC_ERR_UNSUPPORTED;  // beyond the fixed scratch
  cudaStream_t s       = (cudaStream_t)stream;
  // an error left by the caller's earlier work is reported, not consumed
  if (cudaPeekAtLastError() != cudaSuccess) return PIC_ERR_CUDA;
  double* scratch = nullptr;
  int     st      = pic::scratch_for_current_device(s, &scratch);
  if (st != PIC_OK) return st;
  const int    threads = 256, warps = threads / 32;
  const int    blocks  = (int)((rows + warps - 1) / warps);
  if (g->real_bytes == 8) {
    PIC_KL(pic::k_energy_rows<double><<<blocks, threads, 0, s>>>(
      (const double*)EB, g->em_stride[0], g->em_stride[1], g->em_stride[2], g->em_stride[3], g->n[0],
      g->n[1], (int)rows, g->ng, g->dim, dx, scratch));
  } else {
    PIC_KL(pic::k_energy_rows<float><<<blocks, threads, 0, s>>>(
      (const float*)EB, g->em_stride[0], g->em_stride[1], g->em_stride[2], g->em_stride[3], g->n[0],
      g->n[1], (int)rows, g->ng, g->dim, dx, scratch));
  }
  if (cudaGetLastError() != cudaSuccess) return PIC_ERR_CUDA;
  PIC_KL(pic::k_energy_total<<<1, 1024, 0, s>>>((int)rows, scratch));
  if (cudaGetLastError() != cudaSuccess) return PIC_ERR_CUDA;
  if (cudaMemcpyAsync(out, scratch + 2 * pic::kMaxRows, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                      s) != cudaSuccess)
    return PIC_ERR_CUDA;
  return cudaStreamSynchronize(s) == cudaSuccess ? PIC_OK : PIC_ERR_CUDA;
}
