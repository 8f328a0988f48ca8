// Spatial sort and dead-particle removal of one species
// (Particles::SortSpatially / RemoveDead,
// src/framework/containers/particles_sort.cpp:103-253).
//
// The reference bins with Kokkos::BinSort (sort_within_bins = false), whose
// order inside a cell is unspecified. This sort produces the stable order
// (ascending original index inside every cell), which is one of the orders
// the reference may produce, and is deterministic:
//   1. key per particle (PositionToTileIndex, src/global/utils/sorting.h:
//      119-135: (i1*n2 + i2)*n3 + i3; dead -> last bin) and an atomic count
//      per bin whose return value is a provisional rank;
//   2. exclusive scan of the counts -> bin offsets;
//   3. scatter of indices; dead particles get their rank from a scan so the
//      (possibly huge) dead bin is placed in order directly;
//   4. every alive bin's index list is sorted ascending (one thread per bin up
//      to 32 entries, one block per larger bin);
//   5. every particle array is gathered through the permutation and copied
//      back.
// Nothing here synchronises with the host; the dead count stays on the
// device until the caller reads it.
#include <cuda_runtime.h>

#include "sort.cuh"

namespace pic {

namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems   = 8;
constexpr int kScanTile    = kScanThreads * kScanItems;

template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* sh, T& total) {
  // warp inclusive scan
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T         x    = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    T         s  = lane < nw ? sh[lane] : (T)0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) sh[lane] = s;
  }
  __syncthreads();
  const T warp_off = wid > 0 ? sh[wid - 1] : (T)0;
  total            = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_off + x - v;
}

// per-tile sums of in[0..n)
template <typename Tin, typename T>
__global__ void k_tile_sums(const Tin* in, int64_t n, T* sums) {
  __shared__ T  sh[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  T             s    = 0;
#pragma unroll
  for (int it = 0; it < kScanItems; ++it) {
    const int64_t i = base + (int64_t)it * kScanThreads + threadIdx.x;
    if (i < n) s += (T)in[i];
  }
  T total;
  block_exclusive_scan<T>(s, sh, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// exclusive scan of one tile with a carried-in offset per tile
template <typename Tin, typename T>
__global__ void k_tile_scan(const Tin* in, int64_t n, const T* tile_off, T* out) {
  __shared__ T  sh[32];
  __shared__ T  carry;
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  if (threadIdx.x == 0) carry = tile_off ? tile_off[blockIdx.x] : (T)0;
  __syncthreads();
  // each thread owns kScanItems consecutive elements
  T         v[kScanItems];
  T         s  = 0;
  const int t0 = threadIdx.x * kScanItems;
#pragma unroll
  for (int it = 0; it < kScanItems; ++it) {
    const int64_t i = base + t0 + it;
    v[it]           = i < n ? (T)in[i] : (T)0;
    s += v[it];
  }
  T total;
  T pre = block_exclusive_scan<T>(s, sh, total) + carry;
#pragma unroll
  for (int it = 0; it < kScanItems; ++it) {
    const int64_t i = base + t0 + it;
    if (i < n) out[i] = pre;
    pre += v[it];
  }
}

}  // namespace

// exclusive scan (out may alias in only through separate buffers)
template <typename Tin, typename T>
cudaError_t exclusive_scan(const Tin* in, int64_t n, T* out, ScanScratch<T>& scr, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    PIC_KL(k_tile_scan<Tin, T><<<1, kScanThreads, 0, s>>>(in, n, (const T*)nullptr, out));
    return cudaGetLastError();
  }
  T* sums = scr.get(tiles * 2 + 2, s);
  if (!sums) return cudaErrorMemoryAllocation;
  T* offs = sums + tiles + 1;
  PIC_KL(k_tile_sums<Tin, T><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, sums));
  // recursive scan of the tile sums (depth log_4096(n))
  ScanScratch<T> sub;
  cudaError_t    e = exclusive_scan<T, T>(sums, tiles, offs, sub, s);
  if (e != cudaSuccess) {
    sub.release(s);
    return e;
  }
  PIC_KL(k_tile_scan<Tin, T><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, offs, out));
  e = cudaGetLastError();
  sub.release(s);
  return e;
}

template cudaError_t exclusive_scan<int32_t, int64_t>(const int32_t*, int64_t, int64_t*,
                                                      ScanScratch<int64_t>&, cudaStream_t);
template cudaError_t exclusive_scan<uint8_t, int64_t>(const uint8_t*, int64_t, int64_t*,
                                                      ScanScratch<int64_t>&, cudaStream_t);
template cudaError_t exclusive_scan<int64_t, int64_t>(const int64_t*, int64_t, int64_t*,
                                                      ScanScratch<int64_t>&, cudaStream_t);
template cudaError_t exclusive_scan<uint8_t, int32_t>(const uint8_t*, int64_t, int32_t*,
                                                      ScanScratch<int32_t>&, cudaStream_t);
template cudaError_t exclusive_scan<int32_t, int32_t>(const int32_t*, int64_t, int32_t*,
                                                      ScanScratch<int32_t>&, cudaStream_t);

namespace {

// Place of the cell lx within its tile row: the even cells first, then the
// odd ones. A warp's lanes then cover cells two apart, whose order-2 support
// boxes never start on the same node, so fewer of their J-window atomics
// fall on one word; the window reads stay in distinct banks.
__device__ __forceinline__ int tile_row_slot(int lx, int tx) {
  return (lx & 1) ? (tx + 1) / 2 + lx / 2 : lx / 2;
}

// 1. keys + counts + provisional rank
__global__ void k_keys(SortArgs a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.npart; p += stride) {
    const short tag = a.tag[p];
    int32_t     key;
    if (tag != PIC_TAG_ALIVE) {
      key = a.dead_bin;
    } else if (!a.spatial) {
      key = 0;
    } else {
      const int i1 = a.i1[p], i2 = a.i2[p], i3 = a.dim == 3 ? a.i3[p] : 0;
      const bool ok = (i1 >= 0 && i1 < a.n[0] && i2 >= 0 && i2 < a.n[1] &&
                       (a.dim == 2 || (i3 >= 0 && i3 < a.n[2])));
      if (!ok) {
        atomicAdd(a.err + ERR_OUT_OF_GRID, 1ull);
        key = a.dead_bin;  // kept after the alive particles, tag untouched
      } else if (a.tiled) {
        const int tx = i1 / a.tile[0], ty = i2 / a.tile[1], tz = i3 / a.tile[2];
        const int lx = i1 - tx * a.tile[0], ly = i2 - ty * a.tile[1], lz = i3 - tz * a.tile[2];
        const int t  = (tz * a.ntiles[1] + ty) * a.ntiles[0] + tx;
        key = (t * a.tile[2] + lz) * (a.tile[0] * a.tile[1]) + ly * a.tile[0] +
              tile_row_slot(lx, a.tile[0]);
      } else if (a.dim == 2) {
        key = i1 * a.n[1] + i2;
      } else {
        key = (i1 * a.n[1] + i2) * a.n[2] + i3;
      }
    }
    a.key[p]        = key;
    a.is_dead[p]    = (uint8_t)(key == a.dead_bin);
    a.rank[p]       = atomicAdd(a.count + key, 1);
  }
}

// 3. scatter of particle indices into their bins
__global__ void k_scatter(SortArgs a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.npart; p += stride) {
    const int32_t key = a.key[p];
    int64_t       pos;
    if (key == a.dead_bin) {
      pos = a.off[key] + a.dead_rank[p];
    } else if (!a.spatial) {
      pos = p - a.dead_rank[p];  // alive before p, in order
    } else {
      pos = a.off[key] + a.rank[p];
    }
    a.perm[pos] = (int32_t)p;
  }
}

// 4a. per-bin ascending order, small bins
__global__ void k_fix_small(SortArgs a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < a.dead_bin; b += stride) {
    const int64_t lo = a.off[b], hi = a.off[b + 1];
    const int64_t m  = hi - lo;
    if (m <= 1) continue;
    if (m > 32) {
      const int slot = atomicAdd(a.nbig, 1);
      a.big[slot]    = (int32_t)b;
      continue;
    }
    int32_t v[32];
    for (int q = 0; q < m; ++q) v[q] = a.perm[lo + q];
    for (int q = 1; q < m; ++q) {
      const int32_t x = v[q];
      int           r = q - 1;
      while (r >= 0 && v[r] > x) {
        v[r + 1] = v[r];
        --r;
      }
      v[r + 1] = x;
    }
    for (int q = 0; q < m; ++q) a.perm[lo + q] = v[q];
  }
}

// 4b. large bins: rank by counting (O(m^2 / threads)); blocks stride over
// the bins the small-bin pass listed, whose number only the device knows
__global__ void k_fix_big(SortArgs a) {
  const int nbig = *a.nbig;
  for (int bi = blockIdx.x; bi < nbig; bi += gridDim.x) {
    const int     b  = a.big[bi];
    const int64_t lo = a.off[b], hi = a.off[b + 1];
    const int64_t m  = hi - lo;
    for (int64_t q = threadIdx.x; q < m; q += blockDim.x) {
      const int32_t x = a.perm[lo + q];
      int64_t       r = 0;
      for (int64_t z = 0; z < m; ++z) r += (a.perm[lo + z] < x);
      a.perm_tmp[lo + r] = x;
    }
    __syncthreads();
    for (int64_t q = threadIdx.x; q < m; q += blockDim.x) a.perm[lo + q] = a.perm_tmp[lo + q];
    __syncthreads();
  }
}

// 5. one gather per array through perm into its staging buffer, then a
// copy back. (A single kernel gathering every array at once ran at half the
// speed on nearly sorted input: its many concurrent scattered streams lose
// the L2 locality each array's gather has on its own.)
template <typename T>
__global__ void k_gather(const T* __restrict__ src, T* __restrict__ dst, const int32_t* perm,
                         int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    dst[i] = src[perm[i]];
  }
}

__global__ void k_set_tags(int16_t* tag, int64_t np, const int32_t* n_dead) {
  const int64_t nalive = np - *n_dead;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np; i += stride) {
    tag[i] = i < nalive ? (int16_t)PIC_TAG_ALIVE : (int16_t)PIC_TAG_DEAD;
  }
}

dim3 grid_n(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > pic::sm_count() * 64) b = pic::sm_count() * 64;
  if (b < 1) b = 1;
  return dim3((unsigned)b);
}

}  // namespace

cudaError_t sort_build_perm(SortArgs a, cudaStream_t s) {
  cudaError_t e;
  const int64_t nbins = (int64_t)a.dead_bin + 1;
  e = cudaMemsetAsync(a.count, 0, sizeof(int32_t) * (nbins + 1), s);
  if (e != cudaSuccess) return e;
  PIC_KL(k_keys<<<grid_n(a.npart), 256, 0, s>>>(a));
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  ScanScratch<int64_t> scr;
  e = exclusive_scan<int32_t, int64_t>(a.count, nbins + 1, a.off, scr, s);
  scr.release(s);
  if (e != cudaSuccess) return e;
  // the rank of every particle among the dead (and, for the alive-only
  // compaction, the number of dead before it): one scan, whatever the count
  ScanScratch<int32_t> scr2;
  e = exclusive_scan<uint8_t, int32_t>(a.is_dead, a.npart, a.dead_rank, scr2, s);
  scr2.release(s);
  if (e != cudaSuccess) return e;
  PIC_KL(k_scatter<<<grid_n(a.npart), 256, 0, s>>>(a));
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (a.spatial && a.dead_bin > 0) {
    e = cudaMemsetAsync(a.nbig, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return e;
    PIC_KL(k_fix_small<<<grid_n(a.dead_bin), 256, 0, s>>>(a));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    PIC_KL(k_fix_big<<<pic::sm_count() * 2, 256, 0, s>>>(a));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

namespace {
// arr_k[i] -> dst_k[i] = arr_k[perm[i]] for every listed array: the
// permutation is read once per particle for all arrays of the species
struct MultiGather {
  const void* src[kMaxSortArrays];
  void*       dst[kMaxSortArrays];
  int         esz[kMaxSortArrays];
  int64_t     es[kMaxSortArrays];  // element stride of src
  int         n;
};

// N arrays: every value of a particle is loaded before any is stored, so a
// thread keeps N loads in flight instead of one
template <int N>
__global__ void k_gather_multi(MultiGather g, const int32_t* __restrict__ perm, int64_t np) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np; i += stride) {
    const int64_t j = perm[i];
    uint64_t      v[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const int64_t jk = j * g.es[k];
      if (g.esz[k] == 4)      v[k] = (uint32_t)((const int32_t*)g.src[k])[jk];
      else if (g.esz[k] == 8) v[k] = (uint64_t)((const int64_t*)g.src[k])[jk];
      else                    v[k] = (uint16_t)((const int16_t*)g.src[k])[jk];
    }
#pragma unroll
    for (int k = 0; k < N; ++k) {
      if (g.esz[k] == 4)      ((int32_t*)g.dst[k])[i] = (int32_t)(uint32_t)v[k];
      else if (g.esz[k] == 8) ((int64_t*)g.dst[k])[i] = (int64_t)v[k];
      else                    ((int16_t*)g.dst[k])[i] = (int16_t)(uint16_t)v[k];
    }
  }
}

template <int N>
cudaError_t launch_gather_n(const MultiGather& g, const int32_t* perm, int64_t np, dim3 grid,
                            cudaStream_t s) {
  if constexpr (N > kMaxSortArrays) {
    return cudaErrorInvalidValue;
  } else {
    if (g.n != N) return launch_gather_n<N + 1>(g, perm, np, grid, s);
    PIC_KL(k_gather_multi<N><<<grid, 256, 0, s>>>(g, perm, np));
    return cudaGetLastError();
  }
}

// copies of the packed staging areas back into the caller's arrays: packed
// arrays in 16-byte pieces where both ends allow it (chunk c of array k
// covers bytes [c * 16, c * 16 + 16)), strided ones element by element
// (chunk c is element c)
struct MultiCopy {
  const char* src[kMaxSortArrays];
  char*       dst[kMaxSortArrays];
  int64_t     bytes[kMaxSortArrays];
  int64_t     es[kMaxSortArrays];  // element stride of dst
  int         esz[kMaxSortArrays];
  int64_t     first_chunk[kMaxSortArrays + 1];
  int         vec[kMaxSortArrays];  // packed, both pointers 16-byte aligned
  int         n;
};

__global__ void k_copy_multi(MultiCopy m) {
  const int64_t total  = m.first_chunk[m.n];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int           k      = 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < total; c += stride) {
    while (c >= m.first_chunk[k + 1]) ++k;
    const int64_t q = c - m.first_chunk[k];
    if (m.es[k] != 1) {
      const int64_t d = q * m.es[k];
      if (m.esz[k] == 4)      ((int32_t*)m.dst[k])[d] = ((const int32_t*)m.src[k])[q];
      else if (m.esz[k] == 8) ((int64_t*)m.dst[k])[d] = ((const int64_t*)m.src[k])[q];
      else                    ((int16_t*)m.dst[k])[d] = ((const int16_t*)m.src[k])[q];
      continue;
    }
    const int64_t off = q * 16;
    const int64_t len = m.bytes[k] - off < 16 ? m.bytes[k] - off : 16;
    if (m.vec[k] && len == 16) {
      *(int4*)(m.dst[k] + off) = *(const int4*)(m.src[k] + off);
    } else {
      for (int64_t b = 0; b < len; ++b) m.dst[k][off + b] = m.src[k][off + b];
    }
  }
}

// one array through a shared staging buffer, any element stride
template <typename T>
__global__ void k_gather_strided(const T* __restrict__ src, T* __restrict__ dst,
                                 const int32_t* perm, int64_t n, int64_t es) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    dst[i] = src[(int64_t)perm[i] * es];
}
template <typename T>
__global__ void k_unpack_strided(const T* __restrict__ src, T* __restrict__ dst, int64_t n,
                                 int64_t es) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    dst[i * es] = src[i];
}
}  // namespace

cudaError_t sort_apply_all(const GatherSet& g, const int32_t* perm, int64_t n, cudaStream_t s) {
  if (n <= 0 || g.n == 0) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  bool        staged_apart = true;  // every array has its own staging area
  for (int k = 0; k < g.n && staged_apart; ++k)
    for (int q = 0; q < k; ++q) staged_apart = staged_apart && g.tmp[q] != g.tmp[k];
  if (staged_apart) {
    // one gather of all arrays (perm read once), then one copy back
    MultiGather mg{};
    MultiCopy   mc{};
    mg.n = mc.n = g.n;
    mc.first_chunk[0] = 0;
    for (int k = 0; k < g.n; ++k) {
      mg.src[k] = g.arr[k];
      mg.dst[k] = g.tmp[k];
      mg.esz[k] = g.esz[k];
      mg.es[k]  = g.stride[k];
      mc.src[k] = (const char*)g.tmp[k];
      mc.dst[k] = (char*)g.arr[k];
      mc.bytes[k] = n * g.esz[k];
      mc.es[k]    = g.stride[k];
      mc.esz[k]   = g.esz[k];
      mc.vec[k] = g.stride[k] == 1 && ((uintptr_t)g.tmp[k] % 16 == 0) &&
                  ((uintptr_t)g.arr[k] % 16 == 0);
      mc.first_chunk[k + 1] =
        mc.first_chunk[k] + (g.stride[k] == 1 ? (mc.bytes[k] + 15) / 16 : n);
    }
    if ((e = launch_gather_n<1>(mg, perm, n, grid_n(n), s)) != cudaSuccess) return e;
    PIC_KL(k_copy_multi<<<grid_n(mc.first_chunk[g.n]), 256, 0, s>>>(mc));
    return cudaGetLastError();
  }
  // one shared staging buffer: the arrays go in turn
  for (int k = 0; k < g.n; ++k) {
    if (g.stride[k] != 1) {
      if (g.esz[k] == 8) {
        PIC_KL(k_gather_strided<int64_t><<<grid_n(n), 256, 0, s>>>((const int64_t*)g.arr[k], (int64_t*)g.tmp[k], perm, n, g.stride[k]));
        PIC_KL(k_unpack_strided<int64_t><<<grid_n(n), 256, 0, s>>>((const int64_t*)g.tmp[k], (int64_t*)g.arr[k], n, g.stride[k]));
      } else if (g.esz[k] == 4) {
        PIC_KL(k_gather_strided<int32_t><<<grid_n(n), 256, 0, s>>>((const int32_t*)g.arr[k], (int32_t*)g.tmp[k], perm, n, g.stride[k]));
        PIC_KL(k_unpack_strided<int32_t><<<grid_n(n), 256, 0, s>>>((const int32_t*)g.tmp[k], (int32_t*)g.arr[k], n, g.stride[k]));
      } else {
        PIC_KL(k_gather_strided<int16_t><<<grid_n(n), 256, 0, s>>>((const int16_t*)g.arr[k], (int16_t*)g.tmp[k], perm, n, g.stride[k]));
        PIC_KL(k_unpack_strided<int16_t><<<grid_n(n), 256, 0, s>>>((const int16_t*)g.tmp[k], (int16_t*)g.arr[k], n, g.stride[k]));
      }
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      continue;
    }
    if (g.esz[k] == 4)
      PIC_KL(k_gather<int32_t><<<grid_n(n), 256, 0, s>>>((const int32_t*)g.arr[k], (int32_t*)g.tmp[k], perm, n));
    else if (g.esz[k] == 8)
      PIC_KL(k_gather<int64_t><<<grid_n(n), 256, 0, s>>>((const int64_t*)g.arr[k], (int64_t*)g.tmp[k], perm, n));
    else
      PIC_KL(k_gather<int16_t><<<grid_n(n), 256, 0, s>>>((const int16_t*)g.arr[k], (int16_t*)g.tmp[k], perm, n));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    e = cudaMemcpyAsync(g.arr[k], g.tmp[k], (size_t)n * g.esz[k], cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t set_tags_after_removal(int16_t* tag, int64_t np, const int32_t* n_dead,
                                   cudaStream_t s) {
  if (np <= 0) return cudaSuccess;
  PIC_KL(k_set_tags<<<grid_n(np), 256, 0, s>>>(tag, np, n_dead));
  return cudaGetLastError();
}

namespace {
__global__ void k_tile_offsets(const int64_t* off, int64_t tile_cells, int ntiles,
                               int32_t* tile_start) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t <= ntiles) tile_start[t] = (int32_t)off[(int64_t)t * tile_cells];
}
}  // namespace

cudaError_t tile_offsets(const int64_t* off, int64_t tile_cells, int ntiles, int32_t* tile_start,
                         cudaStream_t s) {
  PIC_KL(k_tile_offsets<<<(ntiles + 256) / 256, 256, 0, s>>>(off, tile_cells, ntiles, tile_start));
  return cudaGetLastError();
}

}  // namespace pic
