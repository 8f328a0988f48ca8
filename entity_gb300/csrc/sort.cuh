// Host-side declarations for the sort and scan kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pic_types.h"

namespace pic {

// stream-ordered scratch for the recursive levels of the scan
template <typename T>
struct ScanScratch {
  T*      p   = nullptr;
  int64_t cap = 0;
  T* get(int64_t n, cudaStream_t s) {
    if (n > cap) {
      if (p) cudaFreeAsync(p, s);
      p   = nullptr;
      cap = 0;
      if (cudaMallocAsync((void**)&p, sizeof(T) * n, s) != cudaSuccess) return nullptr;
      cap = n;
    }
    return p;
  }
  void release(cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
    p   = nullptr;
    cap = 0;
  }
};

template <typename Tin, typename T>
cudaError_t exclusive_scan(const Tin* in, int64_t n, T* out, ScanScratch<T>& scr, cudaStream_t s);

struct SortArgs {
  // particle arrays
  const int32_t *i1, *i2, *i3;
  const int16_t *tag;
  int64_t        npart;
  int            dim;
  int            n[3];
  int            spatial;   // 1: cell key, 0: alive/dead only
  int            tiled;     // with spatial: tile-major key (tile, then cell in tile)
  int            tile[3];   // tile shape
  int            ntiles[3]; // tiles per axis
  int32_t        dead_bin;  // index of the last bin
  // scratch
  int32_t*  key;
  int32_t*  rank;
  uint8_t*  is_dead;
  int32_t*  dead_rank;
  int32_t*  count;  // dead_bin + 2 entries
  int64_t*  off;    // dead_bin + 2 entries
  int32_t*  perm;
  int32_t*  perm_tmp;
  int32_t*  big;
  int32_t*  nbig;
  unsigned long long* err;
};

// builds perm (new index -> old index) without host synchronisation; the
// dead count is left in count[dead_bin]
cudaError_t sort_build_perm(SortArgs a, cudaStream_t s);

// every listed array permuted in place: arr_k[i] <- arr_k[perm[i]], staged
// through tmp_k. With a staging area per array, one kernel gathers all
// arrays (the permutation read once) and one copies them back; when the
// tmp_k share one buffer the arrays go in turn
constexpr int kMaxSortArrays = 32;  // 3D with prev arrays needs 17, phi and payloads more
struct GatherSet {
  void*   arr[kMaxSortArrays];
  void*   tmp[kMaxSortArrays];
  int     esz[kMaxSortArrays];     // element bytes: 2, 4 or 8
  int64_t stride[kMaxSortArrays];  // element stride of arr (payload columns); tmp is packed
  int     n = 0;
};
cudaError_t sort_apply_all(const GatherSet& g, const int32_t* perm, int64_t n, cudaStream_t s);

// tags of [0, np - *n_dead) alive and of the rest dead (RemoveDead)
cudaError_t set_tags_after_removal(int16_t* tag, int64_t np, const int32_t* n_dead,
                                   cudaStream_t s);

// tile_start[t] = off[t * tile_cells] for t in [0, ntiles]
cudaError_t tile_offsets(const int64_t* off, int64_t tile_cells, int ntiles, int32_t* tile_start,
                         cudaStream_t s);

}  // namespace pic
