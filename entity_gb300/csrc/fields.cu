// Field kernels of the SR step on a Cartesian (Minkowski) grid: Faraday and
// Ampere Yee updates, the J -> E coupling, the periodic current fold, the
// digital current filter and ghost exchange, and the FP64 energy reduction.
//
// Every kernel maps one thread to one active cell (i1 fastest) and, where the
// reference follows the update with a periodic CommunicateFields, writes the
// cell's new value straight into its ghost images as well, which removes the
// reference's separate halo pass (src/framework/domain/comm_nompi.hpp:44-63).
#include <cuda_runtime.h>

#include "fields.cuh"
#include "pic_common.cuh"

namespace pic {

namespace {

struct CellIter {
  int     n[3];
  int     ng;
  int     dim;
  int64_t count;
  __device__ __forceinline__ void cell(int64_t t, int& i, int& j, int& k) const {
    i = (int)(t % n[0]);
    t /= n[0];
    j = (int)(t % n[1]);
    k = (int)(t / n[1]);
    i += ng;
    j += ng;
    k = (dim == 3) ? k + ng : 0;
  }
};

// visits every ghost image of active cell (i, j, k) across periodic
// dimensions (images: i + n when i < 2 ng, i - n when i >= n)
template <int D, typename F>
__device__ __forceinline__ void for_images(const GridInfo& g, int i, int j, int k, F&& f) {
  int sh[3][2];
  int ns[3];
  const int c[3] = { i, j, k };
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    ns[d]    = 1;
    sh[d][0] = 0;
    if (d < D && g.periodic[d]) {
      if (c[d] < 2 * g.ng) sh[d][ns[d]++] = g.n[d];
      else if (c[d] >= g.n[d]) sh[d][ns[d]++] = -g.n[d];
    }
  }
  for (int a = 0; a < ns[0]; ++a)
    for (int b = 0; b < ns[1]; ++b)
      for (int e = 0; e < ns[2]; ++e) {
        if (a == 0 && b == 0 && e == 0) continue;
        f(i + sh[0][a], j + sh[1][b], k + sh[2][e]);
      }
}

__device__ __forceinline__ bool near_periodic_edge(const GridInfo& g, int D, int i, int j, int k) {
  const int c[3] = { i, j, k };
  for (int d = 0; d < D; ++d) {
    if (g.periodic[d] && (c[d] < 2 * g.ng || c[d] >= g.n[d])) return true;
  }
  return false;
}

CellIter make_iter(const GridInfo& g) {
  CellIter it;
  it.n[0]  = g.n[0];
  it.n[1]  = g.n[1];
  it.n[2]  = g.dim == 3 ? g.n[2] : 1;
  it.ng    = g.ng;
  it.dim   = g.dim;
  it.count = (int64_t)it.n[0] * it.n[1] * it.n[2];
  return it;
}

dim3 grid_for(int64_t count, int threads) {
  int64_t b = (count + threads - 1) / threads;
  if (b > pic::sm_count() * 128) b = pic::sm_count() * 128;
  if (b < 1) b = 1;
  return dim3((unsigned)b);
}

// ---------------------------------------------------------------------------
// Faraday: src/kernels/faraday_mink.hpp:71-166 (+ CommunicateFields(B))
// ---------------------------------------------------------------------------
template <int D, typename real, bool YEE>
__global__ void k_faraday(GridInfo g, CellIter it, FieldView<real> EB, real coeff1, real coeff2,
                          Stencil<real> st) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < it.count; t += stride) {
    int i1, i2, i3;
    it.cell(t, i1, i2, i3);
#define F(a, b, c, comp) EB.p[EB.idx(a, b, c, comp)]
    real nb[3];
    if constexpr (D == 2) {
      const real alphax = (real)1 - (real)2 * st.betaxy - (real)3 * st.deltax;
      const real alphay = (real)1 - (real)2 * st.betayx - (real)3 * st.deltay;
      if constexpr (YEE) {
        nb[0] = F(i1, i2, 0, 3) + coeff1 * (-alphay * (F(i1, i2 + 1, 0, 2) - F(i1, i2, 0, 2)));
        nb[1] = F(i1, i2, 0, 4) + coeff1 * (+alphax * (F(i1 + 1, i2, 0, 2) - F(i1, i2, 0, 2)));
        nb[2] = F(i1, i2, 0, 5) + coeff2 * (+alphay * (F(i1, i2 + 1, 0, 0) - F(i1, i2, 0, 0)) -
                                            alphax * (F(i1 + 1, i2, 0, 1) - F(i1, i2, 0, 1)));
      } else {
        nb[0] = F(i1, i2, 0, 3) +
                coeff1 * (-alphay * (F(i1, i2 + 1, 0, 2) - F(i1, i2, 0, 2)) -
                          st.deltay * (F(i1, i2 + 2, 0, 2) - F(i1, i2 - 1, 0, 2)) -
                          st.betayx * (F(i1 + 1, i2 + 1, 0, 2) - F(i1 + 1, i2, 0, 2)) -
                          st.betayx * (F(i1 - 1, i2 + 1, 0, 2) - F(i1 - 1, i2, 0, 2)));
        nb[1] = F(i1, i2, 0, 4) +
                coeff1 * (+alphax * (F(i1 + 1, i2, 0, 2) - F(i1, i2, 0, 2)) +
                          st.deltax * (F(i1 + 2, i2, 0, 2) - F(i1 - 1, i2, 0, 2)) +
                          st.betaxy * (F(i1 + 1, i2 + 1, 0, 2) - F(i1, i2 + 1, 0, 2)) +
                          st.betaxy * (F(i1 + 1, i2 - 1, 0, 2) - F(i1, i2 - 1, 0, 2)));
        nb[2] = F(i1, i2, 0, 5) +
                coeff2 * (+alphay * (F(i1, i2 + 1, 0, 0) - F(i1, i2, 0, 0)) +
                          st.deltay * (F(i1, i2 + 2, 0, 0) - F(i1, i2 - 1, 0, 0)) +
                          st.betayx * (F(i1 + 1, i2 + 1, 0, 0) - F(i1 + 1, i2, 0, 0)) +
                          st.betayx * (F(i1 - 1, i2 + 1, 0, 0) - F(i1 - 1, i2, 0, 0)) -
                          alphax * (F(i1 + 1, i2, 0, 1) - F(i1, i2, 0, 1)) -
                          st.deltax * (F(i1 + 2, i2, 0, 1) - F(i1 - 1, i2, 0, 1)) -
                          st.betaxy * (F(i1 + 1, i2 + 1, 0, 1) - F(i1, i2 + 1, 0, 1)) -
                          st.betaxy * (F(i1 + 1, i2 - 1, 0, 1) - F(i1, i2 - 1, 0, 1)));
      }
    } else {
      const real alphax = (real)1 - (real)2 * st.betaxy - (real)2 * st.betaxz - (real)3 * st.deltax;
      const real alphay = (real)1 - (real)2 * st.betayx - (real)2 * st.betayz - (real)3 * st.deltay;
      const real alphaz = (real)1 - (real)2 * st.betazx - (real)2 * st.betazy - (real)3 * st.deltaz;
      if constexpr (YEE) {
        nb[0] = F(i1, i2, i3, 3) +
                coeff1 * (+alphaz * (F(i1, i2, i3 + 1, 1) - F(i1, i2, i3, 1)) -
                          alphay * (F(i1, i2 + 1, i3, 2) - F(i1, i2, i3, 2)));
        nb[1] = F(i1, i2, i3, 4) +
                coeff1 * (+alphax * (F(i1 + 1, i2, i3, 2) - F(i1, i2, i3, 2)) -
                          alphaz * (F(i1, i2, i3 + 1, 0) - F(i1, i2, i3, 0)));
        nb[2] = F(i1, i2, i3, 5) +
                coeff1 * (+alphay * (F(i1, i2 + 1, i3, 0) - F(i1, i2, i3, 0)) -
                          alphax * (F(i1 + 1, i2, i3, 1) - F(i1, i2, i3, 1)));
      } else {
        nb[0] = F(i1, i2, i3, 3) +
                coeff1 * (+alphaz * (F(i1, i2, i3 + 1, 1) - F(i1, i2, i3, 1)) +
                          st.deltaz * (F(i1, i2, i3 + 2, 1) - F(i1, i2, i3 - 1, 1)) +
                          st.betazx * (F(i1 + 1, i2, i3 + 1, 1) - F(i1 + 1, i2, i3, 1)) +
                          st.betazx * (F(i1 - 1, i2, i3 + 1, 1) - F(i1 - 1, i2, i3, 1)) +
                          st.betazy * (F(i1, i2 + 1, i3 + 1, 1) - F(i1, i2 + 1, i3, 1)) +
                          st.betazy * (F(i1, i2 - 1, i3 + 1, 1) - F(i1, i2 - 1, i3, 1)) -
                          alphay * (F(i1, i2 + 1, i3, 2) - F(i1, i2, i3, 2)) -
                          st.deltay * (F(i1, i2 + 2, i3, 2) - F(i1, i2 - 1, i3, 2)) -
                          st.betayx * (F(i1 + 1, i2 + 1, i3, 2) - F(i1 + 1, i2, i3, 2)) -
                          st.betayx * (F(i1 - 1, i2 + 1, i3, 2) - F(i1 - 1, i2, i3, 2)) -
                          st.betayz * (F(i1, i2 + 1, i3 + 1, 2) - F(i1, i2, i3 + 1, 2)) -
                          st.betayz * (F(i1, i2 + 1, i3 - 1, 2) - F(i1, i2, i3 - 1, 2)));
        nb[1] = F(i1, i2, i3, 4) +
                coeff1 * (+alphax * (F(i1 + 1, i2, i3, 2) - F(i1, i2, i3, 2)) +
                          st.deltax * (F(i1 + 2, i2, i3, 2) - F(i1 - 1, i2, i3, 2)) +
                          st.betaxy * (F(i1 + 1, i2 + 1, i3, 2) - F(i1, i2 + 1, i3, 2)) +
                          st.betaxy * (F(i1 + 1, i2 - 1, i3, 2) - F(i1, i2 - 1, i3, 2)) +
                          st.betaxz * (F(i1 + 1, i2, i3 + 1, 2) - F(i1, i2, i3 + 1, 2)) +
                          st.betaxz * (F(i1 + 1, i2, i3 - 1, 2) - F(i1, i2, i3 - 1, 2)) -
                          alphaz * (F(i1, i2, i3 + 1, 0) - F(i1, i2, i3, 0)) -
                          st.deltaz * (F(i1, i2, i3 + 2, 0) - F(i1, i2, i3 - 1, 0)) -
                          st.betazx * (F(i1 + 1, i2, i3 + 1, 0) - F(i1 + 1, i2, i3, 0)) -
                          st.betazx * (F(i1 - 1, i2, i3 + 1, 0) - F(i1 - 1, i2, i3, 0)) -
                          st.betazy * (F(i1, i2 + 1, i3 + 1, 0) - F(i1, i2 + 1, i3, 0)) -
                          st.betazy * (F(i1, i2 - 1, i3 + 1, 0) - F(i1, i2 - 1, i3, 0)));
        nb[2] = F(i1, i2, i3, 5) +
                coeff1 * (+alphay * (F(i1, i2 + 1, i3, 0) - F(i1, i2, i3, 0)) +
                          st.deltay * (F(i1, i2 + 2, i3, 0) - F(i1, i2 - 1, i3, 0)) +
                          st.betayx * (F(i1 + 1, i2 + 1, i3, 0) - F(i1 + 1, i2, i3, 0)) +
                          st.betayx * (F(i1 - 1, i2 + 1, i3, 0) - F(i1 - 1, i2, i3, 0)) +
                          st.betayz * (F(i1, i2 + 1, i3 + 1, 0) - F(i1, i2, i3 + 1, 0)) +
                          st.betayz * (F(i1, i2 + 1, i3 - 1, 0) - F(i1, i2, i3 - 1, 0)) -
                          alphax * (F(i1 + 1, i2, i3, 1) - F(i1, i2, i3, 1)) -
                          st.deltax * (F(i1 + 2, i2, i3, 1) - F(i1 - 1, i2, i3, 1)) -
                          st.betaxy * (F(i1 + 1, i2 + 1, i3, 1) - F(i1, i2 + 1, i3, 1)) -
                          st.betaxy * (F(i1 + 1, i2 - 1, i3, 1) - F(i1, i2 - 1, i3, 1)) -
                          st.betaxz * (F(i1 + 1, i2, i3 + 1, 1) - F(i1, i2, i3 + 1, 1)) -
                          st.betaxz * (F(i1 + 1, i2, i3 - 1, 1) - F(i1, i2, i3 - 1, 1)));
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) F(i1, i2, i3, 3 + c) = nb[c];
    for_images<D>(g, i1, i2, i3, [&](int a, int b, int e) {
#pragma unroll
      for (int c = 0; c < 3; ++c) F(a, b, e, 3 + c) = nb[c];
    });
#undef F
  }
}

// ---------------------------------------------------------------------------
// Ampere (ampere_mink.hpp:48-88) + CurrentsAmpere (ampere_mink.hpp:134-214)
// + CommunicateFields(E | J)
// ---------------------------------------------------------------------------
template <int D, typename real, bool CURL, bool CUR, bool FILL>
__global__ void k_ampere(GridInfo g, CellIter it, FieldView<real> EB, FieldView<real> J,
                         real coeff1, real coeff2, real jcoeff, real ppc0) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < it.count; t += stride) {
    int i1, i2, i3;
    it.cell(t, i1, i2, i3);
#define F(a, b, c, comp) EB.p[EB.idx(a, b, c, comp)]
    real ne[3] = { F(i1, i2, i3, 0), F(i1, i2, i3, 1), F(i1, i2, i3, 2) };
    if constexpr (CURL) {
      if constexpr (D == 2) {
        ne[0] += coeff1 * (F(i1, i2, 0, 5) - F(i1, i2 - 1, 0, 5));
        ne[1] += coeff1 * (F(i1 - 1, i2, 0, 5) - F(i1, i2, 0, 5));
        ne[2] += coeff2 * (F(i1, i2 - 1, 0, 3) - F(i1, i2, 0, 3) + F(i1, i2, 0, 4) -
                           F(i1 - 1, i2, 0, 4));
      } else {
        ne[0] += coeff1 * (F(i1, i2, i3 - 1, 4) - F(i1, i2, i3, 4) + F(i1, i2, i3, 5) -
                           F(i1, i2 - 1, i3, 5));
        ne[1] += coeff1 * (F(i1 - 1, i2, i3, 5) - F(i1, i2, i3, 5) + F(i1, i2, i3, 3) -
                           F(i1, i2, i3 - 1, 3));
        ne[2] += coeff1 * (F(i1, i2 - 1, i3, 3) - F(i1, i2, i3, 3) + F(i1, i2, i3, 4) -
                           F(i1 - 1, i2, i3, 4));
      }
    }
    real nj[3];
    if constexpr (CUR) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const real jv = J.p[J.idx(i1, i2, i3, c)];
        ne[c] += jv * jcoeff;
        nj[c] = jv / ppc0;
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) F(i1, i2, i3, c) = ne[c];
    if constexpr (CUR) {
#pragma unroll
      for (int c = 0; c < 3; ++c) J.p[J.idx(i1, i2, i3, c)] = nj[c];
    }
    if constexpr (FILL) {
      for_images<D>(g, i1, i2, i3, [&](int a, int b, int e) {
#pragma unroll
        for (int c = 0; c < 3; ++c) F(a, b, e, c) = ne[c];
        if constexpr (CUR) {
#pragma unroll
          for (int c = 0; c < 3; ++c) J.p[J.idx(a, b, e, c)] = nj[c];
        }
      });
    }
#undef F
  }
}

// ---------------------------------------------------------------------------
// periodic current fold + ghost fill: SynchronizeFields(J) followed by
// CommunicateFields(J) (metadomain_comm.cpp:408-562, 204-367). The sum runs
// over the images in dir::Directions<D>::all order and is added to the
// active value last, as AddBufferedFields does.
// ---------------------------------------------------------------------------
template <int D, typename real>
__global__ void k_sync_currents(GridInfo g, CellIter it, FieldView<real> J) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < it.count; t += stride) {
    int i1, i2, i3;
    it.cell(t, i1, i2, i3);
    if (!near_periodic_edge(g, D, i1, i2, i3)) continue;
    const int c[3] = { i1, i2, i3 };
    real      buf[3] = { 0, 0, 0 };
    // directions v in lexicographic order over {-1,0,1}^D \ {0}; the source
    // of v is c + n*v, valid when v_d = +1 -> c_d < 2ng, v_d = -1 -> c_d >= n
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b)
        for (int e = (D == 3 ? -1 : 0); e <= (D == 3 ? 1 : 0); ++e) {
          if (a == 0 && b == 0 && e == 0) continue;
          const int v[3] = { a, b, e };
          int       src[3];
          bool      ok = true;
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            src[d] = c[d];
            if (v[d] == 0) continue;
            if (d >= D || !g.periodic[d]) {
              ok = false;
            } else if (v[d] == 1) {
              ok = ok && (c[d] < 2 * g.ng);
              src[d] = c[d] + g.n[d];
            } else {
              ok = ok && (c[d] >= g.n[d]);
              src[d] = c[d] - g.n[d];
            }
          }
          if (!ok) continue;
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) buf[cc] += J.p[J.idx(src[0], src[1], src[2], cc)];
        }
    real nv[3];
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
      nv[cc]                          = J.p[J.idx(i1, i2, i3, cc)] + buf[cc];
      J.p[J.idx(i1, i2, i3, cc)] = nv[cc];
    }
    for_images<D>(g, i1, i2, i3, [&](int a, int b, int e) {
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) J.p[J.idx(a, b, e, cc)] = nv[cc];
    });
  }
}

// plain ghost fill of components [c0, c1): images of cells near the edges
template <int D, typename real>
__global__ void k_fill_ghosts(GridInfo g, CellIter it, FieldView<real> f, int c0, int c1) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < it.count; t += stride) {
    int i1, i2, i3;
    it.cell(t, i1, i2, i3);
    if (!near_periodic_edge(g, D, i1, i2, i3)) continue;
    for (int c = c0; c < c1; ++c) {
      const real v = f.p[f.idx(i1, i2, i3, c)];
      for_images<D>(g, i1, i2, i3, [&](int a, int b, int e) { f.p[f.idx(a, b, e, c)] = v; });
    }
  }
}

// ---------------------------------------------------------------------------
// digital filter pass: digital_filter.hpp:183-195 (2D), 352-379 (3D); reads
// src, writes dst at the active cells and their periodic ghost images
// ---------------------------------------------------------------------------
template <int D, typename real>
__global__ void k_filter(GridInfo g, CellIter it, FieldView<real> src, FieldView<real> dst) {
  const real    INV_4 = 0.25, INV_8 = 0.125, INV_16 = 0.0625, INV_32 = 0.03125, INV_64 = 0.015625;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < it.count; t += stride) {
    int i1, i2, i3;
    it.cell(t, i1, i2, i3);
    real nv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#define b(x, y, z) src.p[src.idx(x, y, z, c)]
      if constexpr (D == 2) {
        nv[c] = INV_4 * b(i1, i2, 0) +
                INV_8 * (b(i1 - 1, i2, 0) + b(i1 + 1, i2, 0) + b(i1, i2 - 1, 0) + b(i1, i2 + 1, 0)) +
                INV_16 * (b(i1 - 1, i2 - 1, 0) + b(i1 + 1, i2 + 1, 0) + b(i1 - 1, i2 + 1, 0) +
                          b(i1 + 1, i2 - 1, 0));
      } else {
        // the (i, j, k +- 1) pair appears twice in the 1/32 group, as in
        // digital_filter.hpp:365
        nv[c] = INV_8 * b(i1, i2, i3) +
                INV_16 * (b(i1 - 1, i2, i3) + b(i1 + 1, i2, i3) + b(i1, i2 - 1, i3) +
                          b(i1, i2 + 1, i3) + b(i1, i2, i3 - 1) + b(i1, i2, i3 + 1)) +
                INV_32 * (b(i1 - 1, i2 - 1, i3) + b(i1 + 1, i2 + 1, i3) + b(i1 - 1, i2 + 1, i3) +
                          b(i1 + 1, i2 - 1, i3) + b(i1, i2 - 1, i3 - 1) + b(i1, i2 + 1, i3 + 1) +
                          b(i1, i2, i3 - 1) + b(i1, i2, i3 + 1) + b(i1 - 1, i2, i3 - 1) +
                          b(i1 + 1, i2, i3 + 1) + b(i1 - 1, i2, i3 + 1) + b(i1 + 1, i2, i3 - 1)) +
                INV_64 * (b(i1 - 1, i2 - 1, i3 - 1) + b(i1 + 1, i2 + 1, i3 + 1) +
                          b(i1 - 1, i2 + 1, i3 + 1) + b(i1 + 1, i2 - 1, i3 - 1) +
                          b(i1 - 1, i2 - 1, i3 + 1) + b(i1 + 1, i2 + 1, i3 - 1) +
                          b(i1 - 1, i2 + 1, i3 - 1) + b(i1 + 1, i2 - 1, i3 + 1));
      }
#undef b
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) dst.p[dst.idx(i1, i2, i3, c)] = nv[c];
    for_images<D>(g, i1, i2, i3, [&](int a, int bb, int e) {
#pragma unroll
      for (int c = 0; c < 3; ++c) dst.p[dst.idx(a, bb, e, c)] = nv[c];
    });
  }
}

// The 3D pass staged through shared memory: one CTA per 32 x 8 x 4 block of
// active cells holds the block and a one-cell halo of the three components,
// and each cell's 27-point sum is the expression of k_filter read from the
// stage (same operands, same order: the same bits). The global version
// issues 81 loads per cell through L1.
constexpr int kFltX = 32, kFltY = 8, kFltZ = 4;
template <typename real>
__global__ void __launch_bounds__(256) k_filter3_staged(GridInfo g, FieldView<real> src,
                                                       FieldView<real> dst) {
  constexpr int SX = kFltX + 2, SY = kFltY + 2, SZ = kFltZ + 2;
  __shared__ real sm[3][SZ][SY][SX];
  const real INV_8 = 0.125, INV_16 = 0.0625, INV_32 = 0.03125, INV_64 = 0.015625;
  const int  ng = g.ng;
  // first active cell of the block, ghost-inclusive
  const int x0 = ng + blockIdx.x * kFltX, y0 = ng + blockIdx.y * kFltY, z0 = ng + blockIdx.z * kFltZ;
  const int ex = g.n[0] + 2 * ng, ey = g.n[1] + 2 * ng, ez = g.n[2] + 2 * ng;
  // a fixed trip count, unrolled, so that every thread's loads are in flight
  // together
  constexpr int NS = 3 * SZ * SY * SX, NTH = 256, TRIPS = (NS + NTH - 1) / NTH;
  real          v[TRIPS];
#pragma unroll
  for (int k = 0; k < TRIPS; ++k) {
    const int t = threadIdx.x + k * NTH;
    const int x = t % SX, y = (t / SX) % SY, z = (t / (SX * SY)) % SZ, c = t / (SX * SY * SZ);
    const int gx = x0 - 1 + x, gy = y0 - 1 + y, gz = z0 - 1 + z;
    // cells past the array belong to no active cell of this block
    v[k] = (t < NS && gx < ex && gy < ey && gz < ez) ? src.p[src.idx(gx, gy, gz, c)] : (real)0;
  }
#pragma unroll
  for (int k = 0; k < TRIPS; ++k) {
    const int t = threadIdx.x + k * NTH;
    if (t < NS) (&sm[0][0][0][0])[t] = v[k];
  }
  __syncthreads();
  const int tx = threadIdx.x % kFltX, ty = threadIdx.x / kFltX;
  const int i1 = x0 + tx, i2 = y0 + ty;
  if (i1 >= g.n[0] + ng || i2 >= g.n[1] + ng) return;
  for (int tz = 0; tz < kFltZ; ++tz) {
    const int i3 = z0 + tz;
    if (i3 >= g.n[2] + ng) break;
    real nv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#define b(x, y, z) sm[c][tz + 1 + ((z) - i3)][ty + 1 + ((y) - i2)][tx + 1 + ((x) - i1)]
      // the (i, j, k +- 1) pair appears twice in the 1/32 group, as in
      // digital_filter.hpp:365
      nv[c] = INV_8 * b(i1, i2, i3) +
              INV_16 * (b(i1 - 1, i2, i3) + b(i1 + 1, i2, i3) + b(i1, i2 - 1, i3) +
                        b(i1, i2 + 1, i3) + b(i1, i2, i3 - 1) + b(i1, i2, i3 + 1)) +
              INV_32 * (b(i1 - 1, i2 - 1, i3) + b(i1 + 1, i2 + 1, i3) + b(i1 - 1, i2 + 1, i3) +
                        b(i1 + 1, i2 - 1, i3) + b(i1, i2 - 1, i3 - 1) + b(i1, i2 + 1, i3 + 1) +
                        b(i1, i2, i3 - 1) + b(i1, i2, i3 + 1) + b(i1 - 1, i2, i3 - 1) +
                        b(i1 + 1, i2, i3 + 1) + b(i1 - 1, i2, i3 + 1) + b(i1 + 1, i2, i3 - 1)) +
              INV_64 * (b(i1 - 1, i2 - 1, i3 - 1) + b(i1 + 1, i2 + 1, i3 + 1) +
                        b(i1 - 1, i2 + 1, i3 + 1) + b(i1 + 1, i2 - 1, i3 - 1) +
                        b(i1 - 1, i2 - 1, i3 + 1) + b(i1 + 1, i2 + 1, i3 - 1) +
                        b(i1 - 1, i2 + 1, i3 - 1) + b(i1 + 1, i2 - 1, i3 + 1));
#undef b
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) dst.p[dst.idx(i1, i2, i3, c)] = nv[c];
    for_images<3>(g, i1, i2, i3, [&](int a, int bb, int e) {
#pragma unroll
      for (int c = 0; c < 3; ++c) dst.p[dst.idx(a, bb, e, c)] = nv[c];
    });
  }
}

// copy all cells (ghost-inclusive) of a 3-component field
template <typename real>
__global__ void k_copy3(GridInfo g, FieldView<real> src, FieldView<real> dst) {
  const int     e0 = g.n[0] + 2 * g.ng, e1 = g.n[1] + 2 * g.ng;
  const int     e2 = g.dim == 3 ? g.n[2] + 2 * g.ng : 1;
  const int64_t count  = (int64_t)e0 * e1 * e2 * 3;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += stride) {
    int64_t r = t;
    const int i = (int)(r % e0);
    r /= e0;
    const int j = (int)(r % e1);
    r /= e1;
    const int k = (int)(r % e2);
    const int c = (int)(r / e2);
    dst.p[dst.idx(i, j, k, c)] = src.p[src.idx(i, j, k, c)];
  }
}

// zero all cells of a 3-component field
template <typename real>
__global__ void k_zero3(GridInfo g, FieldView<real> f) {
  const int     e0 = g.n[0] + 2 * g.ng, e1 = g.n[1] + 2 * g.ng;
  const int     e2 = g.dim == 3 ? g.n[2] + 2 * g.ng : 1;
  const int64_t count  = (int64_t)e0 * e1 * e2 * 3;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += stride) {
    int64_t r = t;
    const int i = (int)(r % e0);
    r /= e0;
    const int j = (int)(r % e1);
    r /= e1;
    const int k = (int)(r % e2);
    const int c = (int)(r / e2);
    f.p[f.idx(i, j, k, c)] = (real)0;
  }
}

// FP64 field energy (reduced_stats.hpp:145-187, Minkowski weights)
template <int D, typename real>
__global__ void k_energy(CellIter it, FieldView<real> EB, double dx, double* out) {
  __shared__ double sh[2][32];
  const double  dV     = D == 3 ? dx * dx * dx : dx * dx;
  double        e2 = 0, b2 = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < it.count; t += stride) {
    int i1, i2, i3;
    it.cell(t, i1, i2, i3);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double h  = (c < D) ? dx * dx : 1.0;
      const double ev = (double)EB.p[EB.idx(i1, i2, i3, c)];
      const double bv = (double)EB.p[EB.idx(i1, i2, i3, c + 3)];
      e2 += ev * ev * h * dV;
      b2 += bv * bv * h * dV;
    }
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
      atomicAdd(out, e2);
      atomicAdd(out + 1, b2);
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename real>
cudaError_t launch_faraday(const GridInfo& g, FieldView<real> EB, real c1, real c2,
                           const Stencil<real>& st, bool yee, cudaStream_t s) {
  const CellIter it = make_iter(g);
  const dim3     gr = grid_for(it.count, 256);
  if (g.dim == 2) {
    if (yee) PIC_KL(k_faraday<2, real, true><<<gr, 256, 0, s>>>(g, it, EB, c1, c2, st));
    else     PIC_KL(k_faraday<2, real, false><<<gr, 256, 0, s>>>(g, it, EB, c1, c2, st));
  } else {
    if (yee) PIC_KL(k_faraday<3, real, true><<<gr, 256, 0, s>>>(g, it, EB, c1, c2, st));
    else     PIC_KL(k_faraday<3, real, false><<<gr, 256, 0, s>>>(g, it, EB, c1, c2, st));
  }
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_ampere(const GridInfo& g, FieldView<real> EB, FieldView<real> J, real c1,
                          real c2, real jcoeff, real ppc0, bool curl, bool cur, bool fill,
                          cudaStream_t s) {
  const CellIter it = make_iter(g);
  const dim3     gr = grid_for(it.count, 256);
#define PIC_AMP(DD, A, B, C) PIC_KL(k_ampere<DD, real, A, B, C><<<gr, 256, 0, s>>>(g, it, EB, J, c1, c2, jcoeff, ppc0))
#define PIC_AMP_D(DD)                                                   \
  if (curl && cur && fill) PIC_AMP(DD, true, true, true);              \
  else if (curl && cur) PIC_AMP(DD, true, true, false);                 \
  else if (curl && fill) PIC_AMP(DD, true, false, true);               \
  else if (curl) PIC_AMP(DD, true, false, false);                       \
  else if (cur && fill) PIC_AMP(DD, false, true, true);                 \
  else if (cur) PIC_AMP(DD, false, true, false);
  if (g.dim == 2) {
    PIC_AMP_D(2)
  } else {
    PIC_AMP_D(3)
  }
#undef PIC_AMP_D
#undef PIC_AMP
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_sync_currents(const GridInfo& g, FieldView<real> J, cudaStream_t s) {
  const CellIter it = make_iter(g);
  const dim3     gr = grid_for(it.count, 256);
  if (g.dim == 2) PIC_KL(k_sync_currents<2, real><<<gr, 256, 0, s>>>(g, it, J));
  else            PIC_KL(k_sync_currents<3, real><<<gr, 256, 0, s>>>(g, it, J));
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_fill_ghosts(const GridInfo& g, FieldView<real> f, int c0, int c1, cudaStream_t s) {
  const CellIter it = make_iter(g);
  const dim3     gr = grid_for(it.count, 256);
  if (g.dim == 2) PIC_KL(k_fill_ghosts<2, real><<<gr, 256, 0, s>>>(g, it, f, c0, c1));
  else            PIC_KL(k_fill_ghosts<3, real><<<gr, 256, 0, s>>>(g, it, f, c0, c1));
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_filter(const GridInfo& g, FieldView<real> J, FieldView<real> buff, int npasses,
                          cudaStream_t s) {
  if (npasses <= 0) return cudaSuccess;
  const CellIter it       = make_iter(g);
  const dim3     gr       = grid_for(it.count, 256);
  const bool     all_per  = g.periodic[0] && g.periodic[1] && (g.dim == 2 || g.periodic[2]);
  const int64_t  ncells_g = (int64_t)(g.n[0] + 2 * g.ng) * (g.n[1] + 2 * g.ng) *
                           (g.dim == 3 ? g.n[2] + 2 * g.ng : 1) * 3;
  const dim3     grc      = grid_for(ncells_g, 256);
  const dim3 gs((g.n[0] + kFltX - 1) / kFltX, (g.n[1] + kFltY - 1) / kFltY,
                g.dim == 3 ? (g.n[2] + kFltZ - 1) / kFltZ : 1);
  if (all_per) {
    // ping-pong: every ghost cell is an image and is rewritten each pass
    FieldView<real> a = J, b = buff;
    for (int p = 0; p < npasses; ++p) {
      if (g.dim == 2) PIC_KL(k_filter<2, real><<<gr, 256, 0, s>>>(g, it, a, b));
      else            PIC_KL(k_filter3_staged<real><<<gs, 256, 0, s>>>(g, a, b));
      FieldView<real> t = a;
      a                 = b;
      b                 = t;
    }
    if (npasses % 2 == 1) PIC_KL(k_copy3<real><<<grc, 256, 0, s>>>(g, buff, J));
  } else {
    // reference order: buff <- J (incl. non-periodic ghosts), filter, fill
    for (int p = 0; p < npasses; ++p) {
      PIC_KL(k_copy3<real><<<grc, 256, 0, s>>>(g, J, buff));
      if (g.dim == 2) PIC_KL(k_filter<2, real><<<gr, 256, 0, s>>>(g, it, buff, J));
      else            PIC_KL(k_filter3_staged<real><<<gs, 256, 0, s>>>(g, buff, J));
    }
  }
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_copy3(const GridInfo& g, FieldView<real> src, FieldView<real> dst,
                         cudaStream_t s) {
  const int64_t ncells_g = (int64_t)(g.n[0] + 2 * g.ng) * (g.n[1] + 2 * g.ng) *
                           (g.dim == 3 ? g.n[2] + 2 * g.ng : 1) * 3;
  PIC_KL(k_copy3<real><<<grid_for(ncells_g, 256), 256, 0, s>>>(g, src, dst));
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_zero3(const GridInfo& g, FieldView<real> f, cudaStream_t s) {
  const int64_t ncells_g = (int64_t)(g.n[0] + 2 * g.ng) * (g.n[1] + 2 * g.ng) *
                           (g.dim == 3 ? g.n[2] + 2 * g.ng : 1) * 3;
  PIC_KL(k_zero3<real><<<grid_for(ncells_g, 256), 256, 0, s>>>(g, f));
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_energy(const GridInfo& g, FieldView<real> EB, double dx, double* out,
                          cudaStream_t s) {
  const CellIter it = make_iter(g);
  int64_t        b  = (it.count + 255) / 256;
  if (b > pic::sm_count() * 8) b = pic::sm_count() * 8;
  if (g.dim == 2) PIC_KL(k_energy<2, real><<<(unsigned)b, 256, 0, s>>>(it, EB, dx, out));
  else            PIC_KL(k_energy<3, real><<<(unsigned)b, 256, 0, s>>>(it, EB, dx, out));
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// adjoint (transposed) field operators. Each forward update of the step is a
// periodic linear map on the active cells (ghosts hold images); its transpose
// is applied in gather form to a ghost-filled adjoint field. Yee stencils only.
// ---------------------------------------------------------------------------

// lam(active, c < 3) = 2 h_c dV E_c: the gradient of the E part of the FP64
// energy of k_energy with respect to E; lam(active, c >= 3) = 0
template <int D, typename real>
__global__ void k_adj_seed(CellIter it, FieldView<real> EB, FieldView<real> lam, double dx) {
  const double  dV     = D == 3 ? dx * dx * dx : dx * dx;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < it.count; t += stride) {
    int i1, i2, i3;
    it.cell(t, i1, i2, i3);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double h = (c < D) ? dx * dx : 1.0;
      lam.p[lam.idx(i1, i2, i3, c)] = (real)(2.0 * h * dV * (double)EB.p[EB.idx(i1, i2, i3, c)]);
      lam.p[lam.idx(i1, i2, i3, c + 3)] = (real)0;
    }
  }
}

// transpose of CurrentsAmpere's E += jcoeff * J: lamJ = jcoeff * lamE at the
// active cells and their images
template <int D, typename real>
__global__ void k_adj_currents(GridInfo g, CellIter it, FieldView<real> lam, FieldView<real> lamJ,
                               real jcoeff) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < it.count; t += stride) {
    int i1, i2, i3;
    it.cell(t, i1, i2, i3);
    real v[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v[c]                              = jcoeff * lam.p[lam.idx(i1, i2, i3, c)];
      lamJ.p[lamJ.idx(i1, i2, i3, c)] = v[c];
    }
    for_images<D>(g, i1, i2, i3, [&](int a, int b, int e) {
#pragma unroll
      for (int c = 0; c < 3; ++c) lamJ.p[lamJ.idx(a, b, e, c)] = v[c];
    });
  }
}

// transpose of k_ampere's curl: lamB(active) += A^T lamE (lamE ghost-filled)
template <int D, typename real>
__global__ void k_adj_ampere(CellIter it, FieldView<real> lam, real a1, real a2) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < it.count; t += stride) {
    int i, j, k;
    it.cell(t, i, j, k);
#define L(a, b, c, comp) lam.p[lam.idx(a, b, c, comp)]
    if constexpr (D == 2) {
      L(i, j, 0, 5) += a1 * (L(i, j, 0, 0) - L(i, j + 1, 0, 0)) + a1 * (L(i + 1, j, 0, 1) - L(i, j, 0, 1));
      L(i, j, 0, 3) += a2 * (L(i, j + 1, 0, 2) - L(i, j, 0, 2));
      L(i, j, 0, 4) += a2 * (L(i, j, 0, 2) - L(i + 1, j, 0, 2));
    } else {
      L(i, j, k, 3) += a1 * (L(i, j, k, 1) - L(i, j, k + 1, 1)) + a1 * (L(i, j + 1, k, 2) - L(i, j, k, 2));
      L(i, j, k, 4) += a1 * (L(i, j, k + 1, 0) - L(i, j, k, 0)) + a1 * (L(i, j, k, 2) - L(i + 1, j, k, 2));
      L(i, j, k, 5) += a1 * (L(i, j, k, 0) - L(i, j + 1, k, 0)) + a1 * (L(i + 1, j, k, 1) - L(i, j, k, 1));
    }
#undef L
  }
}

// transpose of k_faraday (Yee): lamE(active) += F^T lamB (lamB ghost-filled)
template <int D, typename real>
__global__ void k_adj_faraday(CellIter it, FieldView<real> lam, real c1, real c2) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < it.count; t += stride) {
    int i, j, k;
    it.cell(t, i, j, k);
#define L(a, b, c, comp) lam.p[lam.idx(a, b, c, comp)]
    if constexpr (D == 2) {
      L(i, j, 0, 2) += c1 * (L(i, j, 0, 3) - L(i, j - 1, 0, 3)) + c1 * (L(i - 1, j, 0, 4) - L(i, j, 0, 4));
      L(i, j, 0, 0) += c2 * (L(i, j - 1, 0, 5) - L(i, j, 0, 5));
      L(i, j, 0, 1) += c2 * (L(i, j, 0, 5) - L(i - 1, j, 0, 5));
    } else {
      L(i, j, k, 0) += c1 * (L(i, j, k, 4) - L(i, j, k - 1, 4)) + c1 * (L(i, j - 1, k, 5) - L(i, j, k, 5));
      L(i, j, k, 1) += c1 * (L(i, j, k - 1, 3) - L(i, j, k, 3)) + c1 * (L(i, j, k, 5) - L(i - 1, j, k, 5));
      L(i, j, k, 2) += c1 * (L(i, j, k, 3) - L(i, j - 1, k, 3)) + c1 * (L(i - 1, j, k, 4) - L(i, j, k, 4));
    }
#undef L
  }
}

// transpose of the ghost fill: every active cell adds the values its ghost
// images accumulated (components [c0, c1)) and clears them
template <int D, typename real>
__global__ void k_adj_fold(GridInfo g, CellIter it, FieldView<real> f, int c0, int c1) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < it.count; t += stride) {
    int i1, i2, i3;
    it.cell(t, i1, i2, i3);
    if (!near_periodic_edge(g, D, i1, i2, i3)) continue;
    // each ghost cell is the image of exactly one active cell, so the
    // thread that folds it may also clear it
    for (int c = c0; c < c1; ++c) {
      real acc = 0;
      for_images<D>(g, i1, i2, i3, [&](int a, int b, int e) {
        real* q = f.p + f.idx(a, b, e, c);
        acc += *q;
        *q = (real)0;
      });
      f.p[f.idx(i1, i2, i3, c)] += acc;
    }
  }
}

// zero the ghost cells of components [c0, c1)
template <typename real>
__global__ void k_zero_ghosts(GridInfo g, FieldView<real> f, int c0, int c1) {
  const int     e0 = g.n[0] + 2 * g.ng, e1 = g.n[1] + 2 * g.ng;
  const int     e2 = g.dim == 3 ? g.n[2] + 2 * g.ng : 1;
  const int64_t count  = (int64_t)e0 * e1 * e2;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += stride) {
    int64_t   r = t;
    const int i = (int)(r % e0);
    r /= e0;
    const int j = (int)(r % e1);
    const int k = (int)(r / e1);
    const bool ghost = i < g.ng || i >= g.n[0] + g.ng || j < g.ng || j >= g.n[1] + g.ng ||
                       (g.dim == 3 && (k < g.ng || k >= g.n[2] + g.ng));
    if (!ghost) continue;
    for (int c = c0; c < c1; ++c) f.p[f.idx(i, j, k, c)] = (real)0;
  }
}

template <typename real>
cudaError_t launch_adj_seed(const GridInfo& g, FieldView<real> EB, FieldView<real> lam, double dx,
                            cudaStream_t s) {
  const CellIter it = make_iter(g);
  if (g.dim == 2) PIC_KL(k_adj_seed<2, real><<<grid_for(it.count, 256), 256, 0, s>>>(it, EB, lam, dx));
  else            PIC_KL(k_adj_seed<3, real><<<grid_for(it.count, 256), 256, 0, s>>>(it, EB, lam, dx));
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_adj_currents(const GridInfo& g, FieldView<real> lam, FieldView<real> lamJ,
                                real jcoeff, cudaStream_t s) {
  const CellIter it = make_iter(g);
  if (g.dim == 2) PIC_KL(k_adj_currents<2, real><<<grid_for(it.count, 256), 256, 0, s>>>(g, it, lam, lamJ, jcoeff));
  else            PIC_KL(k_adj_currents<3, real><<<grid_for(it.count, 256), 256, 0, s>>>(g, it, lam, lamJ, jcoeff));
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_adj_ampere(const GridInfo& g, FieldView<real> lam, real a1, real a2,
                              cudaStream_t s) {
  const CellIter it = make_iter(g);
  if (g.dim == 2) PIC_KL(k_adj_ampere<2, real><<<grid_for(it.count, 256), 256, 0, s>>>(it, lam, a1, a2));
  else            PIC_KL(k_adj_ampere<3, real><<<grid_for(it.count, 256), 256, 0, s>>>(it, lam, a1, a2));
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_adj_faraday(const GridInfo& g, FieldView<real> lam, real c1, real c2,
                               cudaStream_t s) {
  const CellIter it = make_iter(g);
  if (g.dim == 2) PIC_KL(k_adj_faraday<2, real><<<grid_for(it.count, 256), 256, 0, s>>>(it, lam, c1, c2));
  else            PIC_KL(k_adj_faraday<3, real><<<grid_for(it.count, 256), 256, 0, s>>>(it, lam, c1, c2));
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_adj_fold(const GridInfo& g, FieldView<real> f, int c0, int c1, cudaStream_t s) {
  const CellIter it = make_iter(g);
  if (g.dim == 2) PIC_KL(k_adj_fold<2, real><<<grid_for(it.count, 256), 256, 0, s>>>(g, it, f, c0, c1));
  else            PIC_KL(k_adj_fold<3, real><<<grid_for(it.count, 256), 256, 0, s>>>(g, it, f, c0, c1));
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_zero_ghosts(const GridInfo& g, FieldView<real> f, int c0, int c1,
                               cudaStream_t s) {
  const int64_t cells = (int64_t)(g.n[0] + 2 * g.ng) * (g.n[1] + 2 * g.ng) *
                        (g.dim == 3 ? g.n[2] + 2 * g.ng : 1);
  PIC_KL(k_zero_ghosts<real><<<grid_for(cells, 256), 256, 0, s>>>(g, f, c0, c1));
  return cudaGetLastError();
}

#define PIC_INST_ADJ_FIELDS(R)                                                                     \
  template cudaError_t launch_adj_seed<R>(const GridInfo&, FieldView<R>, FieldView<R>, double,     \
                                          cudaStream_t);                                           \
  template cudaError_t launch_adj_currents<R>(const GridInfo&, FieldView<R>, FieldView<R>, R,      \
                                              cudaStream_t);                                       \
  template cudaError_t launch_adj_ampere<R>(const GridInfo&, FieldView<R>, R, R, cudaStream_t);    \
  template cudaError_t launch_adj_faraday<R>(const GridInfo&, FieldView<R>, R, R, cudaStream_t);   \
  template cudaError_t launch_adj_fold<R>(const GridInfo&, FieldView<R>, int, int, cudaStream_t);  \
  template cudaError_t launch_zero_ghosts<R>(const GridInfo&, FieldView<R>, int, int, cudaStream_t);
PIC_INST_ADJ_FIELDS(float)
PIC_INST_ADJ_FIELDS(double)

#define PIC_INST_FIELDS(R)                                                                       \
  template cudaError_t launch_faraday<R>(const GridInfo&, FieldView<R>, R, R, const Stencil<R>&, \
                                         bool, cudaStream_t);                                    \
  template cudaError_t launch_ampere<R>(const GridInfo&, FieldView<R>, FieldView<R>, R, R, R, R, \
                                        bool, bool, bool, cudaStream_t);                         \
  template cudaError_t launch_sync_currents<R>(const GridInfo&, FieldView<R>, cudaStream_t);     \
  template cudaError_t launch_fill_ghosts<R>(const GridInfo&, FieldView<R>, int, int,            \
                                             cudaStream_t);                                      \
  template cudaError_t launch_filter<R>(const GridInfo&, FieldView<R>, FieldView<R>, int,        \
                                        cudaStream_t);                                           \
  template cudaError_t launch_zero3<R>(const GridInfo&, FieldView<R>, cudaStream_t);             \
  template cudaError_t launch_copy3<R>(const GridInfo&, FieldView<R>, FieldView<R>, cudaStream_t); \
  template cudaError_t launch_energy<R>(const GridInfo&, FieldView<R>, double, double*,          \
                                        cudaStream_t);

PIC_INST_FIELDS(float)
PIC_INST_FIELDS(double)

}  // namespace pic
