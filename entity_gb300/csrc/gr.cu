// GR particle-in-cell kernels on a 2D quasi-spherical Kerr-Schild grid
// (r, theta) and their C ABI:
//   - pusher (kernel::gr::Pusher_kernel, src/kernels/pushers/gr.hpp:664-865):
//     shape-order interpolation of D (em) and B (em0), half E push, implicit
//     geodesic momentum push, half E push, implicit coordinate push, the
//     absorbing-r / axis-theta particle boundaries. Particles within a few
//     cells of the horizon (the FP64 island, island_lo <= i1 < island_hi)
//     run the metric and both implicit iterations in double, in a kernel of
//     their own that overlaps the single-precision bulk;
//   - current deposit (DepositCurrents_kernel, GR branch, shape order 1,
//     currents_deposit.hpp:138-159) with the metric out-of-plane velocity;
//   - field kernels (faraday_gr.hpp, ampere_gr.hpp, aux_fields_gr.hpp) and
//     the axis / horizon boundaries (fields_bcs.hpp:825-868, 1188-1240).
// Metric values are evaluated at the staggered points they are needed at;
// one thread per particle or per cell.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx_internal.cuh"
#include "fields.cuh"
#include "gr_host.cuh"
#include "gr_metric.cuh"
#include "pic_common.cuh"

using namespace pic_internal;

namespace pic {

// ---------------------------------------------------------------------------
// pusher
// ---------------------------------------------------------------------------
template <typename real>
struct GRPushArgs {
  SpeciesPtrs     sp;
  FieldView<real> em, em0;
  QKS<double>     m;
  int             n1, n2, ng;
  int             absorb_min, absorb_max, axis_min, axis_max;
  real            dt, ndth;
  int             niter, island_lo, island_hi, massive;
  unsigned long long* err;
  int32_t*        list;        // island indices, or null: no island split
  unsigned*       list_count;  // [0] list length, [1] island work cursor
  unsigned*       mask;        // bit p: particle p is on the list
};

// D from em (components 0..2) and B from em0 (3..5) at the particle
// (gr.hpp:594-662), running sums as fma like the SR interpolation
template <int O, typename real>
__device__ __forceinline__ void interp_db(const FieldView<real>& em, const FieldView<real>& em0,
                                          const int* ic, const real* dc, real* Dv, real* Bv) {
  int  pmin[2], dmin[2];
  real Sp[2][O + 1], Sd[2][O + 1];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    shape<O, false>(ic[a], dc[a], pmin[a], Sp[a]);
    shape<O, true>(ic[a], dc[a], dmin[a], Sd[a]);
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const FieldView<real>& F = c < 3 ? em : em0;
    const int s0 = stag_of(c, 0), s1 = stag_of(c, 1);
    const int m0 = s0 ? dmin[0] : pmin[0], m1 = s1 ? dmin[1] : pmin[1];
    real      v  = 0;
#pragma unroll
    for (int b = 0; b < O + 1; b++) {
      real c0 = 0;
#pragma unroll
      for (int a = 0; a < O + 1; a++) c0 = iacc(s0 ? Sd[0][a] : Sp[0][a], F.ld(m0 + a, m1 + b, 0, c), c0);
      v = iacc(c0, s1 ? Sd[1][b] : Sp[1][b], v);
    }
    if (c < 3) Dv[c] = v;
    else Bv[c - 3] = v;
  }
}

// EMHalfPush (gr.hpp:177-217), metric at the particle
template <typename M>
__device__ __forceinline__ void em_half_push(const QMet<M>& g, M ndth, const M* vp, const M* Dh,
                                             const M* Bh, M* vout) {
  M D0[3] = { Dh[0], Dh[1], Dh[2] }, B0[3] = { Bh[0], Bh[1], Bh[2] }, vh[3], vph[3];
  d_to_t(g, vp, vh);
  M COEFF = ndth * (M)0.5 * g.alpha;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    D0[c] *= COEFF;
    vh[c] += D0[c];
  }
  COEFF *= (M)1 / sqrt((M)1 + vh[0] * vh[0] + vh[1] * vh[1] + vh[2] * vh[2]);
#pragma unroll
  for (int c = 0; c < 3; ++c) B0[c] *= COEFF;
  COEFF  = (M)2 / ((M)1 + B0[0] * B0[0] + B0[1] * B0[1] + B0[2] * B0[2]);
  vph[0] = (vh[0] + vh[1] * B0[2] - vh[2] * B0[1]) * COEFF;
  vph[1] = (vh[1] + vh[2] * B0[0] - vh[0] * B0[2]) * COEFF;
  vph[2] = (vh[2] + vh[0] * B0[1] - vh[1] * B0[0]) * COEFF;
  vh[0] += vph[1] * B0[2] - vph[2] * B0[1] + D0[0];
  vh[1] += vph[2] * B0[0] - vph[0] * B0[2] + D0[1];
  vh[2] += vph[0] * B0[1] - vph[1] * B0[0] + D0[2];
  t_to_d(g, vh, vout);
}

template <typename M>
__device__ __forceinline__ M gamma_of(bool massive, const M* uc, const M* uu) {
  const M s = uc[0] * uu[0] + uc[1] * uu[1] + uc[2] * uu[2];
  return massive ? sqrt((M)1 + s) : sqrt(s);
}

// GeodesicMomentumPush (gr.hpp:260-331): the metric and its derivatives at
// the (fixed) position are formed once for all iterations
template <typename M>
__device__ __forceinline__ void geo_momentum(const QKS<M>& m, bool massive, M dt, int niter,
                                             const M* xp, const M* vp, M* vu) {
  const QPt<M>  p  = qpt(m, xp[0], xp[1]);
  const QMet<M> g  = qmet(m, p);
  const M d_al[2] = { dr_alpha(m, p), dt_alpha(m, p) };
  const M d_be[2] = { dr_beta1(m, p), dt_beta1(m, p) };
  const M d_11[2] = { dr_h11(m, p), dt_h11(m, p) };
  const M d_22[2] = { dr_h22(m, p), dt_h22(m, p) };
  const M d_33[2] = { dr_h33(m, p), dt_h33(m, p) };
  const M d_13[2] = { dr_h13(m, p), dt_h13(m, p) };
  vu[0] = vp[0], vu[1] = vp[1], vu[2] = vp[2];
  for (int it = 0; it < niter; ++it) {
    const M vm[3] = { (M)0.5 * (vp[0] + vu[0]), (M)0.5 * (vp[1] + vu[1]), vp[2] };
    M       vmc[3];
    d_to_u(g, vm, vmc);
    const M u0 = gamma_of(massive, vm, vmc) / g.alpha;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      vu[k] = vp[k] + dt * (-g.alpha * u0 * d_al[k] + vm[0] * d_be[k] -
                            ((M)0.5 / u0) *
                              (d_11[k] * (vm[0] * vm[0]) + d_22[k] * (vm[1] * vm[1]) +
                               d_33[k] * (vm[2] * vm[2]) + (M)2 * d_13[k] * vm[0] * vm[2]));
    }
  }
}

// GeodesicCoordinatePush (gr.hpp:333-383)
template <typename M>
__device__ __forceinline__ void geo_coordinate(const QKS<M>& m, bool massive, M dt, int niter,
                                               const M* xp, const M* vp, M* xu) {
  xu[0] = xp[0], xu[1] = xp[1];
  for (int it = 0; it < niter; ++it) {
    const M       xm0 = (M)0.5 * (xp[0] + xu[0]);
    const M       xm1 = m.clamp_x2((M)0.5 * (xp[1] + xu[1]));
    const QPt<M>  p   = qpt(m, xm0, xm1);
    const QMet<M> g   = qmet(m, p);
    M             vc[3];
    d_to_u(g, vp, vc);
    const M u0 = gamma_of(massive, vp, vc) / g.alpha;
    xu[0] = xp[0] + dt * (vc[0] / u0 - g.beta1);
    xu[1] = xp[1] + dt * (vc[1] / u0);
  }
}

template <typename M>
__device__ __forceinline__ void gr_push_one(const QKS<M>& m, bool massive, M ndth, M dt, int niter,
                                            const M* xp, const M* Dc, const M* Bc, const M* u,
                                            M* xo, M* uo) {
  M vp[3] = { u[0], u[1], u[2] }, vu[3];
  if (massive) {
    const M       xq[2] = { xp[0], m.clamp_x2(xp[1]) };
    const QMet<M> g     = qmet(m, qpt(m, xp[0], xp[1]));
    M             Dh[3], Bh[3];
    u_to_t(g, Dc, Dh);
    u_to_t(g, Bc, Bh);
    em_half_push(g, ndth, vp, Dh, Bh, vu);
    vp[0] = vu[0], vp[1] = vu[1], vp[2] = vu[2];
    geo_momentum(m, true, dt, niter, xq, vp, vu);
    vp[0] = vu[0], vp[1] = vu[1], vp[2] = vu[2];
    em_half_push(g, ndth, vp, Dh, Bh, vu);
    geo_coordinate(m, true, dt, niter, xp, vu, xo);
  } else {
    geo_momentum(m, false, dt, niter, xp, vp, vu);
    geo_coordinate(m, false, dt, niter, xp, vu, xo);
  }
  uo[0] = vu[0], uo[1] = vu[1], uo[2] = vu[2];
}

// one particle: interpolation, the push in the island's or the field
// precision, the particle boundaries (gr.hpp:664-865)
template <int O, bool ISLAND, typename real>
__device__ __forceinline__ void gr_push_particle(const GRPushArgs<real>& a, int64_t p) {
  real* ux[3] = { (real*)a.sp.ux1, (real*)a.sp.ux2, (real*)a.sp.ux3 };
  const int   i1 = a.sp.i1[p], i2 = a.sp.i2[p];
  const float d1 = a.sp.dx1[p], d2 = a.sp.dx2[p];
  if (i1 < 0 || i1 >= a.n1 || i2 < 0 || i2 >= a.n2) {
    atomicAdd(a.err + ERR_OUT_OF_GRID, 1ull);
    return;
  }
  a.sp.i1p[p]  = i1;
  a.sp.i2p[p]  = i2;
  a.sp.dx1p[p] = d1;
  a.sp.dx2p[p] = d2;
  real Dc[3] = { 0, 0, 0 }, Bc[3] = { 0, 0, 0 };
  if (a.massive) {
    const int  ic[2] = { i1 + a.ng, i2 + a.ng };
    const real dc[2] = { (real)d1, (real)d2 };
    interp_db<O, real>(a.em, a.em0, ic, dc, Dc, Bc);
  }
  // i_di_to_Xi in real_t (gr.hpp:45)
  const real X0 = (real)i1 + (real)d1, X1 = (real)i2 + (real)d2;
  real       xo[2], uo[3];
  if (ISLAND) {
    const double xp[2] = { (double)X0, (double)X1 };
    const double Dd[3] = { (double)Dc[0], (double)Dc[1], (double)Dc[2] };
    const double Bd[3] = { (double)Bc[0], (double)Bc[1], (double)Bc[2] };
    const double ud[3] = { (double)ux[0][p], (double)ux[1][p], (double)ux[2][p] };
    double       xd[2], uo_d[3];
    gr_push_one<double>(a.m, a.massive, (double)a.ndth, (double)a.dt, a.niter, xp, Dd, Bd, ud, xd,
                        uo_d);
    xo[0] = (real)xd[0], xo[1] = (real)xd[1];
    uo[0] = (real)uo_d[0], uo[1] = (real)uo_d[1], uo[2] = (real)uo_d[2];
  } else {
    const QKS<real> m     = a.m.template as<real>();
    const real      xp[2] = { X0, X1 };
    const real      ur[3] = { ux[0][p], ux[1][p], ux[2][p] };
    gr_push_one<real>(m, a.massive, a.ndth, a.dt, a.niter, xp, Dc, Bc, ur, xo, uo);
  }
  // from_Xi_to_i_di (gr.hpp:34-43)
  int     j1 = (int)(xo[0] + (real)1) - 1, j2 = (int)(xo[1] + (real)1) - 1;
  float   e1 = (float)xo[0] - (float)j1, e2 = (float)xo[1] - (float)j2;
  int16_t ntag = PIC_TAG_ALIVE;
  // boundaryConditions (gr.hpp:818-865)
  if ((j1 < 0 && a.absorb_min) || (j1 >= a.n1 && a.absorb_max)) ntag = PIC_TAG_DEAD;
  if (j2 < 0) {
    if (a.axis_min) {
      j2    = 0;
      e2    = 1.0f - e2;
      uo[1] = -uo[1];
    }
  } else if (j2 >= a.n2) {
    if (a.axis_max) {
      j2    = a.n2 - 1;
      e2    = 1.0f - e2;
      uo[1] = -uo[1];
    }
  }
  a.sp.i1[p]  = j1;
  a.sp.i2[p]  = j2;
  a.sp.dx1[p] = e1;
  a.sp.dx2[p] = e2;
  ux[0][p] = uo[0], ux[1][p] = uo[1], ux[2][p] = uo[2];
  if (ntag != PIC_TAG_ALIVE) a.sp.tag[p] = ntag;
}

template <typename real>
__device__ __forceinline__ bool in_island(const GRPushArgs<real>& a, int i1) {
  return i1 >= a.island_lo && i1 < a.island_hi;
}

// Live particles of the FP64 island appended to a.list (warp-aggregated
// atomics), ahead of the two push kernels, and marked in a.mask: the two
// kernels run at once and the island kernel moves its particles, so the
// bulk decides membership from the mask, never from i1. A warp covers 32
// consecutive particles starting at a multiple of 32 (block size and grid
// stride are multiples of 32), and its ballot is their mask word.
template <typename real>
__global__ void __launch_bounds__(256) k_gr_island_list(GRPushArgs<real> a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int     lane   = threadIdx.x & 31;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.sp.npart; p += stride) {
    const bool     isl = a.sp.tag[p] == PIC_TAG_ALIVE && in_island(a, a.sp.i1[p]);
    const unsigned act = __activemask();
    const unsigned bal = __ballot_sync(act, isl);
    if (lane == __ffs(act) - 1) a.mask[p >> 5] = bal;
    if (bal) {
      const int leader = __ffs(bal) - 1;
      unsigned  base   = 0;
      if (lane == leader) base = atomicAdd(a.list_count, (unsigned)__popc(bal));
      base = __shfl_sync(act, base, leader);
      if (isl) a.list[base + __popc(bal & ((1u << lane) - 1u))] = (int32_t)p;
    }
  }
}

// The bulk: every live particle outside the island, in the field
// precision. With a.list null (FP64 fields, or no island) every particle is
// pushed here. It asks for three CTAs per SM (80 registers instead of the
// allocator's 120, a 12-byte spill at order 2): the Wald problem's
// push+deposit went from 0.718 to 0.608 ms per step; the island kernel at
// four CTAs of 128 spilled and lost.
template <int O, typename real>
__global__ void __launch_bounds__(256, 3) k_gr_push(GRPushArgs<real> a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.sp.npart; p += stride) {
    const int16_t tag = a.sp.tag[p];
    if (tag != PIC_TAG_ALIVE) {
      if (tag != PIC_TAG_DEAD) atomicAdd(a.err + ERR_BAD_TAG, 1ull);
      continue;
    }
    if (a.list != nullptr && ((a.mask[p >> 5] >> (p & 31)) & 1u)) continue;
    gr_push_particle<O, false, real>(a, p);
  }
}

// The island list, in chunks of 32 entries handed out to warps by a device
// cursor: each warp takes chunks until the list (read once) is exhausted.
// Island particles are cell-sorted into a few contiguous blocks of the
// particle arrays; pushed in place, their FP64 work (GB300 runs FP64 at
// 1/64 of the FP32 rate) would sit on the few SMs holding those blocks. This
// kernel runs on a second stream beside the bulk, so the FP64 and FP32 pipes
// work at once.
template <int O, typename real>
__global__ void __launch_bounds__(128, 3) k_gr_push_island(GRPushArgs<real> a) {
  const int      lane = threadIdx.x & 31;
  const unsigned n    = a.list_count[0];
  for (;;) {
    unsigned chunk = 0;
    if (lane == 0) chunk = atomicAdd(a.list_count + 1, 1u);
    chunk = __shfl_sync(0xffffffffu, chunk, 0);
    if ((uint64_t)chunk * 32u >= n) break;
    const unsigned j = chunk * 32u + (unsigned)lane;
    if (j < n) gr_push_particle<O, true, real>(a, a.list[j]);
  }
}

// ---------------------------------------------------------------------------
// deposit (shape order 1, the reference's GR default)
// ---------------------------------------------------------------------------
template <typename real>
struct GRDepArgs {
  SpeciesPtrs     sp;
  FieldView<real> J;
  QKS<double>     m;
  int             ng, island_lo, island_hi;
  int             ext[3];
  real            inv_dt, charge;
  unsigned long long* err;
};

template <typename M>
__device__ __forceinline__ M gr_vz(const QKS<M>& m, M X0, M X1, const M* u) {
  const QMet<M> g = qmet(m, qpt(m, X0, m.clamp_x2(X1)));
  M             vp[3];
  d_to_u(g, u, vp);
  const M inv_energy = g.alpha / sqrt((M)1 + u[0] * vp[0] + u[1] * vp[1] + u[2] * vp[2]);
  if (isnan(vp[2]) || isinf(vp[2])) vp[2] = (M)0;
  return vp[2] * inv_energy;
}

template <typename real>
__global__ void __launch_bounds__(256) k_gr_deposit(GRDepArgs<real> a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const real*   ux[3]  = { (const real*)a.sp.ux1, (const real*)a.sp.ux2, (const real*)a.sp.ux3 };
  const real*   w      = (const real*)a.sp.w;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.sp.npart; p += stride) {
    if (a.sp.tag[p] == PIC_TAG_DEAD) continue;
    Prtl<real> q;
    q.i[0] = a.sp.i1[p], q.i[1] = a.sp.i2[p], q.i[2] = 0;
    q.dx[0] = a.sp.dx1[p], q.dx[1] = a.sp.dx2[p], q.dx[2] = 0.0f;
    q.ip[0] = a.sp.i1p[p], q.ip[1] = a.sp.i2p[p], q.ip[2] = 0;
    q.dxp[0] = a.sp.dx1p[p], q.dxp[1] = a.sp.dx2p[p], q.dxp[2] = 0.0f;
    const real X0 = (real)q.i[0] + (real)q.dx[0], X1 = (real)q.i[1] + (real)q.dx[1];
    real       vp[3] = { 0, 0, 0 };
    if (q.i[0] >= a.island_lo && q.i[0] < a.island_hi) {
      const double ud[3] = { (double)ux[0][p], (double)ux[1][p], (double)ux[2][p] };
      vp[2]              = (real)gr_vz<double>(a.m, (double)X0, (double)X1, ud);
    } else {
      const real ur[3] = { ux[0][p], ux[1][p], ux[2][p] };
      vp[2]            = gr_vz<real>(a.m.template as<real>(), X0, X1, ur);
    }
    const FieldView<real>& J = a.J;
    const bool ok = deposit_with_velocity<2, 1, real>(q, vp, w[p], a.charge, a.inv_dt, a.ng, a.ext,
                                                      [&](int i, int j, int k, int c, real v) {
                                                        atomicAdd(J.p + J.idx(i, j, k, c), v);
                                                      });
    if (!ok) atomicAdd(a.err + ERR_STENCIL_OUT, 1ull);
  }
}

// ---------------------------------------------------------------------------
// field kernels (one thread per cell of the kernel's range)
// ---------------------------------------------------------------------------
struct Range2 {
  int i0, i1, j0, j1;  // [i0, i1) x [j0, j1), ghost-inclusive indices
  __host__ __device__ __forceinline__ int64_t count() const { return (int64_t)(i1 - i0) * (j1 - j0); }
};

#define GR_CELL_LOOP(R)                                                                    \
  const int64_t stride_ = (int64_t)gridDim.x * blockDim.x;                                 \
  for (int64_t t_ = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t_ < (R).count();      \
       t_ += stride_) {                                                                    \
    const int i1 = (R).i0 + (int)(t_ % ((R).i1 - (R).i0));                                 \
    const int i2 = (R).j0 + (int)(t_ / ((R).i1 - (R).i0));

template <typename real>
struct GRFld {
  QKS<double>     m;
  int             ng, n1, n2, axis_min, axis_max;
};

// Faraday_kernel (faraday_gr.hpp:62-90): Bout = Bin + coeff curl E
template <typename real>
__global__ void k_gr_faraday(GRFld<real> f, Range2 R, FieldView<real> Bin, FieldView<real> Bout,
                             FieldView<real> E, real coeff) {
  const QKS<real> m = f.m.template as<real>();
  const real      H = 0.5;
  GR_CELL_LOOP(R)
    const real i1_ = (real)(i1 - f.ng), i2_ = (real)(i2 - f.ng);
    const real inv_0pH  = (real)1 / sqrt_det_h(m, qpt(m, i1_, i2_ + H));
    const real inv_pHpH = (real)1 / sqrt_det_h(m, qpt(m, i1_ + H, i2_ + H));
    Bout.p[Bout.idx(i1, i2, 0, 3)] = Bin.p[Bin.idx(i1, i2, 0, 3)] +
                                     coeff * inv_0pH * (E.p[E.idx(i1, i2, 0, 2)] - E.p[E.idx(i1, i2 + 1, 0, 2)]);
    if (i2 == f.ng && f.axis_min) {
      Bout.p[Bout.idx(i1, i2, 0, 4)] = (real)0;
    } else {
      const real inv_pH0 = (real)1 / sqrt_det_h(m, qpt(m, i1_ + H, i2_));
      Bout.p[Bout.idx(i1, i2, 0, 4)] =
        Bin.p[Bin.idx(i1, i2, 0, 4)] +
        coeff * inv_pH0 * (E.p[E.idx(i1 + 1, i2, 0, 2)] - E.p[E.idx(i1, i2, 0, 2)]);
    }
    Bout.p[Bout.idx(i1, i2, 0, 5)] =
      Bin.p[Bin.idx(i1, i2, 0, 5)] +
      coeff * inv_pHpH *
        (E.p[E.idx(i1, i2 + 1, 0, 0)] - E.p[E.idx(i1, i2, 0, 0)] + E.p[E.idx(i1, i2, 0, 1)] -
         E.p[E.idx(i1 + 1, i2, 0, 1)]);
  }
}

// Ampere_kernel (ampere_gr.hpp:66-98) except the axis copies of dx1
template <typename real>
__global__ void k_gr_ampere(GRFld<real> f, Range2 R, FieldView<real> Din, FieldView<real> Dout,
                            FieldView<real> Hf, real coeff) {
  const QKS<real> m = f.m.template as<real>();
  const real      H = 0.5;
  const int       i2min = f.ng, i2max = f.n2 + f.ng;
  GR_CELL_LOOP(R)
    const real i1_ = (real)(i1 - f.ng), i2_ = (real)(i2 - f.ng);
#define HH(a, b, c) Hf.p[Hf.idx(a, b, 0, c)]
    if (i2 == i2min && f.axis_min) {
      const real inv = (real)1 / sqrt_det_h(m, qpt(m, i1_, H));
      Dout.p[Dout.idx(i1, i2, 0, 1)] = Din.p[Din.idx(i1, i2, 0, 1)] +
                                       coeff * inv * (HH(i1 - 1, i2, 5) - HH(i1, i2, 5));
    } else if (i2 == i2max && f.axis_max) {
    } else {
      const real inv_0pH = (real)1 / sqrt_det_h(m, qpt(m, i1_, i2_ + H));
      const real inv_00  = (real)1 / sqrt_det_h(m, qpt(m, i1_, i2_));
      const real inv_pH0 = (real)1 / sqrt_det_h(m, qpt(m, i1_ + H, i2_));
      Dout.p[Dout.idx(i1, i2, 0, 0)] = Din.p[Din.idx(i1, i2, 0, 0)] +
                                       coeff * inv_pH0 * (HH(i1, i2, 5) - HH(i1, i2 - 1, 5));
      Dout.p[Dout.idx(i1, i2, 0, 1)] = Din.p[Din.idx(i1, i2, 0, 1)] +
                                       coeff * inv_0pH * (HH(i1 - 1, i2, 5) - HH(i1, i2, 5));
      Dout.p[Dout.idx(i1, i2, 0, 2)] =
        Din.p[Din.idx(i1, i2, 0, 2)] +
        coeff * inv_00 * ((HH(i1, i2 - 1, 3) - HH(i1, i2, 3)) + (HH(i1, i2, 4) - HH(i1 - 1, i2, 4)));
    }
#undef HH
  }
}

// the axis cells' dx1 = the neighbouring row's (read after that row's update)
template <typename real>
__global__ void k_gr_ampere_axis(GRFld<real> f, FieldView<real> Din, FieldView<real> Dout,
                                 bool alias) {
  const int i1 = f.ng + blockIdx.x * blockDim.x + threadIdx.x;
  if (i1 >= f.n1 + f.ng) return;
  const FieldView<real>& src = alias ? Dout : Din;
  if (f.axis_min)
    Dout.p[Dout.idx(i1, f.ng, 0, 0)] = src.p[src.idx(i1, f.ng + 1, 0, 0)];
  if (f.axis_max)
    Dout.p[Dout.idx(i1, f.n2 + f.ng, 0, 0)] = src.p[src.idx(i1, f.n2 + f.ng - 1, 0, 0)];
}

// CurrentsAmpere_kernel (ampere_gr.hpp:143-172)
template <typename real>
__global__ void k_gr_currents_ampere(GRFld<real> f, Range2 R, FieldView<real> D,
                                     FieldView<real> J, real coeff) {
  const QKS<real> m = f.m.template as<real>();
  const real      H = 0.5;
  const int       i2min = f.ng, i2max = f.n2 + f.ng;
  GR_CELL_LOOP(R)
    const real i1_ = (real)(i1 - f.ng), i2_ = (real)(i2 - f.ng);
    const real inv_0pH = (real)1 / sqrt_det_h(m, qpt(m, i1_, i2_ + H));
    if (i2 == i2min && f.axis_min) {
      D.p[D.idx(i1, i2, 0, 0)] += J.p[J.idx(i1, i2, 0, 0)] * H * coeff / polar_area(m, i1_ + H);
      D.p[D.idx(i1, i2, 0, 1)] += J.p[J.idx(i1, i2, 0, 1)] * coeff * inv_0pH;
    } else if (i2 == i2max && f.axis_max) {
      D.p[D.idx(i1, i2, 0, 0)] += J.p[J.idx(i1, i2, 0, 0)] * H * coeff / polar_area(m, i1_ + H);
    } else {
      const real inv_00  = (real)1 / sqrt_det_h(m, qpt(m, i1_, i2_));
      const real inv_pH0 = (real)1 / sqrt_det_h(m, qpt(m, i1_ + H, i2_));
      D.p[D.idx(i1, i2, 0, 0)] += J.p[J.idx(i1, i2, 0, 0)] * coeff * inv_pH0;
      D.p[D.idx(i1, i2, 0, 1)] += J.p[J.idx(i1, i2, 0, 1)] * coeff * inv_0pH;
      D.p[D.idx(i1, i2, 0, 2)] += J.p[J.idx(i1, i2, 0, 2)] * coeff * inv_00;
    }
  }
}

// ComputeAuxE_kernel (aux_fields_gr.hpp:47-109)
template <typename real>
__global__ void k_gr_aux_e(GRFld<real> f, Range2 R, FieldView<real> Df, FieldView<real> Bf,
                           FieldView<real> Ef) {
  const QKS<real> m = f.m.template as<real>();
  const real      H = 0.5;
  GR_CELL_LOOP(R)
    const real i1_ = (real)(i1 - f.ng), i2_ = (real)(i2 - f.ng);
#define DD(a, b, c) Df.p[Df.idx(a, b, 0, c)]
#define BB(a, b, c) Bf.p[Bf.idx(a, b, 0, c)]
    const QPt<real> p_pH0 = qpt(m, i1_ + H, i2_), p_0pH = qpt(m, i1_, i2_ + H);
    const QPt<real> p_00 = qpt(m, i1_, i2_), p_mH0 = qpt(m, i1_ - H, i2_);
    const QPt<real> p_mHpH = qpt(m, i1_ - H, i2_ + H), p_pHpH = qpt(m, i1_ + H, i2_ + H);
    const QPt<real> p_10 = qpt(m, i1_ + (real)1, i2_);
    real w1 = sqrt_det_h_tilde(m, p_mH0), w2 = sqrt_det_h_tilde(m, p_pH0);
    real ww = (real)2 * sqrt_det_h_tilde(m, p_00);
    const real D1_half = (w1 * h_13(m, p_mH0) * DD(i1 - 1, i2, 0) + w2 * h_13(m, p_pH0) * DD(i1, i2, 0)) / ww;
    const real B2_half = (w1 * sqrt_det_h(m, p_mH0) * beta1(m, p_mH0) * BB(i1 - 1, i2, 4) +
                          w2 * sqrt_det_h(m, p_pH0) * beta1(m, p_pH0) * BB(i1, i2, 4)) / ww;
    w1 = sqrt_det_h_tilde(m, p_mHpH), w2 = sqrt_det_h_tilde(m, p_pHpH);
    ww = (real)2 * sqrt_det_h_tilde(m, p_0pH);
    const real B3_half = (w1 * sqrt_det_h(m, p_mHpH) * beta1(m, p_mHpH) * BB(i1 - 1, i2, 5) +
                          w2 * sqrt_det_h(m, p_pHpH) * beta1(m, p_pHpH) * BB(i1, i2, 5)) / ww;
    w1 = sqrt_det_h_tilde(m, p_00), w2 = sqrt_det_h_tilde(m, p_10);
    ww = (real)2 * sqrt_det_h_tilde(m, p_pH0);
    const real D3_half = (w1 * h_13(m, p_00) * DD(i1, i2, 2) + w2 * h_13(m, p_10) * DD(i1 + 1, i2, 2)) / ww;
    const real D1_cov = h_11(m, p_pH0) * DD(i1, i2, 0) + D3_half;
    const real D2_cov = h_22(m, p_0pH) * DD(i1, i2, 1);
    const real D3_cov = h_33(m, p_00) * DD(i1, i2, 2) + D1_half;
    Ef.p[Ef.idx(i1, i2, 0, 0)] = alpha(m, p_pH0) * D1_cov;
    Ef.p[Ef.idx(i1, i2, 0, 1)] = alpha(m, p_0pH) * D2_cov - B3_half;
    Ef.p[Ef.idx(i1, i2, 0, 2)] = alpha(m, p_00) * D3_cov + B2_half;
#undef DD
#undef BB
  }
}

// ComputeAuxH_kernel (aux_fields_gr.hpp:131-193)
template <typename real>
__global__ void k_gr_aux_h(GRFld<real> f, Range2 R, FieldView<real> Df, FieldView<real> Bf,
                           FieldView<real> Hf) {
  const QKS<real> m = f.m.template as<real>();
  const real      H = 0.5;
  GR_CELL_LOOP(R)
    const real i1_ = (real)(i1 - f.ng), i2_ = (real)(i2 - f.ng);
#define DD(a, b, c) Df.p[Df.idx(a, b, 0, c)]
#define BB(a, b, c) Bf.p[Bf.idx(a, b, 0, c)]
    const QPt<real> p_0pH = qpt(m, i1_, i2_ + H), p_pH0 = qpt(m, i1_ + H, i2_);
    const QPt<real> p_pHpH = qpt(m, i1_ + H, i2_ + H), p_1pH = qpt(m, i1_ + (real)1, i2_ + H);
    const QPt<real> p_00 = qpt(m, i1_, i2_), p_10 = qpt(m, i1_ + (real)1, i2_);
    const QPt<real> p_mHpH = qpt(m, i1_ - H, i2_ + H);
    real w1 = sqrt_det_h_tilde(m, p_0pH), w2 = sqrt_det_h_tilde(m, p_1pH);
    real ww = (real)2 * sqrt_det_h_tilde(m, p_pHpH);
    const real B1_half = (w1 * h_13(m, p_0pH) * BB(i1, i2, 3) + w2 * h_13(m, p_1pH) * BB(i1 + 1, i2, 3)) / ww;
    const real D2_half = (w1 * sqrt_det_h(m, p_0pH) * beta1(m, p_0pH) * DD(i1, i2, 1) +
                          w2 * sqrt_det_h(m, p_1pH) * beta1(m, p_1pH) * DD(i1 + 1, i2, 1)) / ww;
    w1 = sqrt_det_h_tilde(m, p_00), w2 = sqrt_det_h_tilde(m, p_10);
    ww = (real)2 * sqrt_det_h_tilde(m, p_pH0);
    const real D3_half = (w1 * sqrt_det_h(m, p_00) * beta1(m, p_00) * DD(i1, i2, 2) +
                          w2 * sqrt_det_h(m, p_10) * beta1(m, p_10) * DD(i1 + 1, i2, 2)) / ww;
    w1 = sqrt_det_h_tilde(m, p_mHpH), w2 = sqrt_det_h_tilde(m, p_pHpH);
    ww = (real)2 * sqrt_det_h_tilde(m, p_0pH);
    const real B3_half = (w1 * h_13(m, p_mHpH) * BB(i1 - 1, i2, 5) + w2 * h_13(m, p_pHpH) * BB(i1, i2, 5)) / ww;
    const real B1_cov = h_11(m, p_0pH) * BB(i1, i2, 3) + B3_half;
    const real B2_cov = h_22(m, p_pH0) * BB(i1, i2, 4);
    const real B3_cov = h_33(m, p_pHpH) * BB(i1, i2, 5) + B1_half;
    Hf.p[Hf.idx(i1, i2, 0, 3)] = alpha(m, p_0pH) * B1_cov;
    Hf.p[Hf.idx(i1, i2, 0, 4)] = alpha(m, p_pH0) * B2_cov + D3_half;
    Hf.p[Hf.idx(i1, i2, 0, 5)] = alpha(m, p_pHpH) * B3_cov - D2_half;
#undef DD
#undef BB
  }
}

// TimeAverageDB / TimeAverageJ (aux_fields_gr.hpp:222-280)
template <typename real>
__global__ void k_gr_average(Range2 R, FieldView<real> a, FieldView<real> b, int ncomp,
                             bool into_b) {
  GR_CELL_LOOP(R)
    for (int c = 0; c < ncomp; ++c) {
      const int64_t ia = a.idx(i1, i2, 0, c), ib = b.idx(i1, i2, 0, c);
      if (into_b) b.p[ib] = (real)0.5 * (b.p[ib] + a.p[ia]);   // f0 = (f0 + f) / 2
      else        a.p[ia] = (real)0.5 * (b.p[ib] + a.p[ia]);   // J = (J0 + J) / 2
    }
  }
}

// one pass of grpic::CurrentsFilter (src/engines/grpic/currents.h:74-101):
// DigitalFilter_kernel's 2D non-Cartesian branch (digital_filter.hpp:196-276)
// writes A from the copy B over i1 in [ng, ng + n1), i2 in [ng, ng + n2]
// (the range runs over the upper axis row); the rows next to an axis take the
// reference's one-sided theta weights, in its operation order
template <typename real>
__global__ void k_gr_filter(GRFld<real> f, Range2 R, FieldView<real> A, FieldView<real> B) {
  const real ZERO = 0, INV_2 = 0.5, INV_4 = 0.25, INV_8 = 0.125, INV_16 = 0.0625;
  const int  i2min = f.ng, i2max = f.n2 + f.ng;
#define BB(a, b, c) B.p[B.idx(a, b, 0, c)]
#define F1(c, a, b) (INV_2 * BB(a, b, c) + INV_4 * (BB((a) - 1, b, c) + BB((a) + 1, b, c)))
  GR_CELL_LOOP(R)
    real c00, c0p1, c0m1;
    if (f.axis_min && i2 == i2min) {
      c00  = F1(0, i1, i2);
      c0p1 = F1(0, i1, i2 + 1);
      A.p[A.idx(i1, i2, 0, 0)] = INV_2 * c00 + INV_2 * c0p1;
      A.p[A.idx(i1, i2, 0, 2)] = ZERO;
      c00  = F1(1, i1, i2);
      c0p1 = F1(1, i1, i2 + 1);
      A.p[A.idx(i1, i2, 0, 1)] = INV_4 * (c00 + c0p1);
    } else if (f.axis_min && i2 == i2min + 1) {
      c00  = F1(0, i1, i2);
      c0p1 = F1(0, i1, i2 + 1);
      c0m1 = F1(0, i1, i2 - 1);
      A.p[A.idx(i1, i2, 0, 0)] = INV_2 * c00 + INV_4 * (c0p1 + c0m1);
      c00  = F1(2, i1, i2);
      c0p1 = F1(2, i1, i2 + 1);
      A.p[A.idx(i1, i2, 0, 2)] = INV_2 * c00 + INV_4 * c0p1;
      c00  = F1(1, i1, i2);
      c0p1 = F1(1, i1, i2 + 1);
      c0m1 = F1(1, i1, i2 - 1);
      A.p[A.idx(i1, i2, 0, 1)] = INV_2 * c00 + INV_4 * (c0m1 + c0p1);
    } else if (f.axis_max && i2 == i2max - 1) {
      c00  = F1(0, i1, i2);
      c0p1 = F1(0, i1, i2 + 1);
      c0m1 = F1(0, i1, i2 - 1);
      A.p[A.idx(i1, i2, 0, 0)] = INV_2 * c00 + INV_4 * (c0m1 + c0p1);
      c00  = F1(2, i1, i2);
      c0m1 = F1(2, i1, i2 - 1);
      A.p[A.idx(i1, i2, 0, 2)] = INV_2 * c00 + INV_4 * c0m1;
      c00  = F1(1, i1, i2);
      c0m1 = F1(1, i1, i2 - 1);
      A.p[A.idx(i1, i2, 0, 1)] = INV_4 * (c00 + c0m1);
    } else if (f.axis_max && i2 == i2max) {
      c00  = F1(0, i1, i2);
      c0m1 = F1(0, i1, i2 - 1);
      A.p[A.idx(i1, i2, 0, 0)] = INV_2 * c00 + INV_2 * c0m1;
      A.p[A.idx(i1, i2, 0, 2)] = ZERO;
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        A.p[A.idx(i1, i2, 0, c)] =
          INV_4 * BB(i1, i2, c) +
          INV_8 * (BB(i1 - 1, i2, c) + BB(i1 + 1, i2, c) + BB(i1, i2 - 1, c) + BB(i1, i2 + 1, c)) +
          INV_16 * (BB(i1 - 1, i2 - 1, c) + BB(i1 + 1, i2 + 1, c) + BB(i1 - 1, i2 + 1, c) +
                    BB(i1 + 1, i2 - 1, c));
      }
    }
  }
#undef F1
#undef BB
}

// AxisBoundaries_kernel (fields_bcs.hpp:825-868), per i1 over all cells
template <typename real>
__global__ void k_gr_axis(GRFld<real> f, FieldView<real> F, int set_e, int set_b) {
  const int i1 = blockIdx.x * blockDim.x + threadIdx.x;
  if (i1 >= f.n1 + 2 * f.ng) return;
#define FF(j, c) F.p[F.idx(i1, j, 0, c)]
  if (f.axis_min) {
    const int e = f.ng;
    if (set_e) {
      FF(e - 1, 1) = -FF(e, 1);
      FF(e, 2)     = (real)0;
      FF(e - 1, 2) = FF(e + 1, 2);
    }
    if (set_b) {
      FF(e - 1, 3) = FF(e, 3);
      FF(e, 4)     = (real)0;
      FF(e - 1, 4) = -FF(e + 1, 4);
      FF(e - 1, 5) = FF(e, 5);
    }
  }
  if (f.axis_max) {
    const int e = f.n2 + f.ng;
    if (set_e) {
      FF(e, 1)     = -FF(e - 1, 1);
      FF(e, 2)     = (real)0;
      FF(e + 1, 2) = FF(e - 1, 2);
    }
    if (set_b) {
      FF(e, 3)     = FF(e - 1, 3);
      FF(e, 4)     = (real)0;
      FF(e + 1, 4) = -FF(e - 1, 4);
      FF(e, 5)     = FF(e - 1, 5);
    }
  }
#undef FF
}

// HorizonBoundaries_kernel (fields_bcs.hpp:1188-1240), per i2
template <typename real>
__global__ void k_gr_horizon(GRFld<real> f, FieldView<real> F, int set_e, int set_b, int nfilter) {
  const int i2 = f.ng + blockIdx.x * blockDim.x + threadIdx.x;
  if (i2 >= f.n2 + f.ng + 1) return;
  const int i1min = f.ng, src = i1min + 1 + nfilter;
  for (int i = 0; i <= 2 + nfilter; ++i) {
    const int dst = i1min - f.ng + i;
    if (set_e)
      for (int c = 0; c < 3; ++c) F.p[F.idx(dst, i2, 0, c)] = F.p[F.idx(src, i2, 0, c)];
    if (set_b)
      for (int c = 3; c < 6; ++c) F.p[F.idx(dst, i2, 0, c)] = F.p[F.idx(src, i2, 0, c)];
  }
}

// MatchBoundaries_kernel, GRPIC branch in 2D with o = x1 (fields_bcs.hpp:
// 181-340) over the cells of the +r layer: each component relaxes toward the
// target field T (the problem generator's field, which the caller stores),
// F = s F + (1 - s) T with s = tanh(4 |r - r_edge| / ds) at the component's
// radius (i + 1/2 for D^r, B^theta, B^phi; i for D^theta, D^phi, B^r). On
// the axis rows D^phi only decays (its target term is skipped there).
template <typename real>
__global__ void k_gr_match(GRFld<real> f, Range2 R, FieldView<real> F, FieldView<real> T,
                           real r_edge, real ds, int set_e, int set_b) {
  const QKS<real> m = f.m.template as<real>();
  const real      H = 0.5, ONE = 1, FOUR = 4;
  const int       N2 = f.n2 + 2 * f.ng;
  auto shape = [&](real x1) {
    const real r = m.r0 + mexp(x1 * m.dchi + m.chi_min);
    return (real)tanh(fabs(r - r_edge) * FOUR / ds);
  };
  GR_CELL_LOOP(R)
    const real i1_ = (real)(i1 - f.ng);
    const real sH = shape(i1_ + H), s0 = shape(i1_);
    auto blend = [&](int c, real sc) {
      real& v = F.p[F.idx(i1, i2, 0, c)];
      v = sc * v + (ONE - sc) * T.p[T.idx(i1, i2, 0, c)];
    };
    if (set_e) {
      blend(0, sH);
      blend(1, s0);
      real& v = F.p[F.idx(i1, i2, 0, 2)];
      v = s0 * v;
      if ((!f.axis_min || i2 > f.ng) && (!f.axis_max || i2 < N2 - f.ng))
        v += (ONE - s0) * T.p[T.idx(i1, i2, 0, 2)];
    }
    if (set_b) {
      blend(3, s0);
      blend(4, sH);
      blend(5, sH);
    }
  }
}

// gr::AbsorbCurrents_kernel<M, 1> (fields_bcs.hpp:1243-1280) over the same
// layer: J *= tanh(|r(i) - r_edge| / (ds / 4)), every component at r(i)
template <typename real>
__global__ void k_gr_absorb_currents(GRFld<real> f, Range2 R, FieldView<real> J, real r_edge,
                                     real ds) {
  const QKS<real> m = f.m.template as<real>();
  const real      INV_4 = 0.25;
  GR_CELL_LOOP(R)
    const real i1_ = (real)(i1 - f.ng);
    const real r   = m.r0 + mexp(i1_ * m.dchi + m.chi_min);
    const real t   = (real)tanh(fabs(r - r_edge) / (INV_4 * ds));
    for (int c = 0; c < 3; ++c) J.p[J.idx(i1, i2, 0, c)] *= t;
  }
}

// metric functions at points (tests and diagnostics)
template <typename real>
__global__ void k_gr_metric_eval(QKS<double> md, const double* x, int64_t n, double* out) {
  const QKS<real> m = md.template as<real>();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const QPt<real> p = qpt(m, (real)x[2 * k], (real)x[2 * k + 1]);
    double*         o = out + k * PIC_GR_NQ;
    o[0] = h_11(m, p), o[1] = h_22(m, p), o[2] = h_33(m, p), o[3] = h_13(m, p);
    o[4] = h11(m, p), o[5] = h22(m, p), o[6] = h33(m, p), o[7] = h13(m, p);
    o[8] = alpha(m, p), o[9] = beta1(m, p), o[10] = sqrt_det_h(m, p);
    o[11] = sqrt_det_h_tilde(m, p), o[12] = dr_alpha(m, p), o[13] = dt_alpha(m, p);
    o[14] = dr_beta1(m, p), o[15] = dt_beta1(m, p), o[16] = dr_h11(m, p), o[17] = dr_h22(m, p);
    o[18] = dr_h33(m, p), o[19] = dr_h13(m, p), o[20] = dt_h11(m, p), o[21] = dt_h22(m, p);
    o[22] = dt_h33(m, p), o[23] = dt_h13(m, p);
  }
}

// vertical seed field (pgens/wald/pgen.hpp InitFields, init_field = vertical):
// B^r at (i, j + 1/2) and B^theta at (i + 1/2, j) from A_3 = (h_33 + 2 a
// h_13 beta^1) / 2; D = 0, B^phi = 0
template <typename real>
__global__ void k_gr_init_vertical(GRFld<real> f, FieldView<real> EB) {
  const QKS<double> m   = f.m;
  const int         N1  = f.n1 + 2 * f.ng, N2 = f.n2 + 2 * f.ng;
  const int64_t     cnt = (int64_t)N1 * N2;
  auto A3 = [&](double x1, double x2) {
    const QPt<double> p = qpt(m, x1, x2);
    return 0.5 * (h_33(m, p) + 2.0 * m.a * h_13(m, p) * beta1(m, p));
  };
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int    i1 = (int)(t % N1), i2 = (int)(t / N1);
    const double x1 = i1 - f.ng, x2 = i2 - f.ng;
    for (int c = 0; c < 6; ++c) EB.p[EB.idx(i1, i2, 0, c)] = (real)0;
    // bx1 at (i, j + 1/2)
    EB.p[EB.idx(i1, i2, 0, 3)] =
      (real)((A3(x1, x2 + 1.0) - A3(x1, x2)) / sqrt_det_h(m, qpt(m, x1, x2 + 0.5)));
    // bx2 at (i + 1/2, j); zero on the axis
    const double th = m.eta2theta(x2 * m.deta + m.eta_min);
    EB.p[EB.idx(i1, i2, 0, 4)] =
      fabs(th) <= QKS<double>::eps()
        ? (real)0
        : (real)(-(A3(x1 + 1.0, x2) - A3(x1, x2)) / sqrt_det_h(m, qpt(m, x1 + 0.5, x2)));
  }
}

// minimum effective cell size (qkerr_schild.h:112-129): 1 / (alpha
// sqrt(h^11 + h^22) + beta^1) over the cell centres; partial minima per block
__global__ void k_gr_dxmin(QKS<double> m, int n1, int n2, double* out) {
  __shared__ double sh[256];
  double            best = 1e300;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)n1 * n2;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double      x1 = (double)(t % n1) + 0.5, x2 = (double)(t / n1) + 0.5;
    const QPt<double> p  = qpt(m, x1, x2);
    const double      dx = 1.0 / (alpha(m, p) * sqrt(h11(m, p) + h22(m, p)) + beta1(m, p));
    best                 = fmin(best, dx);
  }
  sh[threadIdx.x] = best;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmin(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

}  // namespace pic

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
namespace {

using pic::QKS;

template <typename real>
pic::GRFld<real> fld_of(const pic_ctx* c, const pic_gr_metric* g) {
  pic::GRFld<real> f;
  f.m        = make_qks<real>(c, g);
  f.ng       = c->grid.ng;
  f.n1       = c->grid.n[0];
  f.n2       = c->grid.n[1];
  f.axis_min = g->axis_min;
  f.axis_max = g->axis_max;
  return f;
}

unsigned blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > pic::sm_count() * 64) b = pic::sm_count() * 64;
  return (unsigned)(b < 1 ? 1 : b);
}

pic::Range2 active(const pic_ctx* c) {
  const int ng = c->grid.ng;
  return pic::Range2{ ng, c->grid.n[0] + ng, ng, c->grid.n[1] + ng };
}

// the island lists and masks of nsp species (list k: npart_k entries at
// offset off_k; mask k: ceil(npart_k / 32) words after all lists), two
// counters per species, one side stream and join event per species; made or
// grown on first use
int island_resources(pic_ctx* c, int nsp, int64_t words) {
  if (c->gr_island_nsp < nsp) {
    cudaFree(c->gr_island_cnt);
    c->gr_island_cnt = nullptr;
    c->gr_island_nsp = 0;
    if (cudaMalloc((void**)&c->gr_island_cnt, 2 * sizeof(unsigned) * nsp) != cudaSuccess)
      return PIC_ERR_NOMEM;
    c->gr_island_nsp = nsp;
  }
  if (c->gr_island_cap < words) {
    cudaFree(c->gr_island);
    c->gr_island     = nullptr;
    c->gr_island_cap = 0;
    if (cudaMalloc((void**)&c->gr_island, sizeof(int32_t) * words) != cudaSuccess)
      return PIC_ERR_NOMEM;
    c->gr_island_cap = words;
  }
  if (!c->gr_fork && cudaEventCreateWithFlags(&c->gr_fork, cudaEventDisableTiming) != cudaSuccess)
    return PIC_ERR_CUDA;
  while ((int)c->gr_side.size() < nsp) {
    cudaStream_t st = nullptr;
    cudaEvent_t  ev = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return PIC_ERR_CUDA;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      cudaStreamDestroy(st);
      return PIC_ERR_CUDA;
    }
    c->gr_side.push_back(st);
    c->gr_join.push_back(ev);
  }
  return PIC_OK;
}

template <typename real>
pic::GRPushArgs<real> push_args(pic_ctx* c, const pic_gr_metric* g, const pic_species* sp,
                                const void* em, const void* em0, double dt, double omegaB0,
                                int32_t niter, int32_t island_lo, int32_t island_hi) {
  pic::GRPushArgs<real> a;
  a.sp  = sptrs(sp);
  a.em  = em_view<real>(c, em);
  a.em0 = em_view<real>(c, em0);
  a.m   = make_qks<real>(c, g);
  a.n1 = c->grid.n[0], a.n2 = c->grid.n[1], a.ng = c->grid.ng;
  a.absorb_min = c->grid.prtl_bc[0][0] == PIC_BC_ABSORB;
  a.absorb_max = c->grid.prtl_bc[0][1] == PIC_BC_ABSORB;
  a.axis_min   = c->grid.prtl_bc[1][0] == PIC_BC_AXIS;
  a.axis_max   = c->grid.prtl_bc[1][1] == PIC_BC_AXIS;
  a.dt         = (real)dt;
  const float qm = sp->pusher == PIC_PUSHER_PHOTON ? 0.0f : sp->charge / sp->mass;
  a.ndth       = (real)0.5 * (real)qm * (real)omegaB0 * (real)dt;
  a.niter      = niter;
  a.island_lo  = island_lo;
  a.island_hi  = island_hi;
  a.massive    = sp->pusher != PIC_PUSHER_PHOTON;
  a.err        = c->d_err;
  a.list       = nullptr;
  a.list_count = nullptr;
  a.mask       = nullptr;
  return a;
}

// grpic::ParticlePush over the species sp[0..nsp) with npart > 0 and a
// pusher (validated by the caller). FP32 with an island: the island lists
// of all species are built first, then every species' island kernel runs on
// its own side stream while the bulks run on s, and s waits for all of them.
// The islands are latency-bound chains of FP64 work, so running them at once
// costs little more than one.
template <typename real>
int gr_push_species(pic_ctx* c, const pic_gr_metric* g, const pic_species* const* sp, int nsp,
                    const void* em, const void* em0, double dt, double omegaB0, int32_t niter,
                    int32_t island_lo, int32_t island_hi, cudaStream_t s) {
  if (c->grid.order < 1 || c->grid.order > 3) return PIC_ERR_UNSUPPORTED;
  std::vector<pic::GRPushArgs<real>> a(nsp);
  for (int k = 0; k < nsp; ++k)
    a[k] = push_args<real>(c, g, sp[k], em, em0, dt, omegaB0, niter, island_lo, island_hi);
  auto bulk = [&](const pic::GRPushArgs<real>& ak) {
    const unsigned b = blocks_for(ak.sp.npart);
    switch (c->grid.order) {
      case 1: PIC_KL(pic::k_gr_push<1, real><<<b, 256, 0, s>>>(ak)); break;
      case 2: PIC_KL(pic::k_gr_push<2, real><<<b, 256, 0, s>>>(ak)); break;
      default: PIC_KL(pic::k_gr_push<3, real><<<b, 256, 0, s>>>(ak)); break;
    }
  };
  // double fields run everything in double: no split
  if (sizeof(real) == 8 || island_hi <= island_lo) {
    for (int k = 0; k < nsp; ++k) bulk(a[k]);
    return cuda_status(cudaGetLastError());
  }
  int64_t lists = 0, masks = 0;
  for (int k = 0; k < nsp; ++k) {
    // the island lists hold 32-bit particle indices
    if (sp[k]->npart > (int64_t)INT32_MAX) return PIC_ERR_UNSUPPORTED;
    lists += sp[k]->npart;
    masks += (sp[k]->npart + 31) / 32;
  }
  int st = island_resources(c, nsp, lists + masks);
  if (st != PIC_OK) return st;
  if (cudaMemsetAsync(c->gr_island_cnt, 0, 2 * sizeof(unsigned) * nsp, s) != cudaSuccess)
    return PIC_ERR_CUDA;
  int64_t lo = 0, mo = lists;
  for (int k = 0; k < nsp; ++k) {
    a[k].list       = c->gr_island + lo;
    a[k].mask       = reinterpret_cast<unsigned*>(c->gr_island + mo);
    a[k].list_count = c->gr_island_cnt + 2 * k;
    lo += sp[k]->npart;
    mo += (sp[k]->npart + 31) / 32;
    PIC_KL(pic::k_gr_island_list<real><<<blocks_for(sp[k]->npart), 256, 0, s>>>(a[k]));
  }
  if (cudaEventRecord(c->gr_fork, s) != cudaSuccess) return PIC_ERR_CUDA;
  for (int k = 0; k < nsp; ++k) {
    cudaStream_t s2 = c->gr_side[k];
    if (cudaStreamWaitEvent(s2, c->gr_fork, 0) != cudaSuccess) return PIC_ERR_CUDA;
    if constexpr (sizeof(real) == 4) {
      // three 128-thread blocks per SM fit at up to 170 registers per thread
      const unsigned bi = (unsigned)pic::sm_count() * 3;
      switch (c->grid.order) {
        case 1: PIC_KL(pic::k_gr_push_island<1, real><<<bi, 128, 0, s2>>>(a[k])); break;
        case 2: PIC_KL(pic::k_gr_push_island<2, real><<<bi, 128, 0, s2>>>(a[k])); break;
        default: PIC_KL(pic::k_gr_push_island<3, real><<<bi, 128, 0, s2>>>(a[k])); break;
      }
    }
    if (cudaEventRecord(c->gr_join[k], s2) != cudaSuccess) return PIC_ERR_CUDA;
  }
  for (int k = 0; k < nsp; ++k) bulk(a[k]);
  for (int k = 0; k < nsp; ++k)
    if (cudaStreamWaitEvent(s, c->gr_join[k], 0) != cudaSuccess) return PIC_ERR_CUDA;
  return cuda_status(cudaGetLastError());
}

template <typename real>
int gr_deposit(pic_ctx* c, const pic_gr_metric* g, const pic_species* sp, void* J, double dt,
               int32_t island_lo, int32_t island_hi, cudaStream_t s) {
  pic::GRDepArgs<real> a;
  a.sp = sptrs(sp);
  a.J  = cur_view<real>(c, J);
  a.m  = make_qks<real>(c, g);
  a.ng = c->grid.ng;
  // double fields: the field precision is already double
  a.island_lo = sizeof(real) == 8 ? 1 : island_lo;
  a.island_hi = sizeof(real) == 8 ? 0 : island_hi;
  a.ext[0] = c->grid.n[0] + 2 * c->grid.ng;
  a.ext[1] = c->grid.n[1] + 2 * c->grid.ng;
  a.ext[2] = 1;
  a.inv_dt = (real)1 / (real)dt;
  a.charge = (real)sp->charge;
  a.err    = c->d_err;
  PIC_KL(pic::k_gr_deposit<real><<<blocks_for(sp->npart), 256, 0, s>>>(a));
  return cuda_status(cudaGetLastError());
}

// the species of a push that have work, after the checks of pic_gr_push
int push_checks(pic_ctx* c, const pic_gr_metric* g, pic_species* sp, int32_t nsp,
                const void* em, const void* em0, int32_t niter,
                std::vector<const pic_species*>& work) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!em || !em0 || niter < 1 || nsp < 0 || (nsp > 0 && !sp)) return PIC_ERR_ARG;
  for (int32_t k = 0; k < nsp; ++k) {
    st = validate_species(c, sp + k, true);
    if (st != PIC_OK) return st;
    if (sp[k].npart == 0 || sp[k].pusher == PIC_PUSHER_NONE) continue;
    if (sp[k].pusher == PIC_PUSHER_VAY) return PIC_ERR_UNSUPPORTED;
    if (sp[k].pusher == PIC_PUSHER_BORIS && sp[k].mass == 0.0f) return PIC_ERR_ARG;
    work.push_back(sp + k);
  }
  return PIC_OK;
}

int push_entry(pic_ctx* c, const pic_gr_metric* g, pic_species* sp, int32_t nsp, const void* em,
               const void* em0, double dt, double omegaB0, int32_t niter, int32_t island_lo,
               int32_t island_hi, void* stream) {
  std::vector<const pic_species*> work;
  const int st = push_checks(c, g, sp, nsp, em, em0, niter, work);
  if (st != PIC_OK || work.empty()) return st;
  const cudaStream_t s = strm(stream);
  const int          n = (int)work.size();
  return is_f64(c) ? gr_push_species<double>(c, g, work.data(), n, em, em0, dt, omegaB0, niter,
                                             island_lo, island_hi, s)
                   : gr_push_species<float>(c, g, work.data(), n, em, em0, dt, omegaB0, niter,
                                            island_lo, island_hi, s);
}

// the cells of the +x1 match layer (MatchFieldsIn, grpic/fields_bcs.h:53-92,
// and Mesh::ExtentToRange, framework/domain/mesh.h:133-202): x1 over
// [floor(x1(r_max - ds)) + ng, ceil(x1(r_max)) + 2 ng) in real_t, upper ghosts
// included; every x2 cell, ghosts included. The end is clamped to the array.
template <typename real>
pic::Range2 match_range(const pic_ctx* c, const pic_gr_metric* g, double ds) {
  const QKS<double> md = make_qks<real>(c, g);
  const real r0 = (real)md.r0, chi_min = (real)md.chi_min, dchi_inv = (real)md.dchi_inv;
  const real r_lo = (real)g->x1min, r_hi = (real)g->x1max;
  const real lo   = std::min(std::max(r_lo, r_hi - (real)ds), r_hi);
  auto       x1   = [&](real r) { return (std::log(r - r0) - chi_min) * dchi_inv; };
  const int  ng   = c->grid.ng;
  int        i0   = (int)std::floor(x1(lo)) + ng;
  int        i1   = (int)std::ceil(x1(r_hi)) + 2 * ng;
  i0 = std::max(i0, ng);
  i1 = std::min(i1, c->grid.n[0] + 2 * ng);
  return pic::Range2{ i0, std::max(i0, i1), 0, c->grid.n[1] + 2 * ng };
}

}  // namespace

extern "C" {

int pic_gr_metric_eval(pic_ctx* c, const pic_gr_metric* g, const double* x, int64_t n,
                       double* out, void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (n < 0 || (n > 0 && (!x || !out))) return PIC_ERR_ARG;
  if (n == 0) return PIC_OK;
  cudaStream_t s = strm(stream);
  if (is_f64(c)) PIC_KL(pic::k_gr_metric_eval<double><<<blocks_for(n), 256, 0, s>>>(make_qks<double>(c, g), x, n, out));
  else           PIC_KL(pic::k_gr_metric_eval<float><<<blocks_for(n), 256, 0, s>>>(make_qks<float>(c, g), x, n, out));
  return cuda_status(cudaGetLastError());
}

int pic_gr_push(pic_ctx* c, const pic_gr_metric* g, pic_species* sp, const void* em,
                const void* em0, double dt, double omegaB0, int32_t niter, int32_t island_lo,
                int32_t island_hi, void* stream) {
  if (!sp) return PIC_ERR_ARG;
  return push_entry(c, g, sp, 1, em, em0, dt, omegaB0, niter, island_lo, island_hi, stream);
}

int pic_gr_particle_push(pic_ctx* c, const pic_gr_metric* g, pic_species* sp, int32_t nspecies,
                         const void* em, const void* em0, double dt, double omegaB0,
                         int32_t niter, int32_t island_lo, int32_t island_hi, void* stream) {
  return push_entry(c, g, sp, nspecies, em, em0, dt, omegaB0, niter, island_lo, island_hi, stream);
}

int pic_gr_deposit(pic_ctx* c, const pic_gr_metric* g, const pic_species* sp, int32_t nspecies,
                   void* J, double dt, int32_t island_lo, int32_t island_hi, uint32_t flags,
                   void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!J || nspecies < 0 || (nspecies > 0 && !sp)) return PIC_ERR_ARG;
  for (int k = 0; k < nspecies; ++k) {
    st = validate_species(c, sp + k, true);
    if (st != PIC_OK) return st;
  }
  cudaStream_t s = strm(stream);
  if (!(flags & PIC_PD_NO_ZERO)) {
    const auto gi = ginfo(c);
    const cudaError_t e = is_f64(c) ? pic::launch_zero3<double>(gi, cur_view<double>(c, J), s)
                                    : pic::launch_zero3<float>(gi, cur_view<float>(c, J), s);
    if (e != cudaSuccess) return PIC_ERR_CUDA;
  }
  for (int k = 0; k < nspecies; ++k) {
    const pic_species* sk = sp + k;
    if (sk->npart == 0 || sk->pusher == PIC_PUSHER_NONE || sk->charge == 0.0f) continue;
    st = is_f64(c) ? gr_deposit<double>(c, g, sk, J, dt, island_lo, island_hi, s)
                   : gr_deposit<float>(c, g, sk, J, dt, island_lo, island_hi, s);
    if (st != PIC_OK) return st;
  }
  return PIC_OK;
}

#define GR_FLD_DISPATCH(KERNEL_CALL_F, KERNEL_CALL_D) \
  if (is_f64(c)) {                                   \
    KERNEL_CALL_D;                                   \
  } else {                                           \
    KERNEL_CALL_F;                                   \
  }                                                  \
  return cuda_status(cudaGetLastError());

int pic_gr_faraday(pic_ctx* c, const pic_gr_metric* g, const void* Bin, void* Bout, const void* E,
                   double coeff, void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!Bin || !Bout || !E) return PIC_ERR_ARG;
  cudaStream_t      s = strm(stream);
  const pic::Range2 R = active(c);
  const unsigned    b = blocks_for((int64_t)c->grid.n[0] * c->grid.n[1]);
  GR_FLD_DISPATCH(
    PIC_KL(pic::k_gr_faraday<float><<<b, 256, 0, s>>>(fld_of<float>(c, g), R, em_view<float>(c, Bin),
                                                      em_view<float>(c, Bout), em_view<float>(c, E),
                                                      (float)coeff)),
    PIC_KL(pic::k_gr_faraday<double><<<b, 256, 0, s>>>(fld_of<double>(c, g), R, em_view<double>(c, Bin),
                                                       em_view<double>(c, Bout), em_view<double>(c, E),
                                                       coeff)))
}

int pic_gr_ampere(pic_ctx* c, const pic_gr_metric* g, const void* Din, void* Dout, const void* H,
                  double coeff, void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!Din || !Dout || !H) return PIC_ERR_ARG;
  cudaStream_t s  = strm(stream);
  const int    ng = c->grid.ng;
  // ampere range: i2 in [i2min, i2max + 1) (fieldsolvers.h:180-182)
  const pic::Range2 R{ ng, c->grid.n[0] + ng, ng, c->grid.n[1] + ng + 1 };
  const unsigned    b  = blocks_for((int64_t)c->grid.n[0] * (c->grid.n[1] + 1));
  const unsigned    ba = (unsigned)((c->grid.n[0] + 255) / 256);
  const bool        alias = Din == Dout;
  if (is_f64(c)) {
    const auto f = fld_of<double>(c, g);
    PIC_KL(pic::k_gr_ampere<double><<<b, 256, 0, s>>>(f, R, em_view<double>(c, Din), em_view<double>(c, Dout),
                                                      em_view<double>(c, H), coeff));
    PIC_KL(pic::k_gr_ampere_axis<double><<<ba, 256, 0, s>>>(f, em_view<double>(c, Din),
                                                            em_view<double>(c, Dout), alias));
  } else {
    const auto f = fld_of<float>(c, g);
    PIC_KL(pic::k_gr_ampere<float><<<b, 256, 0, s>>>(f, R, em_view<float>(c, Din), em_view<float>(c, Dout),
                                                     em_view<float>(c, H), (float)coeff));
    PIC_KL(pic::k_gr_ampere_axis<float><<<ba, 256, 0, s>>>(f, em_view<float>(c, Din),
                                                           em_view<float>(c, Dout), alias));
  }
  return cuda_status(cudaGetLastError());
}

int pic_gr_currents_ampere(pic_ctx* c, const pic_gr_metric* g, void* D, const void* J,
                           double coeff, void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!D || !J) return PIC_ERR_ARG;
  cudaStream_t      s  = strm(stream);
  const int         ng = c->grid.ng;
  const pic::Range2 R{ ng, c->grid.n[0] + ng, ng, c->grid.n[1] + ng + 1 };
  const unsigned    b = blocks_for((int64_t)c->grid.n[0] * (c->grid.n[1] + 1));
  GR_FLD_DISPATCH(
    PIC_KL(pic::k_gr_currents_ampere<float><<<b, 256, 0, s>>>(fld_of<float>(c, g), R, em_view<float>(c, D),
                                                              cur_view<float>(c, J), (float)coeff)),
    PIC_KL(pic::k_gr_currents_ampere<double><<<b, 256, 0, s>>>(fld_of<double>(c, g), R, em_view<double>(c, D),
                                                               cur_view<double>(c, J), coeff)))
}

int pic_gr_aux(pic_ctx* c, const pic_gr_metric* g, int32_t which, const void* D, const void* B,
               void* out, void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!D || !B || !out || (which != 0 && which != 1)) return PIC_ERR_ARG;
  cudaStream_t s  = strm(stream);
  const int    ng = c->grid.ng;
  // range_with_axis_BCs (fieldsolvers.h:58-81)
  const pic::Range2 R{ ng - 1, c->grid.n[0] + ng, ng, c->grid.n[1] + ng + (g->axis_max ? 1 : 0) };
  const unsigned    b = blocks_for((int64_t)(c->grid.n[0] + 1) * (c->grid.n[1] + 1));
  if (is_f64(c)) {
    const auto f = fld_of<double>(c, g);
    if (which == 0) PIC_KL(pic::k_gr_aux_e<double><<<b, 256, 0, s>>>(f, R, em_view<double>(c, D), em_view<double>(c, B), em_view<double>(c, out)));
    else            PIC_KL(pic::k_gr_aux_h<double><<<b, 256, 0, s>>>(f, R, em_view<double>(c, D), em_view<double>(c, B), em_view<double>(c, out)));
  } else {
    const auto f = fld_of<float>(c, g);
    if (which == 0) PIC_KL(pic::k_gr_aux_e<float><<<b, 256, 0, s>>>(f, R, em_view<float>(c, D), em_view<float>(c, B), em_view<float>(c, out)));
    else            PIC_KL(pic::k_gr_aux_h<float><<<b, 256, 0, s>>>(f, R, em_view<float>(c, D), em_view<float>(c, B), em_view<float>(c, out)));
  }
  return cuda_status(cudaGetLastError());
}

int pic_gr_average(pic_ctx* c, int32_t which, void* a, void* b, void* stream) {
  if (!c || !a || !b || (which != 0 && which != 1)) return PIC_ERR_ARG;
  cudaStream_t      s = strm(stream);
  const pic::Range2 R = active(c);
  const unsigned    nb = blocks_for((int64_t)c->grid.n[0] * c->grid.n[1]);
  // which 0: f0 = (f0 + f) / 2 over the 6 EM components (a = f, b = f0);
  // which 1: J = (J0 + J) / 2 over 3 components (a = J, b = J0)
  if (is_f64(c)) {
    auto va = which == 0 ? em_view<double>(c, a) : cur_view<double>(c, a);
    auto vb = which == 0 ? em_view<double>(c, b) : cur_view<double>(c, b);
    PIC_KL(pic::k_gr_average<double><<<nb, 256, 0, s>>>(R, va, vb, which == 0 ? 6 : 3, which == 0));
  } else {
    auto va = which == 0 ? em_view<float>(c, a) : cur_view<float>(c, a);
    auto vb = which == 0 ? em_view<float>(c, b) : cur_view<float>(c, b);
    PIC_KL(pic::k_gr_average<float><<<nb, 256, 0, s>>>(R, va, vb, which == 0 ? 6 : 3, which == 0));
  }
  return cuda_status(cudaGetLastError());
}

int pic_gr_filter_currents(pic_ctx* c, const pic_gr_metric* g, void* J, void* buff,
                           int32_t npasses, void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!J || !buff || npasses < 0 || J == buff) return PIC_ERR_ARG;
  if (npasses == 0) return PIC_OK;
  cudaStream_t      s  = strm(stream);
  const int         ng = c->grid.ng;
  const pic::Range2 R{ ng, c->grid.n[0] + ng, ng, c->grid.n[1] + ng + 1 };
  const unsigned    b = blocks_for(R.count());
  // bytes spanned by a 3-component field with the cur strides
  int64_t span = 2 * c->grid.cur_stride[3];
  for (int d = 0; d < 2; ++d) span += (int64_t)(c->grid.n[d] + 2 * ng - 1) * c->grid.cur_stride[d];
  const size_t bytes = (size_t)(span + 1) * (size_t)c->grid.real_bytes;
  for (int k = 0; k < npasses; ++k) {
    // buff <- cur0 (currents.h:90), then the stencil back into cur0
    if (cudaMemcpyAsync(buff, J, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return PIC_ERR_CUDA;
    if (is_f64(c)) {
      PIC_KL(pic::k_gr_filter<double><<<b, 256, 0, s>>>(fld_of<double>(c, g), R, cur_view<double>(c, J),
                                                        cur_view<double>(c, buff)));
    } else {
      PIC_KL(pic::k_gr_filter<float><<<b, 256, 0, s>>>(fld_of<float>(c, g), R, cur_view<float>(c, J),
                                                       cur_view<float>(c, buff)));
    }
    if (cudaGetLastError() != cudaSuccess) return PIC_ERR_CUDA;
  }
  return PIC_OK;
}

// the sides in Directions<2>::orth order (grpic/fields_bcs.h:242-252): the
// horizon (-x1) before the axes (-x2, +x2), whose ghost rows then mirror the
// horizon's copies in the corner cells
int pic_gr_field_bcs(pic_ctx* c, const pic_gr_metric* g, void* fld, int32_t set_e, int32_t set_b,
                     int32_t nfilter, void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!fld || nfilter < 0) return PIC_ERR_ARG;
  cudaStream_t   s  = strm(stream);
  const unsigned b1 = (unsigned)((c->grid.n[0] + 2 * c->grid.ng + 255) / 256);
  const unsigned b2 = (unsigned)((c->grid.n[1] + 1 + 255) / 256);
  if (is_f64(c)) {
    const auto f = fld_of<double>(c, g);
    if (g->horizon) PIC_KL(pic::k_gr_horizon<double><<<b2, 256, 0, s>>>(f, em_view<double>(c, fld), set_e, set_b, nfilter));
    if (g->axis_min || g->axis_max) PIC_KL(pic::k_gr_axis<double><<<b1, 256, 0, s>>>(f, em_view<double>(c, fld), set_e, set_b));
  } else {
    const auto f = fld_of<float>(c, g);
    if (g->horizon) PIC_KL(pic::k_gr_horizon<float><<<b2, 256, 0, s>>>(f, em_view<float>(c, fld), set_e, set_b, nfilter));
    if (g->axis_min || g->axis_max) PIC_KL(pic::k_gr_axis<float><<<b1, 256, 0, s>>>(f, em_view<float>(c, fld), set_e, set_b));
  }
  return cuda_status(cudaGetLastError());
}

int pic_gr_match_fields(pic_ctx* c, const pic_gr_metric* g, void* fld, const void* target,
                        double ds, int32_t set_e, int32_t set_b, void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!fld || !target || !(ds > 0.0)) return PIC_ERR_ARG;
  cudaStream_t s = strm(stream);
  if (is_f64(c)) {
    const auto R = match_range<double>(c, g, ds);
    if (R.count() == 0) return PIC_OK;
    PIC_KL(pic::k_gr_match<double><<<blocks_for(R.count()), 256, 0, s>>>(
      fld_of<double>(c, g), R, em_view<double>(c, fld), em_view<double>(c, target),
      (double)g->x1max, ds, set_e, set_b));
  } else {
    const auto R = match_range<float>(c, g, ds);
    if (R.count() == 0) return PIC_OK;
    PIC_KL(pic::k_gr_match<float><<<blocks_for(R.count()), 256, 0, s>>>(
      fld_of<float>(c, g), R, em_view<float>(c, fld), em_view<float>(c, target),
      (float)g->x1max, (float)ds, set_e, set_b));
  }
  return cuda_status(cudaGetLastError());
}

int pic_gr_absorb_currents(pic_ctx* c, const pic_gr_metric* g, void* J, double ds, void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!J || !(ds > 0.0)) return PIC_ERR_ARG;
  cudaStream_t s = strm(stream);
  if (is_f64(c)) {
    const auto R = match_range<double>(c, g, ds);
    if (R.count() == 0) return PIC_OK;
    PIC_KL(pic::k_gr_absorb_currents<double><<<blocks_for(R.count()), 256, 0, s>>>(
      fld_of<double>(c, g), R, cur_view<double>(c, J), (double)g->x1max, ds));
  } else {
    const auto R = match_range<float>(c, g, ds);
    if (R.count() == 0) return PIC_OK;
    PIC_KL(pic::k_gr_absorb_currents<float><<<blocks_for(R.count()), 256, 0, s>>>(
      fld_of<float>(c, g), R, cur_view<float>(c, J), (float)g->x1max, (float)ds));
  }
  return cuda_status(cudaGetLastError());
}

int pic_gr_init_vertical(pic_ctx* c, const pic_gr_metric* g, void* EB, void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!EB) return PIC_ERR_ARG;
  cudaStream_t   s = strm(stream);
  const unsigned b = blocks_for((int64_t)(c->grid.n[0] + 2 * c->grid.ng) * (c->grid.n[1] + 2 * c->grid.ng));
  GR_FLD_DISPATCH(
    PIC_KL(pic::k_gr_init_vertical<float><<<b, 256, 0, s>>>(fld_of<float>(c, g), em_view<float>(c, EB))),
    PIC_KL(pic::k_gr_init_vertical<double><<<b, 256, 0, s>>>(fld_of<double>(c, g), em_view<double>(c, EB))))
}

int pic_gr_min_cell_size(pic_ctx* c, const pic_gr_metric* g, double* out, void* stream) {
  int st = gr_check(c, g);
  if (st != PIC_OK) return st;
  if (!out) return PIC_ERR_ARG;
  cudaStream_t s  = strm(stream);
  const int    nb = pic::sm_count();
  double*      d  = nullptr;
  if (cudaMallocAsync((void**)&d, sizeof(double) * nb, s) != cudaSuccess) return PIC_ERR_NOMEM;
  const QKS<double> m = is_f64(c) ? make_qks<double>(c, g) : make_qks<float>(c, g);
  PIC_KL(pic::k_gr_dxmin<<<nb, 256, 0, s>>>(m, c->grid.n[0], c->grid.n[1], d));
  double h[nb];
  cudaError_t e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFreeAsync(d, s);
  if (e != cudaSuccess) return PIC_ERR_CUDA;
  double best = h[0];
  for (int k = 1; k < nb; ++k) best = best < h[k] ? best : h[k];
  *out = best;
  return PIC_OK;
}

}  // extern "C"
