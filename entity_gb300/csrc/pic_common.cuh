// Device-side building blocks of the SR particle-in-cell step: shape
// functions, field interpolation, Boris/Vay velocity updates, the Cartesian
// position update with particle boundaries, and the zigzag / Esirkepov current
// deposit. Every routine follows the operation order of the reference kernel
// it cites (paths relative to the entity repository) so that, compiled with
// -fmad=false, a particle's new cell, offset and momentum are bit-identical to
// the reference arithmetic; the one deliberate contraction is the running sum
// of the field interpolation at order >= 1, written as an explicit fma.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pic_types.h"

namespace pic {

// ---------------------------------------------------------------------------
// constants per precision: src/global/utils/numeric.h:31-67
// ---------------------------------------------------------------------------
template <typename real>
struct K;
template <>
struct K<float> {
  static constexpr float THIRD = 0.333333f;  // numeric.h:41 (not 1/3)
};
template <>
struct K<double> {
  static constexpr double THIRD = 0.3333333333333333;
};

// one term of an interpolation sum, `c += a * b` as the reference writes it
// (src/kernels/pushers/sr.hpp:1118-1369, gr.hpp:594-662): the product and the
// sum round separately (the library is built with -fmad=false)
template <typename real>
__device__ __forceinline__ real iacc(real a, real b, real c) {
  return c + a * b;
}

// staggering of (ex1, ex2, ex3, bx1, bx2, bx3) per axis: 1 = dual
// (src/kernels/pushers/sr.hpp:1210-1366)
__device__ __forceinline__ int stag_of(int c, int a) {
  // bit (c*3 + a) of the 6x3 table {100, 010, 001, 011, 101, 110}
  constexpr unsigned tbl = (1u << 0) | (1u << 4) | (1u << 8) | (1u << 10) | (1u << 11) |
                           (1u << 12) | (1u << 14) | (1u << 15) | (1u << 16);
  return (tbl >> (c * 3 + a)) & 1u;
}

// ---------------------------------------------------------------------------
// shape functions: src/kernels/particle_shapes.hpp:25-63, 544-614
// ---------------------------------------------------------------------------
template <typename real>
__device__ __forceinline__ real S3f(real x) {
  const real ONE = 1, TWO = 2, HALF = 0.5;
  if (x < ONE) {
    return (real)(2.0 / 3.0) - x * x + HALF * (x * x * x);
  } else if (x < TWO) {
    return (real)(4.0 / 3.0) - TWO * x + x * x - (real)(1.0 / 6.0) * (x * x * x);
  }
  return (real)0;
}

template <int O, bool STAG, typename real>
__device__ __forceinline__ void shape(int i, real di, int& imin, real* S) {
  const real ONE = 1, HALF = 0.5, THREE_FOURTHS = 0.75, THREE_HALFS = 1.5;
  if constexpr (O == 1) {
    if constexpr (!STAG) {
      imin = i;
      S[0] = ONE - di;
      S[1] = di;
    } else {
      if (di < HALF) {
        imin = i - 1;
        S[0] = HALF - di;
        S[1] = ONE - S[0];
      } else {
        imin = i;
        S[0] = THREE_HALFS - di;
        S[1] = ONE - S[0];
      }
    }
  } else if constexpr (O == 2) {
    if constexpr (!STAG) {
      if (di < HALF) {
        imin = i - 1;
        S[0] = HALF * ((HALF - di) * (HALF - di));
        S[1] = THREE_FOURTHS - di * di;
        S[2] = ONE - S[0] - S[1];
      } else {
        imin = i;
        S[0] = HALF * ((THREE_HALFS - di) * (THREE_HALFS - di));
        S[1] = THREE_FOURTHS - (ONE - di) * (ONE - di);
        S[2] = ONE - S[0] - S[1];
      }
    } else {
      imin = i - 1;
      S[0] = HALF * ((ONE - di) * (ONE - di));
      S[2] = HALF * (di * di);
      S[1] = ONE - S[0] - S[2];
    }
  } else {
    static_assert(O == 3, "shape orders 1..3");
    if constexpr (!STAG) {
      imin = i - 1;
#pragma unroll
      for (int n = 0; n < 4; n++) S[n] = S3f<real>(fabs(ONE + di - (real)n));
    } else {
      if (di < HALF) {
        imin = i - 2;
#pragma unroll
        for (int n = 0; n < 4; n++) S[n] = S3f<real>(fabs((real)1.5 + di - (real)n));
      } else {
        imin = i - 1;
#pragma unroll
        for (int n = 0; n < 4; n++) S[n] = S3f<real>(fabs(HALF + di - (real)n));
      }
    }
  }
}

// prtl_shape::for_deposit (particle_shapes.hpp:934-1024)
template <int O, typename real>
__device__ __forceinline__ void for_deposit(int i_init, real di_init, int i_fin, real di_fin,
                                            int& i_min, int& i_max, real* iS, real* fS) {
  int  i_init_min, i_fin_min;
  real iS_[O + 1], fS_[O + 1];
  shape<O, false>(i_init, di_init, i_init_min, iS_);
  shape<O, false>(i_fin, di_fin, i_fin_min, fS_);
  const real ZERO = 0;
  if (i_init_min < i_fin_min) {
    i_min = i_init_min;
    i_max = i_min + O + 1;
#pragma unroll
    for (int j = 0; j < O + 1; j++) iS[j] = iS_[j];
    iS[O + 1] = ZERO;
    fS[0]     = ZERO;
#pragma unroll
    for (int j = 0; j < O + 1; j++) fS[j + 1] = fS_[j];
  } else if (i_init_min > i_fin_min) {
    i_min = i_fin_min;
    i_max = i_min + O + 1;
    iS[0] = ZERO;
#pragma unroll
    for (int j = 0; j < O + 1; j++) iS[j + 1] = iS_[j];
#pragma unroll
    for (int j = 0; j < O + 1; j++) fS[j] = fS_[j];
    fS[O + 1] = ZERO;
  } else {
    i_min = i_init_min;
    i_max = i_min + O;
#pragma unroll
    for (int j = 0; j < O + 1; j++) iS[j] = iS_[j];
    iS[O + 1] = ZERO;
#pragma unroll
    for (int j = 0; j < O + 1; j++) fS[j] = fS_[j];
    fS[O + 1] = ZERO;
  }
}

// The first node of shape<O, false>'s support for the cell i and offset di:
// i at order 1, i - 1 at order 3, and at order 2 the one the offset's half
// of the cell selects (the same comparison shape makes)
template <int O, typename real>
__device__ __forceinline__ int shape_first_node(int i, real di) {
  if constexpr (O == 2) return di < (real)0.5 ? i - 1 : i;
  else                  return O == 3 ? i - 1 : i;
}

// true when for_deposit's initial and final supports start at the same node
// along every simulated axis: the Esirkepov box is then O + 1 nodes wide on
// each axis (for_deposit's third case), never O + 2
template <int D, int O, typename real, typename P>
__device__ __forceinline__ bool support_unmoved(const P& q) {
  bool same = true;
#pragma unroll
  for (int a = 0; a < D; ++a)
    same = same && shape_first_node<O>(q.ip[a], (real)q.dxp[a]) ==
                       shape_first_node<O>(q.i[a], (real)q.dx[a]);
  return same;
}

// for_deposit when both supports start at the same node (support_unmoved):
// its third case, with i_max = i_min + O known to the compiler's caller
template <int O, typename real>
__device__ __forceinline__ void for_deposit_unmoved(int i_init, real di_init, int i_fin,
                                                    real di_fin, int& i_min, real* iS, real* fS) {
  int  i_fin_min;
  real iS_[O + 1], fS_[O + 1];
  shape<O, false>(i_init, di_init, i_min, iS_);
  shape<O, false>(i_fin, di_fin, i_fin_min, fS_);
#pragma unroll
  for (int j = 0; j < O + 1; j++) {
    iS[j] = iS_[j];
    fS[j] = fS_[j];
  }
  iS[O + 1] = (real)0;
  fS[O + 1] = (real)0;
}

// ---------------------------------------------------------------------------
// field access through a small view; ghost-inclusive indices
// ---------------------------------------------------------------------------
template <typename real>
struct FieldView {
  real*   p;
  int64_t s0, s1, s2, s3;
  __device__ __forceinline__ int64_t idx(int i, int j, int k, int c) const {
    return (int64_t)i * s0 + (int64_t)j * s1 + (int64_t)k * s2 + (int64_t)c * s3;
  }
  __device__ __forceinline__ real ld(int i, int j, int k, int c) const {
    return __ldg(p + idx(i, j, k, c));
  }
};

// a window of a field staged in shared memory: ghost-inclusive index g maps
// to window index g - off along every axis; 32-bit strides
template <typename real>
struct SmemView {
  const real* p;
  int         off0, off1, off2;
  int         s1, s2, s3;
  __device__ __forceinline__ real ld(int i, int j, int k, int c) const {
    return p[(i - off0) + (j - off1) * s1 + (k - off2) * s2 + c * s3];
  }
};

// ---------------------------------------------------------------------------
// interpolation: src/kernels/pushers/sr.hpp:851-1369 (V = FieldView or SmemView)
// ---------------------------------------------------------------------------
template <int D, typename real, typename V>
__device__ __forceinline__ void interp_zigzag(const V& EB, const int* ic,
                                              const real* d_, real* e0, real* b0) {
  const real ONE = 1, HALF = 0.5;
  int        ind[3];
  real       wpm[3], wpp[3], wdm[3], wdp[3];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    ind[a] = (int)(d_[a] + HALF);
    wpm[a] = ONE - d_[a];
    wpp[a] = d_[a];
    wdm[a] = (real)(ind[a] + 1) - (d_[a] + HALF);
    wdp[a] = ONE - wdm[a];
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    int  lo[3] = { 0, 0, 0 };
    real wm[3], wp[3];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      if (stag_of(c, a)) {
        lo[a] = ic[a] - 1 + ind[a];
        wm[a] = wdm[a];
        wp[a] = wdp[a];
      } else {
        lo[a] = ic[a];
        wm[a] = wpm[a];
        wp[a] = wpp[a];
      }
    }
    if (D == 3 && c == 5) {
      // the reference's 3D Bx3 (sr.hpp:1100-1116) reads the dual x2 stencil
      // (j - 1 + indy, j + indy) with the primal weights ponpmy / ponppy
      wm[1] = wpm[1];
      wp[1] = wpp[1];
    }
    real v;
    if constexpr (D == 2) {
      // sr.hpp:905-977
      const real c000 = EB.ld(lo[0], lo[1], 0, c);
      const real c100 = EB.ld(lo[0] + 1, lo[1], 0, c);
      const real c010 = EB.ld(lo[0], lo[1] + 1, 0, c);
      const real c110 = EB.ld(lo[0] + 1, lo[1] + 1, 0, c);
      const real c00  = c000 * wm[0] + c100 * wp[0];
      const real c10  = c010 * wm[0] + c110 * wp[0];
      v               = c00 * wm[1] + c10 * wp[1];
    } else {
      // sr.hpp:978-1117
      const real c000 = EB.ld(lo[0], lo[1], lo[2], c);
      const real c100 = EB.ld(lo[0] + 1, lo[1], lo[2], c);
      const real c010 = EB.ld(lo[0], lo[1] + 1, lo[2], c);
      const real c110 = EB.ld(lo[0] + 1, lo[1] + 1, lo[2], c);
      const real c001 = EB.ld(lo[0], lo[1], lo[2] + 1, c);
      const real c101 = EB.ld(lo[0] + 1, lo[1], lo[2] + 1, c);
      const real c011 = EB.ld(lo[0], lo[1] + 1, lo[2] + 1, c);
      const real c111 = EB.ld(lo[0] + 1, lo[1] + 1, lo[2] + 1, c);
      const real c00  = c000 * wm[0] + c100 * wp[0];
      const real c10  = c010 * wm[0] + c110 * wp[0];
      const real c0   = c00 * wm[1] + c10 * wp[1];
      const real c01  = c001 * wm[0] + c101 * wp[0];
      const real c11  = c011 * wm[0] + c111 * wp[0];
      const real c1   = c01 * wm[1] + c11 * wp[1];
      v               = c0 * wm[2] + c1 * wp[2];
    }
    if (c < 3) e0[c] = v; else b0[c - 3] = v;
  }
}

template <int D, int O, typename real, typename V>
__device__ __forceinline__ void interp_shape(const V& EB, const int* ic,
                                             const real* dc, real* e0, real* b0) {
  // sr.hpp:1151-1369; running sums c += S * EB, rounded separately
  int  pmin[3] = { 0, 0, 0 }, dmin[3] = { 0, 0, 0 };
  real Sp[3][O + 1], Sd[3][O + 1];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    shape<O, false>(ic[a], dc[a], pmin[a], Sp[a]);
    shape<O, true>(ic[a], dc[a], dmin[a], Sd[a]);
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const int s0 = stag_of(c, 0), s1 = stag_of(c, 1), s2 = stag_of(c, 2);
    const int m0 = s0 ? dmin[0] : pmin[0];
    const int m1 = s1 ? dmin[1] : pmin[1];
    real      v  = 0;
    if constexpr (D == 2) {
#pragma unroll
      for (int b = 0; b < O + 1; b++) {
        real c0 = 0;
#pragma unroll
        for (int a = 0; a < O + 1; a++) {
          c0 = iacc(s0 ? Sd[0][a] : Sp[0][a], EB.ld(m0 + a, m1 + b, 0, c), c0);
        }
        v = iacc(c0, s1 ? Sd[1][b] : Sp[1][b], v);
      }
    } else {
      const int m2 = s2 ? dmin[2] : pmin[2];
#pragma unroll
      for (int cc = 0; cc < O + 1; cc++) {
        real c0 = 0;
#pragma unroll
        for (int b = 0; b < O + 1; b++) {
          real c00 = 0;
#pragma unroll
          for (int a = 0; a < O + 1; a++) {
            c00 = iacc(s0 ? Sd[0][a] : Sp[0][a], EB.ld(m0 + a, m1 + b, m2 + cc, c), c00);
          }
          c0 = iacc(c00, s1 ? Sd[1][b] : Sp[1][b], c0);
        }
        v = iacc(c0, s2 ? Sd[2][cc] : Sp[2][cc], v);
      }
    }
    if (c < 3) e0[c] = v; else b0[c - 3] = v;
  }
}

// ---------------------------------------------------------------------------
// velocity updates: sr.hpp:337-437
// ---------------------------------------------------------------------------
template <typename real>
__device__ __forceinline__ void boris(real ndth, real* u, real* e0, real* b0) {
  const real ONE = 1, TWO = 2;
  real       COEFF = ndth;
  e0[0] *= COEFF;
  e0[1] *= COEFF;
  e0[2] *= COEFF;
  real u0[3] = { u[0] + e0[0], u[1] + e0[1], u[2] + e0[2] };
  COEFF *= ONE / sqrt(ONE + (u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]));
  b0[0] *= COEFF;
  b0[1] *= COEFF;
  b0[2] *= COEFF;
  COEFF = TWO / (ONE + (b0[0] * b0[0] + b0[1] * b0[1] + b0[2] * b0[2]));
  const real u1[3] = { (u0[0] + (u0[1] * b0[2] - u0[2] * b0[1])) * COEFF,
                       (u0[1] + (u0[2] * b0[0] - u0[0] * b0[2])) * COEFF,
                       (u0[2] + (u0[0] * b0[1] - u0[1] * b0[0])) * COEFF };
  u0[0] += (u1[1] * b0[2] - u1[2] * b0[1]) + e0[0];
  u0[1] += (u1[2] * b0[0] - u1[0] * b0[2]) + e0[1];
  u0[2] += (u1[0] * b0[1] - u1[1] * b0[0]) + e0[2];
  u[0] = u0[0];
  u[1] = u0[1];
  u[2] = u0[2];
}

template <typename real>
__device__ __forceinline__ void vay(real ndth, real* u, real* e0, real* b0) {
  const real ONE = 1, TWO = 2, INV_2 = 0.5;
  real       COEFF = ndth;
  e0[0] *= COEFF;
  e0[1] *= COEFF;
  e0[2] *= COEFF;
  b0[0] *= COEFF;
  b0[1] *= COEFF;
  b0[2] *= COEFF;
  COEFF      = ONE / sqrt(ONE + (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
  real u1[3] = { (u[0] + TWO * e0[0] + (u[1] * b0[2] - u[2] * b0[1]) * COEFF),
                 (u[1] + TWO * e0[1] + (u[2] * b0[0] - u[0] * b0[2]) * COEFF),
                 (u[2] + TWO * e0[2] + (u[0] * b0[1] - u[1] * b0[0]) * COEFF) };
  COEFF       = (u1[0] * b0[0] + u1[1] * b0[1] + u1[2] * b0[2]);
  real COEFF2 = ONE + (u1[0] * u1[0] + u1[1] * u1[1] + u1[2] * u1[2]) -
                (b0[0] * b0[0] + b0[1] * b0[1] + b0[2] * b0[2]);
  COEFF = ONE / sqrt(INV_2 * (COEFF2 + sqrt(COEFF2 * COEFF2 +
                                            (real)4 * (b0[0] * b0[0] + b0[1] * b0[1] +
                                                       b0[2] * b0[2] + COEFF * COEFF))));
  COEFF2 = ONE / (ONE + (b0[0] * COEFF) * (b0[0] * COEFF) + (b0[1] * COEFF) * (b0[1] * COEFF) +
                  (b0[2] * COEFF) * (b0[2] * COEFF));
  const real dotub = (u1[0] * b0[0] + u1[1] * b0[1] + u1[2] * b0[2]);
  u[0] = COEFF2 * (u1[0] + COEFF * dotub * (b0[0] * COEFF) + u1[1] * b0[2] * COEFF -
                   u1[2] * b0[1] * COEFF);
  u[1] = COEFF2 * (u1[1] + COEFF * dotub * (b0[1] * COEFF) + u1[2] * b0[0] * COEFF -
                   u1[0] * b0[2] * COEFF);
  u[2] = COEFF2 * (u1[2] + COEFF * dotub * (b0[2] * COEFF) + u1[0] * b0[1] * COEFF -
                   u1[1] * b0[0] * COEFF);
}

// ---------------------------------------------------------------------------
// one particle's state in registers
// ---------------------------------------------------------------------------
template <typename real>
struct Prtl {
  int   i[3];
  float dx[3];
  int   ip[3];
  float dxp[3];
  real  u[3];
  short tag;
  int   wrap[3];  // periodic shift applied to i and ip by the boundary step
};

// positionPush (Cartesian) + boundaryConditions: sr.hpp:526-572, 659-814.
// `ip`, `dxp` receive the pre-move cell/offset (wrapped with the particle on a
// periodic crossing, as the reference does to i*_prev).
template <int D, typename real>
__device__ __forceinline__ void move_and_bound(Prtl<real>& q, bool massive, real dt, real dx,
                                               const PushConsts& pc) {
  const real ONE = 1, ZERO = 0;
  const real dt_inv_energy =
    massive ? (dt / sqrt(ONE + q.u[0] * q.u[0] + q.u[1] * q.u[1] + q.u[2] * q.u[2]))
            : (dt / sqrt(q.u[0] * q.u[0] + q.u[1] * q.u[1] + q.u[2] * q.u[2]));
#pragma unroll
  for (int a = 0; a < D; ++a) {
    q.ip[a]   = q.i[a];
    q.wrap[a] = 0;
    q.dxp[a] = q.dx[a];
    q.dx[a] += (q.u[a] / dx) * dt_inv_energy;
    q.i[a] += (int)(q.dx[a] >= ONE) - (int)(q.dx[a] < ZERO);
    q.dx[a] -= (q.dx[a] >= ONE);
    q.dx[a] += (q.dx[a] < ZERO);
  }
#pragma unroll
  for (int a = 0; a < D; ++a) {
    bool invert = false;
    if (q.i[a] < 0) {
      const int bc = pc.bc[a][0];
      if (bc == PIC_BC_PERIODIC) {
        q.i[a] += pc.n[a];
        q.ip[a] += pc.n[a];
        q.wrap[a] = pc.n[a];
      } else if (bc == PIC_BC_ABSORB) {
        q.tag = PIC_TAG_DEAD;
      } else if (bc == PIC_BC_REFLECT) {
        q.i[a]  = 0;
        q.dx[a] = ONE - q.dx[a];
        invert  = true;
      } else if (bc == PIC_BC_AXIS && a == 1) {
        q.i[a]  = 0;
        q.dx[a] = ONE - q.dx[a];
      }
    } else if (q.i[a] >= pc.n[a]) {
      const int bc = pc.bc[a][1];
      if (bc == PIC_BC_PERIODIC) {
        q.i[a] -= pc.n[a];
        q.ip[a] -= pc.n[a];
        q.wrap[a] = -pc.n[a];
      } else if (bc == PIC_BC_ABSORB) {
        q.tag = PIC_TAG_DEAD;
      } else if (bc == PIC_BC_REFLECT) {
        q.i[a]  = pc.n[a] - 1;
        q.dx[a] = ONE - q.dx[a];
        invert  = true;
      } else if (bc == PIC_BC_AXIS && a == 1) {
        q.i[a]  = pc.n[a] - 1;
        q.dx[a] = ONE - q.dx[a];
      }
    }
    if (invert) q.u[a] = -q.u[a];
  }
}

// ---------------------------------------------------------------------------
// current deposit of one particle: src/kernels/currents_deposit.hpp:108-761
// `add(i, j, k, c, v)` accumulates v into J at ghost-inclusive (i, j, k).
// ---------------------------------------------------------------------------
// Returns false, touching nothing, when the particle's stencil would reach
// outside the ghost-inclusive extents `ext` (possible only for moves longer
// than the ghost layers allow, i.e. a time step beyond the CFL limit);
// ext == nullptr skips the check (the caller guarantees the window).
template <int D, int O, typename real, bool UNMOVED = false, typename Add>
__device__ __forceinline__ bool deposit_with_velocity(const Prtl<real>& q, const real* vp,
                                                      real weight, real charge, real inv_dt,
                                                      int ng, const int* ext, Add&& add);

// Cartesian velocity of the deposit (currents_deposit.hpp:130-165); only the
// unsimulated direction's component enters a 2D deposit
template <int D, typename real>
__device__ __forceinline__ void deposit_velocity(const Prtl<real>& q, real dx, real* vp) {
  const real ONE = 1, ZERO = 0;
  vp[0] = q.u[0] / dx;
  vp[1] = q.u[1] / dx;
  vp[2] = (D == 3) ? q.u[2] / dx : q.u[2];
  const real inv_energy = ONE / sqrt(ONE + (q.u[0] * q.u[0] + q.u[1] * q.u[1] + q.u[2] * q.u[2]));
  if (isnan(vp[2]) || isinf(vp[2])) vp[2] = ZERO;
  vp[0] *= inv_energy;
  vp[1] *= inv_energy;
  vp[2] *= inv_energy;
}

template <int D, int O, typename real, typename Add>
__device__ __forceinline__ bool deposit_particle(const Prtl<real>& q, real weight, real charge,
                                                 real inv_dt, real dx, int ng, const int* ext,
                                                 Add&& add) {
  real vp[3];
  deposit_velocity<D, real>(q, dx, vp);
  return deposit_with_velocity<D, O, real>(q, vp, weight, charge, inv_dt, ng, ext, add);
}

// the deposit proper, given the particle velocity vp (the GR deposit passes
// its metric velocity, currents_deposit.hpp:138-159). UNMOVED (orders 1-3):
// the caller has checked support_unmoved, so every axis' box is O + 1 nodes
// wide and the stencil's extent is known at compile time; the entries and
// their values are those of the general form.
template <int D, int O, typename real, bool UNMOVED, typename Add>
__device__ __forceinline__ bool deposit_with_velocity(const Prtl<real>& q, const real* vp,
                                                      real weight, real charge, real inv_dt,
                                                      int ng, const int* ext, Add&& add) {
  static_assert(!UNMOVED || O >= 1, "the zigzag deposit has no support box");
  const real ONE = 1, HALF = 0.5, INV_2 = 0.5;
  if constexpr (O == 0) {
    if (ext) {
#pragma unroll
      for (int a = 0; a < D; ++a) {
        if (min(q.ip[a], q.i[a]) + ng < 0 || max(q.ip[a], q.i[a]) + ng + 1 >= ext[a]) return false;
      }
    }
  }
  const real coeff = weight * charge;

  if constexpr (O == 0) {
    // zigzag (currents_deposit.hpp:167-405)
    real W_1[3], W_2[3], F_1[3], F_2[3];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const int   ic = q.i[a], ip = q.ip[a];
      const float dxp_r = (float)(ic == ip) * (q.dx[a] + q.dxp[a]) * (float)INV_2;
      W_1[a] = INV_2 * ((real)(dxp_r + q.dxp[a]) + (real)(ic > ip));
      W_2[a] = INV_2 * ((real)(q.dx[a] + dxp_r) + (real)((int)(ic > ip) + ip - ic));
      F_1[a] = ((real)(ic > ip) + (real)dxp_r - (real)q.dxp[a]) * coeff * inv_dt;
      F_2[a] = ((real)(ic - ip - (int)(ic > ip)) + (real)q.dx[a] - (real)dxp_r) * coeff * inv_dt;
    }
    if constexpr (D == 2) {
      const real Fx3_1 = HALF * vp[2] * coeff;
      const real Fx3_2 = HALF * vp[2] * coeff;
      const int  a = q.ip[0] + ng, b = q.ip[1] + ng, c = q.i[0] + ng, d = q.i[1] + ng;
      add(a, b, 0, 0, F_1[0] * (ONE - W_1[1]));
      add(a, b + 1, 0, 0, F_1[0] * W_1[1]);
      add(c, d, 0, 0, F_2[0] * (ONE - W_2[1]));
      add(c, d + 1, 0, 0, F_2[0] * W_2[1]);
      add(a, b, 0, 1, F_1[1] * (ONE - W_1[0]));
      add(a + 1, b, 0, 1, F_1[1] * W_1[0]);
      add(c, d, 0, 1, F_2[1] * (ONE - W_2[0]));
      add(c + 1, d, 0, 1, F_2[1] * W_2[0]);
      add(a, b, 0, 2, Fx3_1 * (ONE - W_1[0]) * (ONE - W_1[1]));
      add(a + 1, b, 0, 2, Fx3_1 * W_1[0] * (ONE - W_1[1]));
      add(a, b + 1, 0, 2, Fx3_1 * (ONE - W_1[0]) * W_1[1]);
      add(a + 1, b + 1, 0, 2, Fx3_1 * W_1[0] * W_1[1]);
      add(c, d, 0, 2, Fx3_2 * (ONE - W_2[0]) * (ONE - W_2[1]));
      add(c + 1, d, 0, 2, Fx3_2 * W_2[0] * (ONE - W_2[1]));
      add(c, d + 1, 0, 2, Fx3_2 * (ONE - W_2[0]) * W_2[1]);
      add(c + 1, d + 1, 0, 2, Fx3_2 * W_2[0] * W_2[1]);
    } else {
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const int t1 = a == 0 ? 1 : 0;
        const int t2 = a == 2 ? 1 : 2;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int*  o = h == 0 ? q.ip : q.i;
          const real* W = h == 0 ? W_1 : W_2;
          const real  F = h == 0 ? F_1[a] : F_2[a];
#pragma unroll
          for (int s2 = 0; s2 < 2; ++s2) {
#pragma unroll
            for (int s1 = 0; s1 < 2; ++s1) {
              int idx[3] = { o[0] + ng, o[1] + ng, o[2] + ng };
              idx[t1] += s1;
              idx[t2] += s2;
              const real w1 = s1 ? W[t1] : (ONE - W[t1]);
              const real w2 = s2 ? W[t2] : (ONE - W[t2]);
              add(idx[0], idx[1], idx[2], a, F * w1 * w2);
            }
          }
        }
      }
    }
  } else {
    // Esirkepov (currents_deposit.hpp:406-754); jx arrays are formed on the
    // fly as running prefix sums instead of stored tensors
    constexpr int N = O + 2;
    real          iS[D][N], fS[D][N];
    int           imin[3] = { 0, 0, 0 }, imax[3] = { 0, 0, 0 };
#pragma unroll
    for (int a = 0; a < D; ++a) {
      if constexpr (UNMOVED) {
        for_deposit_unmoved<O>(q.ip[a], (real)q.dxp[a], q.i[a], (real)q.dx[a], imin[a], iS[a], fS[a]);
        imax[a] = imin[a] + O;
      } else {
        for_deposit<O>(q.ip[a], (real)q.dxp[a], q.i[a], (real)q.dx[a], imin[a], imax[a], iS[a], fS[a]);
      }
      if (ext && (imin[a] + ng < 0 || imax[a] + ng >= ext[a])) return false;
    }
    const real THIRD = K<real>::THIRD;
    const real Q     = coeff * inv_dt;
    const int  d1 = UNMOVED ? O : imax[0] - imin[0], d2 = UNMOVED ? O : imax[1] - imin[1];
    const int  i0 = imin[0] + ng, j0 = imin[1] + ng;
    // Every entry of the (O+2)-wide stencil is computed and only the add is
    // predicated on the stencil extent: the loops carry no divergent
    // branches. Each entry's arithmetic is the reference's expression; the
    // factors that do not depend on the innermost index are formed once.
    if constexpr (D == 2) {
      const real QVx3 = coeff * vp[2];
      real hd0[N], hs0[N];  // HALF * (fS - iS), HALF * (fS + iS) along x1
#pragma unroll
      for (int i = 0; i < N; ++i) {
        hd0[i] = HALF * (fS[0][i] - iS[0][i]);
        hs0[i] = HALF * (fS[0][i] + iS[0][i]);
      }
      // jx1: prefix over i (currents_deposit.hpp:496-518, 547-551)
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const real s1 = fS[1][j] + iS[1][j];
        real       acc = 0;
#pragma unroll
        for (int i = 0; i < N - 1; ++i) {
          const real W = hd0[i] * s1;
          acc          = (i == 0) ? (-Q * W) : (acc - Q * W);
          if (i < d1 && j <= d2) add(i0 + i, j0 + j, 0, 0, acc);
        }
      }
      // jx2: prefix over j
#pragma unroll
      for (int i = 0; i < N; ++i) {
        real acc = 0;
#pragma unroll
        for (int j = 0; j < N - 1; ++j) {
          const real W = hs0[i] * (fS[1][j] - iS[1][j]);
          acc          = (j == 0) ? (-Q * W) : (acc - Q * W);
          if (i <= d1 && j < d2) add(i0 + i, j0 + j, 0, 1, acc);
        }
      }
      // jx3
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const real ga = HALF * iS[0][i] + fS[0][i];
        const real gb = HALF * fS[0][i] + iS[0][i];
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const real W = THIRD * (fS[1][j] * ga + iS[1][j] * gb);
          if (i <= d1 && j <= d2) add(i0 + i, j0 + j, 0, 2, QVx3 * W);
        }
      }
    } else {
      const int d3 = UNMOVED ? O : imax[2] - imin[2];
      const int k0 = imin[2] + ng;
      real      t0[N], t1[N], t2[N];  // THIRD * (fS - iS) per axis
#pragma unroll
      for (int i = 0; i < N; ++i) {
        t0[i] = THIRD * (fS[0][i] - iS[0][i]);
        t1[i] = THIRD * (fS[1][i] - iS[1][i]);
        t2[i] = THIRD * (fS[2][i] - iS[2][i]);
      }
      // jx1: prefix over i (currents_deposit.hpp:620-700, 716-724)
#pragma unroll
      for (int j = 0; j < N; ++j) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
          const real P = (iS[1][j] * iS[2][k] + fS[1][j] * fS[2][k]) +
                         HALF * (iS[2][k] * fS[1][j] + iS[1][j] * fS[2][k]);
          const bool ok = (j <= d2) && (k <= d3);
          real       acc = 0;
#pragma unroll
          for (int i = 0; i < N - 1; ++i) {
            const real W = t0[i] * P;
            acc          = (i == 0) ? (-Q * W) : (acc - Q * W);
            if (ok && i < d1) add(i0 + i, j0 + j, k0 + k, 0, acc);
          }
        }
      }
      // jx2: prefix over j
#pragma unroll
      for (int i = 0; i < N; ++i) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
          const real P = iS[0][i] * iS[2][k] + fS[0][i] * fS[2][k] +
                         HALF * (iS[2][k] * fS[0][i] + iS[0][i] * fS[2][k]);
          const bool ok = (i <= d1) && (k <= d3);
          real       acc = 0;
#pragma unroll
          for (int j = 0; j < N - 1; ++j) {
            const real W = t1[j] * P;
            acc          = (j == 0) ? (-Q * W) : (acc - Q * W);
            if (ok && j < d2) add(i0 + i, j0 + j, k0 + k, 1, acc);
          }
        }
      }
      // jx3: prefix over k
#pragma unroll
      for (int i = 0; i < N; ++i) {
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const real P = iS[0][i] * iS[1][j] + fS[0][i] * fS[1][j] +
                         HALF * (iS[0][i] * fS[1][j] + iS[1][j] * fS[0][i]);
          const bool ok = (i <= d1) && (j <= d2);
          real       acc = 0;
#pragma unroll
          for (int k = 0; k < N - 1; ++k) {
            const real W = t2[k] * P;
            acc          = (k == 0) ? (-Q * W) : (acc - Q * W);
            if (ok && k < d3) add(i0 + i, j0 + j, k0 + k, 2, acc);
          }
        }
      }
    }
  }
  return true;
}

// true when the cell of every simulated axis lies in [0, n)
template <int D>
__device__ __forceinline__ bool cells_in_grid(const int* i, const int* n) {
  bool ok = true;
#pragma unroll
  for (int a = 0; a < D; ++a) ok = ok && (i[a] >= 0) && (i[a] < n[a]);
  return ok;
}

}  // namespace pic
