// Reverse-mode (adjoint) SR step for 2D Cartesian periodic domains, Boris
// pusher, Esirkepov deposit at shape orders 1-3, Yee field solver.
//
// The forward step is SRPICEngine::step_forward (srpic.hpp:65-188):
//   B' = B + F E                     Faraday, half step
//   u1 = Boris(u0, dx * interp(E, B', X0));  X1 = X0 + (dt/dx) u1 / gamma1
//   J  = deposit(X0, X1, u1, w)      Esirkepov (currents_deposit.hpp:406-754)
//   J  = filter^n(fold(J))
//   B1 = B' + F E;  E1 = E + A B1 + jcoeff J
// Its adjoint runs the transposes in the opposite order. The particle part
// (k_push_deposit_adjoint) recomputes the step's interpolation, Boris update
// and move from the stored state at the start of the step with the forward's
// own device functions (so the linearisation point is the forward's
// trajectory bit for bit), then back-propagates the adjoint of J (through the
// deposit weights and their position derivatives), of the new position (the
// move), of the new momentum (Boris), and of the interpolated fields (shape
// derivatives; the field adjoint is scattered with atomics). The adjoint of
// the weights accumulates over steps (J is linear in w).
//
// Positions are differentiated as continuous coordinates X = i + dx; the
// cell index is piecewise constant. Shape order >= 2 makes the deposit and
// interpolation C^1 in X, so the gradient is almost everywhere smooth.
#include <algorithm>
#include <vector>

#include "ctx_internal.cuh"
#include "fields.cuh"
#include "pic_common.cuh"

using namespace pic_internal;

namespace pic {

// ---------------------------------------------------------------------------
// shape functions with their derivative in the in-cell offset
// (particle_shapes.hpp:25-63, 544-614); values come from the forward's shape
// ---------------------------------------------------------------------------
template <typename real>
__device__ __forceinline__ real S3d(real x) {
  const real ONE = 1, TWO = 2, HALF = 0.5, ONE_HALF = 1.5;
  if (x < ONE) return -TWO * x + ONE_HALF * (x * x);
  if (x < TWO) return -TWO + TWO * x - HALF * (x * x);
  return (real)0;
}

template <int O, bool STAG, typename real>
__device__ __forceinline__ void shape_d(int i, real di, int& imin, real* S, real* dS) {
  shape<O, STAG>(i, di, imin, S);
  const real ONE = 1, HALF = 0.5, TWO = 2;
  if constexpr (O == 1) {
    dS[0] = -ONE;
    dS[1] = ONE;
  } else if constexpr (O == 2) {
    if constexpr (!STAG) {
      if (di < HALF) {
        dS[0] = -(HALF - di);
        dS[1] = -TWO * di;
      } else {
        dS[0] = -((real)1.5 - di);
        dS[1] = TWO * (ONE - di);
      }
      dS[2] = -dS[0] - dS[1];
    } else {
      dS[0] = -(ONE - di);
      dS[2] = di;
      dS[1] = -dS[0] - dS[2];
    }
  } else {
    real c0;
    if constexpr (!STAG) c0 = ONE;
    else c0 = di < HALF ? (real)1.5 : HALF;
#pragma unroll
    for (int n = 0; n < 4; n++) {
      const real x = c0 + di - (real)n;
      dS[n]        = x < (real)0 ? -S3d<real>(-x) : S3d<real>(x);
    }
  }
}

// for_deposit (particle_shapes.hpp:934-1024) with the derivative arrays
// shifted like the values
template <int O, typename real>
__device__ __forceinline__ void for_deposit_d(int i_init, real di_init, int i_fin, real di_fin,
                                              int& i_min, int& i_max, real* iS, real* fS,
                                              real* idS, real* fdS) {
  int  imi, imf;
  real iS_[O + 1], fS_[O + 1], idS_[O + 1], fdS_[O + 1];
  shape_d<O, false>(i_init, di_init, imi, iS_, idS_);
  shape_d<O, false>(i_fin, di_fin, imf, fS_, fdS_);
  const real ZERO = 0;
#pragma unroll
  for (int j = 0; j < O + 2; ++j) {
    iS[j] = fS[j] = idS[j] = fdS[j] = ZERO;
  }
  if (imi < imf) {
    i_min = imi;
    i_max = i_min + O + 1;
#pragma unroll
    for (int j = 0; j < O + 1; j++) {
      iS[j]      = iS_[j];
      idS[j]     = idS_[j];
      fS[j + 1]  = fS_[j];
      fdS[j + 1] = fdS_[j];
    }
  } else if (imi > imf) {
    i_min = imf;
    i_max = i_min + O + 1;
#pragma unroll
    for (int j = 0; j < O + 1; j++) {
      iS[j + 1]  = iS_[j];
      idS[j + 1] = idS_[j];
      fS[j]      = fS_[j];
      fdS[j]     = fdS_[j];
    }
  } else {
    i_min = imi;
    i_max = i_min + O;
#pragma unroll
    for (int j = 0; j < O + 1; j++) {
      iS[j]  = iS_[j];
      idS[j] = idS_[j];
      fS[j]  = fS_[j];
      fdS[j] = fdS_[j];
    }
  }
}

// ---------------------------------------------------------------------------
// vector-Jacobian product of boris() (sr.hpp:337-368):
//   eps = ndth e; um = u0 + eps; k = ndth / sqrt(1 + |um|^2); t = k b;
//   f = 2 / (1 + |t|^2); w = f (um + um x t); u1 = um + w x t + eps
// ---------------------------------------------------------------------------
template <typename real>
__device__ __forceinline__ void cross(const real* a, const real* b, real* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

template <typename real>
__device__ __forceinline__ void boris_vjp(real ndth, const real* u0, const real* e, const real* b,
                                          const real* lu1, real* lu0, real* le, real* lb) {
  const real ONE = 1, TWO = 2;
  real       eps[3], um[3], t[3], v[3], w[3], umt[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    eps[c] = ndth * e[c];
    um[c]  = u0[c] + eps[c];
  }
  const real g = ONE / sqrt(ONE + (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]));
  const real k = ndth * g;
#pragma unroll
  for (int c = 0; c < 3; ++c) t[c] = k * b[c];
  const real f = TWO / (ONE + (t[0] * t[0] + t[1] * t[1] + t[2] * t[2]));
  cross(um, t, umt);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    v[c] = um[c] + umt[c];
    w[c] = f * v[c];
  }
  // u1 = um + w x t + eps
  real eps_b[3], um_b[3], w_b[3], t_b[3], tmp[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    eps_b[c] = lu1[c];
    um_b[c]  = lu1[c];
  }
  cross(t, lu1, w_b);    // d/dw of lu1 . (w x t)
  cross(lu1, w, t_b);    // d/dt
  // w = f v
  const real f_b = w_b[0] * v[0] + w_b[1] * v[1] + w_b[2] * v[2];
  real       v_b[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) v_b[c] = f * w_b[c];
  // v = um + um x t
  cross(t, v_b, tmp);
#pragma unroll
  for (int c = 0; c < 3; ++c) um_b[c] += v_b[c] + tmp[c];
  cross(v_b, um, tmp);
#pragma unroll
  for (int c = 0; c < 3; ++c) t_b[c] += tmp[c];
  // f = 2 / (1 + |t|^2): df/dt = -f^2 t
#pragma unroll
  for (int c = 0; c < 3; ++c) t_b[c] += -f_b * f * f * t[c];
  // t = k b
  const real k_b = t_b[0] * b[0] + t_b[1] * b[1] + t_b[2] * b[2];
#pragma unroll
  for (int c = 0; c < 3; ++c) lb[c] = k * t_b[c];
  // k = ndth (1 + |um|^2)^(-1/2): dk/dum = -k g^2 um
#pragma unroll
  for (int c = 0; c < 3; ++c) um_b[c] += -k_b * k * g * g * um[c];
  // um = u0 + eps; eps = ndth e
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    lu0[c] = um_b[c];
    eps_b[c] += um_b[c];
    le[c] = ndth * eps_b[c];
  }
}

// ---------------------------------------------------------------------------
// one step's particle adjoint, 2D
// ---------------------------------------------------------------------------
template <typename real>
struct AdjArgs {
  SpeciesPtrs     sp;   // state at the start of the step
  real*           lx[2];
  real*           lu[3];
  real*           lw;
  FieldView<real> EB;    // E at the start of the step, B after the first half Faraday
  FieldView<real> lamJ;  // adjoint of the filtered, folded J (ghost-filled)
  FieldView<real> lam;   // adjoint of (E, B'), accumulated (ghost-inclusive)
  PushConsts      pc;
  real            dt, dx, ndth, inv_dt, charge;
};

// FP32 asks for three CTAs per SM (80 registers instead of 128, spilling
// about 200 bytes): on the two-stream problem the gradient went from 489 to
// 464 ms, the forward being 128.6 ms
template <int O, typename real>
__global__ void __launch_bounds__(256, sizeof(real) == 4 ? 3 : 1)
    k_push_deposit_adjoint(AdjArgs<real> a) {
  constexpr int N     = O + 2;
  const real    ONE   = 1, HALF = 0.5;
  const real    THIRD = K<real>::THIRD;
  const int     ng    = a.pc.ng;
  const int     lane  = threadIdx.x & 31;
  const real*   uxa[3] = { (const real*)a.sp.ux1, (const real*)a.sp.ux2, (const real*)a.sp.ux3 };
  const real*   wa     = (const real*)a.sp.w;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // whole warps iterate together (blockDim is a multiple of 32) so that the
  // field-adjoint scatter can be reduced across lanes
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < a.sp.npart; base += stride) {
    const int64_t p     = base + threadIdx.x;
    const bool    valid = p < a.sp.npart && a.sp.tag[p] == PIC_TAG_ALIVE;
    // per-lane state the scatter needs
    int  pmin[2] = { 0, 0 }, dmin[2] = { 0, 0 };
    real Sp[2][O + 1], Sd[2][O + 1], lv6[6];
#pragma unroll
    for (int d = 0; d < 2; ++d)
#pragma unroll
      for (int k = 0; k < O + 1; ++k) Sp[d][k] = Sd[d][k] = (real)0;
#pragma unroll
    for (int c = 0; c < 6; ++c) lv6[c] = (real)0;
    unsigned long long key = ~0ull - (unsigned long long)lane;
    if (valid) {
      Prtl<real> q;
      q.tag     = PIC_TAG_ALIVE;
      q.i[0]    = a.sp.i1[p];
      q.i[1]    = a.sp.i2[p];
      q.i[2]    = 0;
      q.dx[0]   = a.sp.dx1[p];
      q.dx[1]   = a.sp.dx2[p];
      q.dx[2]   = 0.0f;
      real u0[3] = { uxa[0][p], uxa[1][p], uxa[2][p] };
      const real w = wa[p];
      const int  ic[2] = { q.i[0] + ng, q.i[1] + ng };
      const real dc[2] = { (real)q.dx[0], (real)q.dx[1] };
      key = ((unsigned long long)(uint32_t)q.i[0] << 34) | ((unsigned long long)(uint32_t)q.i[1] << 2) |
            ((unsigned long long)(dc[0] < HALF) << 1) | (unsigned long long)(dc[1] < HALF);
      // --- interpolation with its position derivative; the value follows
      // interp_shape's operation order (sr.hpp:1151-1369) bit for bit ------
      real dSp[2][O + 1], dSd[2][O + 1];
#pragma unroll
      for (int d = 0; d < 2; ++d) {
        shape_d<O, false>(ic[d], dc[d], pmin[d], Sp[d], dSp[d]);
        shape_d<O, true>(ic[d], dc[d], dmin[d], Sd[d], dSd[d]);
      }
      real val[6], D0[6], D1[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const int s0 = stag_of(c, 0), s1 = stag_of(c, 1);
        const int m0 = s0 ? dmin[0] : pmin[0];
        const int m1 = s1 ? dmin[1] : pmin[1];
        real      v = 0, d0 = 0, d1 = 0;
#pragma unroll
        for (int bj = 0; bj < O + 1; bj++) {
          real r = 0, rd = 0;
#pragma unroll
          for (int ai = 0; ai < O + 1; ai++) {
            const real F = a.EB.ld(m0 + ai, m1 + bj, 0, c);
            r            = iacc(s0 ? Sd[0][ai] : Sp[0][ai], F, r);
            rd += (s0 ? dSd[0][ai] : dSp[0][ai]) * F;
          }
          v = iacc(r, s1 ? Sd[1][bj] : Sp[1][bj], v);
          d0 += (s1 ? Sd[1][bj] : Sp[1][bj]) * rd;
          d1 += (s1 ? dSd[1][bj] : dSp[1][bj]) * r;
        }
        val[c] = v;
        D0[c]  = d0;
        D1[c]  = d1;
      }
      // transform_xyz (minkowski.h:264-296), Boris and the move, as forward
      real e[3] = { val[0] * a.dx, val[1] * a.dx, val[2] };
      real b[3] = { val[3] * a.dx, val[4] * a.dx, val[5] };
      real ee[3] = { e[0], e[1], e[2] }, bb[3] = { b[0], b[1], b[2] };
#pragma unroll
      for (int c = 0; c < 3; ++c) q.u[c] = u0[c];
      boris<real>(a.ndth, q.u, ee, bb);
      move_and_bound<2, real>(q, true, a.dt, a.dx, a.pc);
      const real u1[3] = { q.u[0], q.u[1], q.u[2] };
      const real ig    = ONE / sqrt(ONE + (u1[0] * u1[0] + u1[1] * u1[1] + u1[2] * u1[2]));

      // --- deposit adjoint -------------------------------------------------
      real iS[2][N], fS[2][N], idS[2][N], fdS[2][N];
      int  imin[2], imax[2];
#pragma unroll
      for (int d = 0; d < 2; ++d)
        for_deposit_d<O, real>(q.ip[d], (real)q.dxp[d], q.i[d], (real)q.dx[d], imin[d], imax[d],
                               iS[d], fS[d], idS[d], fdS[d]);
      const int d1 = imax[0] - imin[0], d2 = imax[1] - imin[1];
      const int i0s = imin[0] + ng, j0s = imin[1] + ng;
      real Gf0[N], Gi0[N], Gf1[N], Gi1[N];
#pragma unroll
      for (int k = 0; k < N; ++k) Gf0[k] = Gi0[k] = Gf1[k] = Gi1[k] = (real)0;
      real Fu = 0;  // sum lamJ . J per unit (weight * charge)
      // jx1: J1(i, j) = -inv_dt sum_{i' <= i} hd0[i'] s1[j] for i < d1, j <= d2;
      // lamJ . J1 = -inv_dt sum_{i', j} hd0[i'] s1[j] A1(i', j) with A1 the
      // suffix sum of lamJ1 over i >= i'
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const real s1 = fS[1][j] + iS[1][j];
        real       A  = 0;
#pragma unroll
        for (int i = N - 2; i >= 0; --i) {
          if (i < d1 && j <= d2) A += a.lamJ.ld(i0s + i, j0s + j, 0, 0);
          const real hd = HALF * (fS[0][i] - iS[0][i]);
          const real tA = -a.inv_dt * A;
          Fu += tA * hd * s1;
          const real gh = tA * s1;
          Gf0[i] += HALF * gh;
          Gi0[i] -= HALF * gh;
          Gf1[j] += tA * hd;
          Gi1[j] += tA * hd;
        }
      }
      // jx2: prefix over j
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const real hs = HALF * (fS[0][i] + iS[0][i]);
        real       A  = 0;
#pragma unroll
        for (int j = N - 2; j >= 0; --j) {
          if (i <= d1 && j < d2) A += a.lamJ.ld(i0s + i, j0s + j, 0, 1);
          const real ds = fS[1][j] - iS[1][j];
          const real tA = -a.inv_dt * A;
          Fu += tA * hs * ds;
          const real gh = tA * ds;
          Gf0[i] += HALF * gh;
          Gi0[i] += HALF * gh;
          Gf1[j] += tA * hs;
          Gi1[j] -= tA * hs;
        }
      }
      // jx3 = vz THIRD (fS1 (iS0/2 + fS0) + iS1 (fS0/2 + iS0))
      real vz = u1[2] * ig;
      if (isnan(vz) || isinf(vz)) vz = 0;
      real F3 = 0;
      {
        real H0f[N], H0i[N], H1f[N], H1i[N];
#pragma unroll
        for (int k = 0; k < N; ++k) H0f[k] = H0i[k] = H1f[k] = H1i[k] = (real)0;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const real ga = HALF * iS[0][i] + fS[0][i];
          const real gb = HALF * fS[0][i] + iS[0][i];
#pragma unroll
          for (int j = 0; j < N; ++j) {
            if (!(i <= d1 && j <= d2)) continue;
            const real l = THIRD * a.lamJ.ld(i0s + i, j0s + j, 0, 2);
            F3 += l * (fS[1][j] * ga + iS[1][j] * gb);
            H1f[j] += l * ga;
            H1i[j] += l * gb;
            H0f[i] += l * (fS[1][j] + HALF * iS[1][j]);
            H0i[i] += l * (HALF * fS[1][j] + iS[1][j]);
          }
        }
#pragma unroll
        for (int k = 0; k < N; ++k) {
          Gf0[k] += vz * H0f[k];
          Gi0[k] += vz * H0i[k];
          Gf1[k] += vz * H1f[k];
          Gi1[k] += vz * H1i[k];
        }
        Fu += vz * F3;
      }
      const real coeff  = w * a.charge;
      real       gX1[2] = { 0, 0 }, gX0[2] = { 0, 0 };
#pragma unroll
      for (int k = 0; k < N; ++k) {
        gX1[0] += Gf0[k] * fdS[0][k];
        gX1[1] += Gf1[k] * fdS[1][k];
        gX0[0] += Gi0[k] * idS[0][k];
        gX0[1] += Gi1[k] * idS[1][k];
      }
      // --- adjoint of the new state ---------------------------------------
      real lX1[2] = { a.lx[0][p] + coeff * gX1[0], a.lx[1][p] + coeff * gX1[1] };
      real lX0[2] = { lX1[0] + coeff * gX0[0], lX1[1] + coeff * gX0[1] };
      real lu1[3] = { a.lu[0][p], a.lu[1][p], a.lu[2][p] };
      const real ig3 = ig * ig * ig;
      {
        // vz = u1_3 / gamma1
        const real gvz = coeff * F3;
        // X1_a = X0_a + (dt / dx) u1_a / gamma1
        const real s = a.dt / a.dx;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          real acc = 0;
#pragma unroll
          for (int d = 0; d < 2; ++d) acc += lX1[d] * ((c == d ? ig : (real)0) - u1[d] * u1[c] * ig3);
          lu1[c] += gvz * ((c == 2 ? ig : (real)0) - u1[2] * u1[c] * ig3) + s * acc;
        }
      }
      real lu0[3], le[3], lb[3];
      boris_vjp<real>(a.ndth, u0, e, b, lu1, lu0, le, lb);
      // --- interpolation adjoint: position part here, field part below ----
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const int cc = c < 3 ? c : c - 3;
        lv6[c]       = (c < 3 ? le[cc] : lb[cc]) * (cc < 2 ? a.dx : ONE);
        lX0[0] += lv6[c] * D0[c];
        lX0[1] += lv6[c] * D1[c];
      }
      a.lx[0][p] = lX0[0];
      a.lx[1][p] = lX0[1];
#pragma unroll
      for (int c = 0; c < 3; ++c) a.lu[c][p] = lu0[c];
      a.lw[p] += a.charge * Fu;
    }
    // --- field-adjoint scatter: lanes with the same cell and the same
    // half-cell side per axis have identical stencils; each run of such lanes
    // is summed with shuffles and its first lane issues the atomics ---------
    const unsigned long long kprev = __shfl_up_sync(0xffffffffu, key, 1);
    const bool               head  = lane == 0 || key != kprev;
    const unsigned           hm    = __ballot_sync(0xffffffffu, head);
    const unsigned           after = lane == 31 ? 0u : (hm & (0xffffffffu << (lane + 1)));
    const int                last  = after ? (__ffs(after) - 2) : 31;
    // no shuffles at all when every lane has its own stencil
    const unsigned runlen = head ? (unsigned)(last - lane + 1) : 1u;
    const unsigned maxrun = __reduce_max_sync(0xffffffffu, runlen);
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const int s0 = stag_of(c, 0), s1 = stag_of(c, 1);
      const int m0 = s0 ? dmin[0] : pmin[0];
      const int m1 = s1 ? dmin[1] : pmin[1];
#pragma unroll
      for (int bj = 0; bj < O + 1; bj++) {
#pragma unroll
        for (int ai = 0; ai < O + 1; ai++) {
          real v = lv6[c] * (s0 ? Sd[0][ai] : Sp[0][ai]) * (s1 ? Sd[1][bj] : Sp[1][bj]);
          if (maxrun > 1) {
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
              const real t = __shfl_down_sync(0xffffffffu, v, off);
              if (lane + off <= last) v += t;
            }
          }
          if (head && valid) atomicAdd(a.lam.p + a.lam.idx(m0 + ai, m1 + bj, 0, c), v);
        }
      }
    }
  }
}

template <typename real>
cudaError_t launch_push_deposit_adjoint(int order, const AdjArgs<real>& a, cudaStream_t s) {
  if (a.sp.npart <= 0) return cudaSuccess;
  int64_t blocks = (a.sp.npart + 255) / 256;
  if (blocks > pic::sm_count() * 32) blocks = pic::sm_count() * 32;
  const unsigned g = (unsigned)blocks;
  switch (order) {
    case 1: PIC_KL(k_push_deposit_adjoint<1, real><<<g, 256, 0, s>>>(a)); break;
    case 2: PIC_KL(k_push_deposit_adjoint<2, real><<<g, 256, 0, s>>>(a)); break;
    case 3: PIC_KL(k_push_deposit_adjoint<3, real><<<g, 256, 0, s>>>(a)); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// checkpoint store: slots of (EB span, per-species i, dx, u, tag), owned by
// the context and grown on demand
// ---------------------------------------------------------------------------
struct Slot {
  void*                 eb = nullptr;
  std::vector<void*>    prt;     // one buffer per species
  std::vector<size_t>   prt_bytes;
  std::vector<int64_t>  npart;
};

struct AdjointScratch {
  std::vector<Slot> slots;
  size_t            eb_bytes = 0;
  void*             lamJ     = nullptr;  // current layout, span of the field
  void*             ebh      = nullptr;  // E, B' scratch, EM layout
  void*             jtmp     = nullptr;  // filter ping-pong partner of lamJ
  size_t            jbytes   = 0;
};

void adjoint_release(AdjointScratch* a) {
  if (!a) return;
  for (auto& s : a->slots) {
    if (s.eb) cudaFree(s.eb);
    for (void* p : s.prt)
      if (p) cudaFree(p);
  }
  if (a->lamJ) cudaFree(a->lamJ);
  if (a->jtmp) cudaFree(a->jtmp);
  if (a->ebh) cudaFree(a->ebh);
  delete a;
}

}  // namespace pic

namespace {

// number of elements spanned by a field with `ncomp` components
int64_t field_span(const pic_grid& g, const int64_t* s, int ncomp) {
  int64_t m = 0;
  for (int d = 0; d < 3; ++d) {
    const int e = d < g.dim ? g.n[d] + 2 * g.ng : 1;
    m += (int64_t)(e - 1) * s[d];
  }
  return m + (int64_t)(ncomp - 1) * s[3] + 1;
}

size_t species_bytes(const pic_grid& g, int64_t n) {
  return (size_t)n * (size_t)(g.dim * 4 + g.dim * 4 + 3 * g.real_bytes + 2);
}

pic::AdjointScratch* scratch_of(pic_ctx* c) {
  if (!c->adjoint) c->adjoint = new pic::AdjointScratch();
  return c->adjoint;
}

int ensure_fields(pic_ctx* c) {
  auto* a = scratch_of(c);
  const size_t eb = (size_t)field_span(c->grid, c->grid.em_stride, 6) * c->grid.real_bytes;
  const size_t jb = (size_t)field_span(c->grid, c->grid.cur_stride, 3) * c->grid.real_bytes;
  if (!a->ebh) {
    if (cudaMalloc(&a->ebh, eb) != cudaSuccess) return PIC_ERR_NOMEM;
    a->eb_bytes = eb;
  }
  if (!a->lamJ) {
    if (cudaMalloc(&a->lamJ, jb) != cudaSuccess) return PIC_ERR_NOMEM;
    if (cudaMalloc(&a->jtmp, jb) != cudaSuccess) return PIC_ERR_NOMEM;
    a->jbytes = jb;
  }
  return PIC_OK;
}

// copies of the per-particle state arrays that a step changes
struct ArrayRef {
  void*  p;
  size_t esz;
};

std::vector<ArrayRef> state_arrays(const pic_grid& g, const pic_species& s) {
  std::vector<ArrayRef> v;
  int32_t* ia[3] = { s.i1, s.i2, s.i3 };
  float*   da[3] = { s.dx1, s.dx2, s.dx3 };
  for (int d = 0; d < g.dim; ++d) v.push_back({ ia[d], 4 });
  for (int d = 0; d < g.dim; ++d) v.push_back({ da[d], 4 });
  v.push_back({ s.ux1, (size_t)g.real_bytes });
  v.push_back({ s.ux2, (size_t)g.real_bytes });
  v.push_back({ s.ux3, (size_t)g.real_bytes });
  v.push_back({ s.tag, 2 });
  return v;
}

template <typename real>
pic::FieldView<real> view_of(const int64_t* s, const void* p) {
  return pic::FieldView<real>{ (real*)p, s[0], s[1], s[2], s[3] };
}

template <typename real>
int step_adjoint(pic_ctx* c, const pic_species* sp, pic_species_adjoint* adj, int nsp,
                 const void* EB, void* lamEB, const pic_step_params* p, cudaStream_t s) {
  auto*          a  = scratch_of(c);
  const auto     g  = ginfo(c);
  const auto     em = c->grid.em_stride;
  const auto     cu = c->grid.cur_stride;
  auto           lam  = view_of<real>(em, lamEB);
  auto           lamJ = view_of<real>(cu, a->lamJ);
  auto           ebh  = view_of<real>(em, a->ebh);
  // coefficients exactly as the forward engine derives them (fieldsolvers.h:36-200)
  const real dT_half = (real)0.5 * (real)p->correction * (real)p->dt;
  const real dT_full = (real)1 * (real)p->correction * (real)p->dt;
  const real h       = (real)p->dx * (real)p->dx;
  const real dx      = std::sqrt(h);
  const real f1      = dT_half / (dx * dx), f2 = dT_half;
  const real a1      = dT_full / (dx * dx), a2 = dT_full;
  const real jcoeff  = -(real)p->dt * (real)p->q0 / ((real)p->B0 * (real)p->V0);
  cudaError_t e;
#define PIC_CK(x)                                  \
  if ((e = (x)) != cudaSuccess) return PIC_ERR_CUDA;
  // E1 = E' + jcoeff J (J filtered and folded): lamJ, then the filter's
  // transpose (the binomial stencils are symmetric) and the fold's (the
  // adjoint of adding ghost images onto active cells is the ghost fill)
  PIC_CK(pic::launch_fill_ghosts<real>(g, lam, 0, 6, s));
  PIC_CK(pic::launch_adj_currents<real>(g, lam, lamJ, jcoeff, s));
  if (p->deposit_enabled && p->nfilter > 0) {
    PIC_CK(pic::launch_filter<real>(g, lamJ, view_of<real>(cu, a->jtmp), p->nfilter, s));
  }
  // E' = E + A B1  ->  lamB1 += A^T lamE
  PIC_CK(pic::launch_adj_ampere<real>(g, lam, a1, a2, s));
  // B1 = B' + F E  ->  lamE += F^T lamB1 (lamB' = lamB1)
  PIC_CK(pic::launch_fill_ghosts<real>(g, lam, 3, 6, s));
  PIC_CK(pic::launch_adj_faraday<real>(g, lam, f1, f2, s));
  PIC_CK(pic::launch_zero_ghosts<real>(g, lam, 0, 6, s));
  // (E, B') of the step: B' = B + F E recomputed with the forward kernel
  PIC_CK(cudaMemcpyAsync(a->ebh, EB, a->eb_bytes, cudaMemcpyDeviceToDevice, s));
  // every forward update leaves ghost images behind it; step 0 fills them
  PIC_CK(pic::launch_fill_ghosts<real>(g, ebh, 0, 6, s));
  {
    pic::Stencil<real> st{};
    PIC_CK(pic::launch_faraday<real>(g, ebh, f1, f2, st, true, s));
  }
  // particles
  for (int k = 0; k < nsp; ++k) {
    const pic_species& sk = sp[k];
    if (sk.pusher == PIC_PUSHER_NONE || sk.npart == 0) continue;
    pic::AdjArgs<real> aa;
    aa.sp    = sptrs(&sk);
    aa.lx[0] = (real*)adj[k].lx1;
    aa.lx[1] = (real*)adj[k].lx2;
    aa.lu[0] = (real*)adj[k].lu1;
    aa.lu[1] = (real*)adj[k].lu2;
    aa.lu[2] = (real*)adj[k].lu3;
    aa.lw    = (real*)adj[k].lw;
    aa.EB    = ebh;
    aa.lamJ  = lamJ;
    aa.lam   = lam;
    for (int d = 0; d < 3; ++d) {
      aa.pc.n[d]     = c->grid.n[d];
      aa.pc.bc[d][0] = c->grid.prtl_bc[d][0];
      aa.pc.bc[d][1] = c->grid.prtl_bc[d][1];
      aa.pc.ext[d]   = d < c->grid.dim ? c->grid.n[d] + 2 * c->grid.ng : 1;
    }
    aa.pc.ng   = c->grid.ng;
    aa.dt      = (real)p->dt;
    aa.dx      = (real)p->dx;
    const float qm = sk.charge / sk.mass;
    aa.ndth    = (real)0.5 * (real)qm * (real)p->omegaB0 * (real)p->dt;
    aa.inv_dt  = (real)1 / (real)p->dt;
    aa.charge  = p->deposit_enabled ? (real)sk.charge : (real)0;
    PIC_CK(pic::launch_push_deposit_adjoint<real>(c->grid.order, aa, s));
  }
  // the interpolation read ghost images of E and B': fold their adjoint back
  PIC_CK(pic::launch_adj_fold<real>(g, lam, 0, 6, s));
  // B' = B + F E  ->  lamE += F^T lamB' (lamB = lamB')
  PIC_CK(pic::launch_fill_ghosts<real>(g, lam, 3, 6, s));
  PIC_CK(pic::launch_adj_faraday<real>(g, lam, f1, f2, s));
  PIC_CK(pic::launch_zero_ghosts<real>(g, lam, 0, 6, s));
#undef PIC_CK
  return PIC_OK;
}

int check_adjoint_support(const pic_ctx* c, const pic_species* sp, int nsp,
                          const pic_step_params* p) {
  if (c->grid.dim != 2) return PIC_ERR_UNSUPPORTED;
  if (c->grid.order < 1 || c->grid.order > 3) return PIC_ERR_UNSUPPORTED;
  for (int d = 0; d < 2; ++d) {
    if (!c->grid.fld_periodic[d]) return PIC_ERR_UNSUPPORTED;
    if (c->grid.prtl_bc[d][0] != PIC_BC_PERIODIC || c->grid.prtl_bc[d][1] != PIC_BC_PERIODIC)
      return PIC_ERR_UNSUPPORTED;
  }
  if (!p->fieldsolver_enabled) return PIC_ERR_UNSUPPORTED;
  for (int k = 0; k < nsp; ++k) {
    const int st = validate_species(c, sp + k, false);
    if (st != PIC_OK) return st;
    if (sp[k].pusher != PIC_PUSHER_NONE && sp[k].pusher != PIC_PUSHER_BORIS)
      return PIC_ERR_UNSUPPORTED;
    if (sp[k].pusher == PIC_PUSHER_BORIS && sp[k].mass == 0.0f) return PIC_ERR_ARG;
  }
  return PIC_OK;
}

}  // namespace

extern "C" {

int pic_checkpoint_save(pic_ctx* c, int32_t slot, const pic_species* sp, int32_t nspecies,
                        const void* EB, void* stream) {
  if (!c || !EB || slot < 0 || nspecies < 0 || (nspecies > 0 && !sp)) return PIC_ERR_ARG;
  for (int k = 0; k < nspecies; ++k) {
    const int st = validate_species(c, sp + k, false);
    if (st != PIC_OK) return st;
  }
  auto*        a  = scratch_of(c);
  cudaStream_t s  = strm(stream);
  const size_t eb = (size_t)field_span(c->grid, c->grid.em_stride, 6) * c->grid.real_bytes;
  if ((int)a->slots.size() <= slot) a->slots.resize(slot + 1);
  pic::Slot& sl = a->slots[slot];
  if (!sl.eb && cudaMalloc(&sl.eb, eb) != cudaSuccess) return PIC_ERR_NOMEM;
  a->eb_bytes = eb;
  if (cudaMemcpyAsync(sl.eb, EB, eb, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return PIC_ERR_CUDA;
  sl.prt.resize(nspecies, nullptr);
  sl.prt_bytes.resize(nspecies, 0);
  sl.npart.resize(nspecies, 0);
  for (int k = 0; k < nspecies; ++k) {
    const size_t need = species_bytes(c->grid, sp[k].npart);
    if (sl.prt_bytes[k] < need) {
      if (sl.prt[k]) cudaFree(sl.prt[k]);
      sl.prt[k] = nullptr;
      if (need && cudaMalloc(&sl.prt[k], need) != cudaSuccess) return PIC_ERR_NOMEM;
      sl.prt_bytes[k] = need;
    }
    sl.npart[k] = sp[k].npart;
    char* dst   = (char*)sl.prt[k];
    for (const auto& r : state_arrays(c->grid, sp[k])) {
      const size_t n = (size_t)sp[k].npart * r.esz;
      if (n && cudaMemcpyAsync(dst, r.p, n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return PIC_ERR_CUDA;
      dst += n;
    }
  }
  return PIC_OK;
}

int pic_checkpoint_restore(pic_ctx* c, int32_t slot, pic_species* sp, int32_t nspecies, void* EB,
                           void* stream) {
  if (!c || !EB || slot < 0 || nspecies < 0 || (nspecies > 0 && !sp)) return PIC_ERR_ARG;
  auto* a = c->adjoint;
  if (!a || (int)a->slots.size() <= slot || !a->slots[slot].eb) return PIC_ERR_ARG;
  pic::Slot& sl = a->slots[slot];
  if ((int)sl.prt.size() != nspecies) return PIC_ERR_ARG;
  cudaStream_t s = strm(stream);
  if (cudaMemcpyAsync(EB, sl.eb, a->eb_bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return PIC_ERR_CUDA;
  for (int k = 0; k < nspecies; ++k) {
    if (sp[k].maxnpart > 0 && sl.npart[k] > sp[k].maxnpart) return PIC_ERR_ARG;
    sp[k].npart = sl.npart[k];
    const char* src = (const char*)sl.prt[k];
    for (const auto& r : state_arrays(c->grid, sp[k])) {
      const size_t n = (size_t)sl.npart[k] * r.esz;
      if (n && cudaMemcpyAsync(r.p, src, n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return PIC_ERR_CUDA;
      src += n;
    }
  }
  return PIC_OK;
}

int pic_checkpoint_view(pic_ctx* c, int32_t slot, const pic_species* like, int32_t nspecies,
                        pic_species* out, void** EB) {
  if (!c || !like || !out || !EB || slot < 0 || nspecies < 0) return PIC_ERR_ARG;
  auto* a = c->adjoint;
  if (!a || (int)a->slots.size() <= slot || !a->slots[slot].eb) return PIC_ERR_ARG;
  pic::Slot& sl = a->slots[slot];
  if ((int)sl.prt.size() != nspecies) return PIC_ERR_ARG;
  *EB = sl.eb;
  for (int k = 0; k < nspecies; ++k) {
    pic_species v = like[k];
    v.npart       = sl.npart[k];
    char*        q = (char*)sl.prt[k];
    const size_t n = (size_t)sl.npart[k];
    int32_t**    ia[3] = { &v.i1, &v.i2, &v.i3 };
    float**      da[3] = { &v.dx1, &v.dx2, &v.dx3 };
    for (int d = 0; d < c->grid.dim; ++d) {
      *ia[d] = (int32_t*)q;
      q += n * 4;
    }
    for (int d = 0; d < c->grid.dim; ++d) {
      *da[d] = (float*)q;
      q += n * 4;
    }
    v.ux1 = q;
    q += n * c->grid.real_bytes;
    v.ux2 = q;
    q += n * c->grid.real_bytes;
    v.ux3 = q;
    q += n * c->grid.real_bytes;
    v.tag = (int16_t*)q;
    v.i1_prev = v.i2_prev = v.i3_prev = nullptr;
    v.dx1_prev = v.dx2_prev = v.dx3_prev = nullptr;
    out[k] = v;
  }
  return PIC_OK;
}

int pic_checkpoint_release(pic_ctx* c) {
  if (!c) return PIC_ERR_ARG;
  if (cudaDeviceSynchronize() != cudaSuccess) return PIC_ERR_CUDA;
  pic::adjoint_release(c->adjoint);
  c->adjoint = nullptr;
  return PIC_OK;
}

int pic_field_energy_adjoint_seed(pic_ctx* c, const void* EB, void* lamEB, double dx,
                                  void* stream) {
  if (!c || !EB || !lamEB) return PIC_ERR_ARG;
  cudaStream_t s    = strm(stream);
  const size_t span = (size_t)field_span(c->grid, c->grid.em_stride, 6) * c->grid.real_bytes;
  if (cudaMemsetAsync(lamEB, 0, span, s) != cudaSuccess) return PIC_ERR_CUDA;
  const auto g = ginfo(c);
  return cuda_status(is_f64(c) ? pic::launch_adj_seed<double>(g, em_view<double>(c, EB),
                                                              em_view<double>(c, lamEB), dx, s)
                               : pic::launch_adj_seed<float>(g, em_view<float>(c, EB),
                                                             em_view<float>(c, lamEB), dx, s));
}

int pic_srpic_step_adjoint(pic_ctx* c, const pic_species* sp, pic_species_adjoint* adj,
                           int32_t nspecies, const void* EB, void* lamEB,
                           const pic_step_params* prm, void* stream) {
  if (!c || !EB || !lamEB || !prm || nspecies < 0 || (nspecies > 0 && (!sp || !adj)))
    return PIC_ERR_ARG;
  int st = check_adjoint_support(c, sp, nspecies, prm);
  if (st != PIC_OK) return st;
  for (int k = 0; k < nspecies; ++k) {
    if (sp[k].pusher == PIC_PUSHER_NONE || sp[k].npart == 0) continue;
    if (!adj[k].lx1 || !adj[k].lx2 || !adj[k].lu1 || !adj[k].lu2 || !adj[k].lu3 || !adj[k].lw)
      return PIC_ERR_ARG;
  }
  st = ensure_fields(c);
  if (st != PIC_OK) return st;
  cudaStream_t s = strm(stream);
  return is_f64(c) ? step_adjoint<double>(c, sp, adj, nspecies, EB, lamEB, prm, s)
                   : step_adjoint<float>(c, sp, adj, nspecies, EB, lamEB, prm, s);
}

}  // extern "C"
