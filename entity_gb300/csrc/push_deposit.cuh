// Particle push and current deposition kernels (SR, Minkowski).
//
// k_push_deposit runs one thread per particle over a grid-stride loop and
// serves three modes: the reference's separate pusher (Pusher_kernel,
// src/kernels/pushers/sr.hpp:117-332), its separate deposit
// (DepositCurrents_kernel, src/kernels/currents_deposit.hpp:108-761), and the
// fused pass that keeps the previous position in registers so the 12
// prev-arrays never round-trip through HBM.
#pragma once

#include "deposit_fixed.cuh"
#include "pic_common.cuh"

namespace pic {

enum Mode { MODE_PUSH = 0, MODE_DEPOSIT = 1, MODE_FUSED = 2 };

template <typename real>
struct PDArgs {
  SpeciesPtrs     sp;
  PushConsts      pc;
  FieldView<real> EB;
  FieldView<real> J;
  real            dt, dx, ndth, inv_dt, charge;
  int             vay;
  int             write_prev;
  unsigned long long* err;
  // optional: process only the particles listed (indices into the arrays),
  // *list_count of them (a device counter)
  const int32_t*  list       = nullptr;
  const unsigned* list_count = nullptr;
  // optional (FP32): deposit into the exact 64-bit accumulator instead of J
  FixedJ          fj;
};

// 2D FP32 asks for three CTAs per SM (80 registers instead of the
// allocator's 96, an 8-byte spill): the never-sorted two-stream adjoint
// problem's forward, which runs here, went from 134.1 to 128.8 ms
template <int D, int O, typename real, int MODE, bool PHOTON>
__global__ void __launch_bounds__(256, (D == 2 && sizeof(real) == 4) ? 3 : 1)
    k_push_deposit(PDArgs<real> a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  real*         ux[3]  = { (real*)a.sp.ux1, (real*)a.sp.ux2, (real*)a.sp.ux3 };
  const real*   w      = (const real*)a.sp.w;
  int32_t*      ia[3]  = { a.sp.i1, a.sp.i2, a.sp.i3 };
  int32_t*      ipa[3] = { a.sp.i1p, a.sp.i2p, a.sp.i3p };
  float*        da[3]  = { a.sp.dx1, a.sp.dx2, a.sp.dx3 };
  float*        dpa[3] = { a.sp.dx1p, a.sp.dx2p, a.sp.dx3p };
  const int64_t n = a.list ? (int64_t)*a.list_count : a.sp.npart;
  // exact accumulator: each contribution is rounded to a multiple of
  // 2^(ex - b) with b = min(30, bits), an int32 conversion (a 64-bit one
  // runs on the FP64 pipe), then shifted to the call's unit 2^(ex - bits)
  float fj_scale = 0.f;
  int   fj_shift = 0;
  if constexpr (sizeof(real) == 4 && MODE != MODE_PUSH) {
    if (a.fj.p) {
      const int b = min(30, a.fj.bits);
      fj_scale    = ldexpf(1.f, b - a.fj.exponent());
      fj_shift    = a.fj.bits - b;
    }
  }
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += stride) {
    const int64_t p = a.list ? (int64_t)a.list[t] : t;
    Prtl<real>    q;
    q.tag = a.sp.tag[p];
    if constexpr (MODE == MODE_DEPOSIT) {
      if (q.tag == PIC_TAG_DEAD) continue;
    } else {
      if (q.tag != PIC_TAG_ALIVE) {
        if (q.tag != PIC_TAG_DEAD) atomicAdd(a.err + ERR_BAD_TAG, 1ull);
        continue;
      }
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
      q.i[d]  = ia[d][p];
      q.dx[d] = da[d][p];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) q.u[d] = ux[d][p];
    if (!cells_in_grid<D>(q.i, a.pc.n)) {
      // a cell outside the grid is invalid input; report it, touch nothing
      atomicAdd(a.err + ERR_OUT_OF_GRID, 1ull);
      continue;
    }
    if constexpr (MODE == MODE_DEPOSIT) {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        q.ip[d]  = ipa[d][p];
        q.dxp[d] = dpa[d][p];
      }
    } else {
      if constexpr (!PHOTON) {
        real e0[3], b0[3];
        int  ic[3] = { q.i[0] + a.pc.ng, q.i[1] + a.pc.ng, D == 3 ? q.i[2] + a.pc.ng : 0 };
        real dc[3] = { (real)q.dx[0], (real)q.dx[1], D == 3 ? (real)q.dx[2] : (real)0 };
        if constexpr (O == 0) {
          interp_zigzag<D, real>(a.EB, ic, dc, e0, b0);
        } else {
          interp_shape<D, O, real>(a.EB, ic, dc, e0, b0);
        }
        // transform_xyz<U, XYZ> (src/metrics/minkowski.h:264-296)
#pragma unroll
        for (int d = 0; d < D; ++d) {
          e0[d] = e0[d] * a.dx;
          b0[d] = b0[d] * a.dx;
        }
        if (a.vay) {
          vay<real>(a.ndth, q.u, e0, b0);
        } else {
          boris<real>(a.ndth, q.u, e0, b0);
        }
      }
      move_and_bound<D, real>(q, !PHOTON, a.dt, a.dx, a.pc);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        ia[d][p] = q.i[d];
        da[d][p] = q.dx[d];
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) ux[d][p] = q.u[d];
      if (q.tag != PIC_TAG_ALIVE) a.sp.tag[p] = q.tag;
      if (MODE == MODE_PUSH || a.write_prev) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
          ipa[d][p] = q.ip[d];
          dpa[d][p] = q.dxp[d];
        }
      }
    }
    if constexpr (MODE != MODE_PUSH) {
      if (q.tag == PIC_TAG_DEAD) continue;
      const FieldView<real>& J    = a.J;
      auto                   to_J = [&](int i, int j, int k, int c, real v) {
        atomicAdd(J.p + J.idx(i, j, k, c), v);
      };
      bool ok;
      if constexpr (sizeof(real) == 4) {
        if (a.fj.p)
          ok = deposit_particle<D, O, real>(q, w[p], a.charge, a.inv_dt, a.dx, a.pc.ng, a.pc.ext,
                                            [&](int i, int j, int k, int c, real v) {
                                              const int x = __float2int_rn(v * fj_scale);
                                              a.fj.add_units(i, j, k, c,
                                                             (long long)((unsigned long long)
                                                                         (long long)x << fj_shift));
                                            });
        else
          ok = deposit_particle<D, O, real>(q, w[p], a.charge, a.inv_dt, a.dx, a.pc.ng, a.pc.ext,
                                            to_J);
      } else {
        ok = deposit_particle<D, O, real>(q, w[p], a.charge, a.inv_dt, a.dx, a.pc.ng, a.pc.ext,
                                          to_J);
      }
      if (!ok) atomicAdd(a.err + ERR_STENCIL_OUT, 1ull);
    }
  }
}

// host-side launcher, explicitly instantiated per (D, O, real)
template <int D, int O, typename real>
cudaError_t launch_push_deposit(const PDArgs<real>& a, int mode, bool photon, cudaStream_t s);

}  // namespace pic
