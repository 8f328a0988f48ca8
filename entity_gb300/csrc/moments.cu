// Particle diagnostics on the device.
//
// k_charge_density: the node charge density that the current deposit
// conserves. Esirkepov's scheme at order O (currents_deposit.hpp:406-754)
// builds its fluxes from differences of the unstaggered order-O shape
// (prtl_shape::order<false, O>, particle_shapes.hpp:544-614), so with
//   rho(n) = sum_p charge * w_p * prod_d S_O(n_d - x_p,d)
// the discrete continuity equation (rho_new - rho_old) / dt + D^- J = 0 holds
// cell by cell (D^- the backward difference of J's staggered components). The
// zigzag deposit (O = 0) conserves the linear (cloud-in-cell) density, so
// order 0 uses S_1.
//
// k_particle_moments: FP64 sums over alive particles of the SR stress-energy
// components of ReducedParticleMoments_kernel<SRPIC, Minkowski, T>
// (src/kernels/reduced_stats.hpp:403-538): T00 = m * gamma, T0i = u_i
// (unweighted, as the reference sums them), plus the weighted kinetic energy
// sum w * m * (gamma - 1) and the weight sum.
#include "moments.cuh"
#include "pic_common.cuh"

namespace pic {

template <int D, int O, typename real>
__global__ void __launch_bounds__(256) k_charge_density(SpeciesPtrs sp, FieldView<real> rho, int ng,
                                                        PushConsts pc, unsigned long long* err) {
  constexpr int OS = O == 0 ? 1 : O;  // shape order of the conserved density
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const real*   w      = (const real*)sp.w;
  const int32_t* ia[3] = { sp.i1, sp.i2, sp.i3 };
  const float*  da[3]  = { sp.dx1, sp.dx2, sp.dx3 };
  const real    charge = (real)sp.charge;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < sp.npart; p += stride) {
    if (sp.tag[p] != PIC_TAG_ALIVE) continue;
    int  imin[3] = { 0, 0, 0 };
    real S[3][OS + 1];
    bool ok = true;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      shape<OS, false>(ia[d][p], (real)da[d][p], imin[d], S[d]);
      if (imin[d] + ng < 0 || imin[d] + OS + ng >= pc.ext[d]) ok = false;
    }
    if (!ok) {
      atomicAdd(err + ERR_STENCIL_OUT, 1ull);
      continue;
    }
    const real q = charge * w[p];
    if constexpr (D == 2) {
#pragma unroll
      for (int j = 0; j <= OS; ++j) {
        const real qj = q * S[1][j];
#pragma unroll
        for (int i = 0; i <= OS; ++i)
          atomicAdd(rho.p + rho.idx(imin[0] + ng + i, imin[1] + ng + j, 0, 0), qj * S[0][i]);
      }
    } else {
#pragma unroll
      for (int k = 0; k <= OS; ++k) {
#pragma unroll
        for (int j = 0; j <= OS; ++j) {
          const real qjk = q * S[2][k] * S[1][j];
#pragma unroll
          for (int i = 0; i <= OS; ++i)
            atomicAdd(rho.p + rho.idx(imin[0] + ng + i, imin[1] + ng + j, imin[2] + ng + k, 0),
                      qjk * S[0][i]);
        }
      }
    }
  }
}

template <typename real>
__global__ void __launch_bounds__(256) k_particle_moments(SpeciesPtrs sp, double* out) {
  constexpr int NM = PIC_NMOMENTS;
  __shared__ double sh[NM][8];
  double        acc[NM] = { 0, 0, 0, 0, 0, 0 };
  const real*   ux[3]   = { (const real*)sp.ux1, (const real*)sp.ux2, (const real*)sp.ux3 };
  const real*   w       = (const real*)sp.w;
  const double  m       = (double)sp.mass;
  const int64_t stride  = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < sp.npart; p += stride) {
    if (sp.tag[p] != PIC_TAG_ALIVE) continue;
    const double u1 = (double)ux[0][p], u2 = (double)ux[1][p], u3 = (double)ux[2][p];
    const double u2s = u1 * u1 + u2 * u2 + u3 * u3;
    const double g   = sqrt(1.0 + u2s);
    const double wp  = (double)w[p];
    acc[0] += m == 0.0 ? sqrt(u2s) : m * g;
    acc[1] += u1;
    acc[2] += u2;
    acc[3] += u3;
    // gamma - 1 = u^2 / (gamma + 1) without the cancellation at small u
    acc[4] += wp * (m == 0.0 ? sqrt(u2s) : m * (u2s / (g + 1.0)));
    acc[5] += wp;
  }
#pragma unroll
  for (int k = 0; k < NM; ++k)
    for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NM; ++k) sh[k][wid] = acc[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NM; ++k) {
      double v = lane < (int)(blockDim.x >> 5) ? sh[k][lane] : 0.0;
      for (int o = 4; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) atomicAdd(out + k, v);
    }
  }
}

template <typename real>
cudaError_t launch_charge_density(int dim, int order, const SpeciesPtrs& sp, FieldView<real> rho,
                                  int ng, const PushConsts& pc, unsigned long long* err,
                                  cudaStream_t s) {
  if (sp.npart <= 0) return cudaSuccess;
  int64_t blocks = (sp.npart + 255) / 256;
  if (blocks > pic::sm_count() * 32) blocks = pic::sm_count() * 32;
  const unsigned b = (unsigned)blocks;
#define PIC_RHO(D, O) PIC_KL(k_charge_density<D, O, real><<<b, 256, 0, s>>>(sp, rho, ng, pc, err))
  if (dim == 2) {
    switch (order) {
      case 0: PIC_RHO(2, 0); break;
      case 1: PIC_RHO(2, 1); break;
      case 2: PIC_RHO(2, 2); break;
      default: PIC_RHO(2, 3); break;
    }
  } else {
    switch (order) {
      case 0: PIC_RHO(3, 0); break;
      case 1: PIC_RHO(3, 1); break;
      case 2: PIC_RHO(3, 2); break;
      default: PIC_RHO(3, 3); break;
    }
  }
#undef PIC_RHO
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_particle_moments(const SpeciesPtrs& sp, double* out, cudaStream_t s) {
  if (sp.npart <= 0) return cudaSuccess;
  int64_t blocks = (sp.npart + 255) / 256;
  if (blocks > pic::sm_count() * 8) blocks = pic::sm_count() * 8;
  PIC_KL(k_particle_moments<real><<<(unsigned)blocks, 256, 0, s>>>(sp, out));
  return cudaGetLastError();
}

template cudaError_t launch_charge_density<float>(int, int, const SpeciesPtrs&, FieldView<float>,
                                                  int, const PushConsts&, unsigned long long*,
                                                  cudaStream_t);
template cudaError_t launch_charge_density<double>(int, int, const SpeciesPtrs&, FieldView<double>,
                                                   int, const PushConsts&, unsigned long long*,
                                                   cudaStream_t);
template cudaError_t launch_particle_moments<float>(const SpeciesPtrs&, double*, cudaStream_t);
template cudaError_t launch_particle_moments<double>(const SpeciesPtrs&, double*, cudaStream_t);

}  // namespace pic
