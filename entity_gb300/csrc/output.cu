// Output preparation on the device (the compute half of the reference's field
// and particle output; the file format is the caller's):
//   - ComputeMoments (src/framework/domain/metadomain_io.cpp:123-170) with
//     ParticleMoments_kernel<SRPIC, Minkowski, F> (src/kernels/
//     particle_moments.hpp:44-405): Rho, Charge, N, Nppc, T^{ab}, V deposited
//     at cell centres with a spline or constant smoothing window;
//   - SynchronizeFields(Comm::Bckp) for periodic axes (the additive ghost fold);
//   - NormalizeVectorByRho_kernel (particle_moments.hpp:407-478);
//   - ComputeDivergence_kernel (src/kernels/divergences.hpp), Cartesian;
//   - DeepCopyFields + FieldsToPhys_kernel<Minkowski> (src/kernels/
//     fields_to_phys.hpp:33-241) fused with the writer's downsampling
//     (src/output/writer.cpp:199-300): one pass from the staggered field to a
//     packed array of cell-centred tetrad components;
//   - PrtlToPhys_kernel<SRPIC, Minkowski, false> (src/kernels/prtls_to_phys.hpp:
//     28-218) as Particles::OutputWrite launches it
//     (src/framework/containers/particles_io.cpp:93-235): every stride-th
//     particle in physical coordinates.
// The moment deposit adds through global atomics, so its sums run in no fixed
// order, like the reference's ScatterView on CUDA.
#include <cmath>

#include "ctx_internal.cuh"

using namespace pic_internal;

namespace pic {
namespace {

// prtl_shape::S1..S6 (src/kernels/particle_shapes.hpp:25-166), x >= 0; the
// constants are rounded to real from their double quotients and every
// product and sum is evaluated in the reference's order
template <typename real>
__device__ real spline(int order, real x) {
  const real ZERO = 0, ONE = 1, TWO = 2, THREE = 3, HALF = 0.5, THREE_HALFS = 1.5;
  const real INV_4 = 0.25, INV_8 = 0.125, THREE_FOURTHS = 0.75;
  const real x2 = x * x, x3 = x * x * x;
  switch (order) {
    case 0: return ONE;
    case 1: return x < ONE ? ONE - x : ZERO;
    case 2:
      if (x < HALF) return (real)0.75 - x2;
      if (x < THREE_HALFS) return HALF * ((THREE_HALFS - x) * (THREE_HALFS - x));
      return ZERO;
    case 3:
      if (x < ONE) return (real)(2.0 / 3.0) - x2 + HALF * x3;
      if (x < TWO) return (real)(4.0 / 3.0) - TWO * x + x2 - (real)(1.0 / 6.0) * x3;
      return ZERO;
    case 4:
      if (x < HALF)
        return (real)(115.0 / 192.0) - (real)(5.0 / 8.0) * x2 + INV_4 * (x2 * x2);
      if (x < THREE_HALFS)
        return (real)(55.0 / 96.0) + (real)(5.0 / 24.0) * x - (real)(5.0 / 4.0) * x2 +
               (real)(5.0 / 6.0) * x3 - (real)(1.0 / 6.0) * (x2 * x2);
      if (x < (real)2.5)
        return (real)(625.0 / 384.0) - (real)(125.0 / 48.0) * x + (real)(25.0 / 16.0) * x2 -
               (real)(5.0 / 12.0) * x3 + (real)(1.0 / 24.0) * (x2 * x2);
      return ZERO;
    case 5:
      if (x <= ONE)
        return (real)(11.0 / 20.0) - HALF * x2 + INV_4 * (x2 * x2) - (real)(1.0 / 12.0) * x3 * x2;
      if (x < TWO)
        return (real)(17.0 / 40.0) + (real)(5.0 / 8.0) * x - (real)(7.0 / 4.0) * x2 +
               (real)(5.0 / 4.0) * x3 - (real)(3.0 / 8.0) * (x2 * x2) +
               (real)(1.0 / 24.0) * x3 * x2;
      if (x < THREE)
        return (real)(81.0 / 40.0) - (real)(27.0 / 8.0) * x + (real)(9.0 / 4.0) * x2 -
               THREE_FOURTHS * x3 + INV_8 * (x2 * x2) - (real)(1.0 / 120.0) * x3 * x2;
      return ZERO;
    case 6:
      if (x <= HALF)
        return (real)(5887.0 / 11520.0) - (real)(77.0 / 192.0) * x2 +
               (real)(7.0 / 48.0) * (x2 * x2) - (real)(1.0 / 36.0) * (x3 * x3);
      if (x < THREE_HALFS)
        return (real)(7861.0 / 15360.0) - (real)(7.0 / 768.0) * x - (real)(91.0 / 256.0) * x2 -
               (real)(35.0 / 288.0) * x3 + (real)(21.0 / 64.0) * (x2 * x2) -
               (real)(7.0 / 48.0) * x3 * x2 + (real)(1.0 / 48.0) * (x3 * x3);
      if (x < (real)2.5)
        return (real)(1379.0 / 7680.0) + (real)(1267.0 / 960.0) * x - (real)(329.0 / 128.0) * x2 +
               (real)(133.0 / 72.0) * x3 - (real)(21.0 / 32.0) * (x2 * x2) +
               (real)(7.0 / 60.0) * x3 * x2 - (real)(1.0 / 120.0) * (x3 * x3);
      if (x < (real)3.5)
        return (real)(117649.0 / 46080.0) - (real)(16807.0 / 3840.0) * x +
               (real)(2401.0 / 768.0) * x2 - (real)(343.0 / 288.0) * x3 +
               (real)(49.0 / 192.0) * (x2 * x2) - (real)(7.0 / 240.0) * x3 * x2 +
               (real)(1.0 / 720.0) * (x3 * x3);
      return ZERO;
  }
  return ZERO;
}

template <typename real>
struct MomArgs {
  SpeciesPtrs     sp;
  FieldView<real> buf;
  int             comp, ng, n[3];
  int             id, c1, c2, order, window, smoothing, use_weights;
  real            inv_n0, dx;
};

// ParticleMoments_kernel::operator() (particle_moments.hpp:291-404), Cartesian
template <int D, typename real>
__global__ void __launch_bounds__(256) k_output_moment(MomArgs<real> a, unsigned long long* err) {
  const real ZERO = 0, ONE = 1, TWO = 2, HALF = 0.5;
  const int64_t  stride = (int64_t)gridDim.x * blockDim.x;
  const int32_t* ia[3]  = { a.sp.i1, a.sp.i2, a.sp.i3 };
  const float*   da[3]  = { a.sp.dx1, a.sp.dx2, a.sp.dx3 };
  const real*    ux[3]  = { (const real*)a.sp.ux1, (const real*)a.sp.ux2, (const real*)a.sp.ux3 };
  const real*    w      = (const real*)a.sp.w;
  const real     mass = (real)a.sp.mass, m_or_1 = a.sp.mass == 0.0f ? ONE : mass;
  // sqrt_det_h of Minkowski<D> (src/metrics/minkowski.h:144-152)
  const real h = D == 2 ? a.dx * a.dx : a.dx * a.dx * a.dx;
  const real cst = ONE / (TWO * (real)a.window + ONE);
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.sp.npart; p += stride) {
    if (a.sp.tag[p] != PIC_TAG_ALIVE) continue;
    int  cell[3] = { 0, 0, 0 };
    bool ok      = true;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      cell[d] = ia[d][p];
      if (cell[d] < 0 || cell[d] >= a.n[d]) ok = false;
    }
    if (!ok) {
      atomicAdd(err + ERR_OUT_OF_GRID, 1ull);
      continue;
    }
    real coeff;
    if (a.id == PIC_MOM_T || a.id == PIC_MOM_V) {
      const real u[3] = { ux[0][p], ux[1][p], ux[2][p] };
      const real nsq  = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
      const real u0   = a.sp.mass == 0.0f ? sqrt(nsq) : sqrt(ONE + nsq);
      if (a.id == PIC_MOM_T) {
        coeff = m_or_1 / u0;
        coeff *= a.c1 > 0 ? u[a.c1 - 1] : u0;
        coeff *= a.c2 > 0 ? u[a.c2 - 1] : u0;
      } else {
        coeff = m_or_1 * u[a.c1 - 1] / u0;
      }
    } else {
      coeff = a.id == PIC_MOM_RHO ? mass : a.id == PIC_MOM_CHARGE ? (real)a.sp.charge : ONE;
    }
    if (a.id != PIC_MOM_NPPC) {
      coeff *= a.inv_n0 / h;
      if (a.use_weights) coeff *= w[p];
    }
    const int W = a.window;
    real      S[3][7];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      for (int q = 0; q <= 2 * W; ++q) {
        if (d >= D) {
          S[d][q] = ONE;
          continue;
        }
        const real dl = fabs((real)da[d][p] - ((real)(q - W) + HALF));
        S[d][q] = a.smoothing == PIC_SMOOTH_SPLINE ? spline<real>(a.order, dl) : cst;
      }
    const int k_hi = D == 3 ? 2 * W : 0;
    for (int k = 0; k <= k_hi; ++k)
      for (int j = 0; j <= 2 * W; ++j)
        for (int i = 0; i <= 2 * W; ++i) {
          real sh = S[0][i] * S[1][j];
          if (D == 3) sh = sh * S[2][k];
          const int t3 = D == 3 ? cell[2] + k - W + a.ng : 0;
          atomicAdd(a.buf.p + a.buf.idx(cell[0] + i - W + a.ng, cell[1] + j - W + a.ng, t3, a.comp),
                    coeff * sh);
        }
  }
  (void)ZERO;
}

// NormalizeVectorByRho_kernel (particle_moments.hpp:407-478): cmp::AlmostZero
// with the real type's epsilon (src/global/utils/comparators.h:37-42)
template <typename real>
__global__ void k_normalize_by_rho(GridInfo g, FieldView<real> f, int cr, int v1, int v2, int v3) {
  const real    eps   = sizeof(real) == 4 ? (real)1.1920928955078125e-07 : (real)2.220446049250313e-16;
  const int     n3    = g.dim == 3 ? g.n[2] : 1;
  const int64_t count = (int64_t)g.n[0] * g.n[1] * n3;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n[0]) + g.ng;
    const int j = (int)((t / g.n[0]) % g.n[1]) + g.ng;
    const int k = g.dim == 3 ? (int)(t / ((int64_t)g.n[0] * g.n[1])) + g.ng : 0;
    const real rho = f.p[f.idx(i, j, k, cr)];
    if (fabs(rho) <= eps) continue;
    f.p[f.idx(i, j, k, v1)] /= rho;
    f.p[f.idx(i, j, k, v2)] /= rho;
    f.p[f.idx(i, j, k, v3)] /= rho;
  }
}

// FieldsToPhys_kernel<Minkowski> (fields_to_phys.hpp:125-236) at the output
// cells (o1, o2, o3) * dwn (writer.cpp:199-300 with first cell 0), written to
// out[c][o3][o2][o1]
template <int D, typename real>
__global__ void k_output_field(GridInfo g, FieldView<real> F, int c0, int ncomp, unsigned flags,
                               real dx, int d1, int d2, int d3, int o1, int o2, int o3,
                               real* out) {
  const real    INV_2 = 0.5, INV_4 = 0.25;
  const int64_t count = (int64_t)o1 * o2 * o3;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(t % o1), b = (int)((t / o1) % o2), e = (int)(t / ((int64_t)o1 * o2));
    const int i = a * d1 + g.ng, j = b * d2 + g.ng, k = D == 3 ? e * d3 + g.ng : 0;
    auto      at = [&](int ii, int jj, int kk, int c) { return F.p[F.idx(ii, jj, kk, c0 + c)]; };
    real      f[3];
    if (ncomp == 1) {
      out[t] = at(i, j, k, 0);
      continue;
    }
    if (flags & PIC_OUT_INTERP_EDGES) {
      if (D == 2) {
        f[0] = INV_2 * (at(i, j, k, 0) + at(i, j + 1, k, 0));
        f[1] = INV_2 * (at(i, j, k, 1) + at(i + 1, j, k, 1));
        f[2] = INV_4 * (at(i, j, k, 2) + at(i + 1, j, k, 2) + at(i, j + 1, k, 2) +
                        at(i + 1, j + 1, k, 2));
      } else {
        f[0] = INV_4 * (at(i, j, k, 0) + at(i, j + 1, k, 0) + at(i, j, k + 1, 0) +
                        at(i, j + 1, k + 1, 0));
        f[1] = INV_4 * (at(i, j, k, 1) + at(i + 1, j, k, 1) + at(i, j, k + 1, 1) +
                        at(i + 1, j, k + 1, 1));
        f[2] = INV_4 * (at(i, j, k, 2) + at(i + 1, j, k, 2) + at(i, j + 1, k, 2) +
                        at(i + 1, j + 1, k, 2));
      }
    } else if (flags & PIC_OUT_INTERP_FACES) {
      f[0] = INV_2 * (at(i, j, k, 0) + at(i + 1, j, k, 0));
      f[1] = INV_2 * (at(i, j, k, 1) + at(i, j + 1, k, 1));
      f[2] = D == 3 ? INV_2 * (at(i, j, k, 2) + at(i, j, k + 1, 2)) : at(i, j, k, 2);
    } else {
      f[0] = at(i, j, k, 0);
      f[1] = at(i, j, k, 1);
      f[2] = at(i, j, k, 2);
    }
    // transform<Idx::U, Idx::T> of Minkowski (minkowski.h:263-300): times
    // sqrt(h_ii) = dx along the simulated axes
    if (flags & PIC_OUT_TO_HAT) {
      f[0] *= dx;
      f[1] *= dx;
      if (D == 3) f[2] *= dx;
    }
    out[t]             = f[0];
    out[t + count]     = f[1];
    out[t + 2 * count] = f[2];
  }
}

// ComputeDivergence_kernel<Minkowski> (src/kernels/divergences.hpp:23-135),
// Cartesian branch: the backward-difference divergence of E over the active
// cells, summed left to right as written there
template <int D, typename real>
__global__ void k_divergence(GridInfo g, FieldView<real> EB, FieldView<real> out, int comp) {
  const int     n3    = D == 3 ? g.n[2] : 1;
  const int64_t count = (int64_t)g.n[0] * g.n[1] * n3;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n[0]) + g.ng;
    const int j = (int)((t / g.n[0]) % g.n[1]) + g.ng;
    const int k = D == 3 ? (int)(t / ((int64_t)g.n[0] * g.n[1])) + g.ng : 0;
    real      v = EB.p[EB.idx(i, j, k, 0)] - EB.p[EB.idx(i - 1, j, k, 0)] +
             EB.p[EB.idx(i, j, k, 1)] - EB.p[EB.idx(i, j - 1, k, 1)];
    if (D == 3) v = v + EB.p[EB.idx(i, j, k, 2)] - EB.p[EB.idx(i, j, k - 1, 2)];
    out.p[out.idx(i, j, k, comp)] = v;
  }
}

template <typename real>
struct PrtlOutArgs {
  SpeciesPtrs sp;
  int64_t     stride, nout;
  int         dim;
  real        dx, xmin[3];
  real*       x[3];
  real*       u[3];
  real*       w;
};

// PrtlToPhys_kernel<SRPIC, Minkowski, false>::operator() (prtls_to_phys.hpp:
// 121-200): convert<Crd::Cd, Crd::Ph> is x * dx + x_min (minkowski.h:161-178),
// and transform_xyz<XYZ, T> leaves Cartesian velocities unchanged
template <typename real>
__global__ void k_output_particles(PrtlOutArgs<real> a) {
  const int32_t* ia[3] = { a.sp.i1, a.sp.i2, a.sp.i3 };
  const float*   da[3] = { a.sp.dx1, a.sp.dx2, a.sp.dx3 };
  const real*    ux[3] = { (const real*)a.sp.ux1, (const real*)a.sp.ux2, (const real*)a.sp.ux3 };
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.nout;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = p * a.stride;
    for (int d = 0; d < a.dim; ++d) {
      const real xc = (real)ia[d][q] + (real)da[d][q];
      a.x[d][p]     = xc * a.dx + a.xmin[d];
    }
    for (int d = 0; d < 3; ++d) a.u[d][p] = ux[d][q];
    a.w[p] = ((const real*)a.sp.w)[q];
  }
}

dim3 blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > pic::sm_count() * 32) b = pic::sm_count() * 32;
  return dim3((unsigned)b);
}

template <typename real>
int output_moment(pic_ctx* c, const pic_species* sp, int nsp, const pic_moment_params* prm,
                  void* bckp, int comp, cudaStream_t s) {
  MomArgs<real> a{};
  a.buf  = em_view<real>(c, bckp);
  a.comp = comp;
  a.ng   = c->grid.ng;
  for (int d = 0; d < 3; ++d) a.n[d] = c->grid.n[d];
  a.id          = prm->id;
  a.c1          = prm->c1;
  a.c2          = prm->c2;
  a.order       = prm->order;
  a.window      = (prm->order + 1) / 2;
  a.smoothing   = prm->smoothing;
  a.use_weights = prm->use_weights;
  a.inv_n0      = (real)prm->inv_n0;
  a.dx          = (real)prm->dx;
  for (int k = 0; k < nsp; ++k) {
    if (sp[k].npart == 0) continue;
    a.sp = sptrs(sp + k);
    if (c->grid.dim == 2)
      PIC_KL(k_output_moment<2, real><<<blocks_for(sp[k].npart), 256, 0, s>>>(a, c->d_err));
    else
      PIC_KL(k_output_moment<3, real><<<blocks_for(sp[k].npart), 256, 0, s>>>(a, c->d_err));
    if (cudaGetLastError() != cudaSuccess) return PIC_ERR_CUDA;
  }
  return PIC_OK;
}

template <typename real>
int output_field(pic_ctx* c, const void* src, int is_em, int c0, int ncomp, unsigned flags,
                 double dx, const int32_t dwn[3], void* out, cudaStream_t s) {
  const GridInfo  g = ginfo(c);
  FieldView<real> F = is_em ? em_view<real>(c, src) : cur_view<real>(c, src);
  int             o[3] = { 1, 1, 1 }, dd[3] = { 1, 1, 1 };
  for (int d = 0; d < g.dim; ++d) {
    dd[d] = dwn[d];
    o[d]  = (g.n[d] + dwn[d] - 1) / dwn[d];
  }
  const int64_t count = (int64_t)o[0] * o[1] * o[2];
  if (g.dim == 2)
    PIC_KL(k_output_field<2, real><<<blocks_for(count), 256, 0, s>>>(
      g, F, c0, ncomp, flags, (real)dx, dd[0], dd[1], dd[2], o[0], o[1], o[2], (real*)out));
  else
    PIC_KL(k_output_field<3, real><<<blocks_for(count), 256, 0, s>>>(
      g, F, c0, ncomp, flags, (real)dx, dd[0], dd[1], dd[2], o[0], o[1], o[2], (real*)out));
  return cuda_status(cudaGetLastError());
}

template <typename real>
int output_particles(pic_ctx* c, const pic_species* sp, int64_t stride, double dx,
                     const double xmin[3], void* const x[3], void* const u[3], void* w,
                     int64_t nout, cudaStream_t s) {
  PrtlOutArgs<real> a{};
  a.sp     = sptrs(sp);
  a.stride = stride;
  a.nout   = nout;
  a.dim    = c->grid.dim;
  a.dx     = (real)dx;
  for (int d = 0; d < 3; ++d) {
    a.xmin[d] = (real)xmin[d];
    a.x[d]    = d < a.dim ? (real*)x[d] : nullptr;
    a.u[d]    = (real*)u[d];
  }
  a.w = (real*)w;
  PIC_KL(k_output_particles<real><<<blocks_for(nout), 256, 0, s>>>(a));
  return cuda_status(cudaGetLastError());
}

}  // namespace
}  // namespace pic

extern "C" {

int pic_output_moment(pic_ctx* c, const pic_species* sp, int32_t nspecies,
                      const pic_moment_params* prm, void* bckp, int32_t comp, void* stream) {
  if (!c || !prm || !bckp || nspecies < 0 || (nspecies > 0 && !sp)) return PIC_ERR_ARG;
  if (comp < 0 || comp >= 6) return PIC_ERR_ARG;
  if (prm->id < PIC_MOM_RHO || prm->id > PIC_MOM_V) return PIC_ERR_ARG;
  // only the spline and constant windows exist (shapeFunction,
  // particle_moments.hpp:111-144); orders beyond 6 need more than 3 ghosts
  if (prm->smoothing != PIC_SMOOTH_SPLINE && prm->smoothing != PIC_SMOOTH_CONST) return PIC_ERR_ARG;
  if (prm->order < 0) return PIC_ERR_ARG;
  if (prm->order > 6) return PIC_ERR_UNSUPPORTED;
  if ((prm->order + 1) / 2 > c->grid.ng) return PIC_ERR_ARG;  // "Window size too large"
  if (prm->id == PIC_MOM_T && (prm->c1 < 0 || prm->c1 > 3 || prm->c2 < 0 || prm->c2 > 3))
    return PIC_ERR_ARG;
  if (prm->id == PIC_MOM_V && (prm->c1 < 1 || prm->c1 > 3)) return PIC_ERR_ARG;
  if (!(prm->dx > 0.0)) return PIC_ERR_ARG;
  for (int k = 0; k < nspecies; ++k) {
    int st = validate_species(c, sp + k, false);
    if (st != PIC_OK) return st;
    // "Rho & Charge for massless particles not defined"
    if ((prm->id == PIC_MOM_RHO || prm->id == PIC_MOM_CHARGE) && sp[k].mass == 0.0f)
      return PIC_ERR_ARG;
  }
  cudaStream_t s = strm(stream);
  return is_f64(c) ? pic::output_moment<double>(c, sp, nspecies, prm, bckp, comp, s)
                   : pic::output_moment<float>(c, sp, nspecies, prm, bckp, comp, s);
}

int pic_sync_moments(pic_ctx* c, void* bckp, int32_t c0, int32_t c1, void* stream) {
  if (!c || !bckp || c0 < 0 || c1 > 6 || c0 >= c1) return PIC_ERR_ARG;
  if (is_f64(c))
    return cuda_status(pic::launch_adj_fold<double>(ginfo(c), em_view<double>(c, bckp), c0, c1,
                                                    strm(stream)));
  return cuda_status(pic::launch_adj_fold<float>(ginfo(c), em_view<float>(c, bckp), c0, c1,
                                                 strm(stream)));
}

int pic_normalize_by_rho(pic_ctx* c, void* bckp, int32_t c_rho, int32_t c_v1, int32_t c_v2,
                         int32_t c_v3, void* stream) {
  if (!c || !bckp) return PIC_ERR_ARG;
  const int cs[4] = { c_rho, c_v1, c_v2, c_v3 };
  for (int a = 0; a < 4; ++a) {
    if (cs[a] < 0 || cs[a] >= 6) return PIC_ERR_ARG;
    for (int b = 0; b < a; ++b)
      if (cs[a] == cs[b]) return PIC_ERR_ARG;
  }
  const GridInfo g     = ginfo(c);
  const int64_t  cells = (int64_t)g.n[0] * g.n[1] * (g.dim == 3 ? g.n[2] : 1);
  cudaStream_t   s     = strm(stream);
  if (is_f64(c))
    PIC_KL(pic::k_normalize_by_rho<double><<<pic::blocks_for(cells), 256, 0, s>>>(
      g, em_view<double>(c, bckp), c_rho, c_v1, c_v2, c_v3));
  else
    PIC_KL(pic::k_normalize_by_rho<float><<<pic::blocks_for(cells), 256, 0, s>>>(
      g, em_view<float>(c, bckp), c_rho, c_v1, c_v2, c_v3));
  return cuda_status(cudaGetLastError());
}

int pic_output_divergence(pic_ctx* c, const void* EB, void* bckp, int32_t comp, void* stream) {
  if (!c || !EB || !bckp || comp < 0 || comp >= 6) return PIC_ERR_ARG;
  if (c->grid.ng < 1) return PIC_ERR_ARG;
  const GridInfo g     = ginfo(c);
  const int64_t  cells = (int64_t)g.n[0] * g.n[1] * (g.dim == 3 ? g.n[2] : 1);
  cudaStream_t   s     = strm(stream);
  if (is_f64(c)) {
    if (g.dim == 2)
      PIC_KL(pic::k_divergence<2, double><<<pic::blocks_for(cells), 256, 0, s>>>(
        g, em_view<double>(c, EB), em_view<double>(c, bckp), comp));
    else
      PIC_KL(pic::k_divergence<3, double><<<pic::blocks_for(cells), 256, 0, s>>>(
        g, em_view<double>(c, EB), em_view<double>(c, bckp), comp));
  } else {
    if (g.dim == 2)
      PIC_KL(pic::k_divergence<2, float><<<pic::blocks_for(cells), 256, 0, s>>>(
        g, em_view<float>(c, EB), em_view<float>(c, bckp), comp));
    else
      PIC_KL(pic::k_divergence<3, float><<<pic::blocks_for(cells), 256, 0, s>>>(
        g, em_view<float>(c, EB), em_view<float>(c, bckp), comp));
  }
  return cuda_status(cudaGetLastError());
}

int pic_output_field(pic_ctx* c, const void* src, int32_t is_em, int32_t c0, int32_t ncomp,
                     uint32_t flags, double dx, const int32_t dwn[3], void* out, void* stream) {
  if (!c || !src || !dwn || !out) return PIC_ERR_ARG;
  const int nc = is_em ? 6 : 3;
  if (ncomp != 1 && ncomp != 3) return PIC_ERR_ARG;
  if (c0 < 0 || c0 + ncomp > nc) return PIC_ERR_ARG;
  if (flags & ~(PIC_OUT_INTERP_EDGES | PIC_OUT_INTERP_FACES | PIC_OUT_TO_HAT)) return PIC_ERR_ARG;
  if ((flags & PIC_OUT_INTERP_EDGES) && (flags & PIC_OUT_INTERP_FACES)) return PIC_ERR_ARG;
  if (ncomp == 1 && flags != 0) return PIC_ERR_ARG;
  // the interpolation reads one cell beyond the active range
  if ((flags & (PIC_OUT_INTERP_EDGES | PIC_OUT_INTERP_FACES)) && c->grid.ng < 1) return PIC_ERR_ARG;
  if ((flags & PIC_OUT_TO_HAT) && !(dx > 0.0)) return PIC_ERR_ARG;
  for (int d = 0; d < c->grid.dim; ++d)
    if (dwn[d] < 1) return PIC_ERR_ARG;
  cudaStream_t s = strm(stream);
  return is_f64(c) ? pic::output_field<double>(c, src, is_em, c0, ncomp, flags, dx, dwn, out, s)
                   : pic::output_field<float>(c, src, is_em, c0, ncomp, flags, dx, dwn, out, s);
}

int pic_output_particles(pic_ctx* c, const pic_species* sp, int64_t stride, double dx,
                         const double xmin[3], void* const x_out[3], void* const u_out[3],
                         void* w_out, int64_t* nout, void* stream) {
  if (!c || !sp || !xmin || !x_out || !u_out || !w_out || !nout || stride < 1) return PIC_ERR_ARG;
  int st = validate_species(c, sp, false);
  if (st != PIC_OK) return st;
  const int64_t n = sp->npart / stride;
  *nout           = n;
  if (n == 0) return PIC_OK;
  for (int d = 0; d < c->grid.dim; ++d)
    if (!x_out[d]) return PIC_ERR_ARG;
  if (!u_out[0] || !u_out[1] || !u_out[2]) return PIC_ERR_ARG;
  cudaStream_t s = strm(stream);
  return is_f64(c) ? pic::output_particles<double>(c, sp, stride, dx, xmin, x_out, u_out, w_out, n, s)
                   : pic::output_particles<float>(c, sp, stride, dx, xmin, x_out, u_out, w_out, n, s);
}

}  // extern "C"
