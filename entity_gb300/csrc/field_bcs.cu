// SR field boundaries on non-periodic sides and their C ABI:
//   - perfect conductor: ConductorBoundaries_kernel (src/kernels/fields_bcs.hpp:
//     522-800) as PerfectConductorFieldsIn launches it
//     (src/engines/srpic/fields_bcs.h:352-472);
//   - MATCH: MatchBoundaries_kernel's SRPIC branch (fields_bcs.hpp:42-520) as
//     MatchFieldsIn selects its cells (srpic/fields_bcs.h:60-202), relaxing
//     toward a caller-held target field;
//   - the digital filter's conductor-wall stencils (DigitalFilter_kernel,
//     src/kernels/digital_filter.hpp:99-379).
// srpic::FieldBoundaries (srpic/fields_bcs.h:622-672) visits the sides in
// Directions<D>::orth order: -x1, -x2, (-x3, +x3,) +x2, +x1.
#include <algorithm>
#include <cmath>

#include "ctx_internal.cuh"

using namespace pic_internal;

namespace pic {

// one side of one axis: offsets k in [0, K) from the wall cell i_edge, every
// cell (ghosts included) of the two other axes. E: the tangential components
// vanish on the wall and the ghosts mirror the active cells (the normal
// component evenly across the face between i_edge - 1 and i_edge, the
// tangential ones oddly about i_edge); B the other way round.
template <typename real>
__global__ void k_conductor(FieldView<real> F, int dim, int axis, int hi, int i_edge, int K,
                            int ea, int eb, int set_e, int set_b) {
  const int64_t cnt = (int64_t)K * ea * eb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int k  = (int)(t % K);
    const int pa = (int)((t / K) % ea);
    const int pb = (int)(t / ((int64_t)K * ea));
    // the other two axes, in increasing order
    const int oa = axis == 0 ? 1 : 0, ob = axis == 2 ? 1 : 2;
    auto at = [&](int i, int c) -> real& {
      int x[3] = { 0, 0, 0 };
      x[axis] = i;
      x[oa]   = pa;
      if (dim == 3) x[ob] = pb;
      return F.p[F.idx(x[0], x[1], x[2], c)];
    };
    const int t1 = oa, t2 = dim == 3 ? ob : 2;  // tangential components
    if (set_e) {
      if (k == 0) {
        at(i_edge, t1) = 0;
        at(i_edge, t2) = 0;
      } else if (!hi) {
        at(i_edge - k, axis) = at(i_edge + k - 1, axis);
        at(i_edge - k, t1)   = -at(i_edge + k, t1);
        at(i_edge - k, t2)   = -at(i_edge + k, t2);
      } else {
        at(i_edge + k - 1, axis) = at(i_edge - k, axis);
        at(i_edge + k, t1)       = -at(i_edge - k, t1);
        at(i_edge + k, t2)       = -at(i_edge - k, t2);
      }
    }
    if (set_b) {
      if (k == 0) {
        at(i_edge, 3 + axis) = 0;
      } else if (!hi) {
        at(i_edge - k, 3 + axis) = -at(i_edge + k, 3 + axis);
        at(i_edge - k, 3 + t1)   = at(i_edge + k - 1, 3 + t1);
        at(i_edge - k, 3 + t2)   = at(i_edge + k - 1, 3 + t2);
      } else {
        at(i_edge + k, 3 + axis)     = -at(i_edge - k, 3 + axis);
        at(i_edge + k - 1, 3 + t1)   = at(i_edge - k, 3 + t1);
        at(i_edge + k - 1, 3 + t2)   = at(i_edge - k, 3 + t2);
      }
    }
  }
}

// MATCH on one side: over the cells [lo, hi) along `axis` (ghosts on the
// outer side included) and every cell of the other axes, each component
// relaxes toward the target T with s = tanh(4 |x - x_edge| / ds), x the
// physical coordinate along `axis` of the component's position (half a cell
// up where the component is staggered along that axis: E_c when c = axis,
// B_c when c != axis)
template <typename real>
__global__ void k_match_sr(FieldView<real> F, FieldView<real> T, int dim, int axis, int lo,
                           int hi, int ea, int eb, int ng, real x0, real dx, real x_edge, real ds,
                           int set_e, int set_b) {
  const int     L   = hi - lo;
  const int64_t cnt = (int64_t)L * ea * eb;
  const real    ONE = 1, FOUR = 4, H = 0.5;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i  = lo + (int)(t % L);
    const int pa = (int)((t / L) % ea);
    const int pb = (int)(t / ((int64_t)L * ea));
    const int oa = axis == 0 ? 1 : 0, ob = axis == 2 ? 1 : 2;
    int       x[3] = { 0, 0, 0 };
    x[axis] = i;
    x[oa]   = pa;
    if (dim == 3) x[ob] = pb;
    const real i_ = (real)(i - ng);
    // Minkowski convert<Cd, Ph>: x_min + x_Cd dx
    const real s0 = (real)tanh(fabs((x0 + i_ * dx) - x_edge) * FOUR / ds);
    const real sH = (real)tanh(fabs((x0 + (i_ + H) * dx) - x_edge) * FOUR / ds);
    for (int c = 0; c < 6; ++c) {
      if (c < 3 ? !set_e : !set_b) continue;
      const bool half = c < 3 ? (c == axis) : (c - 3 != axis);
      const real s    = half ? sH : s0;
      real&      v    = F.p[F.idx(x[0], x[1], x[2], c)];
      v = s * v + (ONE - s) * T.p[T.idx(x[0], x[1], x[2], c)];
    }
  }
}

// DigitalFilter_kernel with conductor walls (digital_filter.hpp:129-379):
// src is the pass's copy of J, dst is J. Active cells next to a conductor
// wall filter along the wall only, with the wall-normal component folded
// onto its inner neighbour; the rest use the full stencil. A cell takes the
// first matching case in the order x1, x2, x3; a case writes only the
// components the reference writes.
struct CondFlags {
  int lo[3], hi[3];
};
template <int D, typename real>
__global__ void k_filter_cond(GridInfo g, CondFlags cf, FieldView<real> B, FieldView<real> A) {
  const real INV_2 = 0.5, INV_4 = 0.25, INV_8 = 0.125, INV_16 = 0.0625, INV_32 = 0.03125,
             INV_64 = 0.015625, THREE = 3;
  const int     ng  = g.ng;
  const int     n0 = g.n[0], n1 = g.n[1], n2 = D == 3 ? g.n[2] : 1;
  const int64_t cnt = (int64_t)n0 * n1 * n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i1 = ng + (int)(t % n0);
    const int i2 = ng + (int)((t / n0) % n1);
    const int i3 = D == 3 ? ng + (int)(t / ((int64_t)n0 * n1)) : 0;
    const int i1min = ng, i1max = n0 + ng, i2min = ng, i2max = n1 + ng, i3min = ng,
              i3max = n2 + ng;
#define b(x, y, z, c) B.p[B.idx((x), (y), (z), (c))]
#define a(c)          A.p[A.idx(i1, i2, i3, (c))]
    if constexpr (D == 2) {
      // FILTER2D_IN_I1 / _I2: the 1-2-1 filter along x1 or x2
#define F_I1(c, I, J) (INV_2 * b((I), (J), 0, c) + INV_4 * (b((I) - 1, (J), 0, c) + b((I) + 1, (J), 0, c)))
#define F_I2(c, I, J) (INV_2 * b((I), (J), 0, c) + INV_4 * (b((I), (J) - 1, 0, c) + b((I), (J) + 1, 0, c)))
      if ((cf.lo[0] && i1 == i1min) || (cf.hi[0] && i1 == i1max - 1)) {
        const int s = cf.lo[0] ? i1 + 1 : i1 - 1;
        a(0) = (THREE * INV_4) * (F_I2(0, i1, i2)) + (INV_4) * (F_I2(0, s, i2));
      } else if ((cf.lo[0] && i1 == i1min + 1) || (cf.hi[0] && i1 == i1max - 2)) {
        const int s = cf.lo[0] ? i1 + 1 : i1 - 1;
        a(0) = INV_2 * (F_I2(0, i1, i2)) + INV_4 * ((F_I2(0, i1 - 1, i2)) + (F_I2(0, i1 + 1, i2)));
        a(1) = (INV_2) * (F_I2(1, i1, i2)) + (INV_4) * (F_I2(1, s, i2));
        a(2) = (INV_2) * (F_I2(2, i1, i2)) + (INV_4) * (F_I2(2, s, i2));
      } else if ((cf.lo[1] && i2 == i2min) || (cf.hi[1] && i2 == i2max - 1)) {
        const int s = cf.lo[1] ? i2 + 1 : i2 - 1;
        a(1) = (THREE * INV_4) * (F_I1(1, i1, i2)) + (INV_4) * (F_I1(1, i1, s));
      } else if ((cf.lo[1] && i2 == i2min + 1) || (cf.hi[1] && i2 == i2max - 2)) {
        const int s = cf.lo[1] ? i2 + 1 : i2 - 1;
        a(0) = INV_2 * (F_I1(0, i1, i2)) + INV_4 * (F_I1(0, i1, s));
        a(1) = INV_2 * (F_I1(1, i1, i2)) + INV_4 * ((F_I1(1, i1, i2 - 1)) + (F_I1(1, i1, i2 + 1)));
        a(2) = INV_2 * (F_I1(2, i1, i2)) + INV_4 * (F_I1(2, i1, s));
      } else {
#pragma unroll
        for (int c = 0; c < 3; ++c)
          a(c) = INV_4 * b(i1, i2, 0, c) +
                 INV_8 * (b(i1 - 1, i2, 0, c) + b(i1 + 1, i2, 0, c) + b(i1, i2 - 1, 0, c) +
                          b(i1, i2 + 1, 0, c)) +
                 INV_16 * (b(i1 - 1, i2 - 1, 0, c) + b(i1 + 1, i2 + 1, 0, c) +
                           b(i1 - 1, i2 + 1, 0, c) + b(i1 + 1, i2 - 1, 0, c));
      }
#undef F_I1
#undef F_I2
    } else {
      // FILTER3D_IN_I2_I3 / _I1_I3 / _I1_I2: the 2D filter in the plane
      // across the wall-normal axis
#define F23(c, I, J, K)                                                                      \
  (INV_4 * b(I, J, K, c) +                                                                   \
   INV_8 * (b((I), (J) - 1, (K), c) + b((I), (J) + 1, (K), c) + b((I), (J), (K) - 1, c) +    \
            b((I), (J), (K) + 1, c)) +                                                       \
   INV_16 * (b((I), (J) - 1, (K) - 1, c) + b((I), (J) + 1, (K) + 1, c) +                     \
             b((I), (J) - 1, (K) + 1, c) + b((I), (J) + 1, (K) - 1, c)))
#define F13(c, I, J, K)                                                                      \
  (INV_4 * b(I, J, K, c) +                                                                   \
   INV_8 * (b((I) - 1, (J), (K), c) + b((I) + 1, (J), (K), c) + b((I), (J), (K) - 1, c) +    \
            b((I), (J), (K) + 1, c)) +                                                       \
   INV_16 * (b((I) - 1, (J), (K) - 1, c) + b((I) + 1, (J), (K) + 1, c) +                     \
             b((I) - 1, (J), (K) + 1, c) + b((I) + 1, (J), (K) - 1, c)))
#define F12(c, I, J, K)                                                                      \
  (INV_4 * b(I, J, K, c) +                                                                   \
   INV_8 * (b((I) - 1, (J), (K), c) + b((I) + 1, (J), (K), c) + b((I), (J) - 1, (K), c) +    \
            b((I), (J) + 1, (K), c)) +                                                       \
   INV_16 * (b((I) - 1, (J) - 1, (K), c) + b((I) + 1, (J) + 1, (K), c) +                     \
             b((I) - 1, (J) + 1, (K), c) + b((I) + 1, (J) - 1, (K), c)))
      if ((cf.lo[0] && i1 == i1min) || (cf.hi[0] && i1 == i1max - 1)) {
        const int s = cf.lo[0] ? i1 + 1 : i1 - 1;
        a(0) = (THREE * INV_4) * (F23(0, i1, i2, i3)) + (INV_4) * (F23(0, s, i2, i3));
      } else if ((cf.lo[0] && i1 == i1min + 1) || (cf.hi[0] && i1 == i1max - 2)) {
        const int s = cf.lo[0] ? i1 + 1 : i1 - 1;
        a(0) = INV_2 * (F23(0, i1, i2, i3)) +
               INV_4 * ((F23(0, i1 - 1, i2, i3)) + (F23(0, i1 + 1, i2, i3)));
        a(1) = INV_2 * (F23(1, i1, i2, i3)) + INV_4 * (F23(1, s, i2, i3));
        a(2) = INV_2 * (F23(2, i1, i2, i3)) + INV_4 * (F23(2, s, i2, i3));
      } else if ((cf.lo[1] && i2 == i2min) || (cf.hi[1] && i2 == i2max - 1)) {
        const int s = cf.lo[1] ? i2 + 1 : i2 - 1;
        a(1) = (THREE * INV_4) * (F13(1, i1, i2, i3)) + (INV_4) * (F13(1, i1, s, i3));
      } else if ((cf.lo[1] && i2 == i2min + 1) || (cf.hi[1] && i2 == i2max - 2)) {
        const int s = cf.lo[1] ? i2 + 1 : i2 - 1;
        a(0) = INV_2 * (F13(0, i1, i2, i3)) + INV_4 * (F13(0, i1, s, i3));
        a(1) = INV_2 * (F13(1, i1, i2, i3)) +
               INV_4 * ((F13(1, i1, i2 - 1, i3)) + (F13(1, i1, i2 + 1, i3)));
        a(2) = INV_2 * (F13(2, i1, i2, i3)) + INV_4 * (F13(2, i1, s, i3));
      } else if ((cf.lo[2] && i3 == i3min) || (cf.hi[2] && i3 == i3max - 1)) {
        const int s = cf.lo[2] ? i3 + 1 : i3 - 1;
        a(2) = (THREE * INV_4) * (F12(2, i1, i2, i3)) + (INV_4) * (F12(2, i1, i2, s));
      } else if ((cf.lo[2] && i3 == i3min + 1) || (cf.hi[2] && i3 == i3max - 2)) {
        const int s = cf.lo[2] ? i3 + 1 : i3 - 1;
        a(0) = INV_2 * (F12(0, i1, i2, i3)) + INV_4 * (F12(0, i1, i2, s));
        a(1) = INV_2 * (F12(1, i1, i2, i3)) + INV_4 * (F12(1, i1, i2, s));
        a(2) = INV_2 * (F12(2, i1, i2, i3)) +
               INV_4 * ((F12(2, i1, i2, i3 - 1)) + (F12(2, i1, i2, i3 + 1)));
      } else {
        // the (i, j, k +- 1) pair appears twice in the 1/32 group, as in
        // digital_filter.hpp:365
#pragma unroll
        for (int c = 0; c < 3; ++c)
          a(c) = INV_8 * b(i1, i2, i3, c) +
                 INV_16 * (b(i1 - 1, i2, i3, c) + b(i1 + 1, i2, i3, c) + b(i1, i2 - 1, i3, c) +
                           b(i1, i2 + 1, i3, c) + b(i1, i2, i3 - 1, c) + b(i1, i2, i3 + 1, c)) +
                 INV_32 * (b(i1 - 1, i2 - 1, i3, c) + b(i1 + 1, i2 + 1, i3, c) +
                           b(i1 - 1, i2 + 1, i3, c) + b(i1 + 1, i2 - 1, i3, c) +
                           b(i1, i2 - 1, i3 - 1, c) + b(i1, i2 + 1, i3 + 1, c) +
                           b(i1, i2, i3 - 1, c) + b(i1, i2, i3 + 1, c) +
                           b(i1 - 1, i2, i3 - 1, c) + b(i1 + 1, i2, i3 + 1, c) +
                           b(i1 - 1, i2, i3 + 1, c) + b(i1 + 1, i2, i3 - 1, c)) +
                 INV_64 * (b(i1 - 1, i2 - 1, i3 - 1, c) + b(i1 + 1, i2 + 1, i3 + 1, c) +
                           b(i1 - 1, i2 + 1, i3 + 1, c) + b(i1 + 1, i2 - 1, i3 - 1, c) +
                           b(i1 - 1, i2 - 1, i3 + 1, c) + b(i1 + 1, i2 + 1, i3 - 1, c) +
                           b(i1 - 1, i2 + 1, i3 - 1, c) + b(i1 + 1, i2 - 1, i3 + 1, c));
      }
#undef F23
#undef F13
#undef F12
    }
#undef a
#undef b
  }
}

template <typename real>
cudaError_t launch_filter_cond(const GridInfo& g, const int lo[3], const int hi[3],
                               FieldView<real> J, FieldView<real> buff, cudaStream_t s) {
  CondFlags cf;
  for (int d = 0; d < 3; ++d) cf.lo[d] = lo[d], cf.hi[d] = hi[d];
  const int64_t cnt = (int64_t)g.n[0] * g.n[1] * (g.dim == 3 ? g.n[2] : 1);
  int64_t       nb  = (cnt + 255) / 256;
  if (nb > pic::sm_count() * 64) nb = pic::sm_count() * 64;
  if (g.dim == 2) PIC_KL(k_filter_cond<2, real><<<(unsigned)nb, 256, 0, s>>>(g, cf, buff, J));
  else            PIC_KL(k_filter_cond<3, real><<<(unsigned)nb, 256, 0, s>>>(g, cf, buff, J));
  return cudaGetLastError();
}
template cudaError_t launch_filter_cond<float>(const GridInfo&, const int*, const int*,
                                               FieldView<float>, FieldView<float>, cudaStream_t);
template cudaError_t launch_filter_cond<double>(const GridInfo&, const int*, const int*,
                                                FieldView<double>, FieldView<double>,
                                                cudaStream_t);

}  // namespace pic

namespace {

unsigned blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > pic::sm_count() * 32) b = pic::sm_count() * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

// MatchFieldsIn's cells along the axis (ExtentToRange, mesh.h:133-202, for
// Minkowski coordinates x = x_min + x_Cd dx): the box [edge - ds, edge] at
// the upper side or [edge, edge + ds] at the lower one, ghosts on the outer
// side included; clamped to the array
template <typename real>
void match_cells(const pic_ctx* c, int axis, int hi, int* lo_out, int* hi_out) {
  const auto& b  = c->fbc;
  const int   ng = c->grid.ng, n = c->grid.n[axis];
  const real  dx = (real)b.dx, x0 = (real)b.x_min[axis], x1 = x0 + (real)n * dx;
  const real  ds = (real)b.match_ds[axis][hi];
  real        lo_x = hi ? x1 - ds : x0, hi_x = hi ? x1 : x0 + ds;
  lo_x = std::min(std::max(x0, lo_x), x1);
  hi_x = std::max(std::min(x1, hi_x), x0);
  real a = std::floor((lo_x - x0) / dx), e = std::ceil((hi_x - x0) / dx);
  int  i0, i1;
  if (hi) {  // incl_ghosts = (false, true)
    a  = std::max(a, (real)0);
    i0 = (int)a + ng;
    i1 = (int)e + 2 * ng;
  } else {  // incl_ghosts = (true, false)
    e  = std::min(e, (real)n);
    i0 = (int)a;
    i1 = (int)e + ng;
  }
  i0 = std::max(i0, 0);
  i1 = std::min(i1, n + 2 * ng);
  *lo_out = i0;
  *hi_out = std::max(i0, i1);
}

template <typename real>
int side_bc(pic_ctx* c, void* EB, int axis, int hi, int set_e, int set_b, cudaStream_t s) {
  const int  kind = c->fbc.kind[axis][hi];
  const auto F    = em_view<real>(c, EB);
  const int  dim = c->grid.dim, ng = c->grid.ng;
  const int  oa = axis == 0 ? 1 : 0, ob = axis == 2 ? 1 : 2;
  const int  ea = c->grid.n[oa] + 2 * ng, eb = dim == 3 ? c->grid.n[ob] + 2 * ng : 1;
  if (kind == PIC_FBC_CONDUCTOR) {
    const int i_edge = hi ? c->grid.n[axis] + ng : ng;
    const int K      = hi ? ng : ng + 1;
    PIC_KL(pic::k_conductor<real><<<blocks((int64_t)K * ea * eb), 256, 0, s>>>(
      F, dim, axis, hi, i_edge, K, ea, eb, set_e, set_b));
  } else if (kind == PIC_FBC_MATCH) {
    int i0, i1;
    match_cells<real>(c, axis, hi, &i0, &i1);
    if (i1 <= i0) return PIC_OK;
    const real x0 = (real)c->fbc.x_min[axis], dx = (real)c->fbc.dx;
    const real x_edge = hi ? x0 + (real)c->grid.n[axis] * dx : x0;
    PIC_KL(pic::k_match_sr<real><<<blocks((int64_t)(i1 - i0) * ea * eb), 256, 0, s>>>(
      F, em_view<real>(c, c->fbc.match_target), dim, axis, i0, i1, ea, eb, ng, x0, dx, x_edge,
      (real)c->fbc.match_ds[axis][hi], set_e, set_b));
  }
  return cuda_status(cudaGetLastError());
}

}  // namespace

extern "C" {

int pic_set_field_bcs(pic_ctx* c, const pic_field_bcs* bcs) {
  if (!c || !bcs) return PIC_ERR_ARG;
  bool match = false;
  for (int d = 0; d < 3; ++d) {
    for (int h = 0; h < 2; ++h) {
      const int k = d < c->grid.dim ? bcs->kind[d][h] : PIC_FBC_PERIODIC;
      if (k < PIC_FBC_PERIODIC || k > PIC_FBC_MATCH) return PIC_ERR_ARG;
      // periodic exactly on the axes the grid was created periodic on
      if (d < c->grid.dim && ((k == PIC_FBC_PERIODIC) != (c->grid.fld_periodic[d] != 0)))
        return PIC_ERR_ARG;
      if (k == PIC_FBC_MATCH) {
        match = true;
        if (!(bcs->match_ds[d][h] > 0.0)) return PIC_ERR_ARG;
      }
    }
  }
  if (match && (!bcs->match_target || !(bcs->dx > 0.0))) return PIC_ERR_ARG;
  c->fbc = *bcs;
  for (int d = c->grid.dim; d < 3; ++d) c->fbc.kind[d][0] = c->fbc.kind[d][1] = PIC_FBC_PERIODIC;
  return PIC_OK;
}

int pic_field_boundaries(pic_ctx* c, void* EB, int32_t set_e, int32_t set_b, void* stream) {
  if (!c || !EB) return PIC_ERR_ARG;
  const cudaStream_t s = strm(stream);
  // Directions<D>::orth: the lower sides in axis order, then the upper ones
  // in reverse axis order
  const int D = c->grid.dim;
  int       order[6][2], m = 0;
  for (int d = 0; d < D; ++d) order[m][0] = d, order[m++][1] = 0;
  for (int d = D - 1; d >= 0; --d) order[m][0] = d, order[m++][1] = 1;
  for (int k = 0; k < m; ++k) {
    const int st = is_f64(c) ? side_bc<double>(c, EB, order[k][0], order[k][1], set_e, set_b, s)
                             : side_bc<float>(c, EB, order[k][0], order[k][1], set_e, set_b, s);
    if (st != PIC_OK) return st;
  }
  return PIC_OK;
}

}  // extern "C"
