// Host-side declarations of the field-kernel launchers.
#pragma once

#include <cuda_runtime.h>

#include "pic_common.cuh"

namespace pic {

struct GridInfo {
  int dim;
  int n[3];
  int ng;
  int periodic[3];
};

// extended-stencil coefficients of Faraday_kernel (faraday_mink.hpp:25-69)
template <typename real>
struct Stencil {
  real deltax, deltay, betaxy, betayx, deltaz, betaxz, betazx, betayz, betazy;
};

template <typename real>
cudaError_t launch_faraday(const GridInfo& g, FieldView<real> EB, real c1, real c2,
                           const Stencil<real>& st, bool yee, cudaStream_t s);
template <typename real>
cudaError_t launch_ampere(const GridInfo& g, FieldView<real> EB, FieldView<real> J, real c1,
                          real c2, real jcoeff, real ppc0, bool curl, bool cur, bool fill,
                          cudaStream_t s);
template <typename real>
cudaError_t launch_sync_currents(const GridInfo& g, FieldView<real> J, cudaStream_t s);
template <typename real>
cudaError_t launch_fill_ghosts(const GridInfo& g, FieldView<real> f, int c0, int c1,
                               cudaStream_t s);
template <typename real>
cudaError_t launch_filter(const GridInfo& g, FieldView<real> J, FieldView<real> buff, int npasses,
                          cudaStream_t s);
template <typename real>
cudaError_t launch_zero3(const GridInfo& g, FieldView<real> f, cudaStream_t s);
// every cell (ghosts included) of a 3-component field
template <typename real>
cudaError_t launch_copy3(const GridInfo& g, FieldView<real> src, FieldView<real> dst,
                         cudaStream_t s);
// one filter pass with conductor walls on the flagged sides (field_bcs.cu):
// reads buff (the pass's copy of J), writes J's active cells
template <typename real>
cudaError_t launch_filter_cond(const GridInfo& g, const int lo[3], const int hi[3],
                               FieldView<real> J, FieldView<real> buff, cudaStream_t s);
template <typename real>
cudaError_t launch_energy(const GridInfo& g, FieldView<real> EB, double dx, double* out,
                          cudaStream_t s);


// adjoint (transposed) field operators, Yee stencils (fields.cu)
template <typename real>
cudaError_t launch_adj_seed(const GridInfo& g, FieldView<real> EB, FieldView<real> lam, double dx,
                            cudaStream_t s);
template <typename real>
cudaError_t launch_adj_currents(const GridInfo& g, FieldView<real> lam, FieldView<real> lamJ,
                                real jcoeff, cudaStream_t s);
template <typename real>
cudaError_t launch_adj_ampere(const GridInfo& g, FieldView<real> lam, real a1, real a2,
                              cudaStream_t s);
template <typename real>
cudaError_t launch_adj_faraday(const GridInfo& g, FieldView<real> lam, real c1, real c2,
                               cudaStream_t s);
template <typename real>
cudaError_t launch_adj_fold(const GridInfo& g, FieldView<real> f, int c0, int c1, cudaStream_t s);
template <typename real>
cudaError_t launch_zero_ghosts(const GridInfo& g, FieldView<real> f, int c0, int c1,
                               cudaStream_t s);

}  // namespace pic
