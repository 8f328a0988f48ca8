// Launchers of the particle diagnostics (charge density, FP64 moments).
#pragma once

#include <cuda_runtime.h>

#include "pic_common.cuh"

namespace pic {

// rho has the current layout; the density goes to component 0
template <typename real>
cudaError_t launch_charge_density(int dim, int order, const SpeciesPtrs& sp, FieldView<real> rho,
                                  int ng, const PushConsts& pc, unsigned long long* err,
                                  cudaStream_t s);

// adds the PIC_NMOMENTS sums of one species to out (device, FP64)
template <typename real>
cudaError_t launch_particle_moments(const SpeciesPtrs& sp, double* out, cudaStream_t s);

}  // namespace pic
