// The reference's own derivation of the simulation scales, compiled from its
// sources (src/framework/parameters/*.cpp, src/global/utils/param_container.cpp)
// against the host Kokkos shim (TEST INFRASTRUCTURE ONLY).
//
// ref_scales() parses an input file's text with the reference's vendored
// toml11, runs SimulationParams::setImmutableParams and setMutableParams as
// ntt::Simulation does for a fresh run (src/framework/simulation.cpp:100-104),
// and returns the derived scales the C ABI's step parameters carry.
#include "global.h"

#include "framework/parameters/parameters.h"

#include <toml11/toml.hpp>

#include <cstring>
#include <exception>
#include <string>

extern "C" {

// out[0..9] = dt, dx0, V0, n0, q0, B0, omegaB0, correction, ppc0, sigma0;
// returns 0, or -1 with the exception's text in err (err_len bytes)
int ref_scales(const char* toml_text, double* out, char* err, int err_len) {
  try {
    const auto raw = toml::parse_str(std::string(toml_text));
    ntt::SimulationParams p;
    p.setRawData(raw);
    p.setImmutableParams(raw);
    p.setMutableParams(raw);
    out[0] = (double)p.get<real_t>("algorithms.timestep.dt");
    out[1] = (double)p.get<real_t>("scales.dx0");
    out[2] = (double)p.get<real_t>("scales.V0");
    out[3] = (double)p.get<real_t>("scales.n0");
    out[4] = (double)p.get<real_t>("scales.q0");
    out[5] = (double)p.get<real_t>("scales.B0");
    out[6] = (double)p.get<real_t>("scales.omegaB0");
    out[7] = (double)p.get<real_t>("algorithms.timestep.correction");
    out[8] = (double)p.get<real_t>("particles.ppc0");
    out[9] = (double)p.get<real_t>("scales.sigma0");
    return 0;
  } catch (const std::exception& e) {
    if (err != nullptr && err_len > 0) {
      std::strncpy(err, e.what(), (std::size_t)err_len - 1);
      err[err_len - 1] = '\0';
    }
    return -1;
  }
}

} // extern "C"
