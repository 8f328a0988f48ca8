// Kokkos API shim (test infrastructure): Kokkos_Sort.hpp is covered by Kokkos_Core.hpp.
#pragma once
#include "Kokkos_Core.hpp"
