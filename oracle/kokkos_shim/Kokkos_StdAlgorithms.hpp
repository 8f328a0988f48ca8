// Kokkos API shim (test infrastructure): the std-algorithm entry points the
// reference's particle containers use.
#pragma once
#include "Kokkos_Core.hpp"

namespace Kokkos {
  namespace Experimental {
    // fill(label, space, view, value): every element of a rank-1 view
    template <class Space, class V, class T>
    inline void fill(const std::string&, const Space&, const V& view, const T& value) {
      for (std::size_t i = 0; i < view.extent(0); ++i) view(i) = value;
    }
    template <class Space, class V, class T>
    inline void fill(const Space&, const V& view, const T& value) {
      for (std::size_t i = 0; i < view.extent(0); ++i) view(i) = value;
    }
  } // namespace Experimental
} // namespace Kokkos
