// Host-only ScatterView for the Kokkos API shim (test infrastructure).
// Serial runs add straight into the target view. Under ENTITY_SHIM_OPENMP
// every thread adds into its own zero-initialised duplicate, and
// contribute() adds the duplicates into the target in thread order, so the
// summation order is fixed by the static schedule.
#pragma once

#include "Kokkos_Core.hpp"

namespace Kokkos {
  namespace Experimental {
    struct ScatterSum {};
    struct ScatterDuplicated {};
    struct ScatterNonDuplicated {};
    struct ScatterAtomic {};
    struct ScatterNonAtomic {};

    template <class DataType, class... Props>
    class ScatterView {
    public:
      using view_type  = View<DataType>;
      using value_type = typename view_type::value_type;

      ScatterView() = default;
      explicit ScatterView(const view_type& v) : m_target(v) {
#if defined(ENTITY_SHIM_OPENMP)
        const int nt = omp_get_max_threads();
        if (nt > 1) {
          m_dups = std::make_shared<std::vector<std::vector<value_type>>>(
            nt, std::vector<value_type>(v.size(), value_type(0)));
        }
#endif
        init_strides();
      }

      struct Ref {
        value_type* p;
        void operator+=(value_type x) const { *p += x; }
        void operator-=(value_type x) const { *p -= x; }
        void operator++() const { *p += 1; }
        void update(value_type x) const { *p += x; }
      };
      struct Access {
        const ScatterView* sv;
        value_type*        base;
        template <class... I>
        Ref operator()(I... i) const {
          const std::size_t idx[] = { static_cast<std::size_t>(static_cast<std::ptrdiff_t>(i))..., 0 };
          std::size_t off = 0;
          for (int r = 0; r < view_type::rank; ++r) {
            off += idx[r] * sv->m_cstride[r];
          }
          return Ref { base + off };
        }
      };

      Access access() const {
        if (!m_dups) {
          // serial: index through the target's own strides
          return Access { this, m_target.data() };
        }
#if defined(ENTITY_SHIM_OPENMP)
        return Access { this, (*m_dups)[omp_get_thread_num()].data() };
#else
        return Access { this, nullptr };
#endif
      }

      void contribute_into(const view_type& dst) const {
        if (!m_dups) {
          return;
        }
        constexpr int R = view_type::rank;
        std::size_t   ext[8];
        for (int r = 0; r < R; ++r) {
          ext[r] = dst.extent(r);
        }
        for (auto& d : *m_dups) {
          shim::for_each_index(ext, R, [&](const std::size_t* i) {
            std::size_t od = 0, oc = 0;
            for (int r = 0; r < R; ++r) {
              od += i[r] * dst.stride(r);
              oc += i[r] * m_cstride[r];
            }
            dst.data()[od] += d[oc];
            d[oc] = value_type(0);
          });
        }
      }
      void reset() {
        if (m_dups) {
          for (auto& d : *m_dups) {
            std::fill(d.begin(), d.end(), value_type(0));
          }
        }
      }

      const view_type& target() const { return m_target; }

    private:
      friend struct Access;
      view_type m_target;
      std::shared_ptr<std::vector<std::vector<value_type>>> m_dups;
      // strides of the duplicates (LayoutRight over the target's extents)
      std::size_t m_cstride[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };

    public:
      void init_strides() {
        if (m_dups) {
          std::size_t s = 1;
          for (int q = view_type::rank - 1; q >= 0; --q) {
            m_cstride[q] = s;
            s *= m_target.extent(q);
          }
        } else {
          for (int q = 0; q < view_type::rank; ++q) {
            m_cstride[q] = m_target.stride(q);
          }
        }
      }
    };

    template <class DT, class... P>
    inline ScatterView<DT> create_scatter_view(const View<DT, P...>& v) {
      return ScatterView<DT> { View<DT>(v) };
    }
    template <class Op, class Dup, class Cont, class DT, class... P>
    inline ScatterView<DT> create_scatter_view(const View<DT, P...>& v) {
      return create_scatter_view(v);
    }
    template <class DT, class... P, class... Q>
    inline void contribute(const View<DT, P...>& dst, const ScatterView<DT, Q...>& s) {
      s.contribute_into(View<DT>(dst));
    }
  } // namespace Experimental
} // namespace Kokkos
