// Kokkos API shim (test infrastructure): bin sorting. BinOp1D maps a key to
// one of max_bins equal bins of [min, max) (one bin per integer when the
// integer range fits the bins); BinSort builds a permutation that orders the
// elements by bin and, within a bin, by their original index (a stable
// counting sort, the order a serial host run gives), and applies it to any
// rank-1 view of the same length. Sorting within bins is not provided (the
// reference asks for none).
#pragma once
#include <type_traits>
#include <vector>

#include "Kokkos_Core.hpp"

namespace Kokkos {
  template <class KeyView>
  struct BinOp1D {
    int    m_bins = 0;
    double m_mul = 0.0, m_min = 0.0;
    template <class A, class B>
    BinOp1D(int max_bins, A min, B max)
      : m_bins(max_bins + 1)
      , m_mul(static_cast<double>(max_bins) / (static_cast<double>(max) - static_cast<double>(min)))
      , m_min(static_cast<double>(min)) {
      using K = std::remove_cv_t<typename KeyView::value_type>;
      if (std::is_integral_v<K> &&
          static_cast<double>(max) - static_cast<double>(min) <= static_cast<double>(max_bins)) {
        m_mul = 1.0;
      }
    }
    template <class V>
    int bin(const V& keys, std::size_t i) const {
      return static_cast<int>(m_mul * (static_cast<double>(keys(i)) - m_min));
    }
    int max_bins() const { return m_bins; }
  };

  template <class KeyView, class BinOp>
  class BinSort {
  public:
    BinSort(const KeyView& keys, const BinOp& op, bool /*sort_within_bins*/ = false)
      : m_keys(keys), m_op(op) {}
    template <class Space>
    BinSort(const Space&, const KeyView& keys, const BinOp& op, bool sw = false)
      : BinSort(keys, op, sw) {}

    void create_permute_vector() {
      const std::size_t n = m_keys.extent(0);
      std::vector<std::size_t> count(static_cast<std::size_t>(m_op.max_bins()) + 1, 0);
      std::vector<int>         bin(n);
      for (std::size_t i = 0; i < n; ++i) {
        bin[i] = m_op.bin(m_keys, i);
        ++count[static_cast<std::size_t>(bin[i]) + 1];
      }
      for (std::size_t b = 1; b < count.size(); ++b) count[b] += count[b - 1];
      m_perm.assign(n, 0);
      for (std::size_t i = 0; i < n; ++i) m_perm[count[static_cast<std::size_t>(bin[i])]++] = i;
    }
    template <class Space>
    void create_permute_vector(const Space&) {
      create_permute_vector();
    }

    // values(i) <- values(perm(i))
    template <class V>
    void sort(const V& values) const {
      using T = std::remove_cv_t<typename V::value_type>;
      std::vector<T> tmp(m_perm.size());
      for (std::size_t i = 0; i < m_perm.size(); ++i) tmp[i] = values(m_perm[i]);
      for (std::size_t i = 0; i < m_perm.size(); ++i) values(i) = tmp[i];
    }
    template <class Space, class V>
    void sort(const Space&, const V& values) const {
      sort(values);
    }

    const std::vector<std::size_t>& permutation() const { return m_perm; }

  private:
    KeyView                  m_keys;
    BinOp                    m_op;
    std::vector<std::size_t> m_perm;
  };
} // namespace Kokkos
