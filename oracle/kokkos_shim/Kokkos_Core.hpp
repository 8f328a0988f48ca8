// Host-only stand-in for the part of the Kokkos API that Entity's hot-path
// kernel headers use (test infrastructure: it lets those headers compile
// unmodified with g++ so the oracle can be checked against them).
//
// What it provides, and how it differs from Kokkos:
// - View<DataType, Props...>: reference-counted (or unmanaged) host arrays of
//   rank 0-4 with dynamic extents first and static extents last, as in
//   `real_t** [6]`. Allocated views use LayoutRight, the Kokkos default on
//   host spaces; wrap_strided() wraps caller memory with any strides.
// - RangePolicy / MDRangePolicy (Rank 2-4, optional work tag) executed by
//   parallel_for in index order; with ENTITY_SHIM_OPENMP the outermost loop
//   is split statically over OpenMP threads.
// - Experimental::ScatterView: serial execution adds straight into the
//   target; under OpenMP each thread adds into its own duplicate and
//   contribute() sums the duplicates in thread order, so results do not
//   depend on scheduling.
// - math functions, pair, atomics, printf/abort/fence, epsilon.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#if defined(ENTITY_SHIM_OPENMP)
  #include <omp.h>
#endif

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [=, *this]

namespace Kokkos {

  // ---------------------------------------------------------------- spaces
  struct HostSpace {
    using execution_space = HostSpace;
    using memory_space    = HostSpace;
  };
  struct Serial {
    using execution_space = Serial;
    using memory_space    = HostSpace;
  };
  struct OpenMP : Serial {};
  using DefaultExecutionSpace     = Serial;
  using DefaultHostExecutionSpace = Serial;

  struct LayoutRight {};
  struct LayoutLeft {};
  struct LayoutStride {};

  enum MemoryTraitsFlags : unsigned {
    Unmanaged    = 0x01,
    RandomAccess = 0x02,
    Atomic       = 0x04,
    Restrict     = 0x08
  };
  template <unsigned F>
  struct MemoryTraits {
    static constexpr unsigned flags = F;
  };

  inline void fence(const std::string& = "") {}
  inline void initialize() {}
  inline void initialize(int&, char**) {}
  struct ScopeGuard {
    ScopeGuard() = default;
    ScopeGuard(int&, char**) {}
  };
  inline void finalize() {}
  inline bool is_initialized() { return true; }

  inline void printf(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vprintf(fmt, ap);
    va_end(ap);
  }
  [[noreturn]] inline void abort(const char* msg) {
    std::fprintf(stderr, "Kokkos shim abort: %s\n", msg);
    std::abort();
  }

  // ------------------------------------------------------------- math
  using std::abs;
  using std::atan;
  using std::atan2;
  using std::ceil;
  using std::cos;
  using std::cosh;
  using std::exp;
  using std::fabs;
  using std::floor;
  using std::fmod;
  using std::isfinite;
  using std::isinf;
  using std::isnan;
  using std::log;
  using std::pow;
  using std::signbit;
  using std::sin;
  using std::sinh;
  using std::sqrt;
  using std::tan;
  using std::tanh;
  using std::acos;
  using std::asin;
  using std::log10;
  using std::round;
  using std::trunc;
  using std::copysign;
  template <class T>
  inline constexpr T min(const T& a, const T& b) {
    return b < a ? b : a;
  }
  template <class T>
  inline constexpr T max(const T& a, const T& b) {
    return a < b ? b : a;
  }

  template <class A, class B>
  using pair = std::pair<A, B>;
  template <class A, class B>
  inline pair<A, B> make_pair(A a, B b) {
    return pair<A, B>(a, b);
  }

  namespace Experimental {
    template <class T>
    struct epsilon {
      static constexpr T value = std::numeric_limits<T>::epsilon();
    };
    template <class T>
    struct infinity {
      static constexpr T value = std::numeric_limits<T>::infinity();
    };
    template <class T>
    struct finite_max {
      static constexpr T value = std::numeric_limits<T>::max();
    };
  } // namespace Experimental

  // ------------------------------------------------------------ atomics
  // Execution is serial or split by thread over disjoint outputs except where
  // the kernels use atomics themselves; the shim makes them real atomics.
  template <class T, class U>
  inline T atomic_fetch_add(T* p, U v) {
    T old;
#pragma omp atomic capture
    {
      old = *p;
      *p += (T)v;
    }
    return old;
  }
  template <class T, class U>
  inline void atomic_add(T* p, U v) {
#pragma omp atomic
    *p += (T)v;
  }
  template <class T, class U>
  inline T atomic_fetch_sub(T* p, U v) {
    return atomic_fetch_add(p, -(T)v);
  }

  // ------------------------------------------------------------ views
  namespace shim {
    // DataType parsing: T, T*, T**, ..., optionally followed by [N] static
    // extents (which Kokkos allows only after the dynamic ones)
    template <class DT>
    struct parse {
      using value_type                  = DT;
      static constexpr int   rank        = 0;
      static constexpr int   rank_dyn    = 0;
      static constexpr int   nstatic     = 0;
      static constexpr std::size_t st[1] = { 0 };
    };
    template <class DT>
    struct parse<DT*> {
      using value_type               = typename parse<DT>::value_type;
      static constexpr int rank      = parse<DT>::rank + 1;
      static constexpr int rank_dyn  = parse<DT>::rank_dyn + 1;
      static constexpr int nstatic   = 0;
      static constexpr std::size_t st[1] = { 0 };
    };
    template <class DT, std::size_t N>
    struct parse<DT[N]> {
      using value_type               = typename parse<DT>::value_type;
      static constexpr int rank      = parse<DT>::rank + 1;
      static constexpr int rank_dyn  = parse<DT>::rank_dyn;
      static constexpr int nstatic   = 1;
      static constexpr std::size_t st[1] = { N };
    };

    template <class... P>
    struct has_unmanaged : std::false_type {};
    template <unsigned F, class... P>
    struct has_unmanaged<MemoryTraits<F>, P...>
      : std::integral_constant<bool, (F & Unmanaged) != 0> {};
    template <class Q, class... P>
    struct has_unmanaged<Q, P...> : has_unmanaged<P...> {};
  } // namespace shim

  template <class DataType, class... Props>
  class View {
    using P = shim::parse<DataType>;

  public:
    using data_type             = DataType;
    using value_type            = typename P::value_type;
    using non_const_value_type  = std::remove_const_t<value_type>;
    using const_value_type      = const non_const_value_type;
    using pointer_type          = value_type*;
    using reference_type        = value_type&;
    using memory_space          = HostSpace;
    using execution_space       = Serial;
    using array_layout          = LayoutRight;
    using size_type             = std::size_t;
    using host_mirror_type      = View<DataType, HostSpace>;
    using HostMirror            = host_mirror_type;
    static constexpr int  rank         = P::rank;
    static constexpr int  rank_dynamic = P::rank_dyn;
    static constexpr unsigned Rank     = P::rank;

    View() = default;

    // allocating constructor: label, then the dynamic extents
    template <class... N,
              std::enable_if_t<(std::is_integral_v<N> && ...), int> = 0>
    explicit View(const std::string& label, N... n) : m_label(label) {
      set_extents({ static_cast<std::size_t>(n)... });
      m_owner = std::shared_ptr<non_const_value_type[]>(
        new non_const_value_type[std::max<std::size_t>(size(), 1)]());
      m_ptr = m_owner.get();
    }
    // unmanaged wrap of caller memory, LayoutRight
    template <class... N,
              std::enable_if_t<(std::is_integral_v<N> && ...), int> = 0>
    explicit View(value_type* ptr, N... n) : m_label("unmanaged") {
      set_extents({ static_cast<std::size_t>(n)... });
      m_ptr = ptr;
    }
    // converting constructor (non-const -> const, other traits)
    template <class DT2, class... P2,
              std::enable_if_t<std::is_convertible_v<typename View<DT2, P2...>::value_type*,
                                                      value_type*> &&
                                 View<DT2, P2...>::rank == rank,
                               int> = 0>
    View(const View<DT2, P2...>& o)
      : m_label(o.label())
      , m_owner(o.impl_owner())
      , m_ptr(o.data()) {
      for (int r = 0; r < 8; ++r) {
        m_ext[r]    = o.extent(r);
        m_stride[r] = o.stride(r);
      }
    }

    // shim-only: wrap caller memory with explicit extents and strides
    // (elements), e.g. a Kokkos LayoutLeft array or a field with padding
    static View wrap_strided(value_type* ptr, const std::size_t* ext, const std::size_t* stride) {
      View v;
      v.m_label = "strided";
      for (int r = 0; r < rank; ++r) {
        v.m_ext[r]    = ext[r];
        v.m_stride[r] = stride[r];
      }
      v.m_ptr = ptr;
      return v;
    }

    template <class... I>
    value_type& operator()(I... i) const {
      static_assert(sizeof...(I) == rank || rank == 0, "View index count");
      const std::size_t idx[] = { static_cast<std::size_t>(static_cast<std::ptrdiff_t>(i))..., 0 };
      std::size_t off = 0;
      for (int r = 0; r < rank; ++r) {
        off += idx[r] * m_stride[r];
      }
      return m_ptr[off];
    }
    template <class I>
    value_type& operator[](I i) const {
      return m_ptr[static_cast<std::size_t>(i) * m_stride[0]];
    }

    std::size_t extent(int r) const { return r < rank ? m_ext[r] : 1; }
    int         extent_int(int r) const { return static_cast<int>(extent(r)); }
    std::size_t stride(int r) const { return r < rank ? m_stride[r] : 0; }
    std::size_t size() const {
      std::size_t s = 1;
      for (int r = 0; r < rank; ++r) {
        s *= m_ext[r];
      }
      return s;
    }
    std::size_t span() const { return size(); }
    value_type* data() const { return m_ptr; }
    bool        is_allocated() const { return m_ptr != nullptr; }
    std::string label() const { return m_label; }
    const std::shared_ptr<non_const_value_type[]>& impl_owner() const { return m_owner; }
    bool span_is_contiguous() const { return true; }

  private:
    void set_extents(std::initializer_list<std::size_t> dyn) {
      int r = 0;
      for (auto n : dyn) {
        if (r < rank) {
          m_ext[r++] = n;
        }
      }
      if constexpr (P::nstatic > 0) {
        m_ext[rank - 1] = P::st[0];
        r               = rank;
      }
      for (; r < rank; ++r) {
        m_ext[r] = 1;
      }
      std::size_t s = 1;
      for (int q = rank - 1; q >= 0; --q) {
        m_stride[q] = s;
        s *= m_ext[q];
      }
    }

    std::string                              m_label;
    std::shared_ptr<non_const_value_type[]>  m_owner;
    value_type*                              m_ptr { nullptr };
    std::size_t                              m_ext[8] { 0, 0, 0, 0, 0, 0, 0, 0 };
    std::size_t                              m_stride[8] { 0, 0, 0, 0, 0, 0, 0, 0 };
  };

  template <class DT, class... P>
  inline View<DT, P...> create_mirror_view(const View<DT, P...>& v) {
    return v;
  }
  template <class Space, class DT, class... P>
  inline View<DT, P...> create_mirror_view(const Space&, const View<DT, P...>& v) {
    return v;
  }
  template <class DT, class... P>
  inline View<DT, P...> create_mirror(const View<DT, P...>& v) {
    View<DT, P...> m(v.label());
    return m;
  }

  namespace shim {
    template <class F>
    inline void for_each_index(const std::size_t* ext, int rank, F&& f) {
      std::size_t idx[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
      std::size_t total  = 1;
      for (int r = 0; r < rank; ++r) {
        total *= ext[r];
      }
      for (std::size_t n = 0; n < total; ++n) {
        std::size_t rem = n;
        for (int r = rank - 1; r >= 0; --r) {
          idx[r] = rem % ext[r];
          rem /= ext[r];
        }
        f(idx);
      }
    }
  } // namespace shim

  template <class DT, class... P, class DT2, class... P2>
  inline void deep_copy(const View<DT, P...>& dst, const View<DT2, P2...>& src) {
    static_assert(View<DT, P...>::rank == View<DT2, P2...>::rank, "deep_copy rank");
    constexpr int R = View<DT, P...>::rank;
    std::size_t   ext[8];
    for (int r = 0; r < R; ++r) {
      if (dst.extent(r) != src.extent(r)) {
        throw std::runtime_error("deep_copy: extents differ");
      }
      ext[r] = dst.extent(r);
    }
    shim::for_each_index(ext, R, [&](const std::size_t* i) {
      std::size_t od = 0, os = 0;
      for (int r = 0; r < R; ++r) {
        od += i[r] * dst.stride(r);
        os += i[r] * src.stride(r);
      }
      dst.data()[od] = src.data()[os];
    });
  }
  template <class DT, class... P, class T,
            std::enable_if_t<std::is_arithmetic_v<T>, int> = 0>
  inline void deep_copy(const View<DT, P...>& dst, const T& value) {
    constexpr int R = View<DT, P...>::rank;
    std::size_t   ext[8];
    for (int r = 0; r < R; ++r) {
      ext[r] = dst.extent(r);
    }
    shim::for_each_index(ext, R, [&](const std::size_t* i) {
      std::size_t od = 0;
      for (int r = 0; r < R; ++r) {
        od += i[r] * dst.stride(r);
      }
      dst.data()[od] = value;
    });
  }
  template <class Space, class A, class B>
  inline void deep_copy(const Space&, const A& dst, const B& src) {
    deep_copy(dst, src);
  }

  // subview(v, a0, a1, ...): each argument is an index (the axis is
  // dropped), a pair (the range [first, second)) or ALL; the result views the
  // same memory with the parent's strides (the parent must outlive it)
  struct ALL_t {};
  inline constexpr ALL_t ALL {};

  namespace shim {
    template <class T, int R>
    struct ptrs {
      using type = typename ptrs<T, R - 1>::type*;
    };
    template <class T>
    struct ptrs<T, 0> {
      using type = T;
    };
    template <class A>
    constexpr bool keeps_axis() {
      return !std::is_integral_v<std::decay_t<A>>;
    }
    template <class A>
    std::pair<std::size_t, std::size_t> sub_range(const A& a, std::size_t n) {
      if constexpr (std::is_same_v<std::decay_t<A>, ALL_t>) {
        return { 0, n };
      } else if constexpr (std::is_integral_v<std::decay_t<A>>) {
        return { static_cast<std::size_t>(a), 1 };
      } else {
        return { static_cast<std::size_t>(a.first),
                 static_cast<std::size_t>(a.second) - static_cast<std::size_t>(a.first) };
      }
    }
  } // namespace shim

  template <class DT, class... P, class... Args>
  auto subview(const View<DT, P...>& v, const Args&... args) {
    using V = View<DT, P...>;
    static_assert(sizeof...(Args) == V::rank, "subview: one argument per axis");
    constexpr int R = (0 + ... + int(shim::keeps_axis<Args>()));
    using Out       = View<typename shim::ptrs<typename V::value_type, R>::type, HostSpace>;
    std::size_t off = 0, ext[8] = {}, str[8] = {};
    int         r = 0, d = 0;
    (
      [&] {
        const auto rg = shim::sub_range(args, v.extent(d));
        off += rg.first * v.stride(d);
        if (shim::keeps_axis<Args>()) {
          ext[r] = rg.second;
          str[r] = v.stride(d);
          ++r;
        }
        ++d;
      }(),
      ...);
    return Out::wrap_strided(v.data() + off, ext, str);
  }

  // ------------------------------------------------------------ policies
  template <unsigned N>
  struct Rank {
    static constexpr unsigned rank = N;
  };

  namespace shim {
    template <class... T>
    struct policy_traits {
      using tag   = void;
      using space = Serial;
    };
    template <class T, class... R>
    struct policy_traits<T, R...> {
      using tail  = policy_traits<R...>;
      using tag   = std::conditional_t<std::is_same_v<T, Serial> || std::is_same_v<T, OpenMP> ||
                                         std::is_same_v<T, HostSpace>,
                                       typename tail::tag, T>;
      using space = Serial;
    };
    template <unsigned N, class... R>
    struct policy_traits<Rank<N>, R...> : policy_traits<R...> {};
  } // namespace shim

  template <class... Args>
  struct RangePolicy {
    using work_tag = typename shim::policy_traits<Args...>::tag;
    std::int64_t begin_ { 0 }, end_ { 0 };
    RangePolicy() = default;
    template <class B, class E>
    RangePolicy(B b, E e) : begin_(static_cast<std::int64_t>(b))
                          , end_(static_cast<std::int64_t>(e)) {}
    template <class S, class B, class E,
              std::enable_if_t<!std::is_integral_v<S>, int> = 0>
    RangePolicy(const S&, B b, E e) : RangePolicy(b, e) {}
    std::int64_t begin() const { return begin_; }
    std::int64_t end() const { return end_; }
  };

  template <class R, class... Args>
  struct MDRangePolicy {
    static constexpr unsigned N = R::rank;
    using work_tag = typename shim::policy_traits<Args...>::tag;
    std::array<std::int64_t, N> lo {}, hi {};
    MDRangePolicy() = default;
    template <class A, class B>
    MDRangePolicy(const A& l, const B& h) {
      std::size_t r = 0;
      for (auto v : l) {
        lo[r++] = static_cast<std::int64_t>(v);
      }
      r = 0;
      for (auto v : h) {
        hi[r++] = static_cast<std::int64_t>(v);
      }
    }
    template <class A, class B>
    MDRangePolicy(std::initializer_list<A> l, std::initializer_list<B> h) {
      std::size_t r = 0;
      for (auto v : l) {
        lo[r++] = static_cast<std::int64_t>(v);
      }
      r = 0;
      for (auto v : h) {
        hi[r++] = static_cast<std::int64_t>(v);
      }
    }
  };

  namespace shim {
    template <class Tag, class F, class... I>
    inline void invoke(const F& f, I&&... i) {
      if constexpr (std::is_void_v<Tag>) {
        f(std::forward<I>(i)...);
      } else {
        f(Tag {}, std::forward<I>(i)...);
      }
    }
    template <class T>
    struct is_md : std::false_type {};
    template <class R, class... A>
    struct is_md<MDRangePolicy<R, A...>> : std::true_type {};
  } // namespace shim

  namespace shim {
    // calls v(i...) for every index of a policy (an integer count, a
    // RangePolicy or an MDRangePolicy) in LayoutRight order, the last index
    // fastest; with ENTITY_SHIM_OPENMP and `par` the outermost loop is split
    // statically over the threads
    // true: every parallel_for runs serially in index order, so that kernels
    // that hand out slots with atomics (stream compaction) give the order a
    // serial host gives (set around calls whose output order is compared)
    inline bool g_serial = false;

    template <bool par, class Policy, class V>
    inline void iterate(const Policy& pol, const V& v) {
      if constexpr (std::is_integral_v<Policy>) {
        const std::int64_t n = static_cast<std::int64_t>(pol);
#if defined(ENTITY_SHIM_OPENMP)
#pragma omp parallel for schedule(static) if (par && !g_serial)
#endif
        for (std::int64_t i = 0; i < n; ++i) {
          v(i);
        }
      } else if constexpr (is_md<Policy>::value) {
        constexpr unsigned N  = Policy::N;
        const auto&        lo = pol.lo;
        const auto&        hi = pol.hi;
#if defined(ENTITY_SHIM_OPENMP)
#pragma omp parallel for schedule(static) if (par && !g_serial)
#endif
        for (std::int64_t i0 = lo[0]; i0 < hi[0]; ++i0) {
          if constexpr (N == 1) {
            v(i0);
          } else {
            for (std::int64_t i1 = lo[1]; i1 < hi[1]; ++i1) {
              if constexpr (N == 2) {
                v(i0, i1);
              } else {
                for (std::int64_t i2 = lo[2]; i2 < hi[2]; ++i2) {
                  if constexpr (N == 3) {
                    v(i0, i1, i2);
                  } else {
                    for (std::int64_t i3 = lo[3]; i3 < hi[3]; ++i3) {
                      v(i0, i1, i2, i3);
                    }
                  }
                }
              }
            }
          }
        }
      } else {
#if defined(ENTITY_SHIM_OPENMP)
#pragma omp parallel for schedule(static) if (par && !g_serial)
#endif
        for (std::int64_t i = pol.begin(); i < pol.end(); ++i) {
          v(i);
        }
      }
    }
    template <class Policy>
    struct tag_of {
      using type = void;
    };
    template <class... A>
    struct tag_of<RangePolicy<A...>> {
      using type = typename RangePolicy<A...>::work_tag;
    };
    template <class R, class... A>
    struct tag_of<MDRangePolicy<R, A...>> {
      using type = typename MDRangePolicy<R, A...>::work_tag;
    };
  } // namespace shim

  template <class Policy, class F>
  inline void parallel_for(const Policy& pol, const F& f) {
    using Tag = typename shim::tag_of<Policy>::type;
    shim::iterate<true>(pol, [&](auto... i) { shim::invoke<Tag>(f, i...); });
  }
  template <class Policy, class F>
  inline void parallel_for(const std::string&, const Policy& pol, const F& f) {
    parallel_for(pol, f);
  }

  // reducers: a plain variable sums; Sum/Min/Max/LAnd/LOr wrap a variable
  template <class T>
  struct Sum {
    T& ref;
    explicit Sum(T& r) : ref(r) {}
    static T    init() { return T(0); }
    static void join(T& a, const T& b) { a += b; }
  };
  template <class T>
  struct Min {
    T& ref;
    explicit Min(T& r) : ref(r) {}
    static T    init() { return std::numeric_limits<T>::max(); }
    static void join(T& a, const T& b) { a = b < a ? b : a; }
  };
  template <class T>
  struct Max {
    T& ref;
    explicit Max(T& r) : ref(r) {}
    static T    init() { return std::numeric_limits<T>::lowest(); }
    static void join(T& a, const T& b) { a = a < b ? b : a; }
  };
  template <class T>
  struct LAnd {
    T& ref;
    explicit LAnd(T& r) : ref(r) {}
    static T    init() { return T(1); }
    static void join(T& a, const T& b) { a = a && b; }
  };
  template <class T>
  struct LOr {
    T& ref;
    explicit LOr(T& r) : ref(r) {}
    static T    init() { return T(0); }
    static void join(T& a, const T& b) { a = a || b; }
  };
  namespace shim {
    template <class T>
    struct is_reducer : std::false_type {};
    template <class T>
    struct is_reducer<Sum<T>> : std::true_type {};
    template <class T>
    struct is_reducer<Min<T>> : std::true_type {};
    template <class T>
    struct is_reducer<Max<T>> : std::true_type {};
    template <class T>
    struct is_reducer<LAnd<T>> : std::true_type {};
    template <class T>
    struct is_reducer<LOr<T>> : std::true_type {};
  } // namespace shim

  // serial in index order, so the result is deterministic
  template <class Policy, class F, class R>
  inline void parallel_reduce(const Policy& pol, const F& f, R&& result) {
    using Tag = typename shim::tag_of<Policy>::type;
    using RR  = std::remove_cv_t<std::remove_reference_t<R>>;
    if constexpr (shim::is_reducer<RR>::value) {
      auto acc = RR::init();
      shim::iterate<false>(pol, [&](auto... i) {
        auto part = RR::init();
        shim::invoke<Tag>(f, i..., part);
        RR::join(acc, part);
      });
      result.ref = acc;
    } else {
      RR acc {};
      shim::iterate<false>(pol, [&](auto... i) { shim::invoke<Tag>(f, i..., acc); });
      result = acc;
    }
  }
  template <class Policy, class F, class R>
  inline void parallel_reduce(const std::string&, const Policy& pol, const F& f, R&& result) {
    parallel_reduce(pol, f, std::forward<R>(result));
  }
  // several plain scalars reduced by sum in one pass (serial, in index order)
  template <class Policy, class F, class R1, class R2, class... Rs>
  inline void parallel_reduce(const std::string&, const Policy& pol, const F& f, R1& r1, R2& r2,
                              Rs&... rs) {
    using Tag = typename shim::tag_of<Policy>::type;
    std::tuple<R1, R2, Rs...> acc {};
    shim::iterate<false>(pol, [&](auto... i) {
      std::apply([&](auto&... a) { shim::invoke<Tag>(f, i..., a...); }, acc);
    });
    std::tie(r1, r2, rs...) = acc;
  }

  // ------------------------------------------------------------ random
  // Only the types appear on the hot path (initial conditions come from the
  // oracle's own generator); the generator is a plain xorshift64*.
  template <class Space>
  class Random_XorShift64_Pool;
  template <class Space>
  class Random_XorShift64 {
  public:
    explicit Random_XorShift64(std::uint64_t s = 1) : m_s(s ? s : 1) {}
    std::uint64_t urand64() {
      m_s ^= m_s >> 12;
      m_s ^= m_s << 25;
      m_s ^= m_s >> 27;
      return m_s * 2685821657736338717ull;
    }
    std::uint32_t urand() { return static_cast<std::uint32_t>(urand64() >> 32); }
    // uniform in [0, range) and [lo, hi)
    std::uint32_t urand(std::uint32_t range) { return range ? urand() % range : 0u; }
    std::uint32_t urand(std::uint32_t lo, std::uint32_t hi) { return lo + urand(hi - lo); }
    float  frand() { return static_cast<float>(urand64() >> 40) * (1.0f / 16777216.0f); }
    double drand() { return static_cast<double>(urand64() >> 11) * (1.0 / 9007199254740992.0); }
    float  frand(float r) { return frand() * r; }
    double drand(double r) { return drand() * r; }
    float  normal() {
      const double u = drand() + 1e-300, v = drand();
      return static_cast<float>(std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v));
    }

  private:
    std::uint64_t m_s;
  };
  template <class Space>
  class Random_XorShift64_Pool {
  public:
    using generator_type = Random_XorShift64<Space>;
    Random_XorShift64_Pool() = default;
    explicit Random_XorShift64_Pool(std::uint64_t seed) : m_seed(seed) {}
    generator_type get_state() const { return generator_type(m_seed); }
    void           free_state(const generator_type&) const {}

  private:
    std::uint64_t m_seed { 1 };
  };

} // namespace Kokkos
