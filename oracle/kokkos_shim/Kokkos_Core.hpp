// Host-only, serial stand-in for the subset of the Kokkos 4.3 API that the
// omega_playground sources use (Views, Range/MDRange policies, parallel_for,
// parallel_reduce with sum and Max, deep_copy, fence).  It exists only so the
// reference's own C++ sources can be compiled unmodified as a CPU pin for the
// oracle; it carries no numerics of its own.  Loops run serially in
// row-major (Iterate::Right) order, so racy writes in the reference (odd-ny
// mesh construction) resolve to the serial last-writer result.
#pragma once
#include <array>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [ =, *this ]
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION

namespace Kokkos {

struct LayoutRight {};
struct HostSpace {};
struct DefaultExecutionSpace {
  using memory_space = HostSpace;
};
template <class A, class B> struct SpaceAccessibility {
  static constexpr bool accessible = true;
};

inline void initialize() {}
inline void initialize(int &, char **) {}
inline void finalize() {}
inline void fence() {}

namespace shim {
template <class T> struct rank_of {
  static constexpr int value = 0;
  using value_type = T;
};
template <class T> struct rank_of<T *> {
  static constexpr int value = rank_of<T>::value + 1;
  using value_type = typename rank_of<T>::value_type;
};
template <class T> struct add_const_data {
  using type = const T;
};
template <class T> struct add_const_data<T *> {
  using type = typename add_const_data<T>::type *;
};
} // namespace shim

template <class DataType, class... Props> class View {
public:
  static constexpr int rank = shim::rank_of<DataType>::value;
  using value_type = typename shim::rank_of<DataType>::value_type;
  using non_const_value_type = std::remove_const_t<value_type>;
  using const_data_type = typename shim::add_const_data<
      std::remove_const_t<typename std::remove_pointer_t<DataType>>>::type *;
  using reference_type = value_type &;

  View() = default;
  explicit View(const std::string &label, size_t n0 = 0, size_t n1 = 0,
                size_t n2 = 0, size_t n3 = 0)
      : m_label(label) {
    size_t n[4] = {n0, n1, n2, n3};
    size_t total = 1;
    for (int r = 0; r < 4; ++r) {
      m_ext[r] = r < rank ? n[r] : 1;
      if (r < rank)
        total *= n[r];
    }
    m_store = std::make_shared<std::vector<non_const_value_type>>(total);
    m_ptr = m_store->data();
    m_size = total;
  }
  template <class D2, class... P2>
  View(const View<D2, P2...> &o)
      : m_store(o.m_store), m_ptr(o.m_ptr), m_size(o.m_size),
        m_label(o.m_label) {
    static_assert(View<D2, P2...>::rank == rank, "rank mismatch");
    for (int r = 0; r < 4; ++r)
      m_ext[r] = o.m_ext[r];
  }

  size_t extent(int r) const { return m_ext[r]; }
  int extent_int(int r) const { return int(m_ext[r]); }
  size_t size() const { return m_size; }
  value_type *data() const { return m_ptr; }
  const std::string &label() const { return m_label; }

  template <class I0> reference_type operator()(I0 i0) const {
    return m_ptr[size_t(i0)];
  }
  template <class I0, class I1>
  reference_type operator()(I0 i0, I1 i1) const {
    return m_ptr[size_t(i0) * m_ext[1] + size_t(i1)];
  }
  template <class I0, class I1, class I2>
  reference_type operator()(I0 i0, I1 i1, I2 i2) const {
    return m_ptr[(size_t(i0) * m_ext[1] + size_t(i1)) * m_ext[2] + size_t(i2)];
  }
  template <class I0, class I1, class I2, class I3>
  reference_type operator()(I0 i0, I1 i1, I2 i2, I3 i3) const {
    return m_ptr[((size_t(i0) * m_ext[1] + size_t(i1)) * m_ext[2] +
                  size_t(i2)) *
                     m_ext[3] +
                 size_t(i3)];
  }

  std::shared_ptr<std::vector<non_const_value_type>> m_store;
  value_type *m_ptr = nullptr;
  size_t m_size = 0;
  size_t m_ext[4] = {0, 1, 1, 1};
  std::string m_label;
};

template <class D, class... P, class S>
std::enable_if_t<std::is_arithmetic<S>::value>
deep_copy(const View<D, P...> &dst, const S &v) {
  for (size_t i = 0; i < dst.size(); ++i)
    dst.data()[i] = v;
}
template <class D, class... P, class D2, class... P2>
void deep_copy(const View<D, P...> &dst, const View<D2, P2...> &src) {
  for (size_t i = 0; i < dst.size(); ++i)
    dst.data()[i] = src.data()[i];
}

template <class... Args> struct RangePolicy {
  long m_begin, m_end;
  RangePolicy(long b, long e) : m_begin(b), m_end(e) {}
};

namespace Iterate {
struct Right {};
struct Left {};
} // namespace Iterate
template <int N, class Outer = Iterate::Right, class Inner = Iterate::Right>
struct Rank {
  static constexpr int value = N;
};

template <class Exec, class R> struct MDRangePolicy {
  static constexpr int N = R::value;
  long m_lo[N], m_hi[N];
  template <class LT, class UT>
  MDRangePolicy(const LT (&lo)[N], const UT (&hi)[N]) {
    for (int r = 0; r < N; ++r) {
      m_lo[r] = lo[r];
      m_hi[r] = hi[r];
    }
  }
  template <class LT, class UT, class TT>
  MDRangePolicy(const LT (&lo)[N], const UT (&hi)[N], const TT (&)[N])
      : MDRangePolicy(lo, hi) {}
};

template <class... Args> struct TeamPolicy {
  struct member_type {};
  TeamPolicy(long, long, long) {}
};
template <class M> inline int TeamThreadRange(const M &, int n) { return n; }
template <class M> inline int ThreadVectorRange(const M &, int n) { return n; }

template <class T> struct Max {
  using value_type = T;
  T &m_ref;
  explicit Max(T &r) : m_ref(r) {}
};

namespace shim {
template <class F, class... I> inline void call(const F &f, I... i) { f(i...); }
} // namespace shim

template <class... A, class F>
void parallel_for(const std::string &, const RangePolicy<A...> &p, const F &f) {
  for (long i = p.m_begin; i < p.m_end; ++i)
    f(int(i));
}
template <class Exec, class R, class F>
void parallel_for(const std::string &, const MDRangePolicy<Exec, R> &p,
                  const F &f) {
  constexpr int N = R::value;
  if constexpr (N == 2) {
    for (long i = p.m_lo[0]; i < p.m_hi[0]; ++i)
      for (long j = p.m_lo[1]; j < p.m_hi[1]; ++j)
        f(int(i), int(j));
  } else if constexpr (N == 3) {
    for (long i = p.m_lo[0]; i < p.m_hi[0]; ++i)
      for (long j = p.m_lo[1]; j < p.m_hi[1]; ++j)
        for (long k = p.m_lo[2]; k < p.m_hi[2]; ++k)
          f(int(i), int(j), int(k));
  } else {
    static_assert(N == 2 || N == 3, "rank");
  }
}
template <class P, class F> void parallel_for(const P &p, const F &f) {
  parallel_for(std::string(), p, f);
}

namespace shim {
template <class T> struct reduce_ops {
  static T init() { return T(0); }
  static void join(T &a, const T &b) { a += b; }
  static T &target(T &r) { return r; }
};
template <class T> struct reduce_ops<Max<T>> {
  static T init() { return std::numeric_limits<T>::lowest(); }
  static void join(T &a, const T &b) { a = b > a ? b : a; }
};
} // namespace shim

template <class... A, class F, class T>
void parallel_reduce(const std::string &, const RangePolicy<A...> &p,
                     const F &f, T &result) {
  T acc = T(0);
  for (long i = p.m_begin; i < p.m_end; ++i)
    f(int(i), acc);
  result = acc;
}
template <class... A, class F, class T>
void parallel_reduce(const std::string &, const RangePolicy<A...> &p,
                     const F &f, Max<T> red) {
  T acc = std::numeric_limits<T>::lowest();
  for (long i = p.m_begin; i < p.m_end; ++i)
    f(int(i), acc);
  red.m_ref = acc;
}
template <class Exec, class R, class F, class T>
void parallel_reduce(const std::string &, const MDRangePolicy<Exec, R> &p,
                     const F &f, T &result) {
  static_assert(R::value == 2, "rank");
  T acc = T(0);
  for (long i = p.m_lo[0]; i < p.m_hi[0]; ++i)
    for (long j = p.m_lo[1]; j < p.m_hi[1]; ++j)
      f(int(i), int(j), acc);
  result = acc;
}
template <class P, class F, class T>
void parallel_reduce(const P &p, const F &f, T &&result) {
  parallel_reduce(std::string(), p, f, std::forward<T>(result));
}

} // namespace Kokkos
