// Minimal single-threaded stand-in for the parts of Kokkos 5.1 that the
// reference's per-particle headers name, so those headers compile unmodified
// with a plain C++20 compiler for the oracle's pin tests.  It is not Kokkos:
// views are host arrays with Kokkos' index layouts (resize keeps elements by
// index), parallel dispatch is a serial loop in index order (league ranks in
// order, one thread per team; tagged policies call the functor with the tag,
// as Kokkos does; reductions start from the value type's zero or the
// reducer's init; a scan is one pass with final = true, as the Serial
// backend runs it), a scatter view writes straight into its view with
// Kokkos' ScatterValue rounding (the right-hand side converted to the
// element type, then added), and the random pool hands out values from a
// caller-filled tape or from a caller's draw provider, which sees the tag,
// league rank and loop index of the code that asks (so a test injects
// exactly the draws it wants).  Math functions forward to the C library with
// Kokkos' overload set (float in, float out), which is what the reference's
// OpenMP (host) build calls.
#ifndef BMC_REFPIN_KOKKOS_SHIM_HPP
#define BMC_REFPIN_KOKKOS_SHIM_HPP

#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [=, *this]

namespace refpin {
// Count of KOKKOS_ASSERT failures seen (the reference's release build
// compiles the asserts out; the pin driver reports them instead of aborting).
inline long& assert_failures() {
  static long n = 0;
  return n;
}
// Where the serial dispatch is: the work tag of the running policy (an
// address unique to the tag type, nullptr untagged), the league rank of the
// running team and the index of the innermost running range loop.
struct Ctx {
  const void* tag = nullptr;
  std::size_t league = 0;
  std::size_t index = 0;
};
inline Ctx& ctx() {
  static Ctx c;
  return c;
}
template <class T>
const void* tag_id() {
  static const char c = 0;
  return &c;
}
// Draw provider: when set, every draw of the random pool asks it (kind 0:
// uniform float, 1: uniform double, 2: standard normal, 3: integer) instead
// of reading the tape.
using DrawFn = double (*)(void* user, int kind);
struct Provider {
  DrawFn fn = nullptr;
  void* user = nullptr;
};
inline Provider& provider() {
  static Provider p;
  return p;
}
}  // namespace refpin
#define KOKKOS_ASSERT(x)                              \
  do {                                                \
    if (!(x)) ++::refpin::assert_failures();          \
  } while (0)

namespace Kokkos {

// ---- memory traits, layouts, spaces ---------------------------------------
enum MemoryTraitsFlags : unsigned { Unmanaged = 0x01, RandomAccess = 0x02, Atomic = 0x04, Restrict = 0x08, Aligned = 0x10 };
template <unsigned T>
struct MemoryTraits {
  static constexpr unsigned impl_value = T;
};
using MemoryUnmanaged = MemoryTraits<Unmanaged>;

struct LayoutLeft {};
struct LayoutRight {};
struct LayoutStride {};

struct HostSpace {
  using memory_space = HostSpace;
};
struct ScratchMemorySpace {
  using memory_space = ScratchMemorySpace;
};
struct Serial {
  using execution_space = Serial;
  using memory_space = HostSpace;
  using array_layout = LayoutRight;  // the host backends' layout
  using scratch_memory_space = ScratchMemorySpace;
  using size_type = std::size_t;
};
using DefaultExecutionSpace = Serial;
using DefaultHostExecutionSpace = Serial;
using SharedSpace = HostSpace;
using SharedHostPinnedSpace = HostSpace;
using OpenMP = Serial;

template <class A, class B>
struct SpaceAccessibility {
  static constexpr bool accessible = true;
  static constexpr bool assignable = true;
};

// ---- views -------------------------------------------------------------------
namespace Impl {
template <class D>
struct DataAnalysis;  // value type, rank, static extents of a View data type
template <class T>
struct DataAnalysis {
  using value_type = T;
  static constexpr int rank = 0;
  static constexpr std::size_t s0 = 0, s1 = 0;
};
template <class T>
struct DataAnalysis<T*> {
  using value_type = T;
  static constexpr int rank = 1;
  static constexpr std::size_t s0 = 0, s1 = 0;
};
template <class T>
struct DataAnalysis<T**> {
  using value_type = T;
  static constexpr int rank = 2;
  static constexpr std::size_t s0 = 0, s1 = 0;
};
template <class T, std::size_t N>
struct DataAnalysis<T* [N]> {
  using value_type = T;
  static constexpr int rank = 2;
  static constexpr std::size_t s0 = 0, s1 = N;
};
template <class T, std::size_t N>
struct DataAnalysis<T[N]> {
  using value_type = T;
  static constexpr int rank = 1;
  static constexpr std::size_t s0 = N, s1 = 0;
};

template <class... P>
struct LayoutOf {
  using type = DefaultExecutionSpace::array_layout;
};
template <class First, class... Rest>
struct LayoutOf<First, Rest...> {
  using type = std::conditional_t<std::is_same_v<First, LayoutLeft> || std::is_same_v<First, LayoutRight>, First,
                                  typename LayoutOf<Rest...>::type>;
};

struct Scratch {
  std::shared_ptr<std::vector<char>> mem = std::make_shared<std::vector<char>>();
};
}  // namespace Impl

struct ALL_t {};
inline constexpr ALL_t ALL{};

struct WithoutInitializing_t {};
inline constexpr WithoutInitializing_t WithoutInitializing{};
namespace Impl {
struct ViewAlloc {
  std::string label;
};
}  // namespace Impl
template <class... A>
Impl::ViewAlloc view_alloc(A... a) {
  Impl::ViewAlloc r;
  ((void)[&](const auto& x) {
    if constexpr (std::is_convertible_v<decltype(x), std::string>) r.label = x;
  }(a), ...);
  return r;
}

template <class DataType, class... Props>
class View {
 public:
  using A = Impl::DataAnalysis<DataType>;
  using value_type = typename A::value_type;
  using non_const_value_type = std::remove_const_t<value_type>;
  using const_value_type = const non_const_value_type;
  using reference_type = value_type&;
  using pointer_type = value_type*;
  using array_layout = typename Impl::LayoutOf<Props...>::type;
  using memory_space = HostSpace;
  using execution_space = DefaultExecutionSpace;
  using size_type = std::size_t;
  static constexpr int rank = A::rank;
  static constexpr bool left = std::is_same_v<array_layout, LayoutLeft>;

  View() {
    ext_[0] = A::s0;
    ext_[1] = A::s1;
  }
  // managed allocation: View("label", n0[, n1])
  explicit View(const std::string& label, std::size_t n0 = 0, std::size_t n1 = 0) : label_(label) {
    set_extents(n0, n1);
    const std::size_t n = span_len();
    holder_ = std::shared_ptr<non_const_value_type[]>(new non_const_value_type[n ? n : 1]());
    ptr_ = holder_.get();
  }
  explicit View(const char* label, std::size_t n0 = 0, std::size_t n1 = 0) : View(std::string(label), n0, n1) {}
  View(const Impl::ViewAlloc& a, std::size_t n0 = 0, std::size_t n1 = 0) : View(a.label, n0, n1) {}
  // unmanaged wrap of caller memory: View(ptr, n0[, n1])
  View(value_type* p, std::size_t n0, std::size_t n1 = 0) : ptr_(p) { set_extents(n0, n1); }
  // team scratch
  View(Impl::Scratch s, std::size_t n0, std::size_t n1 = 0) {
    set_extents(n0, n1);
    s.mem->resize(span_len() * sizeof(value_type));
    scratch_ = s.mem;
    ptr_ = reinterpret_cast<value_type*>(s.mem->data());
  }
  // conversion between views of the same element type (const added, static
  // extents dropped, traits changed)
  template <class D2, class... P2>
  View(const View<D2, P2...>& o) : ptr_(o.impl_ptr()), holder_(o.impl_holder()), scratch_(o.impl_scratch()), label_(o.label()) {
    ext_[0] = o.extent(0);
    ext_[1] = o.extent(1);
  }

  void set_extents(std::size_t n0, std::size_t n1) {
    ext_[0] = A::s0 ? A::s0 : n0;
    ext_[1] = A::s1 ? A::s1 : n1;
  }
  std::size_t span_len() const {
    if (rank == 0) return 1;
    if (rank == 1) return ext_[0];
    return ext_[0] * ext_[1];
  }

  value_type& operator()() const { return ptr_[0]; }
  template <class I>
  value_type& operator()(I i) const {
    return ptr_[static_cast<std::size_t>(i)];
  }
  template <class I, class J>
  value_type& operator()(I i, J j) const {
    const std::size_t a = static_cast<std::size_t>(i), b = static_cast<std::size_t>(j);
    return left ? ptr_[a + b * ext_[0]] : ptr_[a * ext_[1] + b];
  }
  template <class I>
  value_type& operator[](I i) const {
    return ptr_[static_cast<std::size_t>(i)];
  }

  std::size_t extent(int r) const { return r < 2 ? ext_[r] : 1; }
  int extent_int(int r) const { return static_cast<int>(extent(r)); }
  static constexpr std::size_t static_extent(int r) { return r == 0 ? A::s0 : (r == 1 ? A::s1 : 0); }
  std::size_t size() const { return span_len(); }
  std::size_t span() const { return span_len(); }
  value_type* data() const { return ptr_; }
  std::string label() const { return label_; }
  bool is_allocated() const { return ptr_ != nullptr; }

  value_type* impl_ptr() const { return ptr_; }
  std::shared_ptr<non_const_value_type[]> impl_holder() const { return holder_; }
  std::shared_ptr<std::vector<char>> impl_scratch() const { return scratch_; }

 private:
  value_type* ptr_ = nullptr;
  std::shared_ptr<non_const_value_type[]> holder_;
  std::shared_ptr<std::vector<char>> scratch_;
  std::size_t ext_[2] = {0, 0};
  std::string label_;
};

template <class V, class... Args>
using Subview = View<typename V::non_const_value_type*, typename V::array_layout>;

// Kokkos::resize: a new allocation of the new extents holding every element
// whose indices exist in both (LayoutLeft or LayoutRight alike).
template <class D, class... P>
void resize(View<D, P...>& v, std::size_t n0, std::size_t n1 = 0) {
  View<D, P...> w(v.label(), n0, n1);
  const std::size_t e0 = std::min(v.extent(0), w.extent(0)), e1 = std::min(v.extent(1), w.extent(1));
  if constexpr (View<D, P...>::rank == 1) {
    for (std::size_t i = 0; i < e0; ++i) w(i) = v(i);
  } else if constexpr (View<D, P...>::rank == 2) {
    for (std::size_t i = 0; i < e0; ++i)
      for (std::size_t j = 0; j < e1; ++j) w(i, j) = v(i, j);
  }
  v = w;
}
// Kokkos::realloc: a new zeroed allocation (contents not kept).
template <class D, class... P>
void realloc(View<D, P...>& v, std::size_t n0, std::size_t n1 = 0) {
  v = View<D, P...>(v.label(), n0, n1);
}
// subview of a rank-1 view over [a, b)
template <class D, class... P, class I>
View<D, P...> subview(const View<D, P...>& v, std::pair<I, I> r) {
  return View<D, P...>(v.data() + r.first, static_cast<std::size_t>(r.second - r.first));
}

template <class V, class T>
void deep_copy(const V& v, const T& value) {
  for (std::size_t i = 0; i < v.span(); ++i) v.data()[i] = static_cast<typename V::non_const_value_type>(value);
}
template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...>& dst, const View<D2, P2...>& src) {
  for (std::size_t i = 0; i < dst.span(); ++i) dst.data()[i] = src.data()[i];
}

template <class T>
auto create_mirror_view(const T& v) {
  return v;
}
template <class S, class T>
auto create_mirror_view_and_copy(const S&, const T& v) {
  return v;
}

// ---- atomics (single-threaded) ---------------------------------------------------
template <class T, class U>
inline void atomic_add(T* p, U v) {
  *p += static_cast<T>(v);
}
template <class T, class U>
inline T atomic_fetch_add(T* p, U v) {
  T old = *p;
  *p += static_cast<T>(v);
  return old;
}
template <class T>
inline T atomic_fetch_inc(T* p) {
  return (*p)++;
}
template <class T>
inline void atomic_increment(T* p) {
  ++(*p);
}
template <class T>
inline T atomic_load(const T* p) {
  return *p;
}
template <class T, class U>
inline T atomic_exchange(T* p, U v) {
  T old = *p;
  *p = static_cast<T>(v);
  return old;
}

// ---- math: Kokkos' overload set over the C library ------------------------------
#define BMC_REFPIN_UNARY(name)                          \
  inline float name(float x) { return std::name(x); }   \
  inline double name(double x) { return std::name(x); } \
  template <class I, std::enable_if_t<std::is_integral_v<I>, int> = 0> \
  inline double name(I x) { return std::name(static_cast<double>(x)); }
BMC_REFPIN_UNARY(log)
BMC_REFPIN_UNARY(exp)
BMC_REFPIN_UNARY(sqrt)
BMC_REFPIN_UNARY(erf)
BMC_REFPIN_UNARY(erfc)
BMC_REFPIN_UNARY(log10)
BMC_REFPIN_UNARY(cbrt)
BMC_REFPIN_UNARY(tanh)
#undef BMC_REFPIN_UNARY
inline float abs(float x) { return std::fabs(x); }
inline double abs(double x) { return std::fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline long abs(long x) { return x < 0 ? -x : x; }
inline float copysign(float a, float b) { return std::copysign(a, b); }
inline double copysign(double a, double b) { return std::copysign(a, b); }
inline float pow(float a, float b) { return std::pow(a, b); }
inline double pow(double a, double b) { return std::pow(a, b); }
template <class T>
inline bool isfinite(T x) {
  return std::isfinite(x);
}
template <class T>
constexpr const T& min(const T& a, const T& b) {
  return (b < a) ? b : a;
}
template <class T>
constexpr const T& max(const T& a, const T& b) {
  return (a < b) ? b : a;
}
template <class T>
constexpr T min(std::initializer_list<T> l) {
  T m = *l.begin();
  for (const T& v : l) m = (v < m) ? v : m;
  return m;
}
template <class T>
constexpr T max(std::initializer_list<T> l) {
  T m = *l.begin();
  for (const T& v : l) m = (m < v) ? v : m;
  return m;
}
template <class T>
constexpr const T& clamp(const T& v, const T& lo, const T& hi) {
  return (v < lo) ? lo : (hi < v) ? hi : v;
}

namespace numbers {
template <class T>
inline constexpr T pi_v = static_cast<T>(3.141592653589793238462643383279502884L);
template <class T>
inline constexpr T sqrt2_v = static_cast<T>(1.414213562373095048801688724209698079L);
template <class T>
inline constexpr T e_v = static_cast<T>(2.718281828459045235360287471352662498L);
inline constexpr double pi = pi_v<double>;
inline constexpr double sqrt2 = sqrt2_v<double>;
inline constexpr double e = e_v<double>;
}  // namespace numbers

// ---- small aggregates ------------------------------------------------------------
template <class T1, class T2>
struct pair {
  T1 first;
  T2 second;
  constexpr pair() = default;
  constexpr pair(T1 a, T2 b) : first(a), second(b) {}
};
template <class T1, class T2>
pair(T1, T2) -> pair<T1, T2>;

template <class T, std::size_t N>
struct Array {
  T m_internal_implementation_private_member_data[N > 0 ? N : 1];
  constexpr T& operator[](std::size_t i) { return m_internal_implementation_private_member_data[i]; }
  constexpr const T& operator[](std::size_t i) const { return m_internal_implementation_private_member_data[i]; }
  static constexpr std::size_t size() { return N; }
  constexpr T* data() { return m_internal_implementation_private_member_data; }
  constexpr const T* data() const { return m_internal_implementation_private_member_data; }
};

template <class... Args>
inline int printf(const char* fmt, Args... args) {
  if constexpr (sizeof...(Args) == 0)
    return std::fputs(fmt, stdout);
  else
    return std::printf(fmt, args...);
}

// ---- dispatch (serial) ------------------------------------------------------------
struct AUTO_t {
  constexpr const AUTO_t& operator()() const { return *this; }
};
inline constexpr AUTO_t AUTO{};

namespace Impl {
template <class T>
struct IsSpace : std::bool_constant<std::is_same_v<T, Serial>> {};
// work tag of a policy: its first template argument that is not an
// execution space (void when none)
template <class... P>
struct TagOf {
  using type = void;
};
template <class F, class... R>
struct TagOf<F, R...> {
  using type = std::conditional_t<IsSpace<F>::value || std::is_void_v<F>, typename TagOf<R...>::type, F>;
};
template <class Tag, class F, class... A>
void call(const F& f, A&&... a) {
  if constexpr (std::is_void_v<Tag>)
    f(std::forward<A>(a)...);
  else
    f(Tag{}, std::forward<A>(a)...);
}
template <class Tag>
const void* tag_ptr() {
  if constexpr (std::is_void_v<Tag>)
    return nullptr;
  else
    return ::refpin::tag_id<Tag>();
}
}  // namespace Impl

template <class... P>
struct RangePolicy {
  using execution_space = DefaultExecutionSpace;
  using work_tag = typename Impl::TagOf<P...>::type;
  std::size_t b = 0, e = 0;
  RangePolicy(std::size_t b_, std::size_t e_) : b(b_), e(e_) {}
  RangePolicy(const Serial&, std::size_t b_, std::size_t e_) : b(b_), e(e_) {}
};

struct TeamMember {
  std::size_t rank = 0, size = 1;
  int league_rank() const { return static_cast<int>(rank); }
  int league_size() const { return static_cast<int>(size); }
  int team_rank() const { return 0; }
  int team_size() const { return 1; }
  void team_barrier() const {}
  Impl::Scratch team_scratch(int) const { return {}; }
  Impl::Scratch thread_scratch(int) const { return {}; }
};

struct PerTeamTag {
  std::size_t bytes = 0;
};
struct PerThreadTag {
  std::size_t bytes = 0;
};
inline PerTeamTag PerTeam(const TeamMember&) { return {}; }
inline PerThreadTag PerThread(const TeamMember&) { return {}; }
inline PerTeamTag PerTeam(std::size_t b) { return {b}; }
inline PerThreadTag PerThread(std::size_t b) { return {b}; }

template <class... P>
struct TeamPolicy {
  using execution_space = DefaultExecutionSpace;
  using member_type = TeamMember;
  using work_tag = typename Impl::TagOf<P...>::type;
  std::size_t league = 1;
  TeamPolicy() = default;
  template <class N, class... R, std::enable_if_t<std::is_integral_v<N>, int> = 0>
  TeamPolicy(N n, R...) : league(static_cast<std::size_t>(n)) {}
  template <class N, class... R, std::enable_if_t<std::is_integral_v<N>, int> = 0>
  TeamPolicy(const Serial&, N n, R...) : league(static_cast<std::size_t>(n)) {}
  template <class S>
  TeamPolicy set_scratch_size(int, S) const {
    return *this;
  }
  template <class S, class T>
  TeamPolicy set_scratch_size(int, S, T) const {
    return *this;
  }
};

struct ThreadRange {
  std::size_t b = 0, e = 0;
};
inline ThreadRange TeamThreadRange(const TeamMember&, std::size_t b, std::size_t e) { return {b, e}; }
inline ThreadRange TeamThreadRange(const TeamMember&, std::size_t e) { return {0, e}; }
inline ThreadRange TeamVectorRange(const TeamMember&, std::size_t b, std::size_t e) { return {b, e}; }
inline ThreadRange TeamVectorRange(const TeamMember&, std::size_t e) { return {0, e}; }
inline ThreadRange ThreadVectorRange(const TeamMember&, std::size_t b, std::size_t e) { return {b, e}; }
inline ThreadRange ThreadVectorRange(const TeamMember&, std::size_t e) { return {0, e}; }

// nested range loops (inside a team)
template <class F>
void parallel_for(const ThreadRange& r, const F& f) {
  for (std::size_t i = r.b; i < r.e; ++i) {
    ::refpin::ctx().index = i;
    f(i);
  }
}
template <class F, class T>
void parallel_reduce(const ThreadRange& r, const F& f, T& value) {
  value = T{};
  for (std::size_t i = r.b; i < r.e; ++i) {
    ::refpin::ctx().index = i;
    f(i, value);
  }
}

// top-level dispatch
template <class F>
void parallel_for(std::size_t n, const F& f) {
  ::refpin::ctx().tag = nullptr;
  for (std::size_t i = 0; i < n; ++i) {
    ::refpin::ctx().index = i;
    f(i);
  }
}
template <class... P, class F>
void parallel_for(const RangePolicy<P...>& r, const F& f) {
  using Tag = typename RangePolicy<P...>::work_tag;
  ::refpin::ctx().tag = Impl::tag_ptr<Tag>();
  for (std::size_t i = r.b; i < r.e; ++i) {
    ::refpin::ctx().index = i;
    Impl::call<Tag>(f, i);
  }
}
template <class... P, class F>
void parallel_for(const TeamPolicy<P...>& t, const F& f) {
  using Tag = typename TeamPolicy<P...>::work_tag;
  for (std::size_t r = 0; r < t.league; ++r) {
    ::refpin::ctx().tag = Impl::tag_ptr<Tag>();
    ::refpin::ctx().league = r;
    Impl::call<Tag>(f, TeamMember{r, t.league});
  }
}
template <class Pol, class F>
void parallel_for(const std::string&, const Pol& p, const F& f) {
  parallel_for(p, f);
}

namespace Impl {
template <class R, class = void>
struct IsReducer : std::false_type {};
template <class R>
struct IsReducer<R, std::void_t<typename R::reducer>> : std::true_type {};
template <class R, class = void>
struct IsView : std::false_type {};
template <class R>
struct IsView<R, std::void_t<typename R::array_layout, typename R::non_const_value_type>> : std::true_type {};

// runs body(acc) over the policy with the result's type, then stores it
template <class Res, class Body>
void reduce_into(Res&& result, const Body& body) {
  using R = std::decay_t<Res>;
  if constexpr (IsReducer<R>::value) {
    typename R::value_type acc;
    result.init(acc);
    body(acc);
    result.reference() = acc;
  } else if constexpr (IsView<R>::value) {
    typename R::non_const_value_type acc{};
    body(acc);
    result() = acc;
  } else {
    R acc{};
    body(acc);
    result = acc;
  }
}
}  // namespace Impl

template <class... P, class F, class Res>
void parallel_reduce(const RangePolicy<P...>& r, const F& f, Res&& result) {
  using Tag = typename RangePolicy<P...>::work_tag;
  Impl::reduce_into(std::forward<Res>(result), [&](auto& acc) {
    ::refpin::ctx().tag = Impl::tag_ptr<Tag>();
    for (std::size_t i = r.b; i < r.e; ++i) {
      ::refpin::ctx().index = i;
      Impl::call<Tag>(f, i, acc);
    }
  });
}
template <class... P, class F, class Res>
void parallel_reduce(const TeamPolicy<P...>& t, const F& f, Res&& result) {
  using Tag = typename TeamPolicy<P...>::work_tag;
  Impl::reduce_into(std::forward<Res>(result), [&](auto& acc) {
    for (std::size_t r = 0; r < t.league; ++r) {
      ::refpin::ctx().tag = Impl::tag_ptr<Tag>();
      ::refpin::ctx().league = r;
      Impl::call<Tag>(f, TeamMember{r, t.league}, acc);
    }
  });
}
template <class Pol, class F, class Res>
void parallel_reduce(const std::string&, const Pol& p, const F& f, Res&& result) {
  parallel_reduce(p, f, std::forward<Res>(result));
}

// one pass with final = true, as the Serial backend runs a scan
template <class... P, class F>
void parallel_scan(const RangePolicy<P...>& r, const F& f) {
  using Tag = typename RangePolicy<P...>::work_tag;
  ::refpin::ctx().tag = Impl::tag_ptr<Tag>();
  std::size_t update = 0;
  for (std::size_t i = r.b; i < r.e; ++i) {
    ::refpin::ctx().index = i;
    if constexpr (std::is_void_v<Tag>)
      f(static_cast<int>(i), update, true);
    else
      f(Tag{}, static_cast<int>(i), update, true);
  }
}
template <class Pol, class F>
void parallel_scan(const std::string&, const Pol& p, const F& f) {
  parallel_scan(p, f);
}
inline void fence(const std::string& = "") {}

template <class T, class F>
void single(T, const F& f) {
  f();
}

// ---- random numbers: a tape of injected values --------------------------------------
namespace Impl {
// Values a test pushes before a call; each draw takes the next one.  A
// uniform draw in [a, b) returns a + (b - a) * u for the tape value u; a
// normal draw returns mean + stddev * z for the tape value z.
struct DrawTape {
  std::vector<double> v;
  std::size_t pos = 0;
  double next() {
    if (pos >= v.size()) {
      ++::refpin::assert_failures();
      return 0.5;
    }
    return v[pos++];
  }
};
inline DrawTape& tape() {
  static DrawTape t;
  return t;
}
}  // namespace Impl

namespace Impl {
inline double draw(int kind) {
  const auto& p = ::refpin::provider();
  return p.fn ? p.fn(p.user, kind) : tape().next();
}
}  // namespace Impl

template <class Device>
class Random_XorShift1024 {
 public:
  float frand() { return static_cast<float>(Impl::draw(0)); }
  float frand(float b) { return b * frand(); }
  float frand(float a, float b) { return a + (b - a) * frand(); }
  double drand() { return Impl::draw(1); }
  double drand(double b) { return b * drand(); }
  double drand(double a, double b) { return a + (b - a) * drand(); }
  uint64_t urand64() { return static_cast<uint64_t>(Impl::draw(3)); }
  uint64_t urand64(uint64_t b) { return urand64() % (b ? b : 1); }
  uint64_t urand64(uint64_t a, uint64_t b) { return a + urand64(b - a); }
  uint32_t urand() { return static_cast<uint32_t>(Impl::draw(3)); }
  double normal() { return Impl::draw(2); }
  double normal(double mean, double stddev) { return mean + stddev * normal(); }
};

template <class Device>
class Random_XorShift1024_Pool {
 public:
  using generator_type = Random_XorShift1024<Device>;
  using device_type = Device;
  Random_XorShift1024_Pool() = default;
  explicit Random_XorShift1024_Pool(uint64_t) {}
  generator_type get_state() const { return {}; }
  void free_state(const generator_type&) const {}
};

namespace Impl {
template <class ViewType, class RandomPool, int loops, int rank, class IndexType>
struct fill_random_functor_begin_end {
  template <class B, class E>
  fill_random_functor_begin_end(ViewType, RandomPool, B, E) {}
  void operator()(std::size_t) const {}
};
}  // namespace Impl
template <class V, class P, class B, class E>
void fill_random(V, P, B, E) {}

// ---- scatter views: serial, straight into the target view ----------------------------
namespace Experimental {
// Kokkos' ScatterValue::operator+= takes the element type: the right-hand
// side is converted to it, then added.
template <class T>
struct ScatterRef {
  T* p;
  void operator+=(const T& v) const { *p += v; }
  void operator-=(const T& v) const { *p -= v; }
};
template <class DataType, class Layout = LayoutRight, class Exec = DefaultExecutionSpace>
struct ScatterView {
  using view_type = View<DataType, Layout>;
  using value_type = typename view_type::non_const_value_type;
  view_type v;
  ScatterView() = default;
  explicit ScatterView(const view_type& x) : v(x) {}
  void reset() { deep_copy(v, 0); }
  struct Access {
    view_type v;
    template <class... I>
    ScatterRef<value_type> operator()(I... i) const {
      return ScatterRef<value_type>{&v(i...)};
    }
  };
  Access access() const { return Access{v}; }
  template <class V>
  void contribute_into(const V&) const {}
};
template <class D, class... P>
ScatterView<D, typename View<D, P...>::array_layout> create_scatter_view(const View<D, P...>& v) {
  return ScatterView<D, typename View<D, P...>::array_layout>(View<D, typename View<D, P...>::array_layout>(v));
}
template <class V, class S>
void contribute(const V&, const S&) {}
}  // namespace Experimental

// ---- sorting: only the names the container's (unused) sort member spells --------------
template <class V>
struct BinOp1D {
  template <class... A>
  BinOp1D(A...) {}
};
template <class V, class Op>
struct BinSort {
  template <class... A>
  BinSort(A...) {}
};

namespace Profiling {
struct ScopedRegion {
  explicit ScopedRegion(const std::string&) {}
};
}  // namespace Profiling

inline void initialize() {}
inline void finalize() {}
}  // namespace Kokkos

#endif
