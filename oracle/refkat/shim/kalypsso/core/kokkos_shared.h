// Stub of the Kokkos pieces the reference's models/*.h use (Kokkos::Array, the inline-function
// macro, abort) plus kalypsso-core's small index enums. Host-only, for the known-answer bridge.
#pragma once
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <type_traits>
#include <kalypsso/core/real_type.h>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_ASSERT(x) ((void)0)

namespace Kokkos
{
template <typename T, std::size_t N>
struct Array
{
  T m_data[N > 0 ? N : 1];
  T &       operator[](std::size_t i) { return m_data[i]; }
  const T & operator[](std::size_t i) const { return m_data[i]; }
  static constexpr std::size_t size() { return N; }
  T *       begin() { return m_data; }
  T *       end() { return m_data + N; }
  const T * begin() const { return m_data; }
  const T * end() const { return m_data + N; }
};
[[noreturn]] inline void
abort(const char * msg)
{
  std::fprintf(stderr, "Kokkos::abort: %s\n", msg);
  std::abort();
}
template <typename T, std::size_t N>
inline bool
operator==(const Array<T, N> & a, const Array<T, N> & b)
{
  for (std::size_t i = 0; i < N; ++i)
    if (a[i] != b[i])
      return false;
  return true;
}
template <typename T, std::size_t N>
inline Array<T, N>
operator*(const Array<T, N> & a, T s)
{
  Array<T, N> r;
  for (std::size_t i = 0; i < N; ++i)
    r[i] = a[i] * s;
  return r;
}
template <typename T, std::size_t N>
inline Array<T, N>
operator+(const Array<T, N> & a, T s)
{
  Array<T, N> r;
  for (std::size_t i = 0; i < N; ++i)
    r[i] = a[i] + s;
  return r;
}
template <typename T, std::size_t N>
inline Array<T, N>
operator+(const Array<T, N> & a, const Array<T, N> & b)
{
  Array<T, N> r;
  for (std::size_t i = 0; i < N; ++i)
    r[i] = a[i] + b[i];
  return r;
}
template <typename T, std::size_t N>
inline Array<T, N>
operator-(const Array<T, N> & a, const Array<T, N> & b)
{
  Array<T, N> r;
  for (std::size_t i = 0; i < N; ++i)
    r[i] = a[i] - b[i];
  return r;
}
template <typename T, std::size_t N, typename S>
inline Array<T, N>
operator/(const Array<T, N> & a, S s)
{
  Array<T, N> r;
  for (std::size_t i = 0; i < N; ++i)
    r[i] = a[i] / s;
  return r;
}
template <typename T>
struct Max
{
  T & ref;
  explicit Max(T & r) : ref(r) {}
};
template <typename T, std::size_t N>
inline T
dim_prod(const Array<T, N> & a)
{
  T p = 1;
  for (std::size_t i = 0; i < N; ++i)
    p *= a[i];
  return p;
}
// serial stand-ins for the range policy and parallel_for the scheme functors use
template <class Exec, class Tag = void>
struct RangePolicy
{
  long long b, e;
  RangePolicy(long long b_, long long e_) : b(b_), e(e_) {}
};
template <class F, class Exec, class Tag>
void
parallel_for(const char *, RangePolicy<Exec, Tag> p, const F & f)
{
  for (long long i = p.b; i < p.e; ++i)
  {
    if constexpr (std::is_void_v<Tag>)
      f(i);
    else
      f(Tag{}, i);
  }
}
template <class F, class Exec, class Tag, typename T>
void
parallel_reduce(const char *, RangePolicy<Exec, Tag> p, const F & f, Max<T> red)
{
  T v = std::numeric_limits<T>::lowest();
  for (long long i = p.b; i < p.e; ++i)
    f(i, v);
  red.ref = v;
}
} // namespace Kokkos

namespace kalypsso
{
struct DefaultDevice
{
  using execution_space = int;
};
template <typename T>
KOKKOS_INLINE_FUNCTION void
my_swap(T & a, T & b)
{
  T t = a;
  a = b;
  b = t;
}
// component of an edge-centred array by edge direction
enum EdgeAlong : int
{
  ALONG_X = 0,
  ALONG_Y = 1,
  ALONG_Z = 2
};
enum ComponentIndex3D : int
{
  IX = 0,
  IY = 1,
  IZ = 2
};
enum EmfDir : int
{
  EMFX = 0,
  EMFY = 1,
  EMFZ = 2
};
// positions of the four states of the 2D magnetic Riemann problem / of the edge states
enum RiemannProblemPos : int
{
  ILL = 0,
  IRL = 1,
  ILR = 2,
  IRR = 3
};
enum EdgeStatePos : int
{
  IRT = 0,
  IRB = 1,
  ILT = 2,
  ILB = 3
};
} // namespace kalypsso
