// Host-only stand-in for the subset of Kokkos Core that the reference
// euler2d solver uses: View (rank 2 + a static trailing extent of 4), Array,
// deep_copy, create_mirror_view, parallel_for / parallel_reduce over
// RangePolicy and 2-D MDRangePolicy (optionally tagged), the Max and Sum
// reducers, atomic_add / atomic_sub and Profiling regions.
//
// Test infrastructure only (the parity checker for the GPU path).  Views use
// LayoutLeft, i.e. element (i, j, v) of an (n0, n1, 4) view lives at
// i + n0 * (j + n1 * v) -- the layout Kokkos picks on its CUDA backend -- so
// arrays can be exchanged byte for byte with the device code.
//
// With E2D_COMPAT_OPENMP defined, 2-D ranges run as an OpenMP
// `parallel for collapse(2)` and reductions combine per-thread partials.
#pragma once

#include "Kokkos_Macros.hpp"
#include "Kokkos_MathematicalFunctions.hpp"

#include <cfloat>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <memory>
#include <string>
#include <type_traits>

namespace Kokkos
{

// ---------------------------------------------------------------- spaces
struct HostSpace
{
  using memory_space = HostSpace;
};
struct Serial
{
  using execution_space = Serial;
  using memory_space = HostSpace;
  using device_type = Serial;
};
using DefaultExecutionSpace = Serial;
using DefaultHostExecutionSpace = Serial;

template <class Exec, class Mem>
struct Device
{
  using execution_space = Exec;
  using memory_space = Mem;
};

template <unsigned N>
struct MemoryTraits
{};
enum
{
  Atomic = 1
};

inline void
initialize(int &, char **)
{}
inline void
finalize()
{}

namespace Profiling
{
inline void
pushRegion(const std::string &)
{}
inline void
popRegion()
{}
} // namespace Profiling

// ---------------------------------------------------------------- Array
template <class T, unsigned N>
struct Array
{
  T m_data[N];
  T &
  operator[](int k)
  {
    return m_data[k];
  }
  const T &
  operator[](int k) const
  {
    return m_data[k];
  }
  static constexpr unsigned
  size()
  {
    return N;
  }
};

// ---------------------------------------------------------------- View
struct WithoutInitializing_t
{};
constexpr WithoutInitializing_t WithoutInitializing{};

struct ViewAllocProp
{
  std::string label;
  bool        init = true;
};
inline ViewAllocProp
view_alloc(WithoutInitializing_t, const std::string & label)
{
  return ViewAllocProp{ label, false };
}
inline ViewAllocProp
view_alloc(const std::string & label, WithoutInitializing_t)
{
  return ViewAllocProp{ label, false };
}

// Everything is host memory, so every space can access every other.
template <class AccessSpace, class MemorySpace>
struct SpaceAccessibility
{
  static constexpr bool accessible = true;
};

namespace compat_detail
{
// Decompose T** [N] / T* into value type, runtime rank and static extent.
template <class D>
struct traits;
template <class T>
struct traits<T *>
{
  using value_type = T;
  static constexpr int  dyn = 1;
  static constexpr long last = 1;
};
template <class T>
struct traits<T **>
{
  using value_type = T;
  static constexpr int  dyn = 2;
  static constexpr long last = 1;
};
template <class T, long N>
struct traits<T * [N]>
{
  using value_type = T;
  static constexpr int  dyn = 1;
  static constexpr long last = N;
};
template <class T, long N>
struct traits<T ** [N]>
{
  using value_type = T;
  static constexpr int  dyn = 2;
  static constexpr long last = N;
};
} // namespace compat_detail

template <class DataType, class... Props>
class View
{
  using tr = compat_detail::traits<DataType>;

public:
  using value_type = typename tr::value_type;
  using host_mirror_type = View<DataType, Props...>;
  using memory_space = HostSpace;  // every view lives in host memory
  static constexpr int rank = tr::dyn + (tr::last > 1 ? 1 : 0);
  using HostMirror = host_mirror_type;

  View() = default;

  View(const std::string & label, long n0, long n1 = 1)
  {
    allocate(ViewAllocProp{ label, true }, n0, n1);
  }
  View(const ViewAllocProp & prop, long n0, long n1 = 1) { allocate(prop, n0, n1); }

  value_type &
  operator()(long i) const
  {
    return m_ptr[i];
  }
  value_type &
  operator()(long i, long j) const
  {
    return m_ptr[i + m_n0 * j];
  }
  value_type &
  operator()(long i, long j, long v) const
  {
    return m_ptr[i + m_n0 * (j + m_n1 * v)];
  }

  value_type *
  data() const
  {
    return m_ptr;
  }
  long
  extent(int r) const
  {
    return r == 0 ? m_n0 : (r == 1 ? m_n1 : tr::last);
  }
  long
  size() const
  {
    return m_n0 * m_n1 * tr::last;
  }
  const std::string &
  label() const
  {
    return m_label;
  }

private:
  void
  allocate(const ViewAllocProp & prop, long n0, long n1)
  {
    m_label = prop.label;
    m_n0 = n0;
    m_n1 = (tr::dyn == 2) ? n1 : 1;
    const long n = m_n0 * m_n1 * tr::last;
    // 1-D views get zeroed slack after their extent: the radial-profile
    // functor (src/ComputeRadialProfileFunctor.h:150-158) indexes its two
    // histograms with bins up to ~2.5x nbins for the ghost corner cells;
    // the slack absorbs those writes so that bins [0, nbins) are defined.
    const long cap = (tr::dyn == 1 && tr::last == 1) ? 3 * n + 64 : (n > 0 ? n : 1);
    m_owner = std::shared_ptr<value_type>(new value_type[cap], std::default_delete<value_type[]>());
    m_ptr = m_owner.get();
    if (prop.init || cap > n)
      std::memset((void *)m_ptr, 0, sizeof(value_type) * cap);
  }

  std::shared_ptr<value_type> m_owner;
  value_type *                m_ptr = nullptr;
  long                        m_n0 = 0, m_n1 = 0;
  std::string                 m_label;
};

template <class D, class... P>
inline View<D, P...>
create_mirror_view(const View<D, P...> & v)
{
  return v; // host memory already: the mirror aliases the view
}
template <class D, class... P>
inline View<D, P...>
create_mirror_view(WithoutInitializing_t, const View<D, P...> & v)
{
  return v;
}
template <class Space, class D, class... P>
inline View<D, P...>
create_mirror_view_and_copy(const Space &, const View<D, P...> & v)
{
  return v;
}

template <class D1, class... P1, class D2, class... P2>
inline void
deep_copy(const View<D1, P1...> & dst, const View<D2, P2...> & src)
{
  if (dst.data() == src.data())
    return;
  std::memcpy((void *)dst.data(), (const void *)src.data(),
              sizeof(typename View<D1, P1...>::value_type) * dst.size());
}
template <class D, class... P, class S>
inline typename std::enable_if<std::is_arithmetic<S>::value>::type
deep_copy(const View<D, P...> & dst, const S & value)
{
  for (long k = 0; k < dst.size(); ++k)
    dst.data()[k] = value;
}

// ---------------------------------------------------------------- policies
template <unsigned R>
struct Rank
{};

template <class... Args>
struct RangePolicy
{
  long begin, end;
  RangePolicy(long b, long e)
    : begin(b)
    , end(e)
  {}
};

namespace compat_detail
{
template <class... A>
struct tag_of
{
  using type = void;
};
template <class E, class R>
struct tag_of<E, R>
{
  using type = void;
};
template <class E, class R, class Tag>
struct tag_of<E, R, Tag>
{
  using type = Tag;
};
} // namespace compat_detail

template <class... Args>
struct MDRangePolicy
{
  using work_tag = typename compat_detail::tag_of<Args...>::type;
  long lo[2], hi[2];
  MDRangePolicy(std::initializer_list<long> l, std::initializer_list<long> h)
  {
    lo[0] = *l.begin();
    lo[1] = *(l.begin() + 1);
    hi[0] = *h.begin();
    hi[1] = *(h.begin() + 1);
  }
};

// ---------------------------------------------------------------- reducers
template <class T>
struct Max
{
  T & ref;
  explicit Max(T & r)
    : ref(r)
  {}
  static T
  identity()
  {
    return std::numeric_limits<T>::lowest();
  }
  static void
  join(T & a, const T & b)
  {
    if (b > a)
      a = b;
  }
};
template <class T>
struct Sum
{
  T & ref;
  explicit Sum(T & r)
    : ref(r)
  {}
  static T
  identity()
  {
    return T(0);
  }
  static void
  join(T & a, const T & b)
  {
    a += b;
  }
};

namespace compat_detail
{
template <class Tag, class F, class... A>
inline void
call(const F & f, A &&... a)
{
  if constexpr (std::is_void<Tag>::value)
    f(std::forward<A>(a)...);
  else
    f(Tag(), std::forward<A>(a)...);
}
} // namespace compat_detail

template <class... Args, class F>
inline void
parallel_for(const std::string &, const RangePolicy<Args...> & p, const F & f)
{
#ifdef E2D_COMPAT_OPENMP
#  pragma omp parallel for schedule(static)
#endif
  for (long k = p.begin; k < p.end; ++k)
    f((int)k);
}

template <class... Args, class F>
inline void
parallel_for(const std::string &, const MDRangePolicy<Args...> & p, const F & f)
{
  using Tag = typename MDRangePolicy<Args...>::work_tag;
#ifdef E2D_COMPAT_OPENMP
#  pragma omp parallel for collapse(2) schedule(static)
#endif
  for (long j = p.lo[1]; j < p.hi[1]; ++j)
    for (long i = p.lo[0]; i < p.hi[0]; ++i)
    {
      const int ii = (int)i, jj = (int)j;
      compat_detail::call<Tag>(f, ii, jj);
    }
}

template <class... Args, class F, class Reducer>
inline void
parallel_reduce(const std::string &, const MDRangePolicy<Args...> & p, const F & f, Reducer r)
{
  using Tag = typename MDRangePolicy<Args...>::work_tag;
  using T = typename std::remove_reference<decltype(r.ref)>::type;
  T total = Reducer::identity();
#ifdef E2D_COMPAT_OPENMP
#  pragma omp parallel
  {
    T part = Reducer::identity();
#  pragma omp for collapse(2) schedule(static) nowait
    for (long j = p.lo[1]; j < p.hi[1]; ++j)
      for (long i = p.lo[0]; i < p.hi[0]; ++i)
      {
        const int ii = (int)i, jj = (int)j;
        compat_detail::call<Tag>(f, ii, jj, part);
      }
#  pragma omp critical
    Reducer::join(total, part);
  }
#else
  for (long j = p.lo[1]; j < p.hi[1]; ++j)
    for (long i = p.lo[0]; i < p.hi[0]; ++i)
    {
      const int ii = (int)i, jj = (int)j;
      compat_detail::call<Tag>(f, ii, jj, total);
    }
#endif
  r.ref = total;
}

// ---------------------------------------------------------------- atomics
template <class T>
inline void
atomic_add(T * dst, const T v)
{
#ifdef E2D_COMPAT_OPENMP
#  pragma omp atomic
#endif
  *dst += v;
}
template <class T>
inline void
atomic_sub(T * dst, const T v)
{
#ifdef E2D_COMPAT_OPENMP
#  pragma omp atomic
#endif
  *dst -= v;
}

} // namespace Kokkos
