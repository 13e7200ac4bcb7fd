/* Serial stand-in for the few RAJA names the reference's chemistry network and problem files
 * use (src/raja_primordial_network.hpp:46-57, src/raja_primordial_network.cpp,
 * src/primordial_static.cpp): the SERIAL backend's policy types, RAJA::forall over a
 * RangeSegment, 4-d views and three-segment kernels.  Test infrastructure only. */
#ifndef GBMV_SHIM_RAJA_HPP
#define GBMV_SHIM_RAJA_HPP

#define RAJA_DEVICE
#define RAJA_HOST_DEVICE

#include <memory>

namespace RAJA {
struct loop_exec {};
struct loop_reduce {};
template <class... T> struct KernelPolicy {};
namespace statement {
template <int I, class P, class... S> struct For {};
template <int I> struct Lambda {};
}  // namespace statement

struct RangeSegment {
  long b, e;
  RangeSegment(long b_, long e_) : b(b_), e(e_) {}
};

template <class Policy, class Body>
inline void forall(const RangeSegment& r, Body&& body) {
  for (long i = r.b; i < r.e; ++i) body(i);
}

// RAJA::View over a row-major RAJA::Layout<4> (the rightmost index has stride 1), and
// RAJA::kernel over a tuple of three segments as three nested loops, the first segment
// outermost -- the forms the problem files' Dengo-scaling loops use
// (src/primordial_static.cpp:234-318).
template <int N> struct Layout {};
template <class T, class L> struct View;
template <class T> struct View<T, Layout<4> > {
  T* p;
  long n1, n2, n3;
  View(T* p_, long, long n1_, long n2_, long n3_) : p(p_), n1(n1_), n2(n2_), n3(n3_) {}
  T& operator()(long a, long b, long c, long d) const { return p[((a * n1 + b) * n2 + c) * n3 + d]; }
};
struct Segments3 {
  RangeSegment a, b, c;
};
inline Segments3 make_tuple(const RangeSegment& a, const RangeSegment& b,
                            const RangeSegment& c) {
  return Segments3{a, b, c};
}
// a sum reduction usable from a by-value lambda capture, as RAJA's (serial: a shared total)
template <class Policy, class T> struct ReduceSum {
  std::shared_ptr<T> v;
  explicit ReduceSum(T init) : v(new T(init)) {}
  const ReduceSum& operator+=(T x) const { *v += x; return *this; }
  T get() const { return *v; }
  operator T() const { return *v; }
};
template <class Policy, class Body>
inline void kernel(const Segments3& s, Body&& body) {
  for (long a = s.a.b; a < s.a.e; ++a)
    for (long b = s.b.b; b < s.b.e; ++b)
      for (long c = s.c.b; c < s.c.e; ++c) body((int)a, (int)b, (int)c);
}
}  // namespace RAJA

#endif
