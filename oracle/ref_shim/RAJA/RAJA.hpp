/* Serial stand-in for the few RAJA names the reference's chemistry network uses
 * (src/raja_primordial_network.hpp:46-57, src/raja_primordial_network.cpp): the SERIAL
 * backend's policy types and RAJA::forall over a RangeSegment.  Test infrastructure only. */
#ifndef GBMV_SHIM_RAJA_HPP
#define GBMV_SHIM_RAJA_HPP

#define RAJA_DEVICE
#define RAJA_HOST_DEVICE

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
}  // namespace RAJA

#endif
