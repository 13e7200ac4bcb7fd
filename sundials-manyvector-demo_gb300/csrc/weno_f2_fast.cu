// Float-float WENO flux divergence, WV = 1 sweep: the tracer reconstructions take FP32 weights
// and smoothness indicators in correction form (the characteristic fluid fields keep
// float-float weights).  A translation unit of its own so that it compiles beside weno_f2.cu.
#include "weno_f2.cuh"

namespace gbmv {

int feuler_f2_fast(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                   double* scratch, float2* q2, const double* tscale, int* d_status,
                   cudaStream_t s) {
  return feuler_f2_wv<1>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
}

}  // namespace gbmv
