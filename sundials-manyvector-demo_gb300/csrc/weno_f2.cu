// Float-float WENO flux divergence: the per-cell primitive pass and the WV = 0 sweep
// (float-float weights everywhere), with the entry point that picks the weight variant.
#include "weno_f2.cuh"

namespace gbmv {

__global__ void __launch_bounds__(256) prims_f2_kernel(Grid g, Fields w, float2* __restrict__ Q2,
                                                       const double* __restrict__ tscale,
                                                       int* __restrict__ status) {
  const long n = g.ncell;
  int bad = 0;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
       c += (long)gridDim.x * blockDim.x) {
    const double rho = w.f[0][c], mx = w.f[1][c], my = w.f[2][c], mz = w.f[3][c], et = w.f[4][c];
    // one FP64 division per cell: the primitives are multiplied by 1/rho (each within an ulp
    // of the reference's quotients, far inside the float-float representation error)
    const double ir = 1.0 / rho;
    const double p = (g.gamma - 1.0) * (et - (mx * mx + my * my + mz * mz) * 0.5 * ir);
    // legal_state (src/euler3D.hpp:1398-1414) on this pressure: it differs from the quotient
    // form only in the last bit, so only a state with p within rounding of zero can flag
    // differently from the FP64 form
    bad |= (!(rho > 0.0) ? 1 : 0) | (!(et > 0.0) ? 2 : 0) | (!(p > 0.0) ? 4 : 0);
    double q[kQ2Base] = {rho, mx, my, mz, et, p, mx * ir, my * ir, mz * ir,
                         sqrt0(g.gamma * p * ir)};
#pragma unroll
    for (int k = 0; k < kQ2Base; ++k) {
      const f2 v = f2_split(q[k]);
      Q2[k * n + c] = make_float2(v.hi, v.lo);
    }
    for (int v = 0; v < g.nchem; ++v) {
      // tscale: the chemistry component arrives in scaled units (x = chem * scale)
      const long e = v + (long)g.nchem * c;
      const f2 x = f2_split(tscale ? w.f[5][e] * tscale[e] : w.f[5][e]);
      Q2[(kQ2Base + v) * n + c] = make_float2(x.hi, x.lo);
    }
  }
  bad = __reduce_or_sync(0xffffffffu, bad);
  if (bad && (threadIdx.x & 31) == 0) atomicOr(status, bad);
}

int prims_f2(const Grid& g, const Fields& w, float2* q2, const double* tscale, int* d_status,
             cudaStream_t s) {
  ProfScope ps("prims", s);
  prims_f2_kernel<<<sweep_blocks(g.ncell, 256), 256, 0, s>>>(g, w, q2, tscale, d_status);
  GBMV_LAUNCH_CHECK("prims_f2_kernel");
  return GBMV_OK;
}

size_t feuler_f2_prims_floats(const Grid& g) { return (size_t)2 * (kQ2Base + g.nchem) * g.ncell; }

int feuler_f2(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
              double* scratch, float* prims, const double* tscale, int* d_status,
              cudaStream_t s, int fast_weights) {
  float2* q2 = reinterpret_cast<float2*>(prims);
  if (fast_weights) return feuler_f2_fast(g, w, wdot, G, scratch, q2, tscale, d_status, s);
  return feuler_f2_wv<0>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
}

}  // namespace gbmv
