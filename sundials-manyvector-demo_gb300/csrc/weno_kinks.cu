// Branch detection for derivative checks of the FP64 flux divergence (no counterpart in the
// reference).  The WENO face flux is smooth except where the Lax-Friedrichs speed
// alpha = max_j (|u_j| + c_j) over the face's six stencil points changes its maximising point j
// or the sign of that point's velocity (src/utilities.cpp:368-380, the `alpha < s` update keeps
// the first maximising point).  A central difference (f(w + h d) - f(w - h d)) / 2h of a cell's
// tendency is the derivative only if none of the cell's six faces changes that branch between
// w - h d, w and w + h d; this kernel marks the cells where one does, so that derivative tests
// can compare the exact JVP / VJP with finite differences on the smooth entries and count the
// others.  The branch is evaluated with the face kernel's own expressions (eos_t, sqrt0).
#include "weno_face.cuh"
#include "weno_sweep.cuh"

namespace gbmv {
namespace {

// branch word of the face with lower stencil point at axis position p0 - 3 (the face between
// cells p0 - 1 and p0 along DIR, p0 in [0, n_DIR]) at the state w + s dw
template <int DIR>
__device__ __forceinline__ int face_branch(const Grid& g, const Fields& w, const Fields& dw,
                                           double s, long i, long j, long k) {
  const double gm = g.gamma - 1.0;
  double alpha = 0.0;
  int arg = 0, neg = 0;
#pragma unroll
  for (int l = 0; l < 6; ++l) {
    long q[3] = {i, j, k};
    bool nall, nnorm;
    q[DIR] = ghost_src(q[DIR] - 3 + l, g.n[DIR], g.bc[2 * DIR], g.bc[2 * DIR + 1], &nall, &nnorm);
    const long c = q[0] + g.n[0] * (q[1] + g.n[1] * q[2]);
    double v[5];
#pragma unroll
    for (int f = 0; f < 5; ++f) {
      v[f] = __ldg(w.f[f] + c);
      if (s != 0.0) v[f] += s * __ldg(dw.f[f] + c);
    }
    if (nall) {
#pragma unroll
      for (int f = 0; f < 5; ++f) v[f] = -v[f];
    }
    if (nnorm) v[1 + DIR] = -v[1 + DIR];
    const double p = eos_t<double>(gm, v[0], v[1], v[2], v[3], v[4]);
    const double uj = v[1 + DIR] / v[0];
    const double sp = fabs(uj) + sqrt0<double>(g.gamma * p / v[0]);
    if (alpha < sp) {
      alpha = sp;
      arg = l;
      neg = uj < 0.0;
    }
  }
  return arg | (neg << 3);
}

template <int DIR>
__device__ __forceinline__ bool face_kinked(const Grid& g, const Fields& w, const Fields& dw,
                                            double h, long i, long j, long k) {
  const int b0 = face_branch<DIR>(g, w, dw, 0.0, i, j, k);
  return face_branch<DIR>(g, w, dw, h, i, j, k) != b0 ||
         face_branch<DIR>(g, w, dw, -h, i, j, k) != b0;
}

__global__ void __launch_bounds__(128) kink_mask_kernel(Grid g, Fields w, Fields dw, double h,
                                                        unsigned char* __restrict__ mask) {
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < g.ncell;
       c += (long)gridDim.x * blockDim.x) {
    long i, j, k;
    split3(c, g.n[0], g.n[1], i, j, k);
    bool m = face_kinked<0>(g, w, dw, h, i, j, k) || face_kinked<0>(g, w, dw, h, i + 1, j, k) ||
             face_kinked<1>(g, w, dw, h, i, j, k) || face_kinked<1>(g, w, dw, h, i, j + 1, k) ||
             face_kinked<2>(g, w, dw, h, i, j, k) || face_kinked<2>(g, w, dw, h, i, j, k + 1);
    mask[c] = m ? 1 : 0;
  }
}

}  // namespace

int feuler_kink_mask(const Grid& g, const Fields& w, const Fields& dw, double h,
                     unsigned char* mask, cudaStream_t s) {
  kink_mask_kernel<<<sweep_blocks(g.ncell, 128), 128, 0, s>>>(g, w, dw, h, mask);
  GBMV_LAUNCH_CHECK("kink_mask_kernel");
  return GBMV_OK;
}

}  // namespace gbmv
