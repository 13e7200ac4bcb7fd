// Face indexing and stencil gather shared by every face-sweep kernel (the FP64 and float-float
// face fluxes, pack1D, the JVP and VJP sweeps).
//
// A sweep normal to DIR visits every face of the (n_DIR + 1) per row, the lower faces of all
// cells plus the upper boundary faces, as the reference's interior and boundary flux loops do
// together (src/utilities.cpp:17-253).  Face f has coordinates (i, j, k) in the face grid of
// extents n + e_DIR; its stencil points sit at positions i_DIR - 3 .. i_DIR + 2 along DIR and
// take their values through the ghost rule of common.cuh (ghost_src).
#pragma once

#include "common.cuh"
#include "weno.cuh"

namespace gbmv {

// (i, j, k) of the linear index c = i + ex (j + ey k): 32-bit unsigned division while c fits
// (a 64-bit division is a long emulated sequence, comparable to the rest of a cheap pass)
__device__ __forceinline__ void split3(long c, long ex, long ey, long& i, long& j, long& k) {
  if ((unsigned long)c <= 0xffffffffUL) {
    const unsigned u = (unsigned)c, ux = (unsigned)ex, uy = (unsigned)ey;
    const unsigned r = u / ux, q = r / uy;
    i = (long)(u - r * ux);
    j = (long)(r - q * uy);
    k = (long)q;
  } else {
    const long r = c / ex, q = r / ey;
    i = c - r * ex;
    j = r - q * ey;
    k = q;
  }
}

template <int DIR>
__device__ __forceinline__ void face_coords(long f, const Grid& g, long& i, long& j, long& k) {
  split3(f, g.n[0] + (DIR == 0), g.n[1] + (DIR == 1), i, j, k);
}

// cells and ghost signs of the six stencil points of face f
template <int DIR>
__device__ __forceinline__ void stencil(const Grid& g, long f, long (&cell)[6], bool (&nall)[6],
                                        bool (&nnorm)[6], long (&ijk)[3]) {
  long i, j, k;
  face_coords<DIR>(f, g, i, j, k);
  ijk[0] = i;
  ijk[1] = j;
  ijk[2] = k;
#pragma unroll
  for (int l = 0; l < 6; ++l) {
    long q[3] = {i, j, k};
    q[DIR] = ghost_src(q[DIR] - 3 + l, g.n[DIR], g.bc[2 * DIR], g.bc[2 * DIR + 1], &nall[l],
                       &nnorm[l]);
    cell[l] = q[0] + g.n[0] * (q[1] + g.n[1] * q[2]);
  }
}

// the five fluid values of a stencil point in face order (normal momentum in slot 1, the
// direction swap of src/utilities.cpp:283-285), ghost signs applied
template <int DIR>
__device__ __forceinline__ void load_point(const Fields& w, long c, bool nall, bool nnorm,
                                           double (&W)[5]) {
  double q[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) q[v] = __ldg(w.f[v] + c);
  if (nall) {
#pragma unroll
    for (int v = 0; v < 5; ++v) q[v] = -q[v];
  }
  if (nnorm) q[1 + DIR] = -q[1 + DIR];
  W[0] = q[0];
  W[1] = q[1 + DIR];
  W[2] = (DIR == 1) ? q[1] : q[2];
  W[3] = (DIR == 2) ? q[1] : q[3];
  W[4] = q[4];
}

// grid-stride launch size: ceil(n / t) blocks, at least 1, at most 16 per SM
inline int sweep_blocks(long n, int t) {
  long b = (n + t - 1) / t;
  const long cap = (long)kSM * 16;
  return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

// Threads per block of a one-item-per-thread pass over n items whose kernel allows up to
// tmax: the largest of tmax, tmax/2, ..., 32 that still gives every SM two blocks, so that a
// small grid (the Sod tube's ~1200 faces) spreads over as many SMs as it can fill instead of
// queueing its FP64 work on a few of them; large grids keep tmax.  Each item is computed by
// one thread independently, so the results do not depend on the choice.
inline int spread_threads(long n, int tmax) {
  int t = tmax;
  while (t > 32 && n < 2L * kSM * t) t /= 2;
  return t;
}

// the face sweeps' threads per block: the tuned value, else by size
inline int sweep_threads(const Grid& g, long n, int tmax) {
  return g.sweep_threads > 0 && g.sweep_threads <= tmax ? g.sweep_threads
                                                        : spread_threads(n, tmax);
}

// faces normal to x, y, z
inline void face_counts(const Grid& g, long (&nf)[3]) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2];
  nf[0] = (nx + 1) * ny * nz;
  nf[1] = nx * (ny + 1) * nz;
  nf[2] = nx * ny * (nz + 1);
}

}  // namespace gbmv
