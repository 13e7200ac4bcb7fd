// WENO5 flux divergence (part a): the device implementation of fEuler
// (src/utilities.cpp:17-253) with in-kernel ghost synthesis for every boundary type.
//
// FP64 parity form, two passes:
//   1. face_flux_kernel<NCHEM, DIR>: one thread per face normal to DIR (all lower faces plus
//      the upper boundary faces, like the reference's two loops); stencil gathered straight
//      from the SoA fields with ghost synthesis, flux written to a per-direction scratch array
//      F_DIR[v][face] (the xflux/yflux/zflux arrays of EulerData, src/euler3D.hpp:497-499,
//      stored field-major so that the divergence pass reads them coalesced).
//   2. divergence_kernel<NCHEM>: wdot = G - [(Fx+ - Fx-)/dx + (Fy+ - Fy-)/dy + (Fz+ - Fz-)/dz],
//      with the legal-state check (src/euler3D.hpp:1405-1414) OR-ed into a status word.
#include "common.cuh"
#include "weno_fp64.cuh"
#include "weno_mixed.cuh"
#include "weno.cuh"

namespace gbmv {

template <int DIR>
__device__ __forceinline__ void face_coords(long f, const Grid& g, long& i, long& j, long& k) {
  const long ex = g.n[0] + (DIR == 0), ey = g.n[1] + (DIR == 1);
  i = f % ex;
  const long r = f / ex;
  j = r % ey;
  k = r / ey;
}

template <int NCHEM, int DIR>
__global__ void __launch_bounds__(128) face_flux_kernel(Grid g, Fields w, double* __restrict__ F,
                                                        long nfaces) {
  const long nx = g.n[0], ny = g.n[1];
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < nfaces;
       f += (long)gridDim.x * blockDim.x) {
    long i, j, k;
    face_coords<DIR>(f, g, i, j, k);
    const long base[3] = {i, j, k};
    long cell[6];
    bool nall[6], nnorm[6];
#pragma unroll
    for (int l = 0; l < 6; ++l) {
      long p = base[DIR] - 3 + l;
      p = ghost_src(p, g.n[DIR], g.bc[2 * DIR], g.bc[2 * DIR + 1], &nall[l], &nnorm[l]);
      long q[3] = {i, j, k};
      q[DIR] = p;
      cell[l] = q[0] + nx * (q[1] + ny * q[2]);
    }
    double W[6][5];
#pragma unroll
    for (int l = 0; l < 6; ++l) {
      double q[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) q[v] = __ldg(w.f[v] + cell[l]);
      if (nall[l]) {
#pragma unroll
        for (int v = 0; v < 5; ++v) q[v] = -q[v];
      }
      if (nnorm[l]) q[1 + DIR] = -q[1 + DIR];
      // direction swap of src/utilities.cpp:283-285: the normal momentum goes to slot 1
      W[l][0] = q[0];
      W[l][1] = q[1 + DIR];
      W[l][2] = (DIR == 1) ? q[1] : q[2];
      W[l][3] = (DIR == 2) ? q[1] : q[3];
      W[l][4] = q[4];
    }
    FaceState S;
    double out[5];
    fluid_face_flux64(W, g.gamma, S, out);
    // undo the direction swap
    double o1 = out[1], oD = out[1 + DIR];
    out[1] = oD;
    out[1 + DIR] = o1;
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v * nfaces + f] = out[v];
#pragma unroll 1
    for (int c = 0; c < NCHEM; ++c) {
      double cv[6];
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        const double sa = nall[l] ? -1.0 : 1.0;
        cv[l] = sa * __ldg(w.f[5] + c + (long)NCHEM * cell[l]);
      }
      F[(5 + c) * nfaces + f] = tracer_face_flux64(S, cv);
    }
  }
}

template <int NCHEM>
__global__ void __launch_bounds__(256) divergence_kernel(Grid g, Fields w, Fields wdot,
                                                         const double* __restrict__ Fx,
                                                         const double* __restrict__ Fy,
                                                         const double* __restrict__ Fz,
                                                         ForceTerm G, int* __restrict__ status) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const long nfx = (nx + 1) * ny * nz, nfy = nx * (ny + 1) * nz, nfz = nx * ny * (nz + 1);
  int bad = 0;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < g.ncell;
       c += (long)gridDim.x * blockDim.x) {
    const long i = c % nx, r = c / nx, j = r % ny, k = r / ny;
    const long fx = i + (nx + 1) * (j + ny * k);
    const long fy = i + nx * (j + (ny + 1) * k);
    const long fz = c;
    {
      const double rho = w.f[0][c], mx = w.f[1][c], my = w.f[2][c], mz = w.f[3][c],
                   et = w.f[4][c];
      int s = 0;
      if (!(rho > 0.0)) s |= 1;
      if (!(et > 0.0)) s |= 2;
      if (!(eos64(g.gamma, rho, mx, my, mz, et) > 0.0)) s |= 4;
      bad |= s;
    }
#pragma unroll
    for (int v = 0; v < 5 + NCHEM; ++v) {
      const double div = (Fx[v * nfx + fx + 1] - Fx[v * nfx + fx]) / g.d[0] +
                         (Fy[v * nfy + fy + nx] - Fy[v * nfy + fy]) / g.d[1] +
                         (Fz[v * nfz + fz + nx * ny] - Fz[v * nfz + fz]) / g.d[2];
      double* dst = (v < 5) ? (wdot.f[v] + c) : (wdot.f[5] + (v - 5) + (long)NCHEM * c);
      const double base = G.in_wdot ? *dst : G.c[v];
      *dst = base - div;
    }
  }
  // warp-aggregated status
  bad = __reduce_or_sync(0xffffffffu, bad);
  if (bad && (threadIdx.x & 31) == 0) atomicOr(status, bad);
}

template <int NCHEM>
static int launch_fp64(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                       double* scratch, int* d_status, cudaStream_t s) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const long nf[3] = {(nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1)};
  double* F[3] = {scratch, scratch + (long)(5 + NCHEM) * nf[0],
                  scratch + (long)(5 + NCHEM) * (nf[0] + nf[1])};
  auto blocks = [](long n, int t) {
    long b = (n + t - 1) / t;
    const long cap = (long)kSM * 16;
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
  };
  {
  ProfScope ps("face_flux", s);
  face_flux_kernel<NCHEM, 0><<<blocks(nf[0], 128), 128, 0, s>>>(g, w, F[0], nf[0]);
  GBMV_LAUNCH_CHECK("face_flux_kernel<x>");
  }
  {
  ProfScope ps("face_flux", s);
  face_flux_kernel<NCHEM, 1><<<blocks(nf[1], 128), 128, 0, s>>>(g, w, F[1], nf[1]);
  GBMV_LAUNCH_CHECK("face_flux_kernel<y>");
  }
  {
  ProfScope ps("face_flux", s);
  face_flux_kernel<NCHEM, 2><<<blocks(nf[2], 128), 128, 0, s>>>(g, w, F[2], nf[2]);
  GBMV_LAUNCH_CHECK("face_flux_kernel<z>");
  }
  ProfScope ps("divergence", s);
  divergence_kernel<NCHEM><<<blocks(g.ncell, 256), 256, 0, s>>>(g, w, wdot, F[0], F[1], F[2], G,
                                                                d_status);
  GBMV_LAUNCH_CHECK("divergence_kernel");
  return GBMV_OK;
}

size_t feuler_fp64_scratch_doubles(const Grid& g) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2];
  return (size_t)(5 + g.nchem) *
         (size_t)((nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1));
}

int feuler_fp64(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                double* scratch, int* d_status, cudaStream_t s) {
  switch (g.nchem) {
    case 0: return launch_fp64<0>(g, w, wdot, G, scratch, d_status, s);
    case 2: return launch_fp64<2>(g, w, wdot, G, scratch, d_status, s);
    case 4: return launch_fp64<4>(g, w, wdot, G, scratch, d_status, s);
    case 6: return launch_fp64<6>(g, w, wdot, G, scratch, d_status, s);
    case 10: return launch_fp64<10>(g, w, wdot, G, scratch, d_status, s);
    default: set_error("nchem=%d not compiled (0,2,4,6,10)", g.nchem); return GBMV_EUNSUPPORTED;
  }
}

// ------------------------------------------------------------------ mixed-precision form
//
//   prims32_kernel: FP64 state -> FP32 copies (rho, mx, my, mz, et and the FP64-computed
//     pressure, SoA; tracers SoA) + the legal-state check;
//   face_flux_mx_kernel<NCHEM, DIR, WT>: as face_flux_kernel, FP32 arithmetic with WT weights,
//     fluxes stored as FP32;
//   divergence_mx_kernel<NCHEM>: FP64 differences and sums of the FP32 face fluxes.

__global__ void __launch_bounds__(256) prims32_kernel(Grid g, Fields w, float* __restrict__ Q,
                                                      int* __restrict__ status) {
  const long n = g.ncell;
  int bad = 0;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
       c += (long)gridDim.x * blockDim.x) {
    const double rho = w.f[0][c], mx = w.f[1][c], my = w.f[2][c], mz = w.f[3][c], et = w.f[4][c];
    const double p = eos64(g.gamma, rho, mx, my, mz, et);
    int st = 0;
    if (!(rho > 0.0)) st |= 1;
    if (!(et > 0.0)) st |= 2;
    if (!(p > 0.0)) st |= 4;
    bad |= st;
    Q[0 * n + c] = (float)rho;
    Q[1 * n + c] = (float)mx;
    Q[2 * n + c] = (float)my;
    Q[3 * n + c] = (float)mz;
    Q[4 * n + c] = (float)et;
    Q[5 * n + c] = (float)p;
    for (int v = 0; v < g.nchem; ++v) Q[(6 + v) * n + c] = (float)w.f[5][v + (long)g.nchem * c];
  }
  bad = __reduce_or_sync(0xffffffffu, bad);
  if (bad && (threadIdx.x & 31) == 0) atomicOr(status, bad);
}

template <int NCHEM, int DIR, typename WT>
__global__ void __launch_bounds__(128) face_flux_mx_kernel(Grid g, const float* __restrict__ Q,
                                                           float* __restrict__ F, long nfaces) {
  const long nx = g.n[0], ny = g.n[1], n = g.ncell;
  const float gamma = (float)g.gamma;
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < nfaces;
       f += (long)gridDim.x * blockDim.x) {
    long i, j, k;
    face_coords<DIR>(f, g, i, j, k);
    const long base[3] = {i, j, k};
    long cell[6];
    bool nall[6], nnorm[6];
#pragma unroll
    for (int l = 0; l < 6; ++l) {
      long p = base[DIR] - 3 + l;
      p = ghost_src(p, g.n[DIR], g.bc[2 * DIR], g.bc[2 * DIR + 1], &nall[l], &nnorm[l]);
      long q[3] = {i, j, k};
      q[DIR] = p;
      cell[l] = q[0] + nx * (q[1] + ny * q[2]);
    }
    float W[6][5], P[6];
#pragma unroll
    for (int l = 0; l < 6; ++l) {
      float q[6];
#pragma unroll
      for (int v = 0; v < 6; ++v) q[v] = __ldg(Q + v * n + cell[l]);
      if (nall[l]) {
#pragma unroll
        for (int v = 0; v < 6; ++v) q[v] = -q[v];  // homogeneous Dirichlet: p(-w) = -p(w)
      }
      if (nnorm[l]) q[1 + DIR] = -q[1 + DIR];
      W[l][0] = q[0];
      W[l][1] = q[1 + DIR];
      W[l][2] = (DIR == 1) ? q[1] : q[2];
      W[l][3] = (DIR == 2) ? q[1] : q[3];
      W[l][4] = q[4];
      P[l] = q[5];
    }
    FaceState32 S;
    float out[5];
    fluid_face_flux_mx<WT>(W, P, gamma, S, out);
    const float o1 = out[1], oD = out[1 + DIR];
    out[1] = oD;
    out[1 + DIR] = o1;
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v * nfaces + f] = out[v];
#pragma unroll 1
    for (int c = 0; c < NCHEM; ++c) {
      float cv[6];
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        const float x = __ldg(Q + (6 + c) * n + cell[l]);
        cv[l] = nall[l] ? -x : x;
      }
      F[(5 + c) * nfaces + f] = tracer_face_flux_mx<WT>(S, cv);
    }
  }
}

template <int NCHEM>
__global__ void __launch_bounds__(256) divergence_mx_kernel(Grid g, Fields wdot,
                                                            const float* __restrict__ Fx,
                                                            const float* __restrict__ Fy,
                                                            const float* __restrict__ Fz,
                                                            ForceTerm G) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const long nfx = (nx + 1) * ny * nz, nfy = nx * (ny + 1) * nz, nfz = nx * ny * (nz + 1);
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < g.ncell;
       c += (long)gridDim.x * blockDim.x) {
    const long i = c % nx, r = c / nx, j = r % ny, k = r / ny;
    const long fx = i + (nx + 1) * (j + ny * k);
    const long fy = i + nx * (j + (ny + 1) * k);
    const long fz = c;
#pragma unroll
    for (int v = 0; v < 5 + NCHEM; ++v) {
      const double dx = (double)Fx[v * nfx + fx + 1] - (double)Fx[v * nfx + fx];
      const double dy = (double)Fy[v * nfy + fy + nx] - (double)Fy[v * nfy + fy];
      const double dz = (double)Fz[v * nfz + fz + nx * ny] - (double)Fz[v * nfz + fz];
      const double div = dx / g.d[0] + dy / g.d[1] + dz / g.d[2];
      double* dst = (v < 5) ? (wdot.f[v] + c) : (wdot.f[5] + (v - 5) + (long)NCHEM * c);
      const double base = G.in_wdot ? *dst : G.c[v];
      *dst = base - div;
    }
  }
}

template <int NCHEM, typename WT>
static int launch_mixed(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                        float* scratch, int* d_status, cudaStream_t s) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2], n = g.ncell;
  const long nf[3] = {(nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1)};
  float* Q = scratch;
  float* F[3] = {Q + (6 + NCHEM) * n, Q + (6 + NCHEM) * n + (long)(5 + NCHEM) * nf[0],
                 Q + (6 + NCHEM) * n + (long)(5 + NCHEM) * (nf[0] + nf[1])};
  auto blocks = [](long m, int t) {
    long b = (m + t - 1) / t;
    const long cap = (long)kSM * 16;
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
  };
  {
    ProfScope ps("prims", s);
    prims32_kernel<<<blocks(n, 256), 256, 0, s>>>(g, w, Q, d_status);
    GBMV_LAUNCH_CHECK("prims32_kernel");
  }
  {
    ProfScope ps("face_flux", s);
    face_flux_mx_kernel<NCHEM, 0, WT><<<blocks(nf[0], 128), 128, 0, s>>>(g, Q, F[0], nf[0]);
    GBMV_LAUNCH_CHECK("face_flux_mx_kernel<x>");
  }
  {
    ProfScope ps("face_flux", s);
    face_flux_mx_kernel<NCHEM, 1, WT><<<blocks(nf[1], 128), 128, 0, s>>>(g, Q, F[1], nf[1]);
    GBMV_LAUNCH_CHECK("face_flux_mx_kernel<y>");
  }
  {
    ProfScope ps("face_flux", s);
    face_flux_mx_kernel<NCHEM, 2, WT><<<blocks(nf[2], 128), 128, 0, s>>>(g, Q, F[2], nf[2]);
    GBMV_LAUNCH_CHECK("face_flux_mx_kernel<z>");
  }
  ProfScope ps("divergence", s);
  divergence_mx_kernel<NCHEM><<<blocks(n, 256), 256, 0, s>>>(g, wdot, F[0], F[1], F[2], G);
  GBMV_LAUNCH_CHECK("divergence_mx_kernel");
  return GBMV_OK;
}

size_t feuler_mixed_scratch_floats(const Grid& g) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2];
  return (size_t)(6 + g.nchem) * g.ncell +
         (size_t)(5 + g.nchem) *
             (size_t)((nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1));
}

template <typename WT>
static int feuler_mixed_t(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                          float* scratch, int* d_status, cudaStream_t s) {
  switch (g.nchem) {
    case 0: return launch_mixed<0, WT>(g, w, wdot, G, scratch, d_status, s);
    case 2: return launch_mixed<2, WT>(g, w, wdot, G, scratch, d_status, s);
    case 4: return launch_mixed<4, WT>(g, w, wdot, G, scratch, d_status, s);
    case 6: return launch_mixed<6, WT>(g, w, wdot, G, scratch, d_status, s);
    case 10: return launch_mixed<10, WT>(g, w, wdot, G, scratch, d_status, s);
    default: set_error("nchem=%d not compiled (0,2,4,6,10)", g.nchem); return GBMV_EUNSUPPORTED;
  }
}

int feuler_mixed(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                 float* scratch, int* d_status, int fp64_weights, cudaStream_t s) {
  return fp64_weights ? feuler_mixed_t<double>(g, w, wdot, G, scratch, d_status, s)
                      : feuler_mixed_t<f2>(g, w, wdot, G, scratch, d_status, s);
}

}  // namespace gbmv
