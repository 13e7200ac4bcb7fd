// WENO5 flux divergence (part a): the device implementation of fEuler
// (src/utilities.cpp:17-253) with in-kernel ghost synthesis for every boundary type.
//
// Two passes (T = double: the FP64 parity form; T = f2: the float-float mixed form):
//   1. face_flux_kernel<NCHEM, DIR>: one thread per face normal to DIR (all lower faces plus
//      the upper boundary faces, like the reference's two loops); stencil gathered straight
//      from the SoA fields with ghost synthesis, flux written to a per-direction scratch array
//      F_DIR[v][face] (the xflux/yflux/zflux arrays of EulerData, src/euler3D.hpp:497-499,
//      stored field-major so that the divergence pass reads them coalesced).
//   2. divergence_kernel<NCHEM>: wdot = G - [(Fx+ - Fx-)/dx + (Fy+ - Fy-)/dy + (Fz+ - Fz-)/dz],
//      with the legal-state check (src/euler3D.hpp:1405-1414) OR-ed into a status word.
#include <type_traits>

#include "common.cuh"
#include "weno_face.cuh"
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

template <int NCHEM, int DIR, typename T>
__global__ void __launch_bounds__(128) face_flux_kernel(Grid g, Fields w, double* __restrict__ F,
                                                        long nfaces) {
  const long nx = g.n[0], ny = g.n[1];
  T* tag = nullptr;
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
    double Wd[6][5];
    double wmax = 0.0;
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
      Wd[l][0] = q[0];
      Wd[l][1] = q[1 + DIR];
      Wd[l][2] = (DIR == 1) ? q[1] : q[2];
      Wd[l][3] = (DIR == 2) ? q[1] : q[3];
      Wd[l][4] = q[4];
#pragma unroll
      for (int v = 0; v < 5; ++v) wmax = fmax(wmax, fabs(q[v]));
    }
    FaceState<T> S;
    double out[5];
    if (std::is_same<T, double>::value || !(wmax < 1e15)) {
      // FP64 form, or a state outside the float-float range: native FP64
      FaceState<double> S64;
      fluid_face_flux<double>(Wd, g.gamma, S64, out);
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        S.hp[l] = num_from(S64.hp[l], tag);
        S.hm[l] = num_from(S64.hm[l], tag);
      }
    } else {
      T W[6][5], o[5];
#pragma unroll
      for (int l = 0; l < 6; ++l)
#pragma unroll
        for (int v = 0; v < 5; ++v) W[l][v] = num_from(Wd[l][v], tag);
      fluid_face_flux<T>(W, g.gamma, S, o);
#pragma unroll
      for (int v = 0; v < 5; ++v) out[v] = num_to_double(o[v]);
    }
    // undo the direction swap
    double o1 = out[1], oD = out[1 + DIR];
    out[1] = oD;
    out[1 + DIR] = o1;
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v * nfaces + f] = out[v];
#pragma unroll 1
    for (int c = 0; c < NCHEM; ++c) {
      T cv[6];
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        const double x = __ldg(w.f[5] + c + (long)NCHEM * cell[l]);
        cv[l] = num_from(nall[l] ? -x : x, tag);
      }
      F[(5 + c) * nfaces + f] = num_to_double(tracer_face_flux<T>(S, cv));
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
      // (F+ - F-) / d as a multiply by 1/d: the reference divides; the difference is one
      // rounding, and 45 FP64 divisions per cell would cost more than the rest of this pass
      const double div = (Fx[v * nfx + fx + 1] - Fx[v * nfx + fx]) * g.inv_d[0] +
                         (Fy[v * nfy + fy + nx] - Fy[v * nfy + fy]) * g.inv_d[1] +
                         (Fz[v * nfz + fz + nx * ny] - Fz[v * nfz + fz]) * g.inv_d[2];
      double* dst = (v < 5) ? (wdot.f[v] + c) : (wdot.f[5] + (v - 5) + (long)NCHEM * c);
      const double base = G.in_wdot ? *dst : G.c[v];
      *dst = base - div;
    }
  }
  // warp-aggregated status
  bad = __reduce_or_sync(0xffffffffu, bad);
  if (bad && (threadIdx.x & 31) == 0) atomicOr(status, bad);
}

template <int NCHEM, typename T>
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
  face_flux_kernel<NCHEM, 0, T><<<blocks(nf[0], 128), 128, 0, s>>>(g, w, F[0], nf[0]);
  GBMV_LAUNCH_CHECK("face_flux_kernel<x>");
  }
  {
  ProfScope ps("face_flux", s);
  face_flux_kernel<NCHEM, 1, T><<<blocks(nf[1], 128), 128, 0, s>>>(g, w, F[1], nf[1]);
  GBMV_LAUNCH_CHECK("face_flux_kernel<y>");
  }
  {
  ProfScope ps("face_flux", s);
  face_flux_kernel<NCHEM, 2, T><<<blocks(nf[2], 128), 128, 0, s>>>(g, w, F[2], nf[2]);
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

template <typename T>
static int feuler_t(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                    double* scratch, int* d_status, cudaStream_t s) {
  switch (g.nchem) {
    case 0: return launch_fp64<0, T>(g, w, wdot, G, scratch, d_status, s);
    case 2: return launch_fp64<2, T>(g, w, wdot, G, scratch, d_status, s);
    case 4: return launch_fp64<4, T>(g, w, wdot, G, scratch, d_status, s);
    case 6: return launch_fp64<6, T>(g, w, wdot, G, scratch, d_status, s);
    case 10: return launch_fp64<10, T>(g, w, wdot, G, scratch, d_status, s);
    default: set_error("nchem=%d not compiled (0,2,4,6,10)", g.nchem); return GBMV_EUNSUPPORTED;
  }
}

int feuler_fp64(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                double* scratch, int* d_status, cudaStream_t s) {
  return feuler_t<double>(g, w, wdot, G, scratch, d_status, s);
}

int feuler_mixed(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                 double* scratch, int* d_status, cudaStream_t s) {
  return feuler_t<f2>(g, w, wdot, G, scratch, d_status, s);
}

// ------------------------------------------------------------------ float-float (mixed) form
//
//   prims_f2_kernel: once per cell, in FP64 exactly as the reference evaluates them per
//     stencil point -- pressure (eos), the three velocities m/rho and the sound speed
//     sqrt(gamma p / rho) -- then every field and primitive split into float pairs (hi, lo):
//     Q2[q][cell], q = rho, mx, my, mz, et, p, ux, uy, uz, c, tracers...;
//   face_flux_f2_kernel<NCHEM, DIR>: the face flux in float-float arithmetic from Q2 (no FP64
//     instruction on the common path); faces whose states leave the float range, or touch a
//     non-positive density (homogeneous Dirichlet ghosts), are computed in FP64 from w;
//   divergence_kernel: unchanged, FP64.

constexpr int kQ2Base = 10;  // index of the first tracer in Q2

__global__ void __launch_bounds__(256) prims_f2_kernel(Grid g, Fields w, float2* __restrict__ Q2,
                                                       const double* __restrict__ tscale) {
  const long n = g.ncell;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
       c += (long)gridDim.x * blockDim.x) {
    const double rho = w.f[0][c], mx = w.f[1][c], my = w.f[2][c], mz = w.f[3][c], et = w.f[4][c];
    const double p = eos64(g.gamma, rho, mx, my, mz, et);
    double q[kQ2Base] = {rho, mx, my, mz, et, p, mx / rho, my / rho, mz / rho,
                         sqrt0(g.gamma * p / rho)};
#pragma unroll
    for (int k = 0; k < kQ2Base; ++k) {
      const f2 v = f2_from_double(q[k]);
      Q2[k * n + c] = make_float2(v.hi, v.lo);
    }
    for (int v = 0; v < g.nchem; ++v) {
      // tscale: the chemistry component arrives in scaled units (x = chem * scale)
      const long e = v + (long)g.nchem * c;
      const f2 x = f2_from_double(tscale ? w.f[5][e] * tscale[e] : w.f[5][e]);
      Q2[(kQ2Base + v) * n + c] = make_float2(x.hi, x.lo);
    }
  }
}

// WV = 1 (fewer instructions per face) runs faster at 3 resident blocks per SM even with the
// register cap's spills (measured 6.11 -> 5.63 ms per 128^3 RHS); WV = 0 is faster at 2.
template <int NCHEM, int DIR, int WV>
__global__ void __launch_bounds__(128, WV == 1 ? 3 : 1) face_flux_f2_kernel(Grid g, Fields w,
                                                           const float2* __restrict__ Q2,
                                                           double* __restrict__ F, long nfaces) {
  const long nx = g.n[0], ny = g.n[1], n = g.ncell;
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
    f2 W[6][5];
    PointPrims<f2> pre;
    bool ok = true;
#pragma unroll
    for (int l = 0; l < 6; ++l) {
      // slots: rho, m_normal, m_t1, m_t2, et, p, u_normal, c
      const int src[8] = {0, 1 + DIR, DIR == 1 ? 1 : 2, DIR == 2 ? 1 : 3, 4, 5, 6 + DIR, 9};
      f2 q[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const float2 t = __ldg(Q2 + src[m] * n + cell[l]);
        q[m] = f2(t.x, t.y);
      }
      // homogeneous Dirichlet negates every conserved field (so p too; u and c unchanged);
      // reflecting negates the normal momentum (so the normal velocity)
      if (nall[l]) {
#pragma unroll
        for (int m = 0; m < 6; ++m) q[m] = -q[m];
      }
      if (nnorm[l]) {
        q[1] = -q[1];
        q[6] = -q[6];
      }
#pragma unroll
      for (int m = 0; m < 5; ++m) W[l][m] = q[m];
      pre.p[l] = q[5];
      pre.u[l] = q[6];
      pre.c[l] = q[7];
      ok = ok && (q[0].hi > 0.f);
#pragma unroll
      for (int m = 0; m < 6; ++m) ok = ok && (fabsf(q[m].hi) < 1e15f);
    }
    FaceState<f2> S;
    double out[5];
    if (ok) {
      f2 o[5];
      // characteristic fields keep float-float weights in every mixed form: the reference's
      // eigenbasis (conditioning ~1/c^2) amplifies weight rounding in the back-projection
      fluid_face_flux<f2, true, 0>(W, g.gamma, S, o, &pre);
#pragma unroll
      for (int v = 0; v < 5; ++v) out[v] = o[v].to_double();
    } else {  // FP64, exactly the FP64 form's arithmetic
      double Wd[6][5];
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
        Wd[l][0] = q[0];
        Wd[l][1] = q[1 + DIR];
        Wd[l][2] = (DIR == 1) ? q[1] : q[2];
        Wd[l][3] = (DIR == 2) ? q[1] : q[3];
        Wd[l][4] = q[4];
      }
      FaceState<double> S64;
      fluid_face_flux<double>(Wd, g.gamma, S64, out);
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        S.hp[l] = f2_from_double(S64.hp[l]);
        S.hm[l] = f2_from_double(S64.hm[l]);
      }
    }
    const double o1 = out[1], oD = out[1 + DIR];
    out[1] = oD;
    out[1 + DIR] = o1;
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v * nfaces + f] = out[v];
#pragma unroll 1
    for (int c = 0; c < NCHEM; ++c) {
      f2 cv[6];
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        const float2 t = __ldg(Q2 + (kQ2Base + c) * n + cell[l]);
        cv[l] = nall[l] ? f2(-t.x, -t.y) : f2(t.x, t.y);
      }
      F[(5 + c) * nfaces + f] = tracer_face_flux<f2, WV>(S, cv).to_double();
    }
  }
}

template <int NCHEM, int WV>
static int launch_f2(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                     double* scratch, float2* q2, const double* tscale, int* d_status,
                     cudaStream_t s) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const long nf[3] = {(nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1)};
  double* F[3] = {scratch, scratch + (long)(5 + NCHEM) * nf[0],
                  scratch + (long)(5 + NCHEM) * (nf[0] + nf[1])};
  auto blocks = [](long m, int t) {
    long b = (m + t - 1) / t;
    const long cap = (long)kSM * 16;
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
  };
  {
    ProfScope ps("prims", s);
    prims_f2_kernel<<<blocks(g.ncell, 256), 256, 0, s>>>(g, w, q2, tscale);
    GBMV_LAUNCH_CHECK("prims_f2_kernel");
  }
  {
    ProfScope ps("face_flux", s);
    face_flux_f2_kernel<NCHEM, 0, WV><<<blocks(nf[0], 128), 128, 0, s>>>(g, w, q2, F[0], nf[0]);
    GBMV_LAUNCH_CHECK("face_flux_f2_kernel<x>");
  }
  {
    ProfScope ps("face_flux", s);
    face_flux_f2_kernel<NCHEM, 1, WV><<<blocks(nf[1], 128), 128, 0, s>>>(g, w, q2, F[1], nf[1]);
    GBMV_LAUNCH_CHECK("face_flux_f2_kernel<y>");
  }
  {
    ProfScope ps("face_flux", s);
    face_flux_f2_kernel<NCHEM, 2, WV><<<blocks(nf[2], 128), 128, 0, s>>>(g, w, q2, F[2], nf[2]);
    GBMV_LAUNCH_CHECK("face_flux_f2_kernel<z>");
  }
  ProfScope ps("divergence", s);
  divergence_kernel<NCHEM><<<blocks(g.ncell, 256), 256, 0, s>>>(g, w, wdot, F[0], F[1], F[2], G,
                                                                d_status);
  GBMV_LAUNCH_CHECK("divergence_kernel");
  return GBMV_OK;
}

size_t feuler_f2_prims_floats(const Grid& g) { return (size_t)2 * (kQ2Base + g.nchem) * g.ncell; }

template <int WV>
static int feuler_f2_wv(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                        double* scratch, float2* q2, const double* tscale, int* d_status,
                        cudaStream_t s) {
  switch (g.nchem) {
    case 0: return launch_f2<0, WV>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 2: return launch_f2<2, WV>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 4: return launch_f2<4, WV>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 6: return launch_f2<6, WV>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 10: return launch_f2<10, WV>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    default: set_error("nchem=%d not compiled (0,2,4,6,10)", g.nchem); return GBMV_EUNSUPPORTED;
  }
}

int feuler_f2(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
              double* scratch, float* prims, const double* tscale, int* d_status,
              cudaStream_t s, int fast_weights) {
  float2* q2 = reinterpret_cast<float2*>(prims);
  if (fast_weights) return feuler_f2_wv<1>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
  switch (g.nchem) {
    case 0: return launch_f2<0, 0>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 2: return launch_f2<2, 0>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 4: return launch_f2<4, 0>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 6: return launch_f2<6, 0>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 10: return launch_f2<10, 0>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    default: set_error("nchem=%d not compiled (0,2,4,6,10)", g.nchem); return GBMV_EUNSUPPORTED;
  }
}

// ------------------------------------------------------------------ CFL-stable step (stability)
//
// stability (src/utilities.cpp:483-528): alpha = max over cells of |mx/rho| + sqrt(gamma p/rho)
// -- the reference takes |mx/rho| for all three directions -- and
// dt = cfl * min(dx, dy, dz) / alpha.  Non-negative doubles order like their bit patterns, so
// the grid maximum is an atomicMax on the 64-bit integer view; NaN cells are skipped, as the
// reference's std::max(alpha, NaN) keeps alpha.

__global__ void __launch_bounds__(256) wave_speed_max_kernel(Grid g, Fields w,
                                                            unsigned long long* __restrict__ out) {
  double m = 0.0;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < g.ncell;
       c += (long)gridDim.x * blockDim.x) {
    const double rho = w.f[0][c], mx = w.f[1][c];
    const double u = fabs(mx / rho);
    const double p = eos64(g.gamma, rho, mx, w.f[2][c], w.f[3][c], w.f[4][c]);
    const double cs = sqrt0(g.gamma * p / rho);
    const double a = fabs(u + cs);
    m = (m < a) ? a : m;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const double o = __shfl_xor_sync(0xffffffffu, m, off);
    m = (m < o) ? o : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// pack1D_x/y/z and their _bdry variants (src/euler3D.hpp:1197-1378): for every face normal to
// DIR (all (n+1) per row, as the flux loops), the six-point stencil w1d[l][v] the face flux
// reads, ghost rules applied, fields in the ManyVector order (rho, mx, my, mz, et, species),
// written to out[(l * NVAR + v) * nfaces + f].
template <int DIR>
__global__ void __launch_bounds__(128) pack1d_kernel(Grid g, Fields w, double* __restrict__ out,
                                                     long nfaces) {
  const long nx = g.n[0], ny = g.n[1];
  const int nv = 5 + g.nchem;
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < nfaces;
       f += (long)gridDim.x * blockDim.x) {
    long i, j, k;
    face_coords<DIR>(f, g, i, j, k);
    const long base[3] = {i, j, k};
    for (int l = 0; l < 6; ++l) {
      bool nall, nnorm;
      long q[3] = {i, j, k};
      q[DIR] = ghost_src(base[DIR] - 3 + l, g.n[DIR], g.bc[2 * DIR], g.bc[2 * DIR + 1], &nall,
                         &nnorm);
      const long c = q[0] + nx * (q[1] + ny * q[2]);
      for (int v = 0; v < nv; ++v) {
        double x = (v < 5) ? w.f[v][c] : w.f[5][(v - 5) + (long)g.nchem * c];
        if (nall || (nnorm && v == 1 + DIR)) x = -x;
        out[((long)l * nv + v) * nfaces + f] = x;
      }
    }
  }
}

int pack1d(const Grid& g, const Fields& w, int dir, double* out, cudaStream_t s) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const long nf[3] = {(nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1)};
  long b = (nf[dir] + 127) / 128;
  if (b > (long)kSM * 16) b = (long)kSM * 16;
  if (dir == 0) pack1d_kernel<0><<<(int)b, 128, 0, s>>>(g, w, out, nf[0]);
  else if (dir == 1) pack1d_kernel<1><<<(int)b, 128, 0, s>>>(g, w, out, nf[1]);
  else pack1d_kernel<2><<<(int)b, 128, 0, s>>>(g, w, out, nf[2]);
  GBMV_LAUNCH_CHECK("pack1d_kernel");
  return GBMV_OK;
}

// check_conservation (src/io.cpp:503-542): grid totals of rho and et.  Deterministic two-pass
// reduction (fixed grid, per-block partial sums, then one block in a fixed order), FP64 with a
// compensated (two-sum) accumulation per thread.
constexpr int kConsBlocks = 1024;

__device__ __forceinline__ void two_sum_acc(double& s, double& c, double x) {
  const double t = s + x;
  const double bp = t - s;
  c += (s - (t - bp)) + (x - bp);
  s = t;
}

__global__ void __launch_bounds__(256) conservation_partial_kernel(long n, const double* rho,
                                                                   const double* et,
                                                                   double* __restrict__ part) {
  double s0 = 0.0, c0 = 0.0, s1 = 0.0, c1 = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    two_sum_acc(s0, c0, rho[i]);
    two_sum_acc(s1, c1, et[i]);
  }
  double a = s0 + c0, b = s1 + c1;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, off);
    b += __shfl_down_sync(0xffffffffu, b, off);
  }
  __shared__ double wa[8], wb[8];
  if ((threadIdx.x & 31) == 0) {
    wa[threadIdx.x >> 5] = a;
    wb[threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      ta += wa[k];
      tb += wb[k];
    }
    part[blockIdx.x] = ta;
    part[kConsBlocks + blockIdx.x] = tb;
  }
}

__global__ void conservation_final_kernel(const double* __restrict__ part, double* __restrict__ out) {
  if (threadIdx.x == 0) {
    double s0 = 0.0, c0 = 0.0, s1 = 0.0, c1 = 0.0;
    for (int k = 0; k < kConsBlocks; ++k) {
      two_sum_acc(s0, c0, part[k]);
      two_sum_acc(s1, c1, part[kConsBlocks + k]);
    }
    out[0] = s0 + c0;
    out[1] = s1 + c1;
  }
}

int conservation_sums(const Grid& g, const Fields& w, double* d_scratch, cudaStream_t s) {
  conservation_partial_kernel<<<kConsBlocks, 256, 0, s>>>(g.ncell, w.f[0], w.f[4], d_scratch);
  GBMV_LAUNCH_CHECK("conservation_partial_kernel");
  conservation_final_kernel<<<1, 32, 0, s>>>(d_scratch, d_scratch + 2 * kConsBlocks);
  GBMV_LAUNCH_CHECK("conservation_final_kernel");
  return GBMV_OK;
}

size_t conservation_scratch_doubles() { return 2 * kConsBlocks + 2; }

int wave_speed_max(const Grid& g, const Fields& w, unsigned long long* d_out, cudaStream_t s) {
  long b = (g.ncell + 255) / 256;
  if (b > (long)kSM * 8) b = (long)kSM * 8;
  if (b < 1) b = 1;
  GBMV_CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(unsigned long long), s));
  wave_speed_max_kernel<<<(int)b, 256, 0, s>>>(g, w, d_out);
  GBMV_LAUNCH_CHECK("wave_speed_max_kernel");
  return GBMV_OK;
}

}  // namespace gbmv
