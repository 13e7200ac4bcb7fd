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
// The float-float forms (weno_f2*.cu) use divergence_f2_kernel below as their pass 2.  Also
// here: the CFL wave speed, the pack1D stencil gather and the conservation totals.
#include "common.cuh"
#include "weno_face.cuh"
#include "weno_sweep.cuh"
#include "weno.cuh"

namespace gbmv {

template <int NCHEM, int DIR>
__global__ void __launch_bounds__(128) face_flux_kernel(Grid g, Fields w, double* __restrict__ F,
                                                        long nfaces) {
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < nfaces;
       f += (long)gridDim.x * blockDim.x) {
    long cell[6], ijk[3];
    bool nall[6], nnorm[6];
    stencil<DIR>(g, f, cell, nall, nnorm, ijk);
    double Wd[6][5];
#pragma unroll
    for (int l = 0; l < 6; ++l) load_point<DIR>(w, cell[l], nall[l], nnorm[l], Wd[l]);
    FaceState<double> S;
    double out[5];
    fluid_face_flux<double>(Wd, g.gamma, S, out);
    // undo the direction swap
    const double o1 = out[1], oD = out[1 + DIR];
    out[1] = oD;
    out[1 + DIR] = o1;
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v * nfaces + f] = out[v];
#pragma unroll 1
    for (int c = 0; c < NCHEM; ++c) {
      double cv[6];
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        const double x = __ldg(w.f[5] + c + (long)NCHEM * cell[l]);
        cv[l] = nall[l] ? -x : x;
      }
      F[(5 + c) * nfaces + f] = tracer_face_flux<double>(S, cv);
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
    long i, j, k;
    split3(c, nx, ny, i, j, k);
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

int divergence(const Grid& g, const Fields& w, const Fields& wdot, double* const (&F)[3],
               const ForceTerm& G, int* d_status, cudaStream_t s) {
  ProfScope ps("divergence", s);
  const int t = spread_threads(g.ncell, 256);
  const int b = sweep_blocks(g.ncell, t);
  switch (g.nchem) {
    case 0: divergence_kernel<0><<<b, t, 0, s>>>(g, w, wdot, F[0], F[1], F[2], G, d_status); break;
    case 2: divergence_kernel<2><<<b, t, 0, s>>>(g, w, wdot, F[0], F[1], F[2], G, d_status); break;
    case 4: divergence_kernel<4><<<b, t, 0, s>>>(g, w, wdot, F[0], F[1], F[2], G, d_status); break;
    case 6: divergence_kernel<6><<<b, t, 0, s>>>(g, w, wdot, F[0], F[1], F[2], G, d_status); break;
    case 10: divergence_kernel<10><<<b, t, 0, s>>>(g, w, wdot, F[0], F[1], F[2], G, d_status); break;
    default: set_error("nchem=%d not compiled (0,2,4,6,10)", g.nchem); return GBMV_EUNSUPPORTED;
  }
  GBMV_LAUNCH_CHECK("divergence_kernel");
  return GBMV_OK;
}

// Pass 2 of the float-float form: the same divergence over fluxes kept as float pairs.  On
// GB300 the FP64 pipe runs at 1/64 of the FP32 rate, so the divergence's FP64 differences made
// it FP64-bound (81 % of the pipe) at three times its HBM time; here the differences and the
// 1/d scaling are float-float (FP32 pipes) and only G - div is FP64.  The legal-state flags of
// the float-float forms are set by the primitives pass, which already has the pressure, so this
// pass reads no state field and needs no division.
template <int NCHEM>
__global__ void __launch_bounds__(256) divergence_f2_kernel(Grid g, Fields wdot,
                                                            const float2* __restrict__ Fx,
                                                            const float2* __restrict__ Fy,
                                                            const float2* __restrict__ Fz,
                                                            ForceTerm G) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const long nfx = (nx + 1) * ny * nz, nfy = nx * (ny + 1) * nz, nfz = nx * ny * (nz + 1);
  const f2 idx = f2_from_double(g.inv_d[0]), idy = f2_from_double(g.inv_d[1]),
           idz = f2_from_double(g.inv_d[2]);
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < g.ncell;
       c += (long)gridDim.x * blockDim.x) {
    long i, j, k;
    split3(c, nx, ny, i, j, k);
    const long fx = i + (nx + 1) * (j + ny * k);
    const long fy = i + nx * (j + (ny + 1) * k);
    const long fz = c;
#pragma unroll
    for (int v = 0; v < 5 + NCHEM; ++v) {
      const float2 a0 = Fx[v * nfx + fx], a1 = Fx[v * nfx + fx + 1];
      const float2 b0 = Fy[v * nfy + fy], b1 = Fy[v * nfy + fy + nx];
      const float2 c0 = Fz[v * nfz + fz], c1 = Fz[v * nfz + fz + nx * ny];
      const f2 div = (f2(a1.x, a1.y) - f2(a0.x, a0.y)) * idx +
                     (f2(b1.x, b1.y) - f2(b0.x, b0.y)) * idy +
                     (f2(c1.x, c1.y) - f2(c0.x, c0.y)) * idz;
      double* dst = (v < 5) ? (wdot.f[v] + c) : (wdot.f[5] + (v - 5) + (long)NCHEM * c);
      const double base = G.in_wdot ? *dst : G.c[v];
      *dst = base - f2_to_double(div);
    }
  }
}

int divergence_f2(const Grid& g, const Fields& wdot, float2* const (&F)[3], const ForceTerm& G,
                  cudaStream_t s) {
  ProfScope ps("divergence", s);
  const int b = sweep_blocks(g.ncell, 256);
  switch (g.nchem) {
#define GBMV_DIV_F2(NC)                                                     \
  case NC:                                                                  \
    divergence_f2_kernel<NC><<<b, 256, 0, s>>>(g, wdot, F[0], F[1], F[2], G); \
    break;
    GBMV_DIV_F2(0)
    GBMV_DIV_F2(2)
    GBMV_DIV_F2(4)
    GBMV_DIV_F2(6)
    GBMV_DIV_F2(10)
#undef GBMV_DIV_F2
    default: set_error("nchem=%d not compiled (0,2,4,6,10)", g.nchem); return GBMV_EUNSUPPORTED;
  }
  GBMV_LAUNCH_CHECK("divergence_f2_kernel");
  return GBMV_OK;
}

template <int NCHEM>
static int launch_fp64(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                       double* scratch, int* d_status, cudaStream_t s) {
  long nf[3];
  face_counts(g, nf);
  double* F[3] = {scratch, scratch + (long)(5 + NCHEM) * nf[0],
                  scratch + (long)(5 + NCHEM) * (nf[0] + nf[1])};
  {
    ProfScope ps("face_flux", s);
    const int t = sweep_threads(g, nf[0], 128);
    face_flux_kernel<NCHEM, 0><<<sweep_blocks(nf[0], t), t, 0, s>>>(g, w, F[0], nf[0]);
    GBMV_LAUNCH_CHECK("face_flux_kernel<x>");
  }
  {
    ProfScope ps("face_flux", s);
    const int t = sweep_threads(g, nf[1], 128);
    face_flux_kernel<NCHEM, 1><<<sweep_blocks(nf[1], t), t, 0, s>>>(g, w, F[1], nf[1]);
    GBMV_LAUNCH_CHECK("face_flux_kernel<y>");
  }
  {
    ProfScope ps("face_flux", s);
    const int t = sweep_threads(g, nf[2], 128);
    face_flux_kernel<NCHEM, 2><<<sweep_blocks(nf[2], t), t, 0, s>>>(g, w, F[2], nf[2]);
    GBMV_LAUNCH_CHECK("face_flux_kernel<z>");
  }
  return divergence(g, w, wdot, F, G, d_status, s);
}

size_t feuler_fp64_scratch_doubles(const Grid& g) {
  long nf[3];
  face_counts(g, nf);
  return (size_t)(5 + g.nchem) * (size_t)(nf[0] + nf[1] + nf[2]);
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

// N_VWrmsNorm of the six-component ManyVector (the norm ARKODE's error test and Newton
// convergence test take, src/imex_chem_hydro_main.cpp:463): ewt = 1 / (rtol |y| + atol) per
// entry, sum of (v ewt)^2 over the five fluid fields (ncell each) and the chemistry field
// (nchem ncell), divided by the total length, square root.  Same fixed-grid compensated
// two-pass reduction as the conservation totals; partials in scratch[0..kConsBlocks), result
// in scratch[2 kConsBlocks].
__global__ void __launch_bounds__(256) wrms_partial_kernel(long ncell, int nchem, Fields v,
                                                           Fields y, double rtol, double atol,
                                                           double* __restrict__ part) {
  double s0 = 0.0, c0 = 0.0;
  for (int k = 0; k < 6; ++k) {
    const long n = (k < 5) ? ncell : (long)nchem * ncell;
    const double* __restrict__ vk = v.f[k];
    const double* __restrict__ yk = y.f[k];
    if (n == 0) continue;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
      const double ew = 1.0 / (rtol * fabs(yk[i]) + atol);
      const double q = vk[i] * ew;
      two_sum_acc(s0, c0, q * q);
    }
  }
  double a = s0 + c0;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) a += __shfl_down_sync(0xffffffffu, a, off);
  __shared__ double wa[8];
  if ((threadIdx.x & 31) == 0) wa[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) ta += wa[k];
    part[blockIdx.x] = ta;
  }
}

__global__ void wrms_final_kernel(const double* __restrict__ part, double ntotal,
                                  double* __restrict__ out) {
  if (threadIdx.x == 0) {
    double s0 = 0.0, c0 = 0.0;
    for (int k = 0; k < kConsBlocks; ++k) two_sum_acc(s0, c0, part[k]);
    out[0] = sqrt((s0 + c0) / ntotal);
  }
}

int wrms_norm(const Grid& g, const Fields& v, const Fields& y, double rtol, double atol,
              double* d_scratch, cudaStream_t s) {
  wrms_partial_kernel<<<kConsBlocks, 256, 0, s>>>(g.ncell, g.nchem, v, y, rtol, atol, d_scratch);
  GBMV_LAUNCH_CHECK("wrms_partial_kernel");
  const double ntotal = (double)(5 + g.nchem) * (double)g.ncell;
  wrms_final_kernel<<<1, 32, 0, s>>>(d_scratch, ntotal, d_scratch + 2 * kConsBlocks);
  GBMV_LAUNCH_CHECK("wrms_final_kernel");
  return GBMV_OK;
}

// print_stats (src/io.cpp:552-640): per field the root mean square over the grid,
// sqrt(sum_cells (x * units)^2 / ncells), fluid fields in code units times the density,
// momentum and energy units (1 for dimensionless output), the chemistry fields as stored.
// Same fixed-grid compensated two-pass reduction as the conservation totals; partials in
// scratch[v * kConsBlocks + block], results in scratch[16 * kConsBlocks + v].
constexpr int kRmsMaxFields = 16;

template <int NCHEM>
__global__ void __launch_bounds__(256) field_rms_partial_kernel(long n, Fields w, double du,
                                                                double mu, double eu,
                                                                double* __restrict__ part) {
  constexpr int NV = 5 + NCHEM;
  double s[NV], c[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) s[v] = c[v] = 0.0;
  const double u[5] = {du, mu, mu, mu, eu};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double x = w.f[v][i] * u[v];
      two_sum_acc(s[v], c[v], x * x);
    }
#pragma unroll
    for (int v = 0; v < NCHEM; ++v) {
      const double x = w.f[5][v + (long)NCHEM * i];
      two_sum_acc(s[5 + v], c[5 + v], x * x);
    }
  }
  __shared__ double wsum[8][NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    double a = s[v] + c[v];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) a += __shfl_down_sync(0xffffffffu, a, off);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5][v] = a;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += wsum[k][threadIdx.x];
    part[threadIdx.x * kConsBlocks + blockIdx.x] = t;
  }
}

__global__ void field_rms_final_kernel(const double* __restrict__ part, int nv, double ncell,
                                       double* __restrict__ out) {
  const int v = threadIdx.x;
  if (v < nv) {
    double s0 = 0.0, c0 = 0.0;
    for (int k = 0; k < kConsBlocks; ++k) two_sum_acc(s0, c0, part[v * kConsBlocks + k]);
    out[v] = sqrt((s0 + c0) / ncell);
  }
}

size_t reduction_scratch_doubles() { return (size_t)kRmsMaxFields * kConsBlocks + kRmsMaxFields; }

int field_rms(const Grid& g, const Fields& w, double du, double mu, double eu, double* d_scratch,
              cudaStream_t s) {
  switch (g.nchem) {
#define GBMV_RMS(NC)                                                                   \
  case NC:                                                                            \
    field_rms_partial_kernel<NC><<<kConsBlocks, 256, 0, s>>>(g.ncell, w, du, mu, eu,   \
                                                            d_scratch);               \
    break;
    GBMV_RMS(0)
    GBMV_RMS(2)
    GBMV_RMS(4)
    GBMV_RMS(6)
    GBMV_RMS(10)
#undef GBMV_RMS
    default: set_error("nchem=%d not compiled (0,2,4,6,10)", g.nchem); return GBMV_EUNSUPPORTED;
  }
  GBMV_LAUNCH_CHECK("field_rms_partial_kernel");
  field_rms_final_kernel<<<1, 32, 0, s>>>(d_scratch, 5 + g.nchem, (double)g.ncell,
                                         d_scratch + (size_t)kRmsMaxFields * kConsBlocks);
  GBMV_LAUNCH_CHECK("field_rms_final_kernel");
  return GBMV_OK;
}

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

