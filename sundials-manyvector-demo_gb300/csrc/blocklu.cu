// Block-diagonal Newton linear solve (part c): batched LU with partial pivoting of the 10x10
// chemistry blocks (what SUNLinSol_MagmaDense does with MAGMA's batched getrf/getrs under the
// reference's SUNLinSol_RankLocalLS / SUNLinSol_BDMPIMV wrappers,
// src/multirate_chem_hydro_main.cpp:1312-1411, src/imex_chem_hydro_main.cpp:1075-1194).
//
// One thread owns one block; the whole 10x10 block lives in registers (fully unrolled loops
// with compile-time indices), row interchanges are predicated selects.  Blocks are read and
// written through shared memory so that global traffic is coalesced: a warp stages its 32
// consecutive blocks (32 x 800 B, contiguous) with unit-stride loads.
#include "chem.cuh"

namespace gbmv {

constexpr int kLuThreads = 64;

// Coalesced copy of nb_here consecutive blocks between global and a shared tile laid out
// element-major ([e][thread], conflict-free per-thread access).
template <typename T, int NE>
__device__ __forceinline__ void stage_in(const T* __restrict__ g, T* sh, long blk0, int nb_here) {
  const long base = blk0 * NE;
  for (int t = threadIdx.x; t < nb_here * NE; t += blockDim.x) {
    const int b = t / NE, e = t % NE;
    sh[e * kLuThreads + b] = g[base + t];
  }
}
template <typename T, int NE>
__device__ __forceinline__ void stage_out(T* __restrict__ g, const T* sh, long blk0, int nb_here) {
  const long base = blk0 * NE;
  for (int t = threadIdx.x; t < nb_here * NE; t += blockDim.x) {
    const int b = t / NE, e = t % NE;
    g[base + t] = sh[e * kLuThreads + b];
  }
}

// In-register LU with partial pivoting (first maximal |pivot|, full-row interchanges, the
// dgetf2 order).  Returns 0 or 1 + first zero-pivot column.
template <typename R>
__device__ __forceinline__ int lu10_regs(R (&A)[100], int (&piv)[10]) {
  int info = 0;
#pragma unroll
  for (int kk = 0; kk < 10; ++kk) {
    int p = kk;
    R amax = fabs(A[kk * 10 + kk]);
#pragma unroll
    for (int r = kk + 1; r < 10; ++r) {
      const R v = fabs(A[kk * 10 + r]);
      if (v > amax) { amax = v; p = r; }
    }
    piv[kk] = p;
    // predicated interchange of rows kk and p across all columns
#pragma unroll
    for (int r = kk + 1; r < 10; ++r) {
      const bool sw = (r == p);
#pragma unroll
      for (int col = 0; col < 10; ++col) {
        const R a = A[col * 10 + kk], b = A[col * 10 + r];
        A[col * 10 + kk] = sw ? b : a;
        A[col * 10 + r] = sw ? a : b;
      }
    }
    const R d = A[kk * 10 + kk];
    if (d == R(0)) {
      if (!info) info = kk + 1;
    } else {
      const R rp = R(1) / d;
#pragma unroll
      for (int r = kk + 1; r < 10; ++r) A[kk * 10 + r] *= rp;
#pragma unroll
      for (int col = kk + 1; col < 10; ++col) {
        const R a = A[col * 10 + kk];
#pragma unroll
        for (int r = kk + 1; r < 10; ++r) A[col * 10 + r] -= A[kk * 10 + r] * a;
      }
    }
  }
  return info;
}

template <typename R, typename X>
__device__ __forceinline__ void lus10_regs(const R (&A)[100], const int (&piv)[10], X (&x)[10]) {
#pragma unroll
  for (int kk = 0; kk < 10; ++kk) {
#pragma unroll
    for (int r = kk + 1; r < 10; ++r) {
      const bool sw = (r == piv[kk]);
      const X a = x[kk], b = x[r];
      x[kk] = sw ? b : a;
      x[r] = sw ? a : b;
    }
  }
#pragma unroll
  for (int col = 0; col < 10; ++col)
#pragma unroll
    for (int r = col + 1; r < 10; ++r) x[r] -= X(A[col * 10 + r]) * x[col];
#pragma unroll
  for (int col = 9; col >= 0; --col) {
    x[col] /= X(A[col * 10 + col]);
#pragma unroll
    for (int r = 0; r < col; ++r) x[r] -= X(A[col * 10 + r]) * x[col];
  }
}

__global__ void __launch_bounds__(kLuThreads) block_lu_factor_kernel(long nb, double* __restrict__ A,
                                                                     int* __restrict__ piv,
                                                                     int* __restrict__ info_out) {
  extern __shared__ double sh[];  // [100][kLuThreads]
  __shared__ int shp[10 * kLuThreads];
  int bad = 0;
  for (long blk0 = (long)blockIdx.x * kLuThreads; blk0 < nb; blk0 += (long)gridDim.x * kLuThreads) {
    const int nb_here = (int)((nb - blk0) < kLuThreads ? (nb - blk0) : kLuThreads);
    stage_in<double, 100>(A, sh, blk0, nb_here);
    __syncthreads();
    if (threadIdx.x < nb_here) {
      double a[100];
      int p[10];
#pragma unroll
      for (int e = 0; e < 100; ++e) a[e] = sh[e * kLuThreads + threadIdx.x];
      const int info = lu10_regs(a, p);
      if (info && !bad) bad = 1;
#pragma unroll
      for (int e = 0; e < 100; ++e) sh[e * kLuThreads + threadIdx.x] = a[e];
#pragma unroll
      for (int e = 0; e < 10; ++e) shp[e * kLuThreads + threadIdx.x] = p[e];
    }
    __syncthreads();
    stage_out<double, 100>(A, sh, blk0, nb_here);
    stage_out<int, 10>(piv, shp, blk0, nb_here);
    __syncthreads();
  }
  if (bad) atomicMax(info_out, 1);
}

__global__ void __launch_bounds__(kLuThreads) block_lu_solve_kernel(long nb,
                                                                    const double* __restrict__ LU,
                                                                    const int* __restrict__ piv,
                                                                    const double* b,
                                                                    double* x) {
  extern __shared__ double sh[];
  __shared__ int shp[10 * kLuThreads];
  __shared__ double shx[10 * kLuThreads];
  for (long blk0 = (long)blockIdx.x * kLuThreads; blk0 < nb; blk0 += (long)gridDim.x * kLuThreads) {
    const int nb_here = (int)((nb - blk0) < kLuThreads ? (nb - blk0) : kLuThreads);
    stage_in<double, 100>(LU, sh, blk0, nb_here);
    stage_in<int, 10>(piv, shp, blk0, nb_here);
    stage_in<double, 10>(b, shx, blk0, nb_here);
    __syncthreads();
    if (threadIdx.x < nb_here) {
      double a[100], v[10];
      int p[10];
#pragma unroll
      for (int e = 0; e < 100; ++e) a[e] = sh[e * kLuThreads + threadIdx.x];
#pragma unroll
      for (int e = 0; e < 10; ++e) {
        p[e] = shp[e * kLuThreads + threadIdx.x];
        v[e] = shx[e * kLuThreads + threadIdx.x];
      }
      lus10_regs(a, p, v);
#pragma unroll
      for (int e = 0; e < 10; ++e) shx[e * kLuThreads + threadIdx.x] = v[e];
    }
    __syncthreads();
    stage_out<double, 10>(x, shx, blk0, nb_here);
    __syncthreads();
  }
}

// SUNMatScaleAddI(-gamma, J): A = -gamma*J + I on every block.
__global__ void block_form_newton_kernel(long nel, double* __restrict__ J, double c) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nel;
       e += (long)gridDim.x * blockDim.x) {
    const int r = (int)(e % 100);
    const double v = c * J[e];
    J[e] = (r % 11 == 0) ? v + 1.0 : v;
  }
}

static int lu_grid(long nb) {
  long b = (nb + kLuThreads - 1) / kLuThreads;
  const long cap = (long)kSM * 8;
  if (b < 1) b = 1;
  return (int)(b < cap ? b : cap);
}

int block_lu_factor(long nb, double* A, int* piv, int* d_info, cudaStream_t s) {
  const size_t shm = sizeof(double) * 100 * kLuThreads;
  GBMV_CUDA_TRY(cudaFuncSetAttribute(block_lu_factor_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
  ProfScope ps("block_lu_factor", s);
  block_lu_factor_kernel<<<lu_grid(nb), kLuThreads, shm, s>>>(nb, A, piv, d_info);
  GBMV_LAUNCH_CHECK("block_lu_factor_kernel");
  return GBMV_OK;
}

int block_lu_solve(long nb, const double* LU, const int* piv, const double* b, double* x,
                   cudaStream_t s) {
  const size_t shm = sizeof(double) * 100 * kLuThreads;
  GBMV_CUDA_TRY(cudaFuncSetAttribute(block_lu_solve_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
  ProfScope ps("block_lu_solve", s);
  block_lu_solve_kernel<<<lu_grid(nb), kLuThreads, shm, s>>>(nb, LU, piv, b, x);
  GBMV_LAUNCH_CHECK("block_lu_solve_kernel");
  return GBMV_OK;
}

int block_form_newton(long nb, double* J, double gamma, cudaStream_t s) {
  const long nel = 100 * nb;
  long g = (nel + 255) / 256;
  if (g > (long)kSM * 32) g = (long)kSM * 32;
  if (g < 1) g = 1;
  ProfScope ps("glue", s);
  block_form_newton_kernel<<<(int)g, 256, 0, s>>>(nel, J, -gamma);
  GBMV_LAUNCH_CHECK("block_form_newton_kernel");
  return GBMV_OK;
}

}  // namespace gbmv
