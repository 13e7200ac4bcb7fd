// Block-diagonal Newton linear solve (part c): batched LU with partial pivoting of the 10x10
// chemistry blocks (what SUNLinSol_MagmaDense does with MAGMA's batched getrf/getrs under the
// reference's SUNLinSol_RankLocalLS / SUNLinSol_BDMPIMV wrappers,
// src/multirate_chem_hydro_main.cpp:1312-1411, src/imex_chem_hydro_main.cpp:1075-1194).
//
// One thread owns one block; the whole 10x10 block lives in registers (fully unrolled through
// template recursion, compile-time indices), row interchanges are predicated selects.  A CTA
// stages 128 consecutive blocks (102 KB, contiguous in HBM) through shared memory with
// 16-byte coalesced accesses; two CTAs per SM overlap one tile's traffic with the other's
// arithmetic.
#include "chem.cuh"

namespace gbmv {

constexpr int kLuThreads = 64;   // blocks per tile = threads per CTA
constexpr int kLuStride = 101;   // padded per-block stride of the shared tile (doubles)
constexpr int kVecStride = 11;   // the same for the right-hand-side tile

// Coalesced copy of `nb` consecutive blocks of NE doubles between global memory and a shared
// tile with per-block stride SS (16-byte global accesses when NE is even and the address is
// 16-byte aligned -- caller arrays need only be 8-byte aligned).
template <int NE, int SS = kLuStride>
__device__ __forceinline__ void tile_in(const double* __restrict__ g, double* sh, long blk0, int nb) {
  const double* src = g + blk0 * NE;
  if (NE % 2 == 0 && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
    const double2* s2 = reinterpret_cast<const double2*>(src);
    for (int c = threadIdx.x; c < nb * NE / 2; c += blockDim.x) {
      const double2 v = s2[c];
      const int b = (2 * c) / NE, e = (2 * c) % NE;
      sh[b * SS + e] = v.x;
      sh[b * SS + e + 1] = v.y;
    }
  } else {
    for (int c = threadIdx.x; c < nb * NE; c += blockDim.x) sh[(c / NE) * SS + c % NE] = src[c];
  }
}
template <int NE, int SS = kLuStride>
__device__ __forceinline__ void tile_out(double* __restrict__ g, const double* sh, long blk0, int nb) {
  double* dst = g + blk0 * NE;
  if (NE % 2 == 0 && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
    double2* d2 = reinterpret_cast<double2*>(dst);
    for (int c = threadIdx.x; c < nb * NE / 2; c += blockDim.x) {
      const int b = (2 * c) / NE, e = (2 * c) % NE;
      d2[c] = make_double2(sh[b * SS + e], sh[b * SS + e + 1]);
    }
  } else {
    for (int c = threadIdx.x; c < nb * NE; c += blockDim.x) dst[c] = sh[(c / NE) * SS + c % NE];
  }
}

// One elimination step KK of LU with partial pivoting (first maximal |pivot|, full-row
// interchange, the dgetf2 order), fully unrolled through template recursion so the block
// stays in registers.  The factor keeps 1/U(k,k) on the diagonal (the solve only multiplies);
// the factored matrix is private to this solver, as MAGMA's is to its own getrs.
template <int KK, typename R>
__device__ __forceinline__ void lu_step(R (&A)[100], int (&piv)[10], int& info) {
  int p = KK;
  R amax = fabs(A[KK * 10 + KK]);
#pragma unroll
  for (int r = KK + 1; r < 10; ++r) {
    const R v = fabs(A[KK * 10 + r]);
    if (v > amax) { amax = v; p = r; }
  }
  piv[KK] = p;
#pragma unroll
  for (int r = KK + 1; r < 10; ++r) {
    const bool sw = (r == p);
#pragma unroll
    for (int col = 0; col < 10; ++col) {
      const R a = A[col * 10 + KK], b = A[col * 10 + r];
      A[col * 10 + KK] = sw ? b : a;
      A[col * 10 + r] = sw ? a : b;
    }
  }
  const R d = A[KK * 10 + KK];
  if (d == R(0)) {
    if (!info) info = KK + 1;
  } else {
    const R rp = R(1) / d;
    A[KK * 10 + KK] = rp;
#pragma unroll
    for (int r = KK + 1; r < 10; ++r) A[KK * 10 + r] *= rp;
#pragma unroll
    for (int col = KK + 1; col < 10; ++col) {
      const R a = A[col * 10 + KK];
#pragma unroll
      for (int r = KK + 1; r < 10; ++r) A[col * 10 + r] -= A[KK * 10 + r] * a;
    }
  }
  if constexpr (KK < 9) lu_step<KK + 1>(A, piv, info);
}

template <typename R>
__device__ __forceinline__ int lu10_regs(R (&A)[100], int (&piv)[10]) {
  int info = 0;
  lu_step<0>(A, piv, info);
  return info;
}

// Solve with the factor of lu10_regs (row interchanges, unit-lower forward substitution,
// upper back substitution multiplying by the stored reciprocal pivots).
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
    x[col] *= X(A[col * 10 + col]);
#pragma unroll
    for (int r = 0; r < col; ++r) x[r] -= X(A[col * 10 + r]) * x[col];
  }
}

__global__ void __launch_bounds__(kLuThreads, 4) block_lu_factor_kernel(long nb, double* __restrict__ A,
                                                                        int* __restrict__ piv,
                                                                        int* __restrict__ info_out) {
  extern __shared__ double sh[];  // [kLuThreads][kLuStride]
  int bad = 0;
  for (long blk0 = (long)blockIdx.x * kLuThreads; blk0 < nb; blk0 += (long)gridDim.x * kLuThreads) {
    const int nb_here = (int)((nb - blk0) < kLuThreads ? (nb - blk0) : kLuThreads);
    tile_in<100>(A, sh, blk0, nb_here);
    __syncthreads();
    if (threadIdx.x < nb_here) {
      double a[100];
      int p[10];
      const double* mine = sh + threadIdx.x * kLuStride;
#pragma unroll
      for (int e = 0; e < 100; ++e) a[e] = mine[e];
      if (lu10_regs(a, p)) bad = 1;
      double* out = sh + threadIdx.x * kLuStride;
#pragma unroll
      for (int e = 0; e < 100; ++e) out[e] = a[e];
      int* pg = piv + (blk0 + threadIdx.x) * 10;
#pragma unroll
      for (int e = 0; e < 10; ++e) pg[e] = p[e];
    }
    __syncthreads();
    tile_out<100>(A, sh, blk0, nb_here);
    __syncthreads();
  }
  if (bad) atomicMax(info_out, 1);
}

__global__ void __launch_bounds__(kLuThreads, 4) block_lu_solve_kernel(long nb,
                                                                       const double* __restrict__ LU,
                                                                       const int* __restrict__ piv,
                                                                       const double* b, double* x) {
  extern __shared__ double sh[];  // LU tile, then the right-hand sides
  double* shb = sh + kLuThreads * kLuStride;  // [kLuThreads][kVecStride]
  for (long blk0 = (long)blockIdx.x * kLuThreads; blk0 < nb; blk0 += (long)gridDim.x * kLuThreads) {
    const int nb_here = (int)((nb - blk0) < kLuThreads ? (nb - blk0) : kLuThreads);
    tile_in<100>(LU, sh, blk0, nb_here);
    tile_in<10, kVecStride>(b, shb, blk0, nb_here);
    __syncthreads();
    if (threadIdx.x < nb_here) {
      double a[100], v[10];
      int p[10];
      const double* mine = sh + threadIdx.x * kLuStride;
#pragma unroll
      for (int e = 0; e < 100; ++e) a[e] = mine[e];
      const int* pg = piv + (blk0 + threadIdx.x) * 10;
#pragma unroll
      for (int e = 0; e < 10; ++e) {
        p[e] = pg[e];
        v[e] = shb[threadIdx.x * kVecStride + e];
      }
      lus10_regs(a, p, v);
#pragma unroll
      for (int e = 0; e < 10; ++e) shb[threadIdx.x * kVecStride + e] = v[e];
    }
    __syncthreads();
    tile_out<10, kVecStride>(x, shb, blk0, nb_here);
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
  const long cap = (long)kSM * 4;
  if (b < 1) b = 1;
  return (int)(b < cap ? b : cap);
}

int block_lu_factor(long nb, double* A, int* piv, int* d_info, cudaStream_t s) {
  const size_t shm = sizeof(double) * kLuStride * kLuThreads;
  GBMV_CUDA_TRY(cudaFuncSetAttribute(block_lu_factor_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
  ProfScope ps("block_lu_factor", s);
  block_lu_factor_kernel<<<lu_grid(nb), kLuThreads, shm, s>>>(nb, A, piv, d_info);
  GBMV_LAUNCH_CHECK("block_lu_factor_kernel");
  return GBMV_OK;
}

int block_lu_solve(long nb, const double* LU, const int* piv, const double* b, double* x,
                   cudaStream_t s) {
  const size_t shm = sizeof(double) * (kLuStride + kVecStride) * kLuThreads;
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
