// Per-cell 10x10 Newton-matrix helpers shared by the fused Newton kernel (chem_newton.cu) and
// the persistent DIRK integrator (chem_dirk.cu): the network Jacobian's sparsity pattern and an
// LU with partial pivoting on a per-thread strided slice of shared memory.
#pragma once

#include "df64.cuh"

namespace gbmv {

// Casts to and from the factor's precision.  These stay conversion instructions: the Newton
// and DIRK kernels run few warps per SM and are latency-bound, and the integer-instruction
// conversions of df64.cuh (which win in the throughput-bound float-float passes) lengthen
// their dependency chains (measured 1 % slower fused Newton, 8 % slower mixed DIRK).
template <typename LU>
__device__ __forceinline__ LU to_lu(double x) { return (LU)x; }
__device__ __forceinline__ double from_lu(float x) { return (double)x; }
__device__ __forceinline__ double from_lu(double x) { return x; }

// Structural nonzeros (row, col) of the network Jacobian (the CSR pattern of
// src/raja_primordial_network.cpp:1869-1948); every diagonal entry is among them.
__device__ constexpr int kJacPattern[64][2] = {
    {0, 0}, {0, 1}, {0, 2}, {0, 3}, {0, 4}, {0, 8}, {0, 9}, {1, 0}, {1, 1}, {1, 2}, {1, 3},
    {1, 4}, {1, 8}, {1, 9}, {2, 0}, {2, 1}, {2, 2}, {2, 3}, {2, 4}, {2, 8}, {2, 9}, {3, 0},
    {3, 1}, {3, 2}, {3, 3}, {3, 4}, {3, 8}, {3, 9}, {4, 1}, {4, 2}, {4, 3}, {4, 4}, {4, 8},
    {4, 9}, {5, 5}, {5, 6}, {5, 8}, {5, 9}, {6, 5}, {6, 6}, {6, 7}, {6, 8}, {6, 9}, {7, 6},
    {7, 7}, {7, 8}, {7, 9}, {8, 1}, {8, 2}, {8, 3}, {8, 4}, {8, 5}, {8, 6}, {8, 7}, {8, 8},
    {8, 9}, {9, 0}, {9, 2}, {9, 3}, {9, 5}, {9, 6}, {9, 7}, {9, 8}, {9, 9}};

// kJacIndex[row][col] = position of (row, col) in kJacPattern, -1 for a structural zero.
__device__ constexpr signed char kJacIndex[10][10] = {
    {0, 1, 2, 3, 4, -1, -1, -1, 5, 6},         {7, 8, 9, 10, 11, -1, -1, -1, 12, 13},
    {14, 15, 16, 17, 18, -1, -1, -1, 19, 20},  {21, 22, 23, 24, 25, -1, -1, -1, 26, 27},
    {-1, 28, 29, 30, 31, -1, -1, -1, 32, 33},  {-1, -1, -1, -1, -1, 34, 35, -1, 36, 37},
    {-1, -1, -1, -1, -1, 38, 39, 40, 41, 42},  {-1, -1, -1, -1, -1, -1, 43, 44, 45, 46},
    {-1, 47, 48, 49, 50, 51, 52, 53, 54, 55},  {56, -1, 57, 58, -1, 59, 60, 61, 62, 63}};

// In-place LU with partial pivoting on a strided per-thread slice A[e*stride] (column-major
// 10x10), reciprocal pivots on the diagonal; returns 0 or 1 + first zero pivot.
template <typename R>
__device__ __forceinline__ int lu10_strided(R* A, int stride, int (&piv)[10]) {
  int info = 0;
#pragma unroll 1
  for (int kk = 0; kk < 10; ++kk) {
    int p = kk;
    R amax = fabs(A[(kk * 10 + kk) * stride]);
    for (int r = kk + 1; r < 10; ++r) {
      const R v = fabs(A[(kk * 10 + r) * stride]);
      if (v > amax) { amax = v; p = r; }
    }
    piv[kk] = p;
    if (p != kk)
      for (int col = 0; col < 10; ++col) {
        const R t = A[(col * 10 + kk) * stride];
        A[(col * 10 + kk) * stride] = A[(col * 10 + p) * stride];
        A[(col * 10 + p) * stride] = t;
      }
    const R d = A[(kk * 10 + kk) * stride];
    if (d == R(0)) {
      if (!info) info = kk + 1;
      continue;
    }
    const R rp = R(1) / d;
    A[(kk * 10 + kk) * stride] = rp;
    for (int r = kk + 1; r < 10; ++r) A[(kk * 10 + r) * stride] *= rp;
    for (int col = kk + 1; col < 10; ++col) {
      const R a = A[(col * 10 + kk) * stride];
      for (int r = kk + 1; r < 10; ++r) A[(col * 10 + r) * stride] -= A[(kk * 10 + r) * stride] * a;
    }
  }
  return info;
}

// Solve with the factor of lu10_strided: row interchanges, unit-lower and upper sweeps.
template <typename R, typename X>
__device__ __forceinline__ void lus10_strided(const R* A, int stride, const int (&piv)[10],
                                              X (&x)[10]) {
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
    for (int r = col + 1; r < 10; ++r) x[r] -= X(A[(col * 10 + r) * stride]) * x[col];
#pragma unroll
  for (int col = 9; col >= 0; --col) {
    x[col] *= X(A[(col * 10 + col) * stride]);
#pragma unroll
    for (int r = 0; r < col; ++r) x[r] -= X(A[(col * 10 + r) * stride]) * x[col];
  }
}

}  // namespace gbmv
