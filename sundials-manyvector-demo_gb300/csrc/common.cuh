// Shared device/host helpers for the gbmv kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbmv.h"

namespace gbmv {

// Records the last error message and a launch counter (host side, capi.cu).
void set_error(const char* fmt, ...);
void count_launch(long n = 1);
int check_cuda(cudaError_t e, const char* where);
// Grid validation shared by every entry point that takes a gbmv_grid (capi.cu): 0, or
// GBMV_EINVAL / GBMV_EUNSUPPORTED with the reason in gbmv_last_error().
int check_grid(const gbmv_grid* g);

#define GBMV_CUDA_TRY(expr)                                   \
  do {                                                        \
    cudaError_t e_ = (expr);                                  \
    if (e_ != cudaSuccess) return ::gbmv::check_cuda(e_, #expr); \
  } while (0)

#define GBMV_LAUNCH_CHECK(where)                                   \
  do {                                                             \
    ::gbmv::count_launch();                                        \
    cudaError_t e_ = cudaGetLastError();                           \
    if (e_ != cudaSuccess) return ::gbmv::check_cuda(e_, where);   \
  } while (0)

// Optional per-kernel-family timing with CUDA events on the launching stream
// (gbmv_profile_enable); a no-op when disabled.
// Per-family profiling scope around the kernel launches of one entry point: an NVTX range
// (visible to ncu / nsys filters) always, CUDA events while gbmv_profile_enable is on.
struct ProfScope {
  ProfScope(const char* family, cudaStream_t s);
  ~ProfScope();
  int slot;
  cudaStream_t stream;
};

constexpr int kSM = 152;  // GB300 SM count (2 dies x 76)

// Device-side copy of the grid description.
struct Grid {
  long n[3];       // nx, ny, nz
  long ncell;
  int nchem;
  int bc[6];
  double gamma;
  double inv_d[3]; // 1/dx, 1/dy, 1/dz
  double d[3];
  int sweep_threads;  // threads per block of the face sweeps (0: by size, spread_threads)
  int sweep_shared;   // GBMV_MIXED_FAST sweeps sized to share the SMs with another kernel
};

inline Grid make_grid(const gbmv_grid& g) {
  Grid G;
  G.n[0] = g.nx; G.n[1] = g.ny; G.n[2] = g.nz;
  G.ncell = g.nx * g.ny * g.nz;
  G.nchem = g.nchem;
  for (int i = 0; i < 6; ++i) G.bc[i] = g.bc[i];
  G.gamma = g.gamma;
  G.d[0] = g.dx; G.d[1] = g.dy; G.d[2] = g.dz;
  for (int i = 0; i < 3; ++i) G.inv_d[i] = 1.0 / G.d[i];
  G.sweep_threads = 0;
  G.sweep_shared = 0;
  return G;
}

// Ghost synthesis along one axis (the rule of EulerData::ExchangeStart and pack1D_*_bdry,
// src/euler3D.hpp:577-1166 and 1250-1378, on one rank):
//   periodic          : wrap (p+n or p-n)
//   lower, non-periodic: mirror, cell -1-p   (ghost -1 <- cell 0, -2 <- 1, -3 <- 2)
//   upper, non-periodic: shifted copy, cell p-3 (ghost n <- n-3, n+1 <- n-2, n+2 <- n-1)
//   sign: Neumann +, Dirichlet - (all fields), reflecting - on the normal momentum only.
// Returns the source position along the axis; *neg_all / *neg_normal tell the sign rule.
__host__ __device__ inline long ghost_src(long p, long n, int bc_lo, int bc_hi, bool* neg_all,
                                          bool* neg_normal) {
  *neg_all = false;
  *neg_normal = false;
  if (p < 0) {
    if (bc_lo == GBMV_BC_PERIODIC) return p + n;
    *neg_all = (bc_lo == GBMV_BC_DIRICHLET);
    *neg_normal = (bc_lo == GBMV_BC_REFLECTING);
    return -1 - p;
  }
  if (p >= n) {
    if (bc_hi == GBMV_BC_PERIODIC) return p - n;
    *neg_all = (bc_hi == GBMV_BC_DIRICHLET);
    *neg_normal = (bc_hi == GBMV_BC_REFLECTING);
    return p - 3;
  }
  return p;
}

__host__ __device__ constexpr int nvar_of(int nchem) { return 5 + nchem; }

}  // namespace gbmv
