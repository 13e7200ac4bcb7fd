// Declarations shared between the WENO kernels and the C ABI layer.
#pragma once

#include "common.cuh"

namespace gbmv {

// The six ManyVector components as raw device pointers (component 5 may be null if nchem==0).
struct Fields {
  double* f[6];
};

// External forcing: per-field constants, or "wdot already holds G" (GBMV_FORCE_IN_WDOT).
struct ForceTerm {
  double c[16];
  int in_wdot;
};

size_t feuler_fp64_scratch_doubles(const Grid& g);
int feuler_fp64(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                double* scratch, int* d_status, cudaStream_t s);

// pass 2 of every form: wdot = G - div F from the three per-direction face-flux arrays
int divergence(const Grid& g, const Fields& w, const Fields& wdot, double* const (&F)[3],
               const ForceTerm& G, int* d_status, cudaStream_t s);
// the same from fluxes stored as float pairs (hi, lo), differenced in float-float
// (no legal-state check: the float-float forms set those flags in prims_f2)
int divergence_f2(const Grid& g, const Fields& wdot, float2* const (&F)[3], const ForceTerm& G,
                  cudaStream_t s);

int wave_speed_max(const Grid& g, const Fields& w, unsigned long long* d_out, cudaStream_t s);
int pack1d(const Grid& g, const Fields& w, int dir, double* out, cudaStream_t s);
// totals of rho and et into d_scratch[2 * 1024 + 0..1] (scratch: conservation_scratch_doubles)
size_t conservation_scratch_doubles();
int conservation_sums(const Grid& g, const Fields& w, double* d_scratch, cudaStream_t s);
// ManyVector WRMS norm of v with weights 1 / (rtol |y| + atol) into
// d_scratch[conservation_scratch_doubles() - 2] (scratch: conservation_scratch_doubles)
int wrms_norm(const Grid& g, const Fields& v, const Fields& y, double rtol, double atol,
              double* d_scratch, cudaStream_t s);
// per-field RMS (print_stats) into d_scratch[16 * 1024 + v]; every reduction of a handle shares
// one scratch of reduction_scratch_doubles() (>= conservation_scratch_doubles())
size_t reduction_scratch_doubles();
int field_rms(const Grid& g, const Fields& w, double du, double mu, double eu, double* d_scratch,
              cudaStream_t s);

// derivatives of the FP64 flux divergence (weno_jvp.cu, weno_vjp.cu)
size_t feuler_vjp_scratch_doubles(const Grid& g);
int feuler_jvp(const Grid& g, const Fields& w, const Fields& dw, const Fields& out,
               double* scratch, cudaStream_t s);
int feuler_vjp(const Grid& g, const Fields& w, const Fields& v, const Fields& out, double* A,
               cudaStream_t s);

// cells one of whose six faces changes its Lax-Friedrichs branch (maximising stencil point,
// sign of its velocity) between w - h dw, w and w + h dw: mask[cell] = 1 (weno_kinks.cu)
int feuler_kink_mask(const Grid& g, const Fields& w, const Fields& dw, double h,
                     unsigned char* mask, cudaStream_t s);

// float-float form (weno_f2.cu)
size_t feuler_f2_prims_floats(const Grid& g);
// tscale: null, or the per-entry scale of a chemistry component held in scaled units
int feuler_f2(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
              double* scratch, float* prims, const double* tscale, int* d_status,
              cudaStream_t s, int fast_weights = 0);

}  // namespace gbmv
