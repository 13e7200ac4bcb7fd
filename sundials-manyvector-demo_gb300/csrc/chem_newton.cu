// Fused chemistry Newton step (parts b + c in one kernel): for every cell
//   f = TimeUnits * f_chem(y)                      (calculate_rhs_cvklu + N_VScale)
//   J = TimeUnits * df_chem/dy                     (calculate_jacobian_cvklu + scaling)
//   x = (I - gamma J)^{-1} f                       (SUNMatScaleAddI + getrf/getrs)
// without writing J to HBM.  One thread per cell; the cell's FP64 Newton matrix lives in a
// per-thread slice of shared memory ([element][thread], conflict-free).
//   LU = double: factor and solve in FP64 (the plain form fused);
//   LU = float : factor in FP32, solve in FP32, then `refine` steps of iterative refinement
//                with FP64 residuals r = f - A x against the FP64 matrix (the
//                mixed-precision Newton solve); a non-finite FP32 factor falls back to FP64.
// The temperature state (Ts, dTs/dge) is updated as by gbmv_chem_rhs (LU = double: exactly;
// LU = float: the ten Newton iterations run 8 in FP32 and the last 2 in FP64).
#include "chem.cuh"
#include "chem_net.cuh"
#include "chem_lu.cuh"
#include "df64.cuh"

namespace gbmv {

// Threads per block.  Shared memory per cell: the FP32-LU form keeps the 64 structural
// nonzeros of the FP64 Newton matrix (for the refinement residuals) and the 100-entry FP32
// factor, 912 bytes; the FP64-LU form only its 100-entry FP64 factor.  With 32-thread blocks
// seven blocks (seven warps) fit an SM, against six with 64-thread blocks.
constexpr int kNtThreads = 32;

template <typename LU, int BS>
__global__ void __launch_bounds__(BS) chem_newton_kernel(ChemParams P, ChemState S, long n,
                                                         const double* __restrict__ y,
                                                         double* __restrict__ fout,
                                                         double* __restrict__ xout,
                                                         double gamma, double tunit,
                                                         int refine,
                                                         int* __restrict__ info_out,
                                                         const double* __restrict__ bst,
                                                         unsigned long long* __restrict__ queue) {
  extern __shared__ unsigned char smem_raw[];
  constexpr bool kMixed = sizeof(LU) == 4;
  // FP32-LU form: As[e * BS] = FP64 matrix entry e of kJacPattern; L[(col*10+row) * BS] factor
  double* As = reinterpret_cast<double*>(smem_raw) + threadIdx.x;
  LU* L = reinterpret_cast<LU*>(reinterpret_cast<double*>(smem_raw) + (kMixed ? 64 * BS : 0)) +
          threadIdx.x;
  int bad = 0;
  // cells: a grid-stride sweep, or (queue set) 32-cell chunks taken from the shared counter by
  // each one-warp block until every cell is taken (launches on other streams may share it)
  long i = queue ? -1 : blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long stride = (long)gridDim.x * blockDim.x;
  while (true) {
    if (queue) {
      unsigned long long base = 0;
      if (threadIdx.x == 0) base = atomicAdd(queue, (unsigned long long)BS);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= (unsigned long long)n) break;
      i = (long)base + threadIdx.x;
    } else if (i >= n) {
      break;
    }
    if (i < n) {  // (the last chunk's surplus lanes skip the cell and take the next, empty one)
      const long j = i * 10;
      const double* __restrict__ sc = S.scale + j;  // re-read through L1: keeps registers free
      const double* __restrict__ isc = S.inv_scale + j;
      double ya[10];
#pragma unroll
      for (int s = 0; s < 10; ++s) ya[s] = y[j + s] * sc[s];
      double Ts = S.Ts[i], dTs = 0.0;
      // mixed form: up to 8 FP32 iterations, then two in FP64.  (One FP64 iteration where
      // the FP32 stage converged measured 5 % faster but left the carried temperature up to
      // 4e-10 off the FP64 form's ten-iteration value: the adiabatic-index tables are linear
      // in log T per bin, so near a bin edge Newton converges only linearly.)
      if (sizeof(LU) == 4)
        chem_temperature_mixed(P, ya, Ts, dTs, 8);
      else
        chem_temperature(P, ya, Ts, dTs);
      S.Ts[i] = Ts;
      S.dTs_ge[i] = dTs;
      const ChemAux Ax{S.mdens[i], S.imdens[i], S.cie[i], S.h2[i]};
      double f[10];
      {  // source and Newton matrix from one rate evaluation (rates and T slopes)
        double k[kNRates], dk[kNRates];
        chem_rates<true, kMixed>(P, Ts, k, dk);
        const GeRecip Rg = ge_recip(k, ya);  // shared by the source and the Jacobian's ge row
        {
          double r[21], sp[9];
          chem_fluxes(k, ya, r);
          chem_species(r, sp);
#pragma unroll
          for (int s = 0; s < 9; ++s) f[s] = (sp[s] * isc[s]) * tunit;
          double ge = chem_ge_source_r(P, k, ya, Ts, Ax, Rg) * isc[9];
          ge *= Ax.imdens;
          f[9] = ge * tunit;
        }
#pragma unroll
        for (int s = 0; s < 10; ++s) fout[j + s] = f[s];
        // A = I - gamma * (J * inv_scale[row] * scale[col] * tunit), FP64 and a float copy;
        // the ge row's 1/mdensity and the ge column's dT/dge ride on the row and column factors
        double rf[10];  // -gamma * tunit * inv_scale[row]
#pragma unroll
        for (int r = 0; r < 10; ++r) rf[r] = (-gamma * tunit) * isc[r];
        rf[9] *= Ax.imdens;
        const double sc9 = sc[9] * dTs;
#pragma unroll
        for (int e = 0; e < 100; ++e) L[e * BS] = LU(0);  // structural zeros
        // every structural entry (the diagonal included) is put exactly once
        chem_jacobian<true>(P, k, dk, ya, Ts, dTs, Ax, [&](int row, int col, double v) {
          const double a = (v * rf[row]) * (col == 9 ? sc9 : sc[col]) + (row == col ? 1.0 : 0.0);
          if (kMixed) {
            const int e = kJacIndex[row][col];
            if (e >= 0) As[e * BS] = a;
          } else {
            L[(col * 10 + row) * BS] = to_lu<LU>(a);
          }
        }, &Rg);
        if constexpr (kMixed) {  // the FP32 factor's entries, converted with integer
          // instructions after the Jacobian (off the FP64 pipe, which bounds this kernel, and off
          // the Jacobian's dependency chains: 5.45 -> 5.34 ms per 128^3 call; converting inside
          // the entry loop had measured 1 % slower)
#pragma unroll
          for (int e = 0; e < 64; ++e)
            L[(kJacPattern[e][1] * 10 + kJacPattern[e][0]) * BS] = f32_of_f64(As[e * BS]);
        }
      }
#pragma unroll
      for (int s = 0; s < 10; ++s) f[s] = fout[j + s];
      if (bst) {  // implicit-stage form: right-hand side b + gamma f(y)
#pragma unroll
        for (int s = 0; s < 10; ++s) f[s] = fma(gamma, f[s], bst[j + s]);
      }

      int piv[10];
      double x[10];
      // (Power-of-two row, or row and column, equilibration of the FP32 factor was tried: on
      // these matrices it changes the pivot order for the worse -- 2.4e-3 against 1.9e-8 after
      // one refinement on the test blocks, reproduced on the oracle's matrices -- so the factor
      // keeps plain partial pivoting.)
      int info = lu10_strided<LU>(L, BS, piv);
      bool fp64_fallback = (sizeof(LU) == 4) && info != 0;
      if (!fp64_fallback) {
        LU xs[10];
#pragma unroll
        for (int s = 0; s < 10; ++s) xs[s] = to_lu<LU>(f[s]);
        lus10_strided<LU, LU>(L, BS, piv, xs);
        float xmax = 0.f;  // solution size for the stopping tests, from the FP32 solve: the
                           // refinements move it by ~1e-7 relative, far below either threshold
#pragma unroll
        for (int s = 0; s < 10; ++s) {
          x[s] = from_lu(xs[s]);
          xmax = fmaxf(xmax, fabsf((float)xs[s]));
        }
        if (sizeof(LU) == 4) {
          // iterative refinement against FP64 residuals; a cell stops as soon as its correction
          // is below 1e-13 of the solution (well-conditioned cells need one step, the
          // ill-conditioned ones use up to `refine`); a cell whose last correction is still above
          // 1e-6 of its solution (the FP32 factor too poor a preconditioner for its block)
          // takes the FP64 factor below
          float dlast = 0.f;
          for (int it = 0; it < refine; ++it) {
            double rr[10];
#pragma unroll
            for (int row = 0; row < 10; ++row) rr[row] = f[row];
#pragma unroll
            for (int e = 0; e < 64; ++e)  // the 64 structural nonzeros (diagonal included)
              rr[kJacPattern[e][0]] -= As[e * BS] * x[kJacPattern[e][1]];
            LU ds[10];
#pragma unroll
            for (int s = 0; s < 10; ++s) ds[s] = to_lu<LU>(rr[s]);
            lus10_strided<LU, LU>(L, BS, piv, ds);
            float dmax = 0.f;
#pragma unroll
            for (int s = 0; s < 10; ++s) {
              x[s] += from_lu(ds[s]);
              dmax = fmaxf(dmax, fabsf((float)ds[s]));
            }
            dlast = dmax;
            if (dmax <= 1e-13f * xmax) break;
          }
          bool finite = true;
#pragma unroll
          for (int s = 0; s < 10; ++s) finite = finite && isfinite(x[s]);
          fp64_fallback = !finite || !(dlast <= 1e-6f * xmax);
        }
      }
      if (fp64_fallback) {  // FP32 factor singular or out of range: factor the FP64 matrix,
                            // rebuilt densely in (per-thread local) memory -- a rare path
        double Ad[100];
        for (int e = 0; e < 100; ++e) Ad[e] = 0.0;
        for (int e = 0; e < 64; ++e) Ad[kJacPattern[e][1] * 10 + kJacPattern[e][0]] = As[e * BS];
        info = lu10_strided<double>(Ad, 1, piv);
#pragma unroll
        for (int s = 0; s < 10; ++s) x[s] = f[s];
        lus10_strided<double, double>(Ad, 1, piv, x);
      }
      if (info && (sizeof(LU) == 8 || fp64_fallback)) bad = 1;
#pragma unroll
      for (int s = 0; s < 10; ++s) xout[j + s] = x[s];
    }
    if (!queue) i += stride;
  }
  if (bad) atomicMax(info_out, 1);
}

template <typename LU>
static int launch_newton(const ChemParams& P, const ChemState& S, long n, const double* y,
                         double* f, double* x, double gamma, double tunit, int refine,
                         int* d_info, cudaStream_t s, long blocks, const double* b,
                         unsigned long long* queue) {
  constexpr int BS = kNtThreads;
  const size_t shm = (size_t)BS * (sizeof(LU) == 4 ? 64 * sizeof(double) + 100 * sizeof(float)
                                                   : 100 * sizeof(double));
  // a function attribute, not a stream operation: also legal during graph capture
  GBMV_CUDA_TRY(cudaFuncSetAttribute(chem_newton_kernel<LU, BS>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
  chem_newton_kernel<LU, BS><<<(int)blocks, BS, shm, s>>>(P, S, n, y, f, x, gamma, tunit,
                                                          refine, d_info, b, queue);
  GBMV_LAUNCH_CHECK("chem_newton_kernel");
  return GBMV_OK;
}

int chem_newton(const ChemParams& P, const ChemState& S, long n, const double* y, double* f,
                double* x, double gamma, double tunit, int lu_fp32, int refine, int* d_info,
                cudaStream_t s, int blocks_per_sm, const double* b,
                unsigned long long* queue) {
  long blk = (n + kNtThreads - 1) / kNtThreads;
  // default: a deep grid-stride grid; blocks_per_sm > 0: exactly that many resident blocks per
  // SM (a persistent grid leaving room for a kernel running beside it on another stream)
  const long cap = (long)kSM * (blocks_per_sm > 0 ? blocks_per_sm : 48);
  if (blk > cap) blk = cap;
  if (blk < 1) blk = 1;
  ProfScope ps("chem_newton", s);
  if (lu_fp32)
    return launch_newton<float>(P, S, n, y, f, x, gamma, tunit, refine, d_info, s, blk, b,
                                queue);
  return launch_newton<double>(P, S, n, y, f, x, gamma, tunit, refine, d_info, s, blk, b,
                               queue);
}

}  // namespace gbmv
