// Chemistry kernels (part b): per-cell primordial network source and analytic Jacobian, the
// auxiliary setup arrays, and the Dengo scaling glue.  One thread per cell; tables read
// through the read-only path from a bin-major block (all 50 values of a bin contiguous, so a
// cell's two bracketing bins are 800 contiguous bytes; the 400 KB block stays L2-resident).
#include "chem.cuh"
#include "chem_net.cuh"

#include <algorithm>

namespace gbmv {

__global__ void __launch_bounds__(128) chem_rhs_kernel(ChemParams P, ChemState S, long n,
                                                       const double* __restrict__ y,
                                                       double* __restrict__ ydot, double tunit) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const long j = i * 10;
    double ya[10];
#pragma unroll
    for (int s = 0; s < 10; ++s) ya[s] = y[j + s] * S.scale[j + s];
    double Ts = S.Ts[i], dTs = 0.0;
    chem_temperature(P, ya, Ts, dTs);
    S.Ts[i] = Ts;
    S.dTs_ge[i] = dTs;
    double k[kNRates], dk[kNRates];
    chem_rates<false>(P, Ts, k, dk);
    double r[21], sp[9];
    chem_fluxes(k, ya, r);
    chem_species(r, sp);
    const ChemAux A{S.mdens[i], S.imdens[i], S.cie[i], S.h2[i]};
    double out[10];
#pragma unroll
    for (int s = 0; s < 9; ++s) out[s] = sp[s] * S.inv_scale[j + s];
    out[9] = chem_ge_source(P, k, ya, Ts, A) * S.inv_scale[j + 9];
    out[9] *= A.imdens;
#pragma unroll
    for (int s = 0; s < 10; ++s) ydot[j + s] = out[s] * tunit;
  }
}

__global__ void __launch_bounds__(128) chem_jac_kernel(ChemParams P, ChemState S, long n,
                                                       const double* __restrict__ y,
                                                       double* __restrict__ J, double tunit) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const long j = i * 10;
    const double* __restrict__ sc = S.scale + j;
    const double* __restrict__ isc = S.inv_scale + j;
    double ya[10];
#pragma unroll
    for (int s = 0; s < 10; ++s) ya[s] = y[j + s] * sc[s];
    const double T = S.Ts[i];
    double k[kNRates], dk[kNRates];
    chem_rates<true>(P, T, k, dk);
    const ChemAux A{S.mdens[i], S.imdens[i], S.cie[i], S.h2[i]};
    double* out = J + 100 * i;
#pragma unroll
    for (int e = 0; e < 100; ++e) out[e] = 0.0;
    chem_jacobian(P, k, dk, ya, T, S.dTs_ge[i], A, [&](int row, int col, double v) {
      out[col * 10 + row] = (v * (isc[row] * sc[col])) * tunit;
    });
  }
}

// Jacobian-vector products with the chemistry Jacobian of chem_jac_kernel (same entries, same
// rounding of each entry): TRANS = false: out = J dy; TRANS = true: out = J^T v.  The
// derivatives of the chemistry source for Newton-Krylov (JVP) and adjoints (VJP), without
// forming J in HBM.
template <bool TRANS>
__global__ void __launch_bounds__(128) chem_jvp_kernel(ChemParams P, ChemState S, long n,
                                                       const double* __restrict__ y,
                                                       const double* __restrict__ x,
                                                       double* __restrict__ out, double tunit) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const long j = i * 10;
    const double* __restrict__ sc = S.scale + j;
    const double* __restrict__ isc = S.inv_scale + j;
    double ya[10], xv[10], acc[10];
#pragma unroll
    for (int s = 0; s < 10; ++s) {
      ya[s] = y[j + s] * sc[s];
      xv[s] = x[j + s];
      acc[s] = 0.0;
    }
    const double T = S.Ts[i];
    double k[kNRates], dk[kNRates];
    chem_rates<true>(P, T, k, dk);
    const ChemAux A{S.mdens[i], S.imdens[i], S.cie[i], S.h2[i]};
    chem_jacobian(P, k, dk, ya, T, S.dTs_ge[i], A, [&](int row, int col, double v) {
      const double e = (v * (isc[row] * sc[col])) * tunit;
      if (TRANS) acc[col] += e * xv[row];
      else acc[row] += e * xv[col];
    });
#pragma unroll
    for (int s = 0; s < 10; ++s) out[j + s] = acc[s];
  }
}

// setting_up_extra_variables (src/raja_primordial_network.cpp:1969-2018)
__global__ void chem_aux_kernel(ChemState S, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const double* in = S.scale + 10 * i;
    double m = 0.0;
    m += in[0] * 2.0;
    m += in[1] * 2.0;
    m += in[2] * 1.00794;
    m += in[3] * 1.00794;
    m += in[4] * 1.00794;
    m += in[5] * 4.002602;
    m += in[6] * 4.002602;
    m += in[7] * 4.002602;
    m *= 1.67e-24;
    double tau = pow(m / 3.3e-8, 2.8);
    tau = fmax(tau, 1.0e-5);
    S.mdens[i] = m;
    S.imdens[i] = 1.0 / m;
    S.cie[i] = fmin(1.0, (1.0 - exp(-tau)) / tau);
    S.h2[i] = fmin(1.0, pow(m / 1.34e-14, -0.45));
  }
}

// prepare_Dengo_structures (src/primordial_static.cpp:227-259), per element
__global__ void chem_prepare_kernel(ChemState S, double* __restrict__ chem, long nel) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nel;
       e += (long)gridDim.x * blockDim.x) {
    const double c = chem[e];
    S.scale[e] = c;
    S.inv_scale[e] = 1.0 / c;
    chem[e] = 1.0;
  }
}

__global__ void chem_set_scale_kernel(ChemState S, const double* __restrict__ scale, long nel) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nel;
       e += (long)gridDim.x * blockDim.x) {
    const double c = scale[e];
    S.scale[e] = c;
    S.inv_scale[e] = 1.0 / c;
  }
}

// apply (mode 0: chem *= scale) / unapply (mode 1: chem /= scale), src/primordial_static.cpp:264-318
__global__ void chem_scaling_kernel(const double* __restrict__ scale, double* __restrict__ chem,
                                    long nel, int mode) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nel;
       e += (long)gridDim.x * blockDim.x) {
    if (mode == 0) chem[e] *= scale[e];
    else chem[e] /= scale[e];
  }
}

// fslow/fexpl preamble, fused: chem *= scale (apply_Dengo_scaling) and
// et = ge/EnergyUnits + 0.5/rho*|m|^2 (src/multirate_chem_hydro_main.cpp:1028-1042).
// Also PostprocessStep (src/imex_chem_hydro_main.cpp:1032-1041) with apply_only = 0 and
// restore = 1, which leaves chem unscaled: chem*scale/scale, as the reference's apply/unapply pair.
__global__ void energy_sync_kernel(const double* __restrict__ scale, double* __restrict__ chem,
                                   const double* __restrict__ rho, const double* __restrict__ mx,
                                   const double* __restrict__ my, const double* __restrict__ mz,
                                   double* __restrict__ et, long n, int nchem, double eunit_scale,
                                   int restore) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    double* c = chem + (long)nchem * i;
    const double* s = scale + (long)nchem * i;
    double ge;
    if (restore == 2) {  // et only: the chemistry component stays in its scaled units
      ge = c[nchem - 1] * s[nchem - 1];
    } else {
      for (int v = 0; v < nchem; ++v) c[v] *= s[v];
      ge = c[nchem - 1];
    }
    const double r = rho[i], a = mx[i], b = my[i], d = mz[i];
    // the reference's expression with its roundings (no FMA contraction): bit-equal et
    const double m2 = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(d, d));
    et[i] = __dadd_rn(__dmul_rn(ge, eunit_scale), __dmul_rn(0.5 / r, m2));
    if (restore == 1)
      for (int v = 0; v < nchem; ++v) c[v] /= s[v];
  }
}

// fslow/fexpl epilogue: chemdot[ge] = etdot, etdot = 0, chem /= scale
// (src/multirate_chem_hydro_main.cpp:1061-1077).
// exact = 1 divides by scale as the reference's unapply does; exact = 0 multiplies by
// inv_scale (one rounding apart, and no FP64 division); exact = 2: nothing to undo (the
// mixed form applies the scale inside the WENO primitives pass and never rescales w[5]).
__global__ void energy_epilogue_kernel(const double* __restrict__ scale,
                                       const double* __restrict__ inv_scale,
                                       double* __restrict__ chem, double* __restrict__ chemdot,
                                       double* __restrict__ etdot, long n, int nchem, int exact) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    chemdot[(long)nchem * i + nchem - 1] = etdot[i];
    etdot[i] = 0.0;
    double* c = chem + (long)nchem * i;
    if (exact == 1) {
      const double* s = scale + (long)nchem * i;
      for (int v = 0; v < nchem; ++v) c[v] /= s[v];
    } else if (exact == 0) {
      const double* s = inv_scale + (long)nchem * i;
      for (int v = 0; v < nchem; ++v) c[v] *= s[v];
    }  // exact == 2: the chemistry component was never rescaled
  }
}

static int grid_for(long n, int threads) {
  long b = (n + threads - 1) / threads;
  const long cap = (long)kSM * 32;
  if (b < 1) b = 1;
  return (int)(b < cap ? b : cap);
}

int chem_rhs(const ChemParams& P, const ChemState& S, long n, const double* y, double* ydot,
             double tunit, cudaStream_t s) {
  ProfScope ps("chem_rhs", s);
  chem_rhs_kernel<<<grid_for(n, 128), 128, 0, s>>>(P, S, n, y, ydot, tunit);
  GBMV_LAUNCH_CHECK("chem_rhs_kernel");
  return GBMV_OK;
}

int chem_jac(const ChemParams& P, const ChemState& S, long n, const double* y, double* J,
             double tunit, cudaStream_t s) {
  ProfScope ps("chem_jac", s);
  chem_jac_kernel<<<grid_for(n, 128), 128, 0, s>>>(P, S, n, y, J, tunit);
  GBMV_LAUNCH_CHECK("chem_jac_kernel");
  return GBMV_OK;
}

int chem_jvp(const ChemParams& P, const ChemState& S, long n, const double* y, const double* x,
             double* out, double tunit, int transpose, cudaStream_t s) {
  ProfScope ps(transpose ? "vjp" : "jvp", s);
  if (transpose)
    chem_jvp_kernel<true><<<grid_for(n, 128), 128, 0, s>>>(P, S, n, y, x, out, tunit);
  else
    chem_jvp_kernel<false><<<grid_for(n, 128), 128, 0, s>>>(P, S, n, y, x, out, tunit);
  GBMV_LAUNCH_CHECK("chem_jvp_kernel");
  return GBMV_OK;
}

int chem_aux(const ChemState& S, long n, cudaStream_t s) {
  chem_aux_kernel<<<grid_for(n, 256), 256, 0, s>>>(S, n);
  GBMV_LAUNCH_CHECK("chem_aux_kernel");
  return GBMV_OK;
}

int chem_prepare(const ChemState& S, double* chem, long n, cudaStream_t s) {
  chem_prepare_kernel<<<grid_for(10 * n, 256), 256, 0, s>>>(S, chem, 10 * n);
  GBMV_LAUNCH_CHECK("chem_prepare_kernel");
  return chem_aux(S, n, s);
}

int chem_set_scale(const ChemState& S, const double* scale, long n, cudaStream_t s) {
  chem_set_scale_kernel<<<grid_for(10 * n, 256), 256, 0, s>>>(S, scale, 10 * n);
  GBMV_LAUNCH_CHECK("chem_set_scale_kernel");
  return chem_aux(S, n, s);
}

int chem_scaling(const ChemState& S, double* chem, long n, int mode, cudaStream_t s) {
  chem_scaling_kernel<<<grid_for(10 * n, 256), 256, 0, s>>>(S.scale, chem, 10 * n, mode);
  GBMV_LAUNCH_CHECK("chem_scaling_kernel");
  return GBMV_OK;
}

int energy_sync(const ChemState& S, double* const* w, long n, int nchem, double eunit_scale,
                int restore, cudaStream_t s) {
  ProfScope ps("glue", s);
  energy_sync_kernel<<<grid_for(n, 256), 256, 0, s>>>(S.scale, w[5], w[0], w[1], w[2], w[3], w[4],
                                                       n, nchem, eunit_scale, restore);
  GBMV_LAUNCH_CHECK("energy_sync_kernel");
  return GBMV_OK;
}

int energy_epilogue(const ChemState& S, double* chem, double* chemdot, double* etdot, long n,
                    int nchem, int exact, cudaStream_t s) {
  ProfScope ps("glue", s);
  energy_epilogue_kernel<<<grid_for(n, 256), 256, 0, s>>>(S.scale, S.inv_scale, chem, chemdot,
                                                           etdot, n, nchem, exact);
  GBMV_LAUNCH_CHECK("energy_epilogue_kernel");
  return GBMV_OK;
}

}  // namespace gbmv

namespace gbmv {

// MRI forcing of the fast right-hand side (ffast, src/multirate_chem_hydro_main.cpp:921-944):
// for every ManyVector component k, wdot_k <- wdot_k + sum_i c_i forcing_i,k, summed in the
// order of N_VLinearCombination with X[0] == z and c[0] == 1 (z += c_i X_i, i = 1, 2, ...).
// blockIdx.y = component; components 0-4 have ncell entries, component 5 has 10 ncell.
__global__ void mri_forcing_kernel(long ncell, int nf, ForcingSet F, DevFields6 wdot) {
  const int k = blockIdx.y;
  const long len = (k == 5) ? 10 * ncell : ncell;
  double* __restrict__ z = wdot.f[k];
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < len;
       j += (long)gridDim.x * blockDim.x) {
    double acc = z[j];
    for (int i = 0; i < nf; ++i) acc += F.c[i] * F.x[i][k][j];
    z[j] = acc;
  }
}

__global__ void zero_fluid_kernel(long ncell, DevFields6 wdot) {
  const int k = blockIdx.y;
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < ncell;
       j += (long)gridDim.x * blockDim.x)
    wdot.f[k][j] = 0.0;
}

int mri_forcing(long ncell, const ForcingSet& F, int nf, const DevFields6& wdot, bool zero_fluid,
                int ncomp, cudaStream_t s) {
  const int threads = 256;
  const long blocks_x = std::min<long>((10 * ncell + threads - 1) / threads, (long)kSM * 16);
  ProfScope ps("glue", s);
  if (zero_fluid) {
    zero_fluid_kernel<<<dim3((unsigned)std::min<long>((ncell + threads - 1) / threads, (long)kSM * 16), 5),
                        threads, 0, s>>>(ncell, wdot);
    GBMV_LAUNCH_CHECK("zero_fluid_kernel");
  }
  if (nf > 0) {
    mri_forcing_kernel<<<dim3((unsigned)blocks_x, ncomp), threads, 0, s>>>(ncell, nf, F, wdot);
    GBMV_LAUNCH_CHECK("mri_forcing_kernel");
  }
  return GBMV_OK;
}

}  // namespace gbmv
