// Persistent batched DIRK integration of the chemistry network: every cell's 10-species system
//   dz/dt = F(z) = TimeUnits * inv_scale * f_chem(z * scale)
// is advanced from t0 to tout on its own adaptive step sequence, one cell per thread, in one
// launch.  This is the fast-stage work of the reference's chemistry drivers (ARKStep DIRK over
// calculate_rhs_cvklu / calculate_jacobian_cvklu with a block-diagonal direct solver,
// src/primordial_ode_main.cpp, and the rank-local MRI inner stepper of
// src/multirate_chem_hydro_main.cpp:1114-1224), carried to cell granularity.
//
// Method: a stiffly accurate ESDIRK from the table in DirkOpts (explicit first stage, one
// diagonal value gamma, b = last row of a): ARK4(3)7L[2]SA's implicit part, the table the
// reference's chemistry inputs select (`itable = 112`; C. A. Kennedy and M. H. Carpenter, Appl.
// Numer. Math. 136 (2019) 183-205), or TR-BDF2 (`itable = 102`; M. E. Hosea and L. F. Shampine,
// Appl. Numer. Math. 20 (1996) 21-37); the embedded weights give the error estimate.  Stage i
// solves z_i = y + h sum_{j<i} a_ij K_j + h gamma F(z_i) from the previous stage's value.
// Each implicit stage is solved by modified Newton with ARKODE's rules: Newton matrix A = I - gamma J reused
// across steps (set up again when gamma moved by more than dgmax, after msbp steps, or after a
// Newton failure with a matrix from an earlier step), correction scaled by
// 2/(1 + gamma/gamma_p) when gamma differs from the factored one, WRMS convergence test with
// rate estimate crate = max(0.3 crate, del/del_p), success when min(1, crate) del / nlscoef
// <= 1, divergence when del > 2.3 del_p, at most maxcor iterations.  Step control: the error
// estimate's WRMS norm dsm, eta = safety dsm^(-1/p) (p the embedding order) bounded by etamx1
// on the first step,
// growth after it, 1 right after a failure, and below by 0.1 (0.3 at most after repeated
// error failures), h <= hmax; a Newton failure with a current J cuts the step by 0.25.
// oracle/oracle.c (orc_chem_dirk_evolve) restates the same algorithm on the CPU.
//
// Batching: cells converge in uneven numbers of Newton iterations and steps.  Each lane runs a
// small state machine whose every pass evaluates F once (the common, expensive part: the
// temperature solve and 46 rate interpolations) and then acts on its own phase.  A lane whose
// cell reached tout (or failed) retires it and pulls the next cell index from a global counter
// (one warp-aggregated atomic per refill), so warps stay full until the queue drains.
// Unlike ARKODE no Jacobian is kept between matrix setups: each setup evaluates J at the
// step's state (one Jacobian per setup, a few per cent of the F work), which frees 512 bytes
// of shared memory per cell for occupancy.  WRMS weights are kept as floats (the oracle rounds
// them the same way).
// Precision: LU = float factors the Newton matrix in FP32 after power-of-two row and column
// equilibration (the scaled Jacobian spans ~20 decades); REF additionally keeps A in FP64 and
// refines each correction against FP64 residuals.  The residuals G(z), norms and error
// estimates are FP64 in every form, so Newton itself refines against the FP64 equations.
#include <algorithm>

#include "chem.cuh"
#include "chem_lu.cuh"
#include "chem_net.cuh"

namespace gbmv {

namespace {

// Lane state machine phases: F at the step start, a Newton iteration of the current stage,
// F at a converged stage.
enum : int { kPhK1 = 0, kPhNewton = 1, kPhStage = 2 };

// F at a point given in the solver's scaled variables (strided shared-memory slice X) and
// time tf: TimeUnits * f_chem plus the MRI forcing polynomial (ffast's order of summation).
template <int BS>
__device__ __forceinline__ void dirk_F(const ChemParams& P, const ChemState& S, long i,
                                       const double* X, const DirkOpts& O, double tf,
                                       bool mixed_temp, double& Ts, double& dTs,
                                       double (&f)[10]) {
  const double tunit = O.tunit;
  const long j = i * 10;
  double ya[10];
#pragma unroll
  for (int s = 0; s < 10; ++s) ya[s] = X[s * BS] * S.scale[j + s];
  if (mixed_temp)
    chem_temperature_mixed(P, ya, Ts, dTs, 9);  // up to 9 FP32 + 1 FP64 iteration
  else
    chem_temperature(P, ya, Ts, dTs);
  double k[kNRates], dk[kNRates];
  chem_rates<false>(P, Ts, k, dk);
  double r[21], sp[9];
  chem_fluxes(k, ya, r);
  chem_species(r, sp);
  const ChemAux Ax{S.mdens[i], S.imdens[i], S.cie[i], S.h2[i]};
#pragma unroll
  for (int s = 0; s < 9; ++s) f[s] = (sp[s] * S.inv_scale[j + s]) * tunit;
  double ge = chem_ge_source(P, k, ya, Ts, Ax) * S.inv_scale[j + 9];
  ge *= Ax.imdens;
  f[9] = ge * tunit;
  if (O.nforcing > 0) {
    const double tau = (tf - O.tshift) / O.tscale;
    double p = 1.0;
    for (int q = 0; q < O.nforcing; ++q) {
      const double* __restrict__ r = O.fz[q] + j;
#pragma unroll
      for (int s = 0; s < 10; ++s) f[s] += p * r[s];
      p *= tau;
    }
  }
}

}  // namespace

// 2^e as a double (|e| <= 1022): exact power-of-two scaling for the equilibration.
__device__ __forceinline__ double pow2(int e) {
  return __longlong_as_double((long long)(1023 + e) << 52);
}

// Equilibration exponent: -e with m * 2^e = x, m in [0.5, 1) (0 for zero or non-finite x),
// limited so that the combined row + column scale stays a normal double.
__device__ __forceinline__ int eq_exponent(double x) {
  if (!(x > 0.0) || !isfinite(x)) return 0;
  int ex = 0;
  frexp(x, &ex);
  return max(-500, min(500, -ex));
}

// safety dsm^(-1/p): the step-size factor from the embedded error estimate of order p
__device__ __forceinline__ double dirk_eta(double safety, double dsm, int p) {
  return p == 3 ? safety / cbrt(dsm) : (p == 2 ? safety / sqrt(dsm)
                                               : safety * pow(dsm, -1.0 / p));
}
// The same in FP32 (the mixed form): a step-size factor needs a few digits, and the FP64
// root and division cost ~40 FP64-rate instructions, issued in almost every pass of a warp
// for the one or two lanes that finish a step there
__device__ __forceinline__ double dirk_eta_f(double safety, float dsm, int p) {
  const float e = p == 3 ? cbrtf(dsm) : (p == 2 ? sqrtf(dsm) : powf(dsm, 1.f / p));
  return safety * (double)(1.f / e);
}

// Base of stage i: B = Y + sum_{j<i} (h a_ij) K_j, K_0 from shared memory, K_1.. from the
// stage store, terms added in j order (zero coefficients skipped, as the oracle does).
template <int BS>
__device__ __forceinline__ void dirk_stage_base(const DirkOpts& O, int i, double h,
                                                const double* Y, const double* K1,
                                                const double* KG, long kst, double* B) {
  const double c0 = h * O.T.a[i][0];
#pragma unroll
  for (int s = 0; s < 10; ++s) {
    double v = Y[s * BS];
    if (c0 != 0.0) v += c0 * K1[s * BS];
    B[s * BS] = v;
  }
  for (int j = 1; j < i; ++j) {
    const double cj = h * O.T.a[i][j];
    if (cj == 0.0) continue;
#pragma unroll
    for (int s = 0; s < 10; ++s) B[s * BS] += cj * KG[((j - 1) * 10 + s) * kst];
  }
}

template <typename LU, bool REF, int BS>
struct DirkLayout {
  // per-lane slices, element-major [element][BS]
  static constexpr size_t kVec = 40 * sizeof(double);                   // Y, K1, B, Z
  static constexpr size_t kEw = 10 * sizeof(float);                     // weights
  static constexpr size_t kL = 100 * sizeof(LU);                        // factor
  static constexpr size_t kA = REF ? 100 * sizeof(double) : 0;          // FP64 matrix
  static constexpr size_t kEq = sizeof(LU) == 4 ? 20 * sizeof(short) : 0;  // row/col exponents
  static constexpr size_t kPiv = 10;                                    // pivots (bytes)
  static constexpr size_t per_lane = kVec + kEw + kL + kA + kEq + kPiv;
  static constexpr size_t bytes = per_lane * BS;
};

// Newton-matrix setup of one cell: J at (Y, Ts(Y)) from rates with slopes, A = I - gam J,
// for FP32 factors power-of-two equilibrated, factored with partial pivoting; returns the LU
// info (0 or 1 + first zero pivot).
template <typename LU, bool REF, int BS>
__device__ __forceinline__ int dirk_setup(const ChemParams& P, const ChemState& S, long i,
                                       const DirkOpts& O, const double* Y, double* A, LU* L,
                                       short* EQ, double gam, double Tsy, double dTsy,
                                       int (&piv)[10]) {
  const long j = i * 10;
  double ya[10];
#pragma unroll
  for (int s = 0; s < 10; ++s) ya[s] = Y[s * BS] * S.scale[j + s];
  double k[kNRates], dk[kNRates];
  chem_rates<true>(P, Tsy, k, dk);
  const ChemAux Ax{S.mdens[i], S.imdens[i], S.cie[i], S.h2[i]};
  const double* __restrict__ sc = S.scale + j;
  const double* __restrict__ isc = S.inv_scale + j;
  const double mg = -gam * O.tunit;
#pragma unroll
  for (int e = 0; e < 100; ++e) L[e * BS] = LU(0);  // off-pattern entries
  // A = I - gamma * tunit * (isc_r J_rc sc_c): every structural entry is put once
  auto entry = [&](int row, int col, double v) {
    return (row == col ? 1.0 : 0.0) + mg * ((v * isc[row]) * sc[col]);
  };
  if (sizeof(LU) == 8) {
    chem_jacobian(P, k, dk, ya, Tsy, dTsy, Ax, [&](int row, int col, double v) {
      L[(col * 10 + row) * BS] = (LU)entry(row, col, v);
    });
  } else {
    // FP32 factor of R A C with power-of-two row scales R (row maxima to [0.5, 1)) and
    // column scales C (then column maxima to [0.5, 1)), from the FP64 entries
    double rmax[10], cmax[10];
    int er[10], ec[10];
#pragma unroll
    for (int s = 0; s < 10; ++s) rmax[s] = cmax[s] = 0.0;
    if (REF) {
      chem_jacobian(P, k, dk, ya, Tsy, dTsy, Ax, [&](int row, int col, double v) {
        const double a = entry(row, col, v);
        A[(col * 10 + row) * BS] = a;
        rmax[row] = fmax(rmax[row], fabs(a));
      });
    } else {
      chem_jacobian(P, k, dk, ya, Tsy, dTsy, Ax, [&](int row, int col, double v) {
        rmax[row] = fmax(rmax[row], fabs(entry(row, col, v)));
      });
    }
#pragma unroll
    for (int s = 0; s < 10; ++s) er[s] = eq_exponent(rmax[s]);
    if (REF) {
#pragma unroll
      for (int e = 0; e < 64; ++e) {
        const int row = kJacPattern[e][0], col = kJacPattern[e][1];
        cmax[col] = fmax(cmax[col], fabs(A[(col * 10 + row) * BS] * pow2(er[row])));
      }
#pragma unroll
      for (int s = 0; s < 10; ++s) ec[s] = eq_exponent(cmax[s]);
    } else {
      // without an FP64 copy every pass re-evaluates the Jacobian: rows only (scaled partial
      // pivoting), two passes instead of three
#pragma unroll
      for (int s = 0; s < 10; ++s) ec[s] = 0;
    }
#pragma unroll
    for (int s = 0; s < 10; ++s) {
      EQ[s * BS] = (short)er[s];
      EQ[(10 + s) * BS] = (short)ec[s];
    }
    if (REF) {
#pragma unroll
      for (int e = 0; e < 64; ++e) {
        const int row = kJacPattern[e][0], col = kJacPattern[e][1];
        L[(col * 10 + row) * BS] =
            to_lu<LU>(A[(col * 10 + row) * BS] * pow2(er[row] + ec[col]));
      }
    } else {
      chem_jacobian(P, k, dk, ya, Tsy, dTsy, Ax, [&](int row, int col, double v) {
        L[(col * 10 + row) * BS] = to_lu<LU>(entry(row, col, v) * pow2(er[row] + ec[col]));
      });
    }
  }
  return lu10_strided<LU>(L, BS, piv);
}

template <typename LU, bool REF, int BS>
__global__ void __launch_bounds__(BS) chem_dirk_kernel(ChemParams P, ChemState S, long n,
                                                       double* __restrict__ y_io,
                                                       const __grid_constant__ DirkOpts O,
                                                       unsigned long long* __restrict__ next,
                                                       int* __restrict__ stats,
                                                       int* __restrict__ nfail) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using Lay = DirkLayout<LU, REF, BS>;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  unsigned char* p = smem_raw;
  double* const Y = reinterpret_cast<double*>(p) + tid;  // state at the step start
  double* const K1 = Y + 10 * BS;                         // K_0 = F(Y)
  double* const B = K1 + 10 * BS;                         // base of the current stage
  double* const Z = B + 10 * BS;                          // current stage iterate
  // K_1 .. K_{s-2} of this lane in the stage store (L2-resident: lanes x 10 (s-2) doubles)
  const long kst = O.kstore_lanes;
  double* const KG = O.kstore + (long)blockIdx.x * BS + tid;
  p += Lay::kVec * BS;
  double* const A = reinterpret_cast<double*>(p) + tid;   // REF: FP64 Newton matrix
  p += Lay::kA * BS;
  LU* const L = reinterpret_cast<LU*>(p) + tid;           // factor
  p += Lay::kL * BS;
  float* const EW = reinterpret_cast<float*>(p) + tid;    // WRMS weights
  p += Lay::kEw * BS;
  short* const EQ = reinterpret_cast<short*>(p) + tid;    // row exponents [0,10), col [10,20)
  p += Lay::kEq * BS;
  signed char* const PV = reinterpret_cast<signed char*>(p) + tid;  // pivots
  const unsigned full = 0xffffffffu;
  const bool mixed_temp = O.mixed_temp != 0;

  long i = -1;
  bool exhausted = false;
  const int ns = O.T.s;
  int phase = kPhK1, stage = 1, m = 0;
  double t = 0.0, h = 0.0, gp = 0.0, crate = 1.0, delp = 0.0;
  double Tsy = 0.0, dTsy = 0.0, Tsc = 0.0, dTsc = 0.0;
  int nst = 0, nst_lp = 0, nef_s = 0, ncf_s = 0;
  int c_nni = 0, c_netf = 0, c_ncf = 0, c_nsetup = 0, c_nfe = 0;
  bool jcur = false, force_setup = true, last = false;
  // step start requested / Newton-matrix setup pending (the lane waits for its warp's setup
  // pass) / passes waited
  bool setup = false, pend = false;
  int waited = 0;
  const int batch = O.setup_batch;
  const int max_wait = 4 * O.setup_batch;

  while (true) {
    // ---- refill: lanes without a cell take the next indices (one atomic per warp)
    const bool want = (i < 0) && !exhausted;
    const unsigned wm = __ballot_sync(full, want);
    if (wm) {
      const int leader = __ffs(wm) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(next, (unsigned long long)__popc(wm));
      base = __shfl_sync(full, base, leader);
      if (want) {
        const unsigned long long mine =
            base + (unsigned long long)__popc(wm & ((1u << lane) - 1u));
        const unsigned long long count =
            O.list_in ? (unsigned long long)*O.list_in_n : (unsigned long long)n;
        if (mine < count) {
          i = O.list_in ? (long)O.list_in[mine] : (long)mine;
          const long j = i * 10;
          const double* __restrict__ y0 = O.y_init ? O.y_init : y_io;
#pragma unroll
          for (int s = 0; s < 10; ++s) Y[s * BS] = y0[j + s];
          Tsc = O.Ts_init ? O.Ts_init[i] : S.Ts[i];
          dTsc = O.Ts_init ? O.Ts_init[n + i] : S.dTs_ge[i];
          t = O.t0;
          h = O.h0;
          gp = 0.0;
          phase = kPhK1;
          nst = nst_lp = nef_s = ncf_s = 0;
          c_nni = c_netf = c_ncf = c_nsetup = c_nfe = 0;
          jcur = false;
          force_setup = true;
          last = false;
          setup = pend = false;
        } else {
          exhausted = true;
        }
      }
    }
    if (__all_sync(full, i < 0)) break;
    bool retire = false, failed = false;

    // ---- step start (or restart) at (t, Y): weights, predictor; a lane whose Newton matrix
    // must be set up waits for the warp's setup pass below
    if (i >= 0 && setup) {
      setup = false;
      last = (t + h >= O.tout);
      if (last) h = O.tout - t;
      Tsc = Tsy;
      dTsc = dTsy;
#pragma unroll
      for (int s = 0; s < 10; ++s) {
        const double ys = Y[s * BS];
        EW[s * BS] = (float)(1.0 / (O.rtol * fabs(ys) + O.atol));
        Z[s * BS] = ys;  // trivial predictor
      }
      const double gam = h * O.T.gamma;
      if (force_setup || nst >= nst_lp + O.msbp || !(fabs(gam / gp - 1.0) <= O.dgmax)) {
        pend = true;
        waited = 0;
      } else {
        stage = 1;
        dirk_stage_base<BS>(O, stage, h, Y, K1, KG, kst, B);
        m = 0;
        phase = kPhNewton;
      }
    }

    // ---- the warp's setup pass: the waiting lanes set up together once enough of them wait
    // (a setup costs about two F evaluations and every lane of the warp pays for it in time,
    // so one lane setting up alone stalls the other 31)
    const unsigned pm = __ballot_sync(full, pend);
    if (pm) {
      const int npend = __popc(pm);
      const int nact = __popc(__ballot_sync(full, i >= 0));
      const int wmax = __reduce_max_sync(full, pend ? waited : 0);
      const bool drained = __any_sync(full, exhausted);
      if (npend >= batch || npend == nact || wmax >= max_wait || drained) {
        if (pend) {
          pend = false;
          // Newton matrix I - gamma J with J evaluated at (Y, Ts(Y)), factored (inline: an
          // out-of-line call measured 4 % slower in the mixed form)
          const double gam = h * O.T.gamma;
          int piv[10];
          const int info =
              dirk_setup<LU, REF, BS>(P, S, i, O, Y, A, L, EQ, gam, Tsy, dTsy, piv);
#pragma unroll
          for (int s = 0; s < 10; ++s) PV[s * BS] = (signed char)piv[s];
          gp = gam;
          nst_lp = nst;
          crate = 1.0;
          jcur = true;
          force_setup = false;
          ++c_nsetup;
          if (info) {  // singular Newton matrix: a recoverable failure, cut the step and retry
            ++ncf_s;
            ++c_ncf;
            if (ncf_s >= O.maxncf || (O.maxncf_total > 0 && c_ncf >= O.maxncf_total)) {
              retire = failed = true;
            } else {
              h *= 0.25;
              force_setup = true;
              setup = true;
            }
          } else {
            stage = 1;
            dirk_stage_base<BS>(O, stage, h, Y, K1, KG, kst, B);
            m = 0;
            phase = kPhNewton;
          }
        }
      } else if (pend) {
        ++waited;
      }
    }

    // ---- one evaluation of F per pass (at Y for the first stage, else at the iterate)
    if (i >= 0 && !pend && !setup && !retire) {
      double f[10];
      const double tf = (phase == kPhK1) ? t : t + O.T.c[stage] * h;
      dirk_F<BS>(P, S, i, phase == kPhK1 ? Y : Z, O, tf, mixed_temp, Tsc, dTsc, f);
      ++c_nfe;

      if (phase == kPhK1) {
#pragma unroll
        for (int s = 0; s < 10; ++s) K1[s * BS] = f[s];
        Tsy = Tsc;
        dTsy = dTsc;
        if (h <= 0.0) {  // initial step from the derivative size
          double s2 = 0.0;
#pragma unroll
          for (int s = 0; s < 10; ++s) {
            const double v = f[s] / (O.rtol * fabs(Y[s * BS]) + O.atol);
            s2 += v * v;
          }
          const double fn = sqrt(s2 / 10.0);
          h = (fn > 0.0) ? O.h0fac / fn : O.tout - t;
        }
        if (O.hmax > 0.0 && h > O.hmax) h = O.hmax;
        setup = true;
      } else if (phase == kPhNewton) {
        const double gam = h * O.T.gamma;
        double g[10];
#pragma unroll
        for (int s = 0; s < 10; ++s) g[s] = B[s * BS] + gam * f[s] - Z[s * BS];
        int piv[10];
#pragma unroll
        for (int s = 0; s < 10; ++s) piv[s] = PV[s * BS];
        double dl[10];
        if (sizeof(LU) == 8) {
#pragma unroll
          for (int s = 0; s < 10; ++s) dl[s] = g[s];
          lus10_strided<LU, double>(L, BS, piv, dl);
        } else {
          // equilibrated FP32 solve: (R A C) u = R g, dl = C u
          LU u[10];
#pragma unroll
          for (int s = 0; s < 10; ++s) u[s] = to_lu<LU>(g[s] * pow2(EQ[s * BS]));
          lus10_strided<LU, LU>(L, BS, piv, u);
#pragma unroll
          for (int s = 0; s < 10; ++s) dl[s] = from_lu(u[s]) * pow2(EQ[(10 + s) * BS]);
          if (REF) {
            for (int it = 0; it < O.refine; ++it) {  // r = g - A dl in FP64, solve, update
              double r[10];
#pragma unroll
              for (int s = 0; s < 10; ++s) r[s] = g[s];
#pragma unroll
              for (int e = 0; e < 64; ++e) {
                const int row = kJacPattern[e][0], col = kJacPattern[e][1];
                r[row] -= A[(col * 10 + row) * BS] * dl[col];
              }
#pragma unroll
              for (int s = 0; s < 10; ++s) u[s] = to_lu<LU>(r[s] * pow2(EQ[s * BS]));
              lus10_strided<LU, LU>(L, BS, piv, u);
#pragma unroll
              for (int s = 0; s < 10; ++s) dl[s] += from_lu(u[s]) * pow2(EQ[(10 + s) * BS]);
            }
          }
        }
        if (gam != gp) {
          const double sc = 2.0 / (1.0 + gam / gp);
#pragma unroll
          for (int s = 0; s < 10; ++s) dl[s] *= sc;
        }
        double del;
        if (sizeof(LU) == 4) {  // the convergence measure in FP32 (a decision quantity)
          float s2 = 0.f;
#pragma unroll
          for (int s = 0; s < 10; ++s) {
            Z[s * BS] += dl[s];
            const float v = (float)dl[s] * EW[s * BS];
            s2 = fmaf(v, v, s2);
          }
          del = (double)sqrtf(0.1f * s2);
        } else {
          double s2 = 0.0;
#pragma unroll
          for (int s = 0; s < 10; ++s) {
            Z[s * BS] += dl[s];
            const double v = dl[s] * (double)EW[s * BS];
            s2 += v * v;
          }
          del = sqrt(s2 / 10.0);
        }
        ++m;
        ++c_nni;
        if (m > 1) crate = fmax(0.3 * crate, del / delp);
        const double dcon = fmin(crate, 1.0) * del / O.nlscoef;
        if (dcon <= 1.0 && O.deduce && stage < ns - 1) {
          // converged intermediate stage, derivative deduced from the stage equation:
          // K_stage = (z - base) / (h gamma), no F evaluation; next stage in this pass.  One
          // reciprocal and ten products: nearly every pass of a warp has a lane deducing, and
          // ten FP64 divisions there cost as much FP64-pipe time as the F evaluations saved
          const double rg = 1.0 / gam;
#pragma unroll
          for (int s = 0; s < 10; ++s)
            KG[((stage - 1) * 10 + s) * kst] = (Z[s * BS] - B[s * BS]) * rg;
          ++stage;
          dirk_stage_base<BS>(O, stage, h, Y, K1, KG, kst, B);
          m = 0;
        } else if (dcon <= 1.0) {
          phase = kPhStage;
        } else if ((m > 1 && del > 2.3 * delp) || m >= O.maxcor || !(del == del)) {
          // Newton failure: with a matrix from an earlier step set up a current one at the
          // same h, else cut the step
          ++ncf_s;
          ++c_ncf;
          if (ncf_s >= O.maxncf || (O.maxncf_total > 0 && c_ncf >= O.maxncf_total)) {
            retire = failed = true;
          } else {
            if (jcur) h *= 0.25;
            else force_setup = true;
            setup = true;
          }
        } else {
          delp = del;
        }
      } else if (stage < ns - 1) {  // kPhStage, not the last stage: keep K_stage, next stage
#pragma unroll
        for (int s = 0; s < 10; ++s) KG[((stage - 1) * 10 + s) * kst] = f[s];
        ++stage;  // predictor: the converged value of this stage, already in Z
        dirk_stage_base<BS>(O, stage, h, Y, K1, KG, kst, B);
        m = 0;
        phase = kPhNewton;
      } else {  // kPhStage of the last stage: error test
        double acc[10];
        const double e0 = O.T.e[0];
#pragma unroll
        for (int s = 0; s < 10; ++s) acc[s] = e0 * K1[s * BS];
        for (int j = 1; j < ns - 1; ++j) {
          const double ej = O.T.e[j];
          if (ej == 0.0) continue;
#pragma unroll
          for (int s = 0; s < 10; ++s) acc[s] += ej * KG[((j - 1) * 10 + s) * kst];
        }
        const double el = O.T.e[ns - 1];
        double dsm;
        float dsmf = 0.f;
        if (sizeof(LU) == 4) {  // the error norm in FP32 (an accept test and a step factor)
          float s2 = 0.f;
#pragma unroll
          for (int s = 0; s < 10; ++s) {
            const float v = (float)(h * (acc[s] + el * f[s])) * EW[s * BS];
            s2 = fmaf(v, v, s2);
          }
          dsmf = sqrtf(0.1f * s2);
          dsm = (double)dsmf;
        } else {
          double s2 = 0.0;
#pragma unroll
          for (int s = 0; s < 10; ++s) {
            const double e = h * (acc[s] + el * f[s]);
            const double v = e * (double)EW[s * BS];
            s2 += v * v;
          }
          dsm = sqrt(s2 / 10.0);
        }
        if (dsm <= 1.0) {
          ++nst;
          t = last ? O.tout : t + h;
#pragma unroll
          for (int s = 0; s < 10; ++s) {
            Y[s * BS] = Z[s * BS];
            K1[s * BS] = f[s];  // stiffly accurate: F(last stage) = F(y_{n+1})
          }
          Tsy = Tsc;
          dTsy = dTsc;
          jcur = false;
          double eta = !(dsm > 0.0) ? 1.0e300
                       : (sizeof(LU) == 4 ? dirk_eta_f(O.safety, dsmf, O.T.p)
                                          : dirk_eta(O.safety, dsm, O.T.p));
          eta = fmin(eta, nst == 1 ? O.etamx1 : O.growth);
          if (nef_s > 0 || ncf_s > 0) eta = fmin(eta, 1.0);
          h *= eta;
          if (O.hmax > 0.0 && h > O.hmax) h = O.hmax;
          nef_s = ncf_s = 0;
          if (last) retire = true;
          else if (nst >= O.max_steps) retire = failed = true;
          else setup = true;
        } else {
          ++nef_s;
          ++c_netf;
          if (nef_s >= O.maxnef) {
            retire = failed = true;
          } else {
            double eta = fmax(0.1, sizeof(LU) == 4 ? dirk_eta_f(O.safety, dsmf, O.T.p)
                                                   : dirk_eta(O.safety, dsm, O.T.p));
            if (nef_s >= 2) eta = fmin(eta, 0.3);
            h *= eta;
            setup = true;
          }
        }
      }
    }

    if (retire) {
      const long j = i * 10;
#pragma unroll
      for (int s = 0; s < 10; ++s) y_io[j + s] = Y[s * BS];
      S.Ts[i] = Tsy;
      S.dTs_ge[i] = dTsy;
      if (stats) {
        int* st = stats + i * kDirkStats;
        st[0] = nst;
        st[1] = c_nni;
        st[2] = c_netf;
        st[3] = c_ncf;
        st[4] = c_nsetup;
        st[5] = c_nsetup;  // every setup evaluates the Jacobian
        st[6] = c_nfe;
        st[7] = failed ? 1 : 0;
      }
      if (failed) {
        if (O.list_out) O.list_out[atomicAdd(O.list_out_n, 1)] = (int)i;  // second pass
        else atomicAdd(nfail, 1);
      }
      i = -1;
      setup = pend = false;
    }
  }
}

// Resident blocks per SM of one instantiation (0 if it does not fit).
template <typename LU, bool REF, int BS>
static int dirk_blocks_per_sm(int* per_sm) {
  const size_t shm = DirkLayout<LU, REF, BS>::bytes;
  GBMV_CUDA_TRY(cudaFuncSetAttribute(chem_dirk_kernel<LU, REF, BS>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
  GBMV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      per_sm, chem_dirk_kernel<LU, REF, BS>, BS, shm));
  return GBMV_OK;
}

template <typename LU, bool REF, int BS>
static int launch_dirk(const ChemParams& P, const ChemState& S, long n, double* y,
                       const DirkOpts& O, unsigned long long* d_next, int* stats, int* d_nfail,
                       int nsm, cudaStream_t s) {
  const size_t shm = DirkLayout<LU, REF, BS>::bytes;
  int per_sm = 0;
  int rc = dirk_blocks_per_sm<LU, REF, BS>(&per_sm);
  if (rc) return rc;
  if (per_sm < 1) return GBMV_EUNSUPPORTED;
  long blocks = (long)nsm * per_sm;
  const long need = (n + BS - 1) / BS;
  if (blocks > need) blocks = need;
  if (O.T.s > 2 && (!O.kstore || blocks * BS > O.kstore_lanes)) {
    set_error("DIRK stage store of %ld lanes is smaller than the launch (%ld lanes)",
              O.kstore_lanes, blocks * BS);
    return GBMV_EINVAL;
  }
  chem_dirk_kernel<LU, REF, BS><<<(int)blocks, BS, shm, s>>>(P, S, n, y, O, d_next, stats,
                                                             d_nfail);
  GBMV_LAUNCH_CHECK("chem_dirk_kernel");
  return GBMV_OK;
}

template <typename LU, bool REF>
static int launch_dirk_bs(int block, const ChemParams& P, const ChemState& S, long n, double* y,
                          const DirkOpts& O, unsigned long long* d_next, int* stats,
                          int* d_nfail, int nsm, cudaStream_t s) {
  switch (block) {
    case 32: return launch_dirk<LU, REF, 32>(P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
    case 64: return launch_dirk<LU, REF, 64>(P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
    case 128: return launch_dirk<LU, REF, 128>(P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
    default: return GBMV_EINVAL;
  }
}

template <typename LU, bool REF>
static int max_lanes_bs(int nsm, long* lanes) {
  const int bs[3] = {32, 64, 128};
  for (int k = 0; k < 3; ++k) {
    int per_sm = 0;
    int rc = k == 0 ? dirk_blocks_per_sm<LU, REF, 32>(&per_sm)
                    : (k == 1 ? dirk_blocks_per_sm<LU, REF, 64>(&per_sm)
                              : dirk_blocks_per_sm<LU, REF, 128>(&per_sm));
    if (rc) return rc;
    const long l = (long)nsm * per_sm * bs[k];
    if (l > *lanes) *lanes = l;
  }
  return GBMV_OK;
}

long chem_dirk_max_lanes() {
  int dev = 0, nsm = kSM;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  long lanes = 0;
  if (max_lanes_bs<double, false>(nsm, &lanes) || max_lanes_bs<float, false>(nsm, &lanes) ||
      max_lanes_bs<float, true>(nsm, &lanes))
    return -1;
  return lanes;
}

// ---- cost order: cells with the largest initial derivative first
//
// A persistent launch ends when its last lane finishes, and the cells' costs differ by 30x
// (tens to thousands of Newton iterations), so cells pulled last in index order leave most
// lanes idle at the end.  The initial derivative's WRMS size ||F(z0)|| ranks the cells' costs
// well (Spearman 0.71 against their F-evaluation counts on the static-chemistry inputs), so
// the cells are bucketed by it (4 buckets per decade) and taken largest first: a greedy-refill
// model with the measured per-cell costs puts the makespan 17 % lower (true-cost order: 21 %).
// Per-cell work does not depend on the order, so results are the same bit for bit.
__global__ void __launch_bounds__(128) dirk_order_key_kernel(ChemParams P, ChemState S, long n,
                                                             const double* __restrict__ y,
                                                             const __grid_constant__ DirkOpts O,
                                                             unsigned char* __restrict__ bucket,
                                                             int* __restrict__ hist) {
  __shared__ int sh[kDirkOrderBuckets];
  for (int b = threadIdx.x; b < kDirkOrderBuckets; b += blockDim.x) sh[b] = 0;
  __syncthreads();
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
       c += (long)gridDim.x * blockDim.x) {
    const long i = O.list_in ? (long)O.list_in[c] : c;
    double z[10], f[10];
#pragma unroll
    for (int s = 0; s < 10; ++s) z[s] = y[i * 10 + s];
    double Ts = S.Ts[i], dTs = 0.0;  // a copy: the carried state is not touched
    dirk_F<1>(P, S, i, z, O, O.t0, true, Ts, dTs, f);
    float s2 = 0.f;
#pragma unroll
    for (int s = 0; s < 10; ++s) {
      const float v = (float)(f[s] / (O.rtol * fabs(z[s]) + O.atol));
      s2 = fmaf(v, v, s2);
    }
    // bucket 0 for ||F|| >= 1e12, one per quarter decade below, the last for 0 or NaN
    const float lg = log10f(sqrtf(0.1f * s2));
    int b = (lg == lg) ? (int)floorf(4.f * (12.f - lg)) : kDirkOrderBuckets - 1;
    b = b < 0 ? 0 : (b >= kDirkOrderBuckets ? kDirkOrderBuckets - 1 : b);
    bucket[c] = (unsigned char)b;
    atomicAdd(&sh[b], 1);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kDirkOrderBuckets; b += blockDim.x)
    if (sh[b]) atomicAdd(&hist[b], sh[b]);
}

__global__ void dirk_order_scan_kernel(long n, const int* __restrict__ hist,
                                       int* __restrict__ offset, int* __restrict__ count) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int acc = 0;
    for (int b = 0; b < kDirkOrderBuckets; ++b) {
      offset[b] = acc;
      acc += hist[b];
    }
    *count = (int)n;
  }
}

__global__ void __launch_bounds__(256) dirk_order_scatter_kernel(
    long n, const int* __restrict__ cells, const unsigned char* __restrict__ bucket,
    int* __restrict__ offset, int* __restrict__ list) {
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
       c += (long)gridDim.x * blockDim.x)
    list[atomicAdd(&offset[bucket[c]], 1)] = cells ? cells[c] : (int)c;
}

// the cell list of O in cost order (O.list_in, when set, is reordered; else cells 0..n-1)
static int dirk_order(const ChemParams& P, const ChemState& S, long n, const double* y,
                      const DirkOpts& O, const DirkOrder& B, int nsm, cudaStream_t s) {
  GBMV_CUDA_TRY(cudaMemsetAsync(B.hist, 0, sizeof(int) * kDirkOrderBuckets, s));
  const int blocks = (int)std::min<long>((n + 127) / 128, (long)nsm * 8);
  dirk_order_key_kernel<<<std::max(blocks, 1), 128, 0, s>>>(P, S, n, y, O, B.bucket, B.hist);
  GBMV_LAUNCH_CHECK("dirk_order_key_kernel");
  dirk_order_scan_kernel<<<1, 32, 0, s>>>(n, B.hist, B.offset, B.count);
  GBMV_LAUNCH_CHECK("dirk_order_scan_kernel");
  const int sb = (int)std::min<long>((n + 255) / 256, (long)nsm * 8);
  dirk_order_scatter_kernel<<<std::max(sb, 1), 256, 0, s>>>(n, O.list_in, B.bucket, B.offset,
                                                            B.list);
  GBMV_LAUNCH_CHECK("dirk_order_scatter_kernel");
  return GBMV_OK;
}

int chem_dirk(const ChemParams& P, const ChemState& S, long n, double* y, const DirkOpts& Oin,
              int lu_fp32, int block, unsigned long long* d_next, int* stats, int* d_nfail,
              cudaStream_t s, const DirkRetry* retry, const DirkOrder* order) {
  GBMV_CUDA_TRY(cudaMemsetAsync(d_next, 0, sizeof(unsigned long long), s));
  int dev = 0, nsm = kSM;
  GBMV_CUDA_TRY(cudaGetDevice(&dev));
  GBMV_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  ProfScope ps("chem_dirk", s);
  DirkOpts O = Oin;
  if (order && Oin.order && !Oin.list_in && n > 0) {
    const int rc = dirk_order(P, S, n, y, Oin, *order, nsm, s);
    if (rc) return rc;
    O.list_in = order->list;
    O.list_in_n = order->count;
  }
  if (!lu_fp32)
    return launch_dirk_bs<double, false>(block, P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
  if (O.refine > 0)
    return launch_dirk_bs<float, true>(block, P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
  if (!retry)
    return launch_dirk_bs<float, false>(block, P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
  // FP32 pass over every cell, its start state kept; a cell it cannot finish (its Newton
  // iterations keep failing on an FP32 factor too poor for the block) is listed, and a pass
  // with the FP64 factor integrates the listed cells again from their start state.  Both
  // passes are asynchronous launches; the second finds an empty list when nothing failed.
  GBMV_CUDA_TRY(cudaMemcpyAsync(retry->y0, y, sizeof(double) * 10 * n, cudaMemcpyDeviceToDevice,
                                s));
  GBMV_CUDA_TRY(cudaMemcpyAsync(retry->ts0, S.Ts, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                s));
  GBMV_CUDA_TRY(cudaMemcpyAsync(retry->ts0 + n, S.dTs_ge, sizeof(double) * n,
                                cudaMemcpyDeviceToDevice, s));
  GBMV_CUDA_TRY(cudaMemsetAsync(retry->count, 0, sizeof(int), s));
  DirkOpts Om = O;
  Om.list_out = retry->list;
  Om.list_out_n = retry->count;
  // The FP32 pass gives a cell up after kDirkFp32MaxNcf Newton failures in one step (the
  // caller's maxncf applies in the second pass).  With the mixed F's single FP64 temperature
  // iteration the FP32 pass is faster per cell, but the few cells whose FP32 factor keeps
  // failing would otherwise crawl on in tiny steps and become the launch's tail (64^3: FP32
  // pass alone 1.78 s with the caller's 10; 1.14 s for both passes at 5, 195 cells retried;
  // 1.18 s at 2 and 3)
  Om.maxncf = O.maxncf < kDirkFp32MaxNcf ? O.maxncf : kDirkFp32MaxNcf;
  // With deduced stage derivatives the FP32 factor's inexact corrections enter the next
  // stages' bases, and on the few blocks whose species span ~50 decades that shows as repeated
  // Newton failures (64^3: two cells with 10 and 14 over the run, against 0-1 for every other
  // form, ending 2e-3 and 3e-2 from a tight-tolerance solution; with the FP64 factor 4e-5 and
  // 1.4e-4, as the evaluated forms).  So the FP32 pass also gives up a cell after
  // kDirkFp32MaxNcfTotal Newton failures in all, and the FP64 factor integrates it
  Om.maxncf_total = O.deduce ? kDirkFp32MaxNcfTotal : 0;
  int rc = launch_dirk_bs<float, false>(block, P, S, n, y, Om, d_next, stats, d_nfail, nsm, s);
  if (rc) return rc;
  GBMV_CUDA_TRY(cudaMemsetAsync(d_next, 0, sizeof(unsigned long long), s));
  DirkOpts Of = O;
  Of.list_in = retry->list;
  Of.list_in_n = retry->count;
  Of.y_init = retry->y0;
  Of.Ts_init = retry->ts0;
  // the retried cells keep the mixed temperature solve (up to 9 FP32 + 1 FP64 iterations)
  // with the FP64 factor: a few hundred hard cells, one lane each, whose pass is
  // latency-bound by its F evaluations -- the ten FP64 temperature iterations of the FP64 form
  // were 70 % of them (retry pass 210 -> 95 ms, 64^3 call 1.31 -> 1.19 s)
  Of.mixed_temp = 1;
  return launch_dirk<double, false, 64>(P, S, n, y, Of, d_next, stats, d_nfail, nsm, s);
}

}  // namespace gbmv
