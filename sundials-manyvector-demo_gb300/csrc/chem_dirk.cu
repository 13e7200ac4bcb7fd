// Persistent batched DIRK integration of the chemistry network: every cell's 10-species system
//   dz/dt = F(z) = TimeUnits * inv_scale * f_chem(z * scale)
// is advanced from t0 to tout on its own adaptive step sequence, one cell per thread, in one
// launch.  This is the fast-stage work of the reference's chemistry drivers (ARKStep DIRK over
// calculate_rhs_cvklu / calculate_jacobian_cvklu with a block-diagonal direct solver,
// src/primordial_ode_main.cpp, and the rank-local MRI inner stepper of
// src/multirate_chem_hydro_main.cpp:1114-1224), carried to cell granularity.
//
// Method: TR-BDF2 written as an ESDIRK (explicit first stage, equal diagonal gd = 1 - 1/sqrt 2,
// stiffly accurate, L-stable), its order-3 companion weights giving the embedded error
// estimate (M. E. Hosea and L. F. Shampine, Appl. Numer. Math. 20 (1996) 21-37).  Each implicit
// stage is solved by modified Newton with ARKODE's rules: Newton matrix A = I - gamma J reused
// across steps (refactored when gamma moved by more than dgmax or after msbp steps, J
// re-evaluated after msbj steps or a Newton failure with a stale J), correction scaled by
// 2/(1 + gamma/gamma_p) when gamma differs from the factored one, WRMS convergence test with
// rate estimate crate = max(0.3 crate, del/del_p), success when min(1, crate) del / nlscoef
// <= 1, divergence when del > 2.3 del_p, at most maxcor iterations.  Step control: the error
// estimate's WRMS norm dsm, eta = safety / cbrt(dsm) bounded by etamx1 on the first step,
// growth after it, 1 right after a failure, and below by 0.1 (0.3 at most after repeated
// error failures), h <= hmax; a Newton failure with a current J cuts the step by 0.25.
// oracle/oracle.c (orc_chem_dirk_evolve) restates the same algorithm on the CPU.
//
// Batching: cells converge in uneven numbers of Newton iterations and steps.  Each lane runs a
// small state machine whose every pass evaluates F once (the common, expensive part: the
// temperature solve and 46 rate interpolations) and then acts on its own phase.  A lane whose
// cell reached tout (or failed) retires it and pulls the next cell index from a global counter
// (one warp-aggregated atomic per refill), so warps stay full until the queue drains.
// Precision: LU = float factors the Newton matrix in FP32 and (with refine > 0) refines the
// correction against FP64 residuals of A computed from the FP64 Jacobian; residuals G(z),
// norms and error estimates are FP64 in both forms.
#include "chem.cuh"
#include "chem_lu.cuh"
#include "chem_net.cuh"

namespace gbmv {

namespace {

// TR-BDF2 coefficients (ESDIRK form): A = [[0,0,0],[gd,gd,0],[w,w,gd]], b = (w, w, gd),
// bhat = ((1-w)/3, (3w+1)/3, gd/3); e = b - bhat.
constexpr double kSqrt2 = 1.4142135623730951;
constexpr double kGd = (2.0 - kSqrt2) / 2.0;
constexpr double kW = kSqrt2 / 4.0;
constexpr double kE1 = kW - (1.0 - kW) / 3.0;
constexpr double kE2 = kW - (3.0 * kW + 1.0) / 3.0;
constexpr double kE3 = kGd - kGd / 3.0;

enum : int { kPhK1 = 0, kPhNewton = 1, kPhK2 = 2, kPhK3 = 3 };

// F at a point given in the solver's scaled variables (strided shared-memory slice X).
template <int BS>
__device__ __forceinline__ void dirk_F(const ChemParams& P, const ChemState& S, long i,
                                       const double* X, double tunit, bool mixed_temp,
                                       double& Ts, double& dTs, double (&f)[10]) {
  const long j = i * 10;
  double ya[10];
#pragma unroll
  for (int s = 0; s < 10; ++s) ya[s] = X[s * BS] * S.scale[j + s];
  if (mixed_temp)
    chem_temperature_mixed(P, ya, Ts, dTs, 8);
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
}

}  // namespace

template <typename LU, int BS>
__global__ void __launch_bounds__(BS) chem_dirk_kernel(ChemParams P, ChemState S, long n,
                                                       double* __restrict__ y_io, DirkOpts O,
                                                       unsigned long long* __restrict__ next,
                                                       int* __restrict__ stats,
                                                       int* __restrict__ nfail) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  double* const dbase = reinterpret_cast<double*>(smem_raw);
  double* const Jm = dbase + tid;            // [64][BS] scaled Jacobian dF/dz (pattern order)
  double* const Y = dbase + 64 * BS + tid;   // [10][BS] state at the step start
  double* const K1 = Y + 10 * BS;            // F(Y)
  double* const K2 = K1 + 10 * BS;           // F(stage 2)
  double* const EW = K2 + 10 * BS;           // WRMS weights 1 / (rtol |Y| + atol)
  double* const Z = EW + 10 * BS;            // current stage iterate
  LU* const L = reinterpret_cast<LU*>(dbase + 114 * BS) + tid;  // [100][BS] factor
  int* const PV = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(dbase + 114 * BS) +
                                         sizeof(LU) * 100 * BS) + tid;  // [10][BS] pivots
  const unsigned full = 0xffffffffu;
  const bool mixed_temp = O.mixed_temp != 0;

  long i = -1;
  bool exhausted = false;
  int phase = kPhK1, stage = 2, m = 0;
  double t = 0.0, h = 0.0, gp = 0.0, crate = 1.0, delp = 0.0;
  double Tsy = 0.0, dTsy = 0.0, Tsc = 0.0, dTsc = 0.0;
  int nst = 0, nst_lp = 0, nst_lj = 0, nef_s = 0, ncf_s = 0;
  int c_nni = 0, c_netf = 0, c_ncf = 0, c_nsetup = 0, c_nje = 0, c_nfe = 0;
  bool jcur = false, need_jac = true, last = false;

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
        if (mine < (unsigned long long)n) {
          i = (long)mine;
          const long j = i * 10;
#pragma unroll
          for (int s = 0; s < 10; ++s) Y[s * BS] = y_io[j + s];
          Tsc = S.Ts[i];
          dTsc = S.dTs_ge[i];
          t = O.t0;
          h = O.h0;
          gp = 0.0;
          phase = kPhK1;
          nst = nst_lp = nst_lj = nef_s = ncf_s = 0;
          c_nni = c_netf = c_ncf = c_nsetup = c_nje = c_nfe = 0;
          jcur = false;
          need_jac = true;
          last = false;
        } else {
          exhausted = true;
        }
      }
    }
    if (__all_sync(full, i < 0)) break;
    if (i < 0) continue;

    // ---- one evaluation of F per pass (at Y for the first stage, else at the iterate)
    double f[10];
    dirk_F<BS>(P, S, i, phase == kPhK1 ? Y : Z, O.tunit, mixed_temp, Tsc, dTsc, f);
    ++c_nfe;

    bool setup = false, retire = false, failed = false;
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
      const double gam = h * kGd;
      double g[10];
      if (stage == 2) {
#pragma unroll
        for (int s = 0; s < 10; ++s)
          g[s] = (Y[s * BS] + gam * K1[s * BS]) + gam * f[s] - Z[s * BS];
      } else {
        const double hw = h * kW;
#pragma unroll
        for (int s = 0; s < 10; ++s)
          g[s] = (Y[s * BS] + hw * (K1[s * BS] + K2[s * BS])) + gam * f[s] - Z[s * BS];
      }
      int piv[10];
#pragma unroll
      for (int s = 0; s < 10; ++s) piv[s] = PV[s * BS];
      double dl[10];
      {
        LU xs[10];
#pragma unroll
        for (int s = 0; s < 10; ++s) xs[s] = (LU)g[s];
        lus10_strided<LU, LU>(L, BS, piv, xs);
#pragma unroll
        for (int s = 0; s < 10; ++s) dl[s] = (double)xs[s];
      }
      if (sizeof(LU) == 4) {
        for (int it = 0; it < O.refine; ++it) {  // residual of A_p dl = g in FP64
          double r[10];
#pragma unroll
          for (int s = 0; s < 10; ++s) r[s] = 0.0;
#pragma unroll
          for (int e = 0; e < 64; ++e) r[kJacPattern[e][0]] += Jm[e * BS] * dl[kJacPattern[e][1]];
          LU ds[10];
#pragma unroll
          for (int s = 0; s < 10; ++s) ds[s] = (LU)(g[s] - (dl[s] - gp * r[s]));
          lus10_strided<LU, LU>(L, BS, piv, ds);
#pragma unroll
          for (int s = 0; s < 10; ++s) dl[s] += (double)ds[s];
        }
      }
      if (gam != gp) {
        const double sc = 2.0 / (1.0 + gam / gp);
#pragma unroll
        for (int s = 0; s < 10; ++s) dl[s] *= sc;
      }
      double s2 = 0.0;
#pragma unroll
      for (int s = 0; s < 10; ++s) {
        Z[s * BS] += dl[s];
        const double v = dl[s] * EW[s * BS];
        s2 += v * v;
      }
      const double del = sqrt(s2 / 10.0);
      ++m;
      ++c_nni;
      if (m > 1) crate = fmax(0.3 * crate, del / delp);
      const double dcon = fmin(crate, 1.0) * del / O.nlscoef;
      if (dcon <= 1.0) {
        phase = (stage == 2) ? kPhK2 : kPhK3;
      } else if ((m > 1 && del > 2.3 * delp) || m >= O.maxcor || !(del == del)) {
        // Newton failure: with a stale Jacobian retry at the same h with a fresh one, else
        // cut the step
        ++ncf_s;
        ++c_ncf;
        if (ncf_s >= O.maxncf) {
          retire = failed = true;
        } else {
          if (jcur) h *= 0.25;
          else need_jac = true;
          setup = true;
        }
      } else {
        delp = del;
      }
    } else if (phase == kPhK2) {
#pragma unroll
      for (int s = 0; s < 10; ++s) K2[s * BS] = f[s];
      stage = 3;  // predictor: the stage-2 value already in Z
      m = 0;
      phase = kPhNewton;
    } else {  // kPhK3: error test
      double s2 = 0.0;
#pragma unroll
      for (int s = 0; s < 10; ++s) {
        const double e = h * ((kE1 * K1[s * BS] + kE2 * K2[s * BS]) + kE3 * f[s]);
        const double v = e * EW[s * BS];
        s2 += v * v;
      }
      const double dsm = sqrt(s2 / 10.0);
      if (dsm <= 1.0) {
        ++nst;
        t = last ? O.tout : t + h;
#pragma unroll
        for (int s = 0; s < 10; ++s) {
          Y[s * BS] = Z[s * BS];
          K1[s * BS] = f[s];  // stiffly accurate: F(stage 3) = F(y_{n+1})
        }
        Tsy = Tsc;
        dTsy = dTsc;
        jcur = false;
        double eta = (dsm > 0.0) ? O.safety / cbrt(dsm) : 1.0e300;
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
          double eta = fmax(0.1, O.safety / cbrt(dsm));
          if (nef_s >= 2) eta = fmin(eta, 0.3);
          h *= eta;
          setup = true;
        }
      }
    }

    while (setup && !retire) {  // start (or restart) a step at (t, Y)
      setup = false;
      last = (t + h >= O.tout);
      if (last) h = O.tout - t;
      Tsc = Tsy;
      dTsc = dTsy;
#pragma unroll
      for (int s = 0; s < 10; ++s) {
        const double ys = Y[s * BS];
        EW[s * BS] = 1.0 / (O.rtol * fabs(ys) + O.atol);
        Z[s * BS] = ys;  // trivial predictor
      }
      const double gam = h * kGd;
      bool refactor = false;
      if (need_jac || nst >= nst_lj + O.msbj) {
        const long j = i * 10;
        double ya[10];
#pragma unroll
        for (int s = 0; s < 10; ++s) ya[s] = Y[s * BS] * S.scale[j + s];
        double k[kNRates], dk[kNRates];
        chem_rates<true>(P, Tsy, k, dk);
        const ChemAux Ax{S.mdens[i], S.imdens[i], S.cie[i], S.h2[i]};
        const double* __restrict__ sc = S.scale + j;
        const double* __restrict__ isc = S.inv_scale + j;
        const double tu = O.tunit;
        chem_jacobian(P, k, dk, ya, Tsy, dTsy, Ax, [&](int row, int col, double v) {
          const int e = kJacIndex[row][col];  // every entry put is structural (folded)
          if (e >= 0) Jm[e * BS] = ((v * isc[row]) * sc[col]) * tu;
        });
        ++c_nje;
        nst_lj = nst;
        jcur = true;
        need_jac = false;
        refactor = true;
      }
      if (refactor || nst >= nst_lp + O.msbp || !(fabs(gam / gp - 1.0) <= O.dgmax)) {
#pragma unroll
        for (int e = 0; e < 100; ++e) L[e * BS] = (e % 11 == 0) ? LU(1) : LU(0);
#pragma unroll
        for (int e = 0; e < 64; ++e) {
          const int row = kJacPattern[e][0], col = kJacPattern[e][1];
          L[(col * 10 + row) * BS] = (LU)((row == col ? 1.0 : 0.0) - gam * Jm[e * BS]);
        }
        int piv[10];
        const int info = lu10_strided<LU>(L, BS, piv);
#pragma unroll
        for (int s = 0; s < 10; ++s) PV[s * BS] = piv[s];
        gp = gam;
        nst_lp = nst;
        crate = 1.0;
        ++c_nsetup;
        if (info) {  // singular Newton matrix: a recoverable failure, cut the step and retry
          ++ncf_s;
          ++c_ncf;
          if (ncf_s >= O.maxncf) {
            retire = failed = true;
          } else {
            h *= 0.25;
            if (!jcur) need_jac = true;
            gp = 0.0;  // forces a refactor
            setup = true;
          }
        }
      }
      stage = 2;
      m = 0;
      phase = kPhNewton;
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
        st[5] = c_nje;
        st[6] = c_nfe;
        st[7] = failed ? 1 : 0;
      }
      if (failed) atomicAdd(nfail, 1);
      i = -1;
    }
  }
}

template <typename LU, int BS>
static int launch_dirk(const ChemParams& P, const ChemState& S, long n, double* y,
                       const DirkOpts& O, unsigned long long* d_next, int* stats, int* d_nfail,
                       int nsm, cudaStream_t s) {
  const size_t shm = (size_t)BS * (114 * sizeof(double) + 100 * sizeof(LU) + 10 * sizeof(int));
  GBMV_CUDA_TRY(cudaFuncSetAttribute(chem_dirk_kernel<LU, BS>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
  int per_sm = 0;
  GBMV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chem_dirk_kernel<LU, BS>,
                                                              BS, shm));
  if (per_sm < 1) return GBMV_EUNSUPPORTED;
  long blocks = (long)nsm * per_sm;
  const long need = (n + BS - 1) / BS;
  if (blocks > need) blocks = need;
  chem_dirk_kernel<LU, BS><<<(int)blocks, BS, shm, s>>>(P, S, n, y, O, d_next, stats, d_nfail);
  GBMV_LAUNCH_CHECK("chem_dirk_kernel");
  return GBMV_OK;
}

int chem_dirk(const ChemParams& P, const ChemState& S, long n, double* y, const DirkOpts& O,
              int lu_fp32, int block, unsigned long long* d_next, int* stats, int* d_nfail,
              cudaStream_t s) {
  GBMV_CUDA_TRY(cudaMemsetAsync(d_next, 0, sizeof(unsigned long long), s));
  int dev = 0, nsm = kSM;
  GBMV_CUDA_TRY(cudaGetDevice(&dev));
  GBMV_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  ProfScope ps("chem_dirk", s);
  switch ((lu_fp32 ? 1000 : 0) + block) {
    case 32: return launch_dirk<double, 32>(P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
    case 64: return launch_dirk<double, 64>(P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
    case 128: return launch_dirk<double, 128>(P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
    case 1032: return launch_dirk<float, 32>(P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
    case 1064: return launch_dirk<float, 64>(P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
    case 1128: return launch_dirk<float, 128>(P, S, n, y, O, d_next, stats, d_nfail, nsm, s);
    default: return GBMV_EINVAL;
  }
}

}  // namespace gbmv
