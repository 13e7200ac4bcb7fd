// Declarations for the chemistry kernels (part b) and the block solves (part c).
#pragma once

#include "chem_net.cuh"
#include "common.cuh"

namespace gbmv {

// Persistent per-cell network state (device arrays), the per-cell members of cvklu_data
// (src/raja_primordial_network.hpp:168-270) that the source/Jacobian actually need.
struct ChemState {
  double* scale;      // 10 per cell
  double* inv_scale;  // 10 per cell
  double* Ts;         // temperature, carried from call to call
  double* dTs_ge;     // dT/dge from the last source evaluation
  double* mdens;
  double* imdens;
  double* cie;        // CIE cooling optical-depth factor
  double* h2;         // H2 line cooling optical-depth factor
};

int chem_rhs(const ChemParams& P, const ChemState& S, long n, const double* y, double* ydot,
             double tunit, cudaStream_t s);
int chem_jac(const ChemParams& P, const ChemState& S, long n, const double* y, double* J,
             double tunit, cudaStream_t s);
int chem_aux(const ChemState& S, long n, cudaStream_t s);
int chem_jvp(const ChemParams& P, const ChemState& S, long n, const double* y, const double* x,
             double* out, double tunit, int transpose, cudaStream_t s);
int chem_prepare(const ChemState& S, double* chem, long n, cudaStream_t s);
int chem_set_scale(const ChemState& S, const double* scale, long n, cudaStream_t s);
int chem_scaling(const ChemState& S, double* chem, long n, int mode, cudaStream_t s);
int energy_sync(const ChemState& S, double* const* w, long n, int nchem, double eunit_scale,
                int restore, cudaStream_t s);
int energy_epilogue(const ChemState& S, double* chem, double* chemdot, double* etdot, long n,
                    int nchem, int exact, cudaStream_t s);

// MRI forcing of the fast RHS (ffast): wdot_k += sum_i c_i x_i,k over the six components
constexpr int kMaxForcing = 8;
struct DevFields6 {
  double* f[6];
};
struct ForcingSet {
  double c[kMaxForcing];                 // tau^i
  const double* x[kMaxForcing][6];       // forcing vector i, component k
};
int mri_forcing(long ncell, const ForcingSet& F, int nf, const DevFields6& wdot, bool zero_fluid,
                int ncomp, cudaStream_t s);

// fused source + Jacobian + Newton matrix + LU solve (chem_newton.cu)
// b: null, or the implicit-stage right-hand side base: x = (I - gamma J)^{-1} (b + gamma f)
// queue: null (a grid-stride sweep) or a caller-zeroed cell counter shared by launches
int chem_newton(const ChemParams& P, const ChemState& S, long n, const double* y, double* f,
                double* x, double gamma, double tunit, int lu_fp32, int refine, int* d_info,
                cudaStream_t s, int blocks_per_sm = 0, const double* b = nullptr,
                unsigned long long* queue = nullptr);

// The stiffly accurate ESDIRK the persistent DIRK runs (explicit first stage, one diagonal
// value gamma, b = last row of a): stage i of s solves z_i = y + h sum_{j<i} a_ij K_j
// + h gamma F(z_i); e = b - bhat gives the embedded error estimate of order p.
constexpr int kDirkMaxStages = 7;
struct DirkTable {
  int s, p;
  double gamma;
  double c[kDirkMaxStages];
  double a[kDirkMaxStages][kDirkMaxStages];
  double e[kDirkMaxStages];
};

// persistent per-cell DIRK integration from t0 to tout (chem_dirk.cu)
struct DirkOpts {
  double t0, tout, tunit;
  double rtol, atol;  // WRMS weights 1 / (rtol |z| + atol) on the scaled variables
  double nlscoef;     // Newton tolerance factor
  double h0;          // first step; <= 0: h0fac / ||F(z0)||_WRMS
  double h0fac;
  double safety;      // step-size safety factor
  double dgmax;       // refactor when |gamma / gamma_p - 1| > dgmax
  double growth, etamx1, hmax;  // step growth bounds (after the first step / on it); hmax <= 0: none
  int maxcor, max_steps, msbp, maxnef, maxncf;
  int refine;      // FP32 LU: refinement steps per Newton solve
  int setup_batch; // waiting lanes of a warp that trigger its matrix setups (1: no waiting)
  int order;       // 1: cells taken largest initial derivative first (DirkOrder), 0: by index
  int deduce;      // 1: intermediate stage derivatives from the stage equation, not F
  int maxncf_total;  // Newton failures of a cell before it counts as failed (0: no limit)
  int mixed_temp;  // F evaluations' temperature solve: up to 9 FP32 iterations + 1 FP64
  // MRI forcing added to F: sum_i tau^i fz[i] (chemistry components, 10 per cell),
  // tau = (t - tshift) / tscale
  int nforcing;
  double tshift, tscale;
  const double* fz[8];
  DirkTable T;
  // stage derivatives K_1 .. K_{s-2} of every lane (element-major [(j-1)*10 + species][lane]),
  // kstore_lanes lanes; K_0 stays in shared memory
  double* kstore;
  long kstore_lanes;
  // cell lists.  list_in: null = cells 0..n-1, else the *list_in_n cells list_in[...], each
  // started from y_init / Ts_init (Ts at [cell], dTs/dge at [n + cell]) instead of the in-out
  // state.  list_out: null = failed cells are counted in nfail, else appended to list_out.
  const int* list_in;
  const int* list_in_n;
  const double* y_init;
  const double* Ts_init;
  int* list_out;
  int* list_out_n;
};

// Buffers of the FP32 form's second pass: the cells the FP32 pass could not finish are
// integrated again from their start state in FP64 (chem_dirk).
struct DirkRetry {
  double* y0;   // 10 n: the start state
  double* ts0;  // 2 n: Ts, dTs/dge at the start
  int* list;    // n: failed cells of the FP32 pass
  int* count;   // 1
};
// Buffers of the cost order: a bucket per cell (kDirkOrderBuckets, 4 per decade of the cell's
// initial WRMS derivative size, largest first), the bucket counts and offsets, the ordered
// cell list and its length.
constexpr int kDirkOrderBuckets = 64;
struct DirkOrder {
  unsigned char* bucket;  // n
  int* hist;              // kDirkOrderBuckets
  int* offset;            // kDirkOrderBuckets
  int* count;             // 1
  int* list;              // n
};
constexpr int kDirkFp32MaxNcf = 5;  // the mixed DIRK's FP32 pass: Newton failures per step
constexpr int kDirkFp32MaxNcfTotal = 8;  // and per cell, with deduced stage derivatives
constexpr int kDirkStats = 8;  // per cell: steps, Newton iters, error fails, Newton fails,
                               // matrix setups, Jacobians (= setups), F evaluations, failed
// retry: null, or (FP32 form without refinement) the buffers of the FP64 second pass
int chem_dirk(const ChemParams& P, const ChemState& S, long n, double* y, const DirkOpts& O,
              int lu_fp32, int block, unsigned long long* d_next, int* stats, int* d_nfail,
              cudaStream_t s, const DirkRetry* retry = nullptr, const DirkOrder* order = nullptr);
// Largest number of lanes (threads) any launch shape of chem_dirk runs on this device: the
// stage store must hold kstore_lanes >= this many lanes.
long chem_dirk_max_lanes();

// batched 10x10 LU (blocklu.cu)
int block_lu_factor(long nb, double* A, int* piv, int* d_info, cudaStream_t s);
int block_lu_solve(long nb, const double* LU, const int* piv, const double* b, double* x,
                   cudaStream_t s);
int block_form_newton(long nb, double* J, double gamma, cudaStream_t s);

}  // namespace gbmv
