// The C ABI (include/gbmv.h): handles mirroring EulerData / cvklu_data, argument checking,
// dispatch to the kernels, ARKODE-convention return codes.
#include <nvtx3/nvToolsExt.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "butcher.cuh"
#include "chem.cuh"
#include "weno.cuh"

namespace gbmv {

static thread_local char g_err[512];
static std::atomic<long> g_launches{0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}
void count_launch(long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
int check_cuda(cudaError_t e, const char* where) {
  set_error("%s: %s", where, cudaGetErrorString(e));
  return GBMV_ECUDA;
}

// ---- per-family event profiler
struct ProfRec {
  const char* family;
  cudaEvent_t e0, e1;
};
static std::mutex g_prof_mu;
static bool g_prof_on = false;
static std::vector<ProfRec> g_prof;

ProfScope::ProfScope(const char* family, cudaStream_t s) : slot(-1), stream(s) {
  nvtxRangePushA(family);
  if (!g_prof_on) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return;  // no timing events inside a graph capture
  }
  ProfRec r{family, nullptr, nullptr};
  if (cudaEventCreate(&r.e0) != cudaSuccess || cudaEventCreate(&r.e1) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  cudaEventRecord(r.e0, s);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  slot = (int)g_prof.size();
  g_prof.push_back(r);
}
ProfScope::~ProfScope() {
  if (slot >= 0) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEventRecord(g_prof[slot].e1, stream);
  }
  nvtxRangePop();
}

}  // namespace gbmv

using namespace gbmv;

struct gbmv_hydro_s {
  Grid g;
  ForceTerm force;
  double* scratch = nullptr;
  size_t scratch_doubles = 0;
  float* prims = nullptr;  // float-float per-cell primitives of the mixed form (first use)
  double* adj = nullptr;   // per-face stencil cotangents of the VJP (first use)
  double* cons = nullptr;  // conservation-sum partials (first use)
  int* d_status = nullptr;
  int sweep_threads[3] = {0, 0, 0};  // face-sweep threads per block per precision (0: by size)
  int sweep_shared = 0;               // GBMV_SWEEPS_SHARED register budget
};

struct gbmv_chem_s {
  long n = 0;
  ChemParams P{};
  ChemState S{};
  double* tab = nullptr;
  double* cell = nullptr;  // one allocation for all per-cell arrays
  int* d_info = nullptr;               // first word of a 64-byte control block:
  int* d_nfail = nullptr;              //   [0] info, [1] failed cells,
  unsigned long long* d_next = nullptr;  //   [16] DIRK work counter
  int dirk_block[2] = {0, 0};          // autotuned block size per precision (0 = not yet)
  double* dirk_k = nullptr;            // DIRK stage store (first DIRK call), dirk_k_lanes lanes
  long dirk_k_lanes = 0;
  double* dirk_retry = nullptr;        // FP32 DIRK's second pass: start state, Ts, cell list
  DirkRetry retry{};
  int* dirk_order_buf = nullptr;       // DIRK cost order: buckets, counts, ordered cell list
  DirkOrder order{};
  int newton_bps = 0;                  // fused Newton: resident blocks per SM (0 = default)
};

int gbmv::check_grid(const gbmv_grid* g) {
  if (!g) { set_error("null grid"); return GBMV_EINVAL; }
  if (g->nx < 3 || g->ny < 3 || g->nz < 3) {
    set_error("every extent must be >= 3 (got %ld x %ld x %ld)", g->nx, g->ny, g->nz);
    return GBMV_EINVAL;
  }
  if (!(g->nchem == 0 || g->nchem == 2 || g->nchem == 4 || g->nchem == 6 || g->nchem == 10)) {
    set_error("nchem=%d not supported (0,2,4,6,10)", g->nchem);
    return GBMV_EUNSUPPORTED;
  }
  for (int a = 0; a < 3; ++a) {
    const int lo = g->bc[2 * a], hi = g->bc[2 * a + 1];
    if (lo < 0 || lo > 3 || hi < 0 || hi > 3) { set_error("bad boundary code"); return GBMV_EINVAL; }
    if ((lo == GBMV_BC_PERIODIC) != (hi == GBMV_BC_PERIODIC)) {
      set_error("axis %d: only one face periodic", a);
      return GBMV_EINVAL;
    }
  }
  if (!(g->dx > 0) || !(g->dy > 0) || !(g->dz > 0) || !(g->gamma > 1.0)) {
    set_error("bad spacing or gamma");
    return GBMV_EINVAL;
  }
  return GBMV_OK;
}

static bool fields_ok(const double* const* w, int nchem) {
  if (!w) return false;
  for (int v = 0; v < 5; ++v)
    if (!w[v]) return false;
  return nchem == 0 || w[5] != nullptr;
}

// Median of five event-timed runs of fn (after one untimed run), in ms; < 0 on error.
template <class Fn>
static float time_runs(cudaStream_t s, Fn fn) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    return -1.f;
  }
  float ms[5] = {0, 0, 0, 0, 0};
  int rc = fn();
  for (int k = 0; k < 5 && !rc; ++k) {
    cudaEventRecord(e0, s);
    rc = fn();
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = GBMV_ECUDA;
    else cudaEventElapsedTime(&ms[k], e0, e1);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return -1.f;
  for (int a = 0; a < 5; ++a)
    for (int b = a + 1; b < 5; ++b)
      if (ms[b] < ms[a]) { float t = ms[a]; ms[a] = ms[b]; ms[b] = t; }
  return ms[2];
}

extern "C" {

const char* gbmv_version(void) { return "gbmv 0.1 (sm_103a)"; }

int gbmv_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_on = on != 0;
  return GBMV_OK;
}

int gbmv_profile_reset(void) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (auto& r : g_prof) {
    cudaEventDestroy(r.e0);
    cudaEventDestroy(r.e1);
  }
  g_prof.clear();
  return GBMV_OK;
}

int gbmv_profile_get(const char* family, double* total_ms, long* launches) {
  if (!family || !total_ms || !launches) return GBMV_EINVAL;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  double tot = 0.0;
  long n = 0;
  for (auto& r : g_prof) {
    if (std::string(r.family) != family) continue;
    GBMV_CUDA_TRY(cudaEventSynchronize(r.e1));
    float ms = 0.f;
    GBMV_CUDA_TRY(cudaEventElapsedTime(&ms, r.e0, r.e1));
    tot += ms;
    ++n;
  }
  *total_ms = tot;
  *launches = n;
  return GBMV_OK;
}
const char* gbmv_last_error(void) { return g_err; }
long gbmv_launch_count(void) { return g_launches.load(); }

int gbmv_hydro_create(const gbmv_grid* grid, gbmv_hydro* out) {
  if (!out) return GBMV_EINVAL;
  *out = nullptr;
  int rc = check_grid(grid);
  if (rc) return rc;
  gbmv_hydro h = new (std::nothrow) gbmv_hydro_s();
  if (!h) return GBMV_ENOMEM;
  h->g = make_grid(*grid);
  memset(&h->force, 0, sizeof h->force);
  h->scratch_doubles = feuler_fp64_scratch_doubles(h->g);
  if (cudaMalloc(&h->scratch, h->scratch_doubles * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&h->d_status, 2 * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    set_error("device allocation of %zu flux doubles failed", h->scratch_doubles);
    cudaFree(h->scratch);
    delete h;
    return GBMV_ENOMEM;
  }
  *out = h;
  return GBMV_OK;
}

int gbmv_hydro_destroy(gbmv_hydro h) {
  if (!h) return GBMV_OK;
  cudaFree(h->scratch);
  cudaFree(h->prims);
  cudaFree(h->adj);
  cudaFree(h->cons);
  cudaFree(h->d_status);
  delete h;
  return GBMV_OK;
}

int gbmv_hydro_set_force(gbmv_hydro h, const double* force) {
  if (!h) return GBMV_EINVAL;
  for (int v = 0; v < 16; ++v) h->force.c[v] = (force && v < 5 + h->g.nchem) ? force[v] : 0.0;
  return GBMV_OK;
}

static bool capturing(cudaStream_t s);

// fEuler dispatch; tscale (mixed form only): the chemistry component is in scaled units and
// is multiplied by tscale where the WENO reads it.
static int feuler_dispatch(gbmv_hydro h, const double* const* w, double* const* wdot,
                           int precision, int flags, int* d_status, cudaStream_t s,
                           const double* tscale);

int gbmv_feuler_async(gbmv_hydro h, double t, const double* const* w, double* const* wdot,
                      int precision, int flags, int* d_status, void* stream) {
  (void)t;
  return feuler_dispatch(h, w, wdot, precision, flags, d_status, (cudaStream_t)stream, nullptr);
}

static int feuler_dispatch(gbmv_hydro h, const double* const* w, double* const* wdot,
                           int precision, int flags, int* d_status, cudaStream_t s,
                           const double* tscale) {
  if (!h || !fields_ok(w, h->g.nchem) || !fields_ok(wdot, h->g.nchem) || !d_status) {
    set_error("null handle, field or status pointer");
    return GBMV_EINVAL;
  }
  if (precision != GBMV_FP64 && precision != GBMV_MIXED && precision != GBMV_MIXED_FAST) {
    set_error("unknown precision %d", precision);
    return GBMV_EINVAL;
  }
  Fields W, Wd;
  for (int v = 0; v < 6; ++v) {
    W.f[v] = const_cast<double*>(w[v]);
    Wd.f[v] = (v < 5 || h->g.nchem) ? wdot[v] : nullptr;
  }
  if (!h->g.nchem) W.f[5] = nullptr;
  ForceTerm G = h->force;
  G.in_wdot = (flags & GBMV_FORCE_IN_WDOT) ? 1 : 0;
  Grid g = h->g;
  g.sweep_threads = h->sweep_threads[precision];
  g.sweep_shared = h->sweep_shared;
  if (precision == GBMV_FP64) return feuler_fp64(g, W, Wd, G, h->scratch, d_status, s);
  if (!h->prims) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      set_error("the first GBMV_MIXED call on a handle allocates its buffers: make it before "
                "any stream capture");
      return GBMV_EINVAL;
    }
    const size_t nf = feuler_f2_prims_floats(h->g);
    if (cudaMalloc(&h->prims, nf * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      h->prims = nullptr;
      set_error("device allocation of %zu mixed-form primitive floats failed", nf);
      return GBMV_ENOMEM;
    }
  }
  return feuler_f2(g, W, Wd, G, h->scratch, h->prims, tscale, d_status, s,
                   precision == GBMV_MIXED_FAST);
}

int gbmv_hydro_autotune(gbmv_hydro h, const double* const* w, int precision, int* threads,
                        void* stream) {
  if (!h || !fields_ok(w, h->g.nchem) ||
      (precision != GBMV_FP64 && precision != GBMV_MIXED && precision != GBMV_MIXED_FAST)) {
    set_error("null handle or field, or unknown precision");
    return GBMV_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (capturing(s)) {
    set_error("the face-sweep autotuner times launches: call it outside any stream capture");
    return GBMV_EINVAL;
  }
  const long n = h->g.ncell;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * (5 + h->g.nchem) * n) != cudaSuccess) {
    cudaGetLastError();
    set_error("autotune output allocation failed");
    return GBMV_ENOMEM;
  }
  double* wd[6];
  for (int k = 0; k < 6; ++k) wd[k] = (k < 5 || h->g.nchem) ? out + (long)k * n : nullptr;
  const int cand[3] = {32, 64, 128};
  int best = 0, rc = GBMV_OK;
  float best_ms = 0.f;
  for (int c = 0; c < 3 && !rc; ++c) {
    h->sweep_threads[precision] = cand[c];
    const float ms = time_runs(s, [&]() {
      return feuler_dispatch(h, w, wd, precision, 0, h->d_status, s, nullptr);
    });
    if (ms < 0.f) { rc = GBMV_ECUDA; break; }
    if (best == 0 || ms < best_ms) { best = cand[c]; best_ms = ms; }
  }
  cudaFree(out);
  h->sweep_threads[precision] = rc ? 0 : best;
  if (rc) return rc;
  if (threads) *threads = best;
  return GBMV_OK;
}

int gbmv_hydro_set_sweep_threads(gbmv_hydro h, int precision, int threads) {
  if (!h || precision < GBMV_FP64 || precision > GBMV_MIXED_FAST ||
      (threads != 0 && threads != 32 && threads != 64 && threads != 128)) {
    set_error("null handle, unknown precision or threads not 0/32/64/128");
    return GBMV_EINVAL;
  }
  h->sweep_threads[precision] = threads;
  return GBMV_OK;
}

int gbmv_hydro_set_sweep_budget(gbmv_hydro h, int budget) {
  if (!h || (budget != GBMV_SWEEPS_ALONE && budget != GBMV_SWEEPS_SHARED)) {
    set_error("null handle or unknown sweep budget (GBMV_SWEEPS_ALONE, GBMV_SWEEPS_SHARED)");
    return GBMV_EINVAL;
  }
  h->sweep_shared = budget == GBMV_SWEEPS_SHARED;
  return GBMV_OK;
}

int gbmv_feuler(gbmv_hydro h, double t, const double* const* w, double* const* wdot,
                int precision, void* stream) {
  if (!h) return GBMV_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  GBMV_CUDA_TRY(cudaMemsetAsync(h->d_status, 0, sizeof(int), s));
  int rc = gbmv_feuler_async(h, t, w, wdot, precision, 0, h->d_status, stream);
  if (rc) return rc;
  int st = 0;
  GBMV_CUDA_TRY(cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  if (st) {
    set_error("illegal state (mask %d: 1 density, 2 energy, 4 pressure)", st);
    return GBMV_ILLEGAL_STATE;
  }
  return GBMV_OK;
}

/* ------------------------------------------------------------------ chemistry */

int gbmv_chem_create(long ncells, const double* tables_host, double current_z, gbmv_chem* out) {
  if (!out || ncells <= 0 || !tables_host) { set_error("bad chem_create arguments"); return GBMV_EINVAL; }
  *out = nullptr;
  gbmv_chem c = new (std::nothrow) gbmv_chem_s();
  if (!c) return GBMV_ENOMEM;
  c->n = ncells;
  // bin-major re-layout of the (50 x 1024) table block
  double* h = (double*)malloc(sizeof(double) * kNT * kTSize);
  if (!h) { delete c; return GBMV_ENOMEM; }
  for (int b = 0; b < kTSize; ++b)
    for (int r = 0; r < kNT; ++r) h[b * kNT + r] = tables_host[(long)r * kTSize + b];
  // after the double table: the per-bin differences next - value in FP64 (dtab), then float
  // copies of the four H2 adiabatic-index tables for the FP32 temperature iterations: per bin
  // (value, next - value) of gammaH2_2, dgammaH2_2_dT, gammaH2_1, dgammaH2_1_dT, each rounded
  // to float once
  const size_t tab_doubles = (size_t)kNT * kTSize;
  const size_t gtab_floats = (size_t)8 * kTSize;
  float* gh = (float*)calloc(gtab_floats, sizeof(float));
  double* dh = (double*)calloc(tab_doubles, sizeof(double));
  if (!gh || !dh) { free(h); free(gh); free(dh); delete c; return GBMV_ENOMEM; }
  for (int b = 0; b + 1 < kTSize; ++b)
    for (int r = 0; r < kNT; ++r) dh[b * kNT + r] = h[(b + 1) * kNT + r] - h[b * kNT + r];
  const int grow[4] = {GAMMAH2_2, DGAMMAH2_2, GAMMAH2_1, DGAMMAH2_1};
  for (int b = 0; b + 1 < kTSize; ++b)
    for (int q = 0; q < 4; ++q) {
      const double lo = h[b * kNT + grow[q]], hi = h[(b + 1) * kNT + grow[q]];
      gh[b * 8 + 2 * q] = (float)lo;
      gh[b * 8 + 2 * q + 1] = (float)(hi - lo);
    }
  const size_t per_cell = 10 + 10 + 6;
  if (cudaMalloc(&c->tab, sizeof(double) * 2 * tab_doubles + sizeof(float) * gtab_floats) !=
          cudaSuccess ||
      cudaMalloc(&c->cell, sizeof(double) * per_cell * ncells) != cudaSuccess ||
      cudaMalloc(&c->d_info, 64) != cudaSuccess) {
    cudaGetLastError();
    free(h);
    free(gh);
    free(dh);
    cudaFree(c->tab);
    cudaFree(c->cell);
    delete c;
    set_error("device allocation failed for %ld cells", ncells);
    return GBMV_ENOMEM;
  }
  c->d_nfail = c->d_info + 1;
  c->d_next = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(c->d_info) + 16);
  cudaMemcpy(c->tab, h, sizeof(double) * tab_doubles, cudaMemcpyHostToDevice);
  cudaMemcpy(c->tab + tab_doubles, dh, sizeof(double) * tab_doubles, cudaMemcpyHostToDevice);
  cudaMemcpy(c->tab + 2 * tab_doubles, gh, sizeof(float) * gtab_floats, cudaMemcpyHostToDevice);
  free(h);
  free(gh);
  free(dh);
  // constants of cvklu_setup_data (src/raja_primordial_network.cpp:190-194)
  ChemParams& P = c->P;
  P.tab = c->tab;
  P.dtab = c->tab + tab_doubles;
  P.tlo = 1.0;
  P.thi = 100000.0;
  P.nbins = kTSize - 1;
  P.lb = log(P.tlo);
  P.dbin = (log(P.thi) - log(P.tlo)) / P.nbins;
  P.idbin = (double)(1.0L / (long double)P.dbin);
  P.gtab = reinterpret_cast<const float*>(c->tab + 2 * tab_doubles);  // 16-byte aligned
  P.dbinf = (float)P.dbin;
  P.idbinf = (float)P.idbin;
  P.lbf = (float)P.lb;
  P.z = current_z;
  P.zp1_4 = pow(current_z + 1.0, 4);
  ChemState& S = c->S;
  double* p = c->cell;
  S.scale = p; p += 10 * ncells;
  S.inv_scale = p; p += 10 * ncells;
  S.Ts = p; p += ncells;
  S.dTs_ge = p; p += ncells;
  S.mdens = p; p += ncells;
  S.imdens = p; p += ncells;
  S.cie = p; p += ncells;
  S.h2 = p; p += ncells;
  // Ts = 1000 K, scale = inv_scale = 1 (src/raja_primordial_network.cpp:185-188,
  // src/primordial_static.cpp:193-200), aux from scale
  double* init = (double*)malloc(sizeof(double) * per_cell * ncells);
  if (!init) { gbmv_chem_destroy(c); return GBMV_ENOMEM; }
  for (long i = 0; i < 20 * ncells; ++i) init[i] = 1.0;
  for (long i = 0; i < ncells; ++i) init[20 * ncells + i] = 1000.0;
  for (long i = 21 * ncells; i < (long)per_cell * ncells; ++i) init[i] = 0.0;
  cudaError_t e = cudaMemcpy(c->cell, init, sizeof(double) * per_cell * ncells,
                             cudaMemcpyHostToDevice);
  free(init);
  if (e != cudaSuccess) { gbmv_chem_destroy(c); return check_cuda(e, "chem_create upload"); }
  int rc = chem_aux(S, ncells, 0);
  if (rc) { gbmv_chem_destroy(c); return rc; }
  GBMV_CUDA_TRY(cudaDeviceSynchronize());
  *out = c;
  return GBMV_OK;
}

int gbmv_chem_destroy(gbmv_chem c) {
  if (!c) return GBMV_OK;
  cudaFree(c->tab);
  cudaFree(c->cell);
  cudaFree(c->d_info);
  cudaFree(c->dirk_k);
  cudaFree(c->dirk_retry);
  cudaFree(c->dirk_order_buf);
  delete c;
  return GBMV_OK;
}

double* gbmv_chem_state(gbmv_chem c, int which) {
  if (!c) return nullptr;
  switch (which) {
    case 0: return c->S.Ts;
    case 1: return c->S.dTs_ge;
    case 2: return c->S.mdens;
    case 3: return c->S.imdens;
    case 4: return c->S.cie;
    case 5: return c->S.h2;
    case 6: return c->S.scale;
    case 7: return c->S.inv_scale;
    default: return nullptr;
  }
}

int gbmv_chem_prepare(gbmv_chem c, double* chem, void* stream) {
  if (!c || !chem) return GBMV_EINVAL;
  return chem_prepare(c->S, chem, c->n, (cudaStream_t)stream);
}

int gbmv_chem_set_scale(gbmv_chem c, const double* scale, void* stream) {
  if (!c || !scale) return GBMV_EINVAL;
  return chem_set_scale(c->S, scale, c->n, (cudaStream_t)stream);
}

int gbmv_chem_apply_scaling(gbmv_chem c, double* chem, void* stream) {
  if (!c || !chem) return GBMV_EINVAL;
  return chem_scaling(c->S, chem, c->n, 0, (cudaStream_t)stream);
}

int gbmv_chem_unapply_scaling(gbmv_chem c, double* chem, void* stream) {
  if (!c || !chem) return GBMV_EINVAL;
  return chem_scaling(c->S, chem, c->n, 1, (cudaStream_t)stream);
}

int gbmv_chem_rhs(gbmv_chem c, double t, const double* y, double* ydot, double time_units,
                  void* stream) {
  (void)t;
  if (!c || !y || !ydot) { set_error("null argument"); return GBMV_EINVAL; }
  return chem_rhs(c->P, c->S, c->n, y, ydot, time_units, (cudaStream_t)stream);
}

int gbmv_chem_jac(gbmv_chem c, double t, const double* y, double* J, double time_units,
                  void* stream) {
  (void)t;
  if (!c || !y || !J) { set_error("null argument"); return GBMV_EINVAL; }
  return chem_jac(c->P, c->S, c->n, y, J, time_units, (cudaStream_t)stream);
}

int gbmv_chem_newton_async(gbmv_chem c, double t, const double* y, double* f, double* x,
                           double gamma, double time_units, int lu_precision, int refine,
                           int* d_info, void* stream) {
  (void)t;
  if (!c || !y || !f || !x || !d_info || refine < 0 || refine > 8 ||
      (lu_precision != GBMV_FP64 && lu_precision != GBMV_MIXED)) {
    set_error("bad chem_newton arguments");
    return GBMV_EINVAL;
  }
  return chem_newton(c->P, c->S, c->n, y, f, x, gamma, time_units, lu_precision == GBMV_MIXED,
                     refine, d_info, (cudaStream_t)stream, c->newton_bps);
}

int gbmv_chem_newton_queue_async(gbmv_chem c, double t, const double* y, double* f, double* x,
                                 double gamma, double time_units, int lu_precision, int refine,
                                 unsigned long long* d_queue, int blocks_per_sm, int* d_info,
                                 void* stream) {
  (void)t;
  if (!c || !y || !f || !x || !d_info || !d_queue || refine < 0 || refine > 8 ||
      blocks_per_sm < 0 || blocks_per_sm > 32 ||
      (lu_precision != GBMV_FP64 && lu_precision != GBMV_MIXED)) {
    set_error("bad chem_newton_queue arguments");
    return GBMV_EINVAL;
  }
  return chem_newton(c->P, c->S, c->n, y, f, x, gamma, time_units, lu_precision == GBMV_MIXED,
                     refine, d_info, (cudaStream_t)stream, blocks_per_sm, nullptr, d_queue);
}

}  // extern "C"

// synchronous fused Newton (b null: gbmv_chem_newton; b set: its implicit-stage form)
static int newton_sync(gbmv_chem c, const double* y, const double* b, double* f, double* x,
                       double gamma, double time_units, int lu_precision, int refine,
                       void* stream) {
  if (!c || !y || !f || !x || refine < 0 || refine > 8 ||
      (lu_precision != GBMV_FP64 && lu_precision != GBMV_MIXED)) {
    set_error("bad chem_newton arguments");
    return GBMV_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  GBMV_CUDA_TRY(cudaMemsetAsync(c->d_info, 0, sizeof(int), s));
  int rc = chem_newton(c->P, c->S, c->n, y, f, x, gamma, time_units, lu_precision == GBMV_MIXED,
                       refine, c->d_info, s, c->newton_bps, b);
  if (rc) return rc;
  int h = 0;
  GBMV_CUDA_TRY(cudaMemcpyAsync(&h, c->d_info, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  if (h) { set_error("singular Newton block"); return 1; }
  return GBMV_OK;
}

extern "C" {

int gbmv_chem_newton(gbmv_chem c, double t, const double* y, double* f, double* x,
                     double gamma, double time_units, int lu_precision, int refine,
                     void* stream) {
  (void)t;
  return newton_sync(c, y, nullptr, f, x, gamma, time_units, lu_precision, refine, stream);
}

int gbmv_chem_newton_stage(gbmv_chem c, double t, const double* y, const double* b, double* f,
                           double* x, double gamma, double time_units, int lu_precision,
                           int refine, void* stream) {
  (void)t;
  if (!b) {
    set_error("chem_newton_stage needs the stage base b");
    return GBMV_EINVAL;
  }
  return newton_sync(c, y, b, f, x, gamma, time_units, lu_precision, refine, stream);
}

/* ------------------------------------------------------------------ DIRK integrator */

void gbmv_dirk_opts_default(gbmv_dirk_opts* o) {
  if (!o) return;
  o->rtol = 1e-6;
  o->atol = 1e-10;
  o->nlscoef = 0.1;
  o->h0 = 0.0;
  o->safety = 0.9;
  o->dgmax = 0.2;
  o->growth = 20.0;
  o->etamx1 = 10000.0;
  o->hmax = 0.0;
  o->maxcor = 3;
  o->max_steps = 5000;
  o->msbp = 20;
  o->maxnef = 7;
  o->maxncf = 10;
  o->precision = GBMV_FP64;
  o->refine = 0;
  o->block = 0;
  o->table = 0;
  o->setup_batch = 8;
  o->order = 1;
  o->deduce = 0;
}

// The DIRK table of the options (0: ARK437L2SA_DIRK_7_3_4, the reference's chemistry inputs'
// itable), checked to be a stiffly accurate ESDIRK with one diagonal value.
static int dirk_table(int id, DirkTable* D) {
  const int tid = id ? id : 112;
  const ButcherTable* T = butcher_table(tid);
  bool ok = T && T->s >= 2 && T->s <= kDirkMaxStages && T->A[0][0] == 0.0 && T->A[1][1] > 0.0;
  for (int i = 1; ok && i < T->s; ++i) ok = T->A[i][i] == T->A[1][1];
  for (int j = 0; ok && j < T->s; ++j) ok = T->b[j] == T->A[T->s - 1][j];
  if (!ok) {
    set_error("DIRK table %d is not a stiffly accurate ESDIRK of gbmv_butcher_table (use 112 "
              "or 102)", tid);
    return GBMV_EUNSUPPORTED;
  }
  memset(D, 0, sizeof *D);
  D->s = T->s;
  D->p = T->p;
  D->gamma = T->A[1][1];
  for (int i = 0; i < T->s; ++i) {
    D->c[i] = T->c[i];
    D->e[i] = T->b[i] - T->bhat[i];
    for (int j = 0; j < T->s; ++j) D->a[i][j] = T->A[i][j];
  }
  return GBMV_OK;
}


// The stage store of the handle's DIRK (K_1 .. K_{s-2} of every lane), allocated at the first
// call that needs it, for the most lanes any launch shape of the kernel runs.
static int dirk_store(gbmv_chem c, DirkOpts* O, cudaStream_t s) {
  if (O->T.s > 2 && !c->dirk_k) {
    if (capturing(s)) {
      set_error("the first DIRK call allocates its stage store: make it before any capture");
      return GBMV_EINVAL;
    }
    const long lanes = chem_dirk_max_lanes();
    if (lanes <= 0) return check_cuda(cudaGetLastError(), "DIRK occupancy query");
    if (cudaMalloc(&c->dirk_k, sizeof(double) * 10 * (kDirkMaxStages - 2) * lanes) !=
        cudaSuccess) {
      cudaGetLastError();
      c->dirk_k = nullptr;
      set_error("device allocation of the DIRK stage store (%ld lanes) failed", lanes);
      return GBMV_ENOMEM;
    }
    c->dirk_k_lanes = lanes;
  }
  O->kstore = c->dirk_k;
  O->kstore_lanes = c->dirk_k_lanes;
  if (!c->dirk_retry) {  // the FP32 form's second pass: start state, Ts, failed-cell list
    if (capturing(s)) {
      set_error("the first DIRK call allocates its buffers: make it before any capture");
      return GBMV_EINVAL;
    }
    const long n = c->n;
    if (cudaMalloc(&c->dirk_retry, sizeof(double) * 12 * n + sizeof(int) * (n + 1)) !=
        cudaSuccess) {
      cudaGetLastError();
      c->dirk_retry = nullptr;
      set_error("device allocation of the DIRK retry buffers failed");
      return GBMV_ENOMEM;
    }
    c->retry.y0 = c->dirk_retry;
    c->retry.ts0 = c->dirk_retry + 10 * n;
    c->retry.list = reinterpret_cast<int*>(c->dirk_retry + 12 * n);
    c->retry.count = c->retry.list + n;
  }
  if (!c->dirk_order_buf) {  // the cost order's buckets, counts and cell list
    if (capturing(s)) {
      set_error("the first DIRK call allocates its buffers: make it before any capture");
      return GBMV_EINVAL;
    }
    const long n = c->n;
    const size_t ints = (size_t)n + 2 * kDirkOrderBuckets + 1 + ((size_t)n + 3) / 4;
    if (cudaMalloc(&c->dirk_order_buf, sizeof(int) * ints) != cudaSuccess) {
      cudaGetLastError();
      c->dirk_order_buf = nullptr;
      set_error("device allocation of the DIRK order buffers failed");
      return GBMV_ENOMEM;
    }
    c->order.list = c->dirk_order_buf;
    c->order.hist = c->order.list + n;
    c->order.offset = c->order.hist + kDirkOrderBuckets;
    c->order.count = c->order.offset + kDirkOrderBuckets;
    c->order.bucket = reinterpret_cast<unsigned char*>(c->order.count + 1);
  }
  return GBMV_OK;
}

static int dirk_opts(const gbmv_dirk_opts* o, double t0, double tout, double tunit, DirkOpts* O) {
  if (!o || !(o->rtol > 0.0) || !(o->atol > 0.0) || !(o->nlscoef > 0.0) || !(o->safety > 0.0) ||
      !(o->dgmax >= 0.0) || !(o->growth >= 1.0) || !(o->etamx1 >= 1.0) || !(o->hmax >= 0.0) ||
      o->maxcor < 1 || o->max_steps < 1 || o->msbp < 1 ||
      o->maxnef < 1 || o->maxncf < 1 || o->refine < 0 || o->refine > 8 ||
      (o->precision != GBMV_FP64 && o->precision != GBMV_MIXED) ||
      (o->block != 0 && o->block != 32 && o->block != 64 && o->block != 128) ||
      o->setup_batch < 1 || o->setup_batch > 32 || (o->order != 0 && o->order != 1) ||
      (o->deduce != 0 && o->deduce != 1) || !(tout > t0) || !(tunit > 0.0)) {
    set_error("bad DIRK options (tolerances > 0, growth >= 1, hmax >= 0, counts >= 1, refine 0-8, "
              "block 0/32/64/128, setup_batch 1-32, order 0/1, deduce 0/1, tout > t0, "
              "time_units > 0)");
    return GBMV_EINVAL;
  }
  O->t0 = t0;
  O->tout = tout;
  O->tunit = tunit;
  O->rtol = o->rtol;
  O->atol = o->atol;
  O->nlscoef = o->nlscoef;
  O->h0 = o->h0;
  O->h0fac = 0.5 * pow(o->rtol, -2.0 / 3.0);  // h0 = rtol^(1/3) x (time scale |z|/|F|) / 2
  O->safety = o->safety;
  O->dgmax = o->dgmax;
  O->growth = o->growth;
  O->etamx1 = o->etamx1;
  O->hmax = o->hmax;
  O->maxcor = o->maxcor;
  O->max_steps = o->max_steps;
  O->msbp = o->msbp;
  O->maxnef = o->maxnef;
  O->maxncf = o->maxncf;
  O->refine = o->precision == GBMV_MIXED ? o->refine : 0;
  O->setup_batch = o->setup_batch;
  O->order = o->order;
  O->deduce = o->deduce;
  O->maxncf_total = 0;
  O->mixed_temp = o->precision == GBMV_MIXED;
  O->nforcing = 0;
  O->tshift = 0.0;
  O->tscale = 1.0;
  for (int q = 0; q < 8; ++q) O->fz[q] = nullptr;
  O->kstore = nullptr;
  O->kstore_lanes = 0;
  O->list_in = nullptr;
  O->list_in_n = nullptr;
  O->y_init = nullptr;
  O->Ts_init = nullptr;
  O->list_out = nullptr;
  O->list_out_n = nullptr;
  return dirk_table(o->table, &O->T);
}

static int ck(cudaError_t e, const char* where) {
  return e == cudaSuccess ? GBMV_OK : check_cuda(e, where);
}

// Block-size autotuner: integrates a sample of the cells (the first min(n, 65536), their
// temperature state saved and restored) once per candidate, 32 and 64 threads, and keeps the
// fastest.  (128 is accepted as an explicit option but not a candidate: on the 64^3
// static-chemistry run it measured 2.49 s against 2.27-2.30 s for 32 and 64 in the FP64 form
// and no better in the mixed one, while a sample run -- under two cells per lane, so mostly
// its slowest cells -- cannot tell them apart.)
static int dirk_autotune(gbmv_chem c, const double* y, const DirkOpts& O, int mixed,
                         cudaStream_t s) {
  const long ns = c->n < 65536 ? c->n : 65536;
  double *ybuf = nullptr, *tsave = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int best = 64;
  float best_ms = 0.f;
  int rc = GBMV_OK;
  if (cudaMalloc(&ybuf, sizeof(double) * 10 * ns) != cudaSuccess ||
      cudaMalloc(&tsave, sizeof(double) * 2 * ns) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    rc = check_cuda(cudaErrorMemoryAllocation, "DIRK autotune buffers");
  }
  if (!rc) rc = ck(cudaMemcpyAsync(tsave, c->S.Ts, sizeof(double) * ns,
                                           cudaMemcpyDeviceToDevice, s), "autotune save");
  if (!rc) rc = ck(cudaMemcpyAsync(tsave + ns, c->S.dTs_ge, sizeof(double) * ns,
                                           cudaMemcpyDeviceToDevice, s), "autotune save");
  const int cand[2] = {32, 64};
  for (int k = 0; k < 2 && !rc; ++k) {
    rc = ck(cudaMemcpyAsync(ybuf, y, sizeof(double) * 10 * ns, cudaMemcpyDeviceToDevice, s),
                    "autotune sample");
    if (!rc) rc = ck(cudaMemcpyAsync(c->S.Ts, tsave, sizeof(double) * ns,
                                             cudaMemcpyDeviceToDevice, s), "autotune restore");
    if (!rc) rc = ck(cudaMemcpyAsync(c->S.dTs_ge, tsave + ns, sizeof(double) * ns,
                                             cudaMemcpyDeviceToDevice, s), "autotune restore");
    if (!rc) rc = ck(cudaEventRecord(e0, s), "autotune event");
    if (rc) break;
    const int r = chem_dirk(c->P, c->S, ns, ybuf, O, mixed, cand[k], c->d_next, nullptr,
                            c->d_info, s, nullptr, &c->order);  // failures: a scratch word
    if (r == GBMV_EUNSUPPORTED) continue;  // does not fit on an SM
    if (r) { rc = r; break; }
    rc = ck(cudaEventRecord(e1, s), "autotune event");
    if (!rc) rc = ck(cudaEventSynchronize(e1), "autotune run");
    float ms = 0.f;
    if (!rc) rc = ck(cudaEventElapsedTime(&ms, e0, e1), "autotune time");
    if (!rc && (best_ms == 0.f || ms < best_ms)) { best_ms = ms; best = cand[k]; }
  }
  if (!rc) {
    rc = ck(cudaMemcpyAsync(c->S.Ts, tsave, sizeof(double) * ns, cudaMemcpyDeviceToDevice, s),
                    "autotune restore");
    if (!rc) rc = ck(cudaMemcpyAsync(c->S.dTs_ge, tsave + ns, sizeof(double) * ns,
                                             cudaMemcpyDeviceToDevice, s), "autotune restore");
    if (!rc) rc = ck(cudaStreamSynchronize(s), "autotune restore");
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(ybuf);
  cudaFree(tsave);
  if (rc) return rc;
  c->dirk_block[mixed] = best;
  return GBMV_OK;
}

static int dirk_launch(gbmv_chem c, double t0, double tout, double* y, double time_units,
                       const gbmv_dirk_opts* opts, int* stats, int* d_nfail, cudaStream_t s,
                       bool may_tune) {
  if (!c || !y || !d_nfail) { set_error("null argument"); return GBMV_EINVAL; }
  DirkOpts O;
  int rc = dirk_opts(opts, t0, tout, time_units, &O);
  if (!rc) rc = dirk_store(c, &O, s);
  if (rc) return rc;
  const int mixed = opts->precision == GBMV_MIXED;
  int block = opts->block ? opts->block : c->dirk_block[mixed];
  if (!block) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (!may_tune ||
        (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)) {
      set_error("DIRK block size not tuned yet: set opts->block or make a synchronous call first");
      return GBMV_EINVAL;
    }
    rc = dirk_autotune(c, y, O, mixed, s);
    if (rc) return rc;
    block = c->dirk_block[mixed];
  }
  rc = chem_dirk(c->P, c->S, c->n, y, O, mixed, block, c->d_next, stats, d_nfail, s,
                 &c->retry, &c->order);
  if (rc == GBMV_EUNSUPPORTED) set_error("DIRK block of %d threads does not fit on an SM", block);
  return rc;
}

int gbmv_chem_dirk_evolve(gbmv_chem c, double t0, double tout, double* y, double time_units,
                          const gbmv_dirk_opts* opts, int* stats, void* stream) {
  if (!c) { set_error("null handle"); return GBMV_EINVAL; }
  cudaStream_t s = (cudaStream_t)stream;
  GBMV_CUDA_TRY(cudaMemsetAsync(c->d_nfail, 0, sizeof(int), s));
  int rc = dirk_launch(c, t0, tout, y, time_units, opts, stats, c->d_nfail, s, true);
  if (rc) return rc;
  int h = 0;
  GBMV_CUDA_TRY(cudaMemcpyAsync(&h, c->d_nfail, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  return h;
}

int gbmv_chem_dirk_evolve_async(gbmv_chem c, double t0, double tout, double* y,
                                double time_units, const gbmv_dirk_opts* opts, int* stats,
                                int* d_nfail, void* stream) {
  return dirk_launch(c, t0, tout, y, time_units, opts, stats, d_nfail, (cudaStream_t)stream,
                     false);
}

int gbmv_chem_set_newton_occupancy(gbmv_chem c, int blocks_per_sm) {
  if (!c || blocks_per_sm < 0 || blocks_per_sm > 32) {
    set_error("blocks_per_sm must be 0 (default) to 32");
    return GBMV_EINVAL;
  }
  c->newton_bps = blocks_per_sm;
  return GBMV_OK;
}

int gbmv_chem_newton_autotune(gbmv_chem c, const double* y, double gamma, double time_units,
                              int lu_precision, int refine, int* blocks_per_sm, void* stream) {
  if (!c || !y || (lu_precision != GBMV_FP64 && lu_precision != GBMV_MIXED) || refine < 0) {
    set_error("bad Newton autotune arguments");
    return GBMV_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (capturing(s)) {
    set_error("the Newton autotuner times launches: call it outside any stream capture");
    return GBMV_EINVAL;
  }
  const long n = c->n;
  double *buf = nullptr;  // f, x, saved Ts and dTs/dge
  if (cudaMalloc(&buf, sizeof(double) * 22 * n) != cudaSuccess) {
    cudaGetLastError();
    set_error("autotune buffer allocation failed");
    return GBMV_ENOMEM;
  }
  double *f = buf, *x = buf + 10 * n, *ts = buf + 20 * n;
  int rc = ck(cudaMemcpyAsync(ts, c->S.Ts, sizeof(double) * n, cudaMemcpyDeviceToDevice, s),
              "autotune save");
  if (!rc) rc = ck(cudaMemcpyAsync(ts + n, c->S.dTs_ge, sizeof(double) * n,
                                   cudaMemcpyDeviceToDevice, s), "autotune save");
  const int cand[7] = {0, 2, 3, 4, 5, 6, 8};  // 0: the deep grid-stride grid
  int best = -1;
  float best_ms = 0.f;
  for (int k = 0; k < 7 && !rc; ++k) {
    const float ms = time_runs(s, [&]() {
      GBMV_CUDA_TRY(cudaMemcpyAsync(c->S.Ts, ts, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                    s));
      return chem_newton(c->P, c->S, n, y, f, x, gamma, time_units,
                         lu_precision == GBMV_MIXED, refine, c->d_info, s, cand[k]);
    });
    if (ms < 0.f) { rc = GBMV_ECUDA; break; }
    if (best < 0 || ms < best_ms) { best = cand[k]; best_ms = ms; }
  }
  if (!rc) rc = ck(cudaMemcpyAsync(c->S.Ts, ts, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                   s), "autotune restore");
  if (!rc) rc = ck(cudaMemcpyAsync(c->S.dTs_ge, ts + n, sizeof(double) * n,
                                   cudaMemcpyDeviceToDevice, s), "autotune restore");
  if (!rc) rc = ck(cudaStreamSynchronize(s), "autotune restore");
  cudaFree(buf);
  if (rc) return rc;
  c->newton_bps = best;
  if (blocks_per_sm) *blocks_per_sm = best;
  return GBMV_OK;
}

int gbmv_chem_dirk_retried(gbmv_chem c, int* cells, int max_cells, void* stream) {
  if (!c) { set_error("null handle"); return GBMV_EINVAL; }
  if (!c->dirk_retry) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  int count = 0;
  GBMV_CUDA_TRY(cudaMemcpyAsync(&count, c->retry.count, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  const int k = cells ? (count < max_cells ? count : max_cells) : 0;
  if (k > 0) {
    GBMV_CUDA_TRY(cudaMemcpyAsync(cells, c->retry.list, sizeof(int) * k, cudaMemcpyDeviceToHost, s));
    GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return count;
}

int gbmv_chem_dirk_block(gbmv_chem c, int precision) {
  if (!c || (precision != GBMV_FP64 && precision != GBMV_MIXED)) return 0;
  return c->dirk_block[precision == GBMV_MIXED];
}

/* ------------------------------------------------------------------ block solve */

// Status word of gbmv_block_lu_factor, which takes no handle: one word per (host thread,
// device), allocated on that device at the thread's first factorisation there.  A call resets,
// fills and reads its word before it returns, so calls of one thread never overlap, calls of
// different threads use different words, and a word is never read on another device.
// (4 bytes per thread and device stay allocated until the process exits.)
static int* lu_info_buffer() {
  constexpr int kMaxDev = 64;
  static thread_local int* buf[kMaxDev] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) {
    cudaGetLastError();
    set_error("no usable current device for the block factorisation status word");
    return nullptr;
  }
  if (!buf[dev] && cudaMalloc(&buf[dev], sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    buf[dev] = nullptr;
    set_error("device allocation of the block factorisation status word failed");
    return nullptr;
  }
  return buf[dev];
}

int gbmv_block_lu_factor(long nblocks, double* A, int* pivots, void* stream) {
  if (nblocks <= 0 || !A || !pivots) { set_error("bad factor arguments"); return GBMV_EINVAL; }
  int* info = lu_info_buffer();
  if (!info) return GBMV_ENOMEM;
  cudaStream_t s = (cudaStream_t)stream;
  GBMV_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(int), s));
  int rc = block_lu_factor(nblocks, A, pivots, info, s);
  if (rc) return rc;
  int h = 0;
  GBMV_CUDA_TRY(cudaMemcpyAsync(&h, info, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  if (h) { set_error("singular block"); return 1; }
  return GBMV_OK;
}

// Block linear solver handle: owns the pivots and its own singular-block word.
struct gbmv_block_ls_s {
  long nblocks = 0;
  int* pivots = nullptr;
  int* d_info = nullptr;
};

int gbmv_block_ls_create(long nblocks, gbmv_block_ls* out) {
  if (!out || nblocks <= 0) { set_error("bad block solver arguments"); return GBMV_EINVAL; }
  *out = nullptr;
  gbmv_block_ls L = new (std::nothrow) gbmv_block_ls_s();
  if (!L) return GBMV_ENOMEM;
  L->nblocks = nblocks;
  if (cudaMalloc(&L->pivots, sizeof(int) * 10 * nblocks) != cudaSuccess ||
      cudaMalloc(&L->d_info, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(L->pivots);
    delete L;
    set_error("device allocation of the block solver's pivots failed");
    return GBMV_ENOMEM;
  }
  *out = L;
  return GBMV_OK;
}

int gbmv_block_ls_destroy(gbmv_block_ls L) {
  if (!L) return GBMV_OK;
  cudaFree(L->pivots);
  cudaFree(L->d_info);
  delete L;
  return GBMV_OK;
}

int gbmv_block_ls_setup(gbmv_block_ls L, double* A, void* stream) {
  if (!L || !A) { set_error("null block solver or matrix"); return GBMV_EINVAL; }
  cudaStream_t s = (cudaStream_t)stream;
  GBMV_CUDA_TRY(cudaMemsetAsync(L->d_info, 0, sizeof(int), s));
  int rc = block_lu_factor(L->nblocks, A, L->pivots, L->d_info, s);
  if (rc) return rc;
  int h = 0;
  GBMV_CUDA_TRY(cudaMemcpyAsync(&h, L->d_info, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  if (h) { set_error("singular block"); return 1; }
  return GBMV_OK;
}

int gbmv_block_ls_solve(gbmv_block_ls L, const double* LU, const double* b, double* x,
                        void* stream) {
  if (!L || !LU || !b || !x) { set_error("bad block solve arguments"); return GBMV_EINVAL; }
  return block_lu_solve(L->nblocks, LU, L->pivots, b, x, (cudaStream_t)stream);
}

int gbmv_block_lu_solve(long nblocks, const double* LU, const int* pivots, const double* b,
                        double* x, void* stream) {
  if (nblocks <= 0 || !LU || !pivots || !b || !x) { set_error("bad solve arguments"); return GBMV_EINVAL; }
  return block_lu_solve(nblocks, LU, pivots, b, x, (cudaStream_t)stream);
}

int gbmv_block_form_newton(long nblocks, double* J, double gamma, void* stream) {
  if (nblocks <= 0 || !J) return GBMV_EINVAL;
  return block_form_newton(nblocks, J, gamma, (cudaStream_t)stream);
}

/* ------------------------------------------------------------------ glue */

int gbmv_fexpl_async(gbmv_hydro h, gbmv_chem c, double t, double* const* w,
                     double* const* wdot, double energy_units, int precision, int* d_status,
                     void* stream) {
  if (!h || !c || h->g.nchem != 10 || c->n != h->g.ncell || !d_status) {
    set_error("fexpl needs a 10-species hydro grid matching the chemistry cell count");
    return GBMV_EINVAL;
  }
  if (!fields_ok(w, 10) || !fields_ok(wdot, 10)) return GBMV_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  (void)t;
  // FP64 form: the reference's in-place scale / unscale of the chemistry component (its
  // rounding included); mixed form: w[5] is left untouched (the scale is applied where the
  // WENO reads it), so a concurrent chemistry branch may read w[5] during the sweep
  const bool fp64 = precision == GBMV_FP64;
  int rc = energy_sync(c->S, w, c->n, 10, 1.0 / energy_units, fp64 ? 0 : 2, s);
  if (rc) return rc;
  rc = feuler_dispatch(h, (const double* const*)w, wdot, precision, 0, d_status, s,
                       fp64 ? nullptr : c->S.scale);
  if (rc) return rc;
  return energy_epilogue(c->S, w[5], wdot[5], wdot[4], c->n, 10, fp64 ? 1 : 2, s);
}

int gbmv_fexpl(gbmv_hydro h, gbmv_chem c, double t, double* const* w, double* const* wdot,
               double energy_units, int precision, void* stream) {
  if (!h || !c || h->g.nchem != 10 || c->n != h->g.ncell) {
    set_error("fexpl needs a 10-species hydro grid matching the chemistry cell count");
    return GBMV_EINVAL;
  }
  if (!fields_ok(w, 10) || !fields_ok(wdot, 10)) return GBMV_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  GBMV_CUDA_TRY(cudaMemsetAsync(h->d_status, 0, sizeof(int), s));
  int rc = gbmv_fexpl_async(h, c, t, w, wdot, energy_units, precision, h->d_status, stream);
  if (rc) return rc;
  int st = 0;
  GBMV_CUDA_TRY(cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  if (st) {
    set_error("illegal state (mask %d: 1 density, 2 energy, 4 pressure)", st);
    return GBMV_ILLEGAL_STATE;
  }
  return GBMV_OK;
}

int gbmv_ffast(gbmv_hydro h, gbmv_chem c, double t, const double* const* w, double* const* wdot,
               double time_units, int nforcing, const double* const* forcing, double tshift,
               double tscale, void* stream) {
  if (!h || !c || h->g.nchem != 10 || c->n != h->g.ncell) {
    set_error("ffast needs a 10-species hydro grid matching the chemistry cell count");
    return GBMV_EINVAL;
  }
  if (!fields_ok(w, 10) || !fields_ok(wdot, 10) || nforcing < 0 || nforcing > kMaxForcing ||
      (nforcing > 0 && (!forcing || !(tscale != 0.0)))) {
    set_error("bad ffast arguments (nforcing 0-%d, forcing pointers, tscale != 0)", kMaxForcing);
    return GBMV_EINVAL;
  }
  ForcingSet F{};
  const double tau = nforcing > 0 ? (t - tshift) / tscale : 0.0;
  for (int i = 0; i < nforcing; ++i) {
    double p = 1.0;  // SUNRpowerI(tau, i): repeated multiplication
    for (int q = 0; q < i; ++q) p *= tau;
    F.c[i] = p;
    for (int k = 0; k < 6; ++k) {
      F.x[i][k] = forcing[i * 6 + k];
      if (!F.x[i][k]) { set_error("null forcing vector %d component %d", i, k); return GBMV_EINVAL; }
    }
  }
  cudaStream_t s = (cudaStream_t)stream;
  DevFields6 D;
  for (int k = 0; k < 6; ++k) D.f[k] = wdot[k];
  int rc = chem_rhs(c->P, c->S, c->n, w[5], wdot[5], time_units, s);  // wdot[5] fully written
  if (rc) return rc;
  return mri_forcing(c->n, F, nforcing, D, true, 6, s);
}

// The fast evolve shared by gbmv_mri_fast_evolve (synchronous, may tune the DIRK block size)
// and gbmv_mri_fast_evolve_async (graph-capturable: failures added to *d_nfail).
static int mri_fast_launch(gbmv_hydro h, gbmv_chem c, double t0, double tout, double* const* w,
                           double time_units, int nforcing, const double* const* forcing,
                           double tshift, double tscale, const gbmv_dirk_opts* opts, int* stats,
                           int* d_nfail, cudaStream_t s, bool may_tune) {
  if (!h || !c || h->g.nchem != 10 || c->n != h->g.ncell || !fields_ok(w, 10)) {
    set_error("mri_fast_evolve needs a 10-species hydro grid matching the chemistry cells");
    return GBMV_EINVAL;
  }
  if (nforcing < 0 || nforcing > kMaxForcing || (nforcing > 0 && (!forcing || !(tscale != 0.0)))) {
    set_error("bad forcing arguments (nforcing 0-%d, forcing pointers, tscale != 0)", kMaxForcing);
    return GBMV_EINVAL;
  }
  DirkOpts O;
  int rc = dirk_opts(opts, t0, tout, time_units, &O);
  if (!rc) rc = dirk_store(c, &O, s);
  if (rc) return rc;
  ForcingSet Ff{};
  const double tau0 = nforcing > 0 ? (t0 - tshift) / tscale : 0.0;
  const double tau1 = nforcing > 0 ? (tout - tshift) / tscale : 0.0;
  double p0 = tau0, p1 = tau1;  // tau^(i+1)
  for (int i = 0; i < nforcing; ++i) {
    for (int k = 0; k < 6; ++k)
      if (!forcing[i * 6 + k]) { set_error("null forcing vector %d component %d", i, k); return GBMV_EINVAL; }
    // fluid components: exact integral of the forcing polynomial over [t0, tout]
    Ff.c[i] = tscale * (p1 - p0) / (double)(i + 1);
    for (int k = 0; k < 6; ++k) Ff.x[i][k] = forcing[i * 6 + k];
    O.fz[i] = forcing[i * 6 + 5];  // chemistry component: inside the DIRK right-hand side
    p0 *= tau0;
    p1 *= tau1;
  }
  O.nforcing = nforcing;
  O.tshift = tshift;
  O.tscale = tscale;
  const int mixed = opts->precision == GBMV_MIXED;
  int block = opts->block ? opts->block : c->dirk_block[mixed];
  if (!block) {
    if (!may_tune || capturing(s)) {
      set_error("DIRK block size not tuned yet: set opts->block or make a synchronous call first");
      return GBMV_EINVAL;
    }
    O.nforcing = 0;  // tune on the unforced problem (same work per evaluation within a few %)
    rc = dirk_autotune(c, w[5], O, mixed, s);
    if (rc) return rc;
    O.nforcing = nforcing;
    block = c->dirk_block[mixed];
  }
  if (nforcing > 0) {
    DevFields6 D;
    for (int k = 0; k < 6; ++k) D.f[k] = w[k];
    rc = mri_forcing(c->n, Ff, nforcing, D, false, 5, s);  // components 0-4 only
    if (rc) return rc;
  }
  return chem_dirk(c->P, c->S, c->n, w[5], O, mixed, block, c->d_next, stats, d_nfail, s,
                   &c->retry, &c->order);
}

int gbmv_mri_fast_evolve(gbmv_hydro h, gbmv_chem c, double t0, double tout, double* const* w,
                         double time_units, int nforcing, const double* const* forcing,
                         double tshift, double tscale, const gbmv_dirk_opts* opts, int* stats,
                         void* stream) {
  if (!c) { set_error("null handle"); return GBMV_EINVAL; }
  cudaStream_t s = (cudaStream_t)stream;
  GBMV_CUDA_TRY(cudaMemsetAsync(c->d_nfail, 0, sizeof(int), s));
  int rc = mri_fast_launch(h, c, t0, tout, w, time_units, nforcing, forcing, tshift, tscale,
                           opts, stats, c->d_nfail, s, true);
  if (rc) return rc;
  int nf = 0;
  GBMV_CUDA_TRY(cudaMemcpyAsync(&nf, c->d_nfail, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  return nf;
}

int gbmv_mri_fast_evolve_async(gbmv_hydro h, gbmv_chem c, double t0, double tout,
                               double* const* w, double time_units, int nforcing,
                               const double* const* forcing, double tshift, double tscale,
                               const gbmv_dirk_opts* opts, int* stats, int* d_nfail,
                               void* stream) {
  if (!d_nfail) { set_error("null failure counter"); return GBMV_EINVAL; }
  return mri_fast_launch(h, c, t0, tout, w, time_units, nforcing, forcing, tshift, tscale,
                         opts, stats, d_nfail, (cudaStream_t)stream, false);
}

static bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

int gbmv_feuler_jvp(gbmv_hydro h, double t, const double* const* w, const double* const* dw,
                    double* const* jv, void* stream) {
  (void)t;
  if (!h || !fields_ok(w, h->g.nchem) || !fields_ok(dw, h->g.nchem) ||
      !fields_ok(jv, h->g.nchem)) {
    set_error("null handle or field pointer");
    return GBMV_EINVAL;
  }
  Fields W, D, O;
  for (int v = 0; v < 6; ++v) {
    W.f[v] = const_cast<double*>(w[v]);
    D.f[v] = const_cast<double*>(dw[v]);
    O.f[v] = jv[v];
  }
  return feuler_jvp(h->g, W, D, O, h->scratch, (cudaStream_t)stream);
}

int gbmv_feuler_vjp(gbmv_hydro h, double t, const double* const* w, const double* const* v,
                    double* const* u, void* stream) {
  (void)t;
  if (!h || !fields_ok(w, h->g.nchem) || !fields_ok(v, h->g.nchem) ||
      !fields_ok(u, h->g.nchem)) {
    set_error("null handle or field pointer");
    return GBMV_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (!h->adj) {
    if (capturing(s)) {
      set_error("the first gbmv_feuler_vjp call on a handle allocates its buffer: make it "
                "before any stream capture");
      return GBMV_EINVAL;
    }
    const size_t nd = feuler_vjp_scratch_doubles(h->g);
    if (cudaMalloc(&h->adj, nd * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      h->adj = nullptr;
      set_error("device allocation of %zu adjoint doubles failed", nd);
      return GBMV_ENOMEM;
    }
  }
  Fields W, V, U;
  for (int k = 0; k < 6; ++k) {
    W.f[k] = const_cast<double*>(w[k]);
    V.f[k] = const_cast<double*>(v[k]);
    U.f[k] = u[k];
  }
  return feuler_vjp(h->g, W, V, U, h->adj, s);
}

int gbmv_chem_jvp(gbmv_chem c, double t, const double* y, const double* dy, double* jv,
                  double time_units, void* stream) {
  (void)t;
  if (!c || !y || !dy || !jv) { set_error("null argument"); return GBMV_EINVAL; }
  return chem_jvp(c->P, c->S, c->n, y, dy, jv, time_units, 0, (cudaStream_t)stream);
}

int gbmv_chem_vjp(gbmv_chem c, double t, const double* y, const double* v, double* u,
                  double time_units, void* stream) {
  (void)t;
  if (!c || !y || !v || !u) { set_error("null argument"); return GBMV_EINVAL; }
  return chem_jvp(c->P, c->S, c->n, y, v, u, time_units, 1, (cudaStream_t)stream);
}

int gbmv_postprocess_step(gbmv_hydro h, gbmv_chem c, double* const* w, double energy_units,
                          void* stream) {
  if (!h || !c || h->g.nchem != 10 || !fields_ok(w, 10)) return GBMV_EINVAL;
  return energy_sync(c->S, w, c->n, 10, 1.0 / energy_units, 1, (cudaStream_t)stream);
}

int gbmv_pack1d(gbmv_hydro h, const double* const* w, int dir, double* out, void* stream) {
  if (!h || !fields_ok(w, h->g.nchem) || !out || dir < 0 || dir > 2) {
    set_error("bad pack1d arguments (dir 0, 1 or 2)");
    return GBMV_EINVAL;
  }
  Fields W;
  for (int v = 0; v < 6; ++v) W.f[v] = (v < 5 || h->g.nchem) ? const_cast<double*>(w[v]) : nullptr;
  return pack1d(h->g, W, dir, out, (cudaStream_t)stream);
}

// the reduction scratch of a hydro handle (conservation totals, WRMS norms), allocated on
// first use
static int reduction_scratch(gbmv_hydro h, cudaStream_t s, const char* who) {
  if (h->cons) return GBMV_OK;
  if (capturing(s)) {
    set_error("the first %s call on a handle allocates its buffer: make it before any stream "
              "capture", who);
    return GBMV_EINVAL;
  }
  if (cudaMalloc(&h->cons, reduction_scratch_doubles() * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    h->cons = nullptr;
    return check_cuda(cudaErrorMemoryAllocation, "reduction scratch");
  }
  return GBMV_OK;
}

int gbmv_conservation(gbmv_hydro h, const double* const* w, double mass_factor,
                      double energy_factor, double* totals, void* stream) {
  if (!h || !fields_ok(w, 0) || !totals) {
    set_error("null handle, field or output pointer");
    return GBMV_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (int rc = reduction_scratch(h, s, "gbmv_conservation")) return rc;
  Fields W;
  for (int v = 0; v < 6; ++v) W.f[v] = (v < 5) ? const_cast<double*>(w[v]) : nullptr;
  int rc = conservation_sums(h->g, W, h->cons, s);
  if (rc) return rc;
  double t[2];
  GBMV_CUDA_TRY(cudaMemcpyAsync(t, h->cons + conservation_scratch_doubles() - 2, sizeof t,
                                cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  totals[0] = t[0] * mass_factor;
  totals[1] = t[1] * energy_factor;
  return GBMV_OK;
}

int gbmv_wrms_norm(gbmv_hydro h, const double* const* v, const double* const* y, double rtol,
                   double atol, double* norm, void* stream) {
  if (!h || !fields_ok(v, h->g.nchem) || !fields_ok(y, h->g.nchem) || !norm) {
    set_error("null handle, field or output pointer");
    return GBMV_EINVAL;
  }
  if (!(rtol >= 0.0) || !(atol >= 0.0) || !(rtol > 0.0 || atol > 0.0)) {
    set_error("rtol, atol must be >= 0 and not both 0");
    return GBMV_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (int rc = reduction_scratch(h, s, "gbmv_wrms_norm")) return rc;
  Fields V, Y;
  for (int k = 0; k < 6; ++k) {
    V.f[k] = const_cast<double*>(v[k]);
    Y.f[k] = const_cast<double*>(y[k]);
  }
  int rc = wrms_norm(h->g, V, Y, rtol, atol, h->cons, s);
  if (rc) return rc;
  GBMV_CUDA_TRY(cudaMemcpyAsync(norm, h->cons + conservation_scratch_doubles() - 2,
                                sizeof(double), cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  return GBMV_OK;
}

int gbmv_feuler_kink_mask(gbmv_hydro h, const double* const* w, const double* const* dw,
                          double eps, unsigned char* mask, void* stream) {
  if (!h || !fields_ok(w, h->g.nchem) || !fields_ok(dw, h->g.nchem) || !mask ||
      !(eps >= 0.0)) {
    set_error("null handle, field or mask pointer, or eps < 0");
    return GBMV_EINVAL;
  }
  Fields W, D;
  for (int k = 0; k < 6; ++k) {
    W.f[k] = const_cast<double*>(w[k]);
    D.f[k] = const_cast<double*>(dw[k]);
  }
  return feuler_kink_mask(h->g, W, D, eps, mask, (cudaStream_t)stream);
}

int gbmv_wrms_norm_async(gbmv_hydro h, const double* const* v, const double* const* y,
                         double rtol, double atol, double* d_norm, void* stream) {
  if (!h || !fields_ok(v, h->g.nchem) || !fields_ok(y, h->g.nchem) || !d_norm) {
    set_error("null handle, field or output pointer");
    return GBMV_EINVAL;
  }
  if (!(rtol >= 0.0) || !(atol >= 0.0) || !(rtol > 0.0 || atol > 0.0)) {
    set_error("rtol, atol must be >= 0 and not both 0");
    return GBMV_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (int rc = reduction_scratch(h, s, "gbmv_wrms_norm_async")) return rc;
  Fields V, Y;
  for (int k = 0; k < 6; ++k) {
    V.f[k] = const_cast<double*>(v[k]);
    Y.f[k] = const_cast<double*>(y[k]);
  }
  int rc = wrms_norm(h->g, V, Y, rtol, atol, h->cons, s);
  if (rc) return rc;
  GBMV_CUDA_TRY(cudaMemcpyAsync(d_norm, h->cons + conservation_scratch_doubles() - 2,
                                sizeof(double), cudaMemcpyDeviceToDevice, s));
  return GBMV_OK;
}

int gbmv_print_stats(gbmv_hydro h, const double* const* w, double density_units,
                     double momentum_units, double energy_units, double* rms, void* stream) {
  if (!h || !fields_ok(w, h->g.nchem) || !rms) {
    set_error("null handle, field or output pointer");
    return GBMV_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (int rc = reduction_scratch(h, s, "gbmv_print_stats")) return rc;
  Fields W;
  for (int k = 0; k < 6; ++k) W.f[k] = (k < 5 || h->g.nchem) ? const_cast<double*>(w[k]) : nullptr;
  int rc = field_rms(h->g, W, density_units, momentum_units, energy_units, h->cons, s);
  if (rc) return rc;
  const int nv = 5 + h->g.nchem;
  GBMV_CUDA_TRY(cudaMemcpyAsync(rms, h->cons + reduction_scratch_doubles() - 16,
                                sizeof(double) * nv, cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  return GBMV_OK;
}

int gbmv_stability(gbmv_hydro h, const double* const* w, double cfl, double* dt_stab,
                   void* stream) {
  if (!h || !fields_ok(w, 0) || !dt_stab) return GBMV_EINVAL;
  Fields W;
  for (int v = 0; v < 6; ++v) W.f[v] = (v < 5) ? const_cast<double*>(w[v]) : nullptr;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long* d = reinterpret_cast<unsigned long long*>(h->d_status);  // 8-byte slot
  int rc = wave_speed_max(h->g, W, d, s);
  if (rc) return rc;
  unsigned long long bits = 0;
  GBMV_CUDA_TRY(cudaMemcpyAsync(&bits, d, sizeof bits, cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  double alpha;
  memcpy(&alpha, &bits, sizeof alpha);
  const double dmin = fmin(fmin(h->g.d[0], h->g.d[1]), h->g.d[2]);
  *dt_stab = cfl * dmin / alpha;
  return GBMV_OK;
}

}  // extern "C"
