// Device-resident adaptive step control for integrators whose whole step is a CUDA graph: the
// accept / reject decision, ARKODE's step-size controllers and the end-of-interval clamp run in
// one-thread kernels on the integration stream, so a host loop replays step graphs without
// reading anything back until it wants to (no counterpart in the reference, whose ARKStep
// makes these decisions on the host after a synchronising norm).
//
// The controller is ARKODE's (arkode_adapt.c conventions): e = bias * dsm,
//   eta = safety * e_n^(-k1/k) * e_{n-1}^(k2/k) * e_{n-2}^(-k3/k)   (k the embedding order),
// bounded by etamx1 on the first step and growth after, kept at 1 inside [1, 1.5) and after
// a failure, at least 0.1; after an error-test failure eta = max(0.1, min(1, safety
// e^(-1/k))), at most etamxf from the small_nef-th failure of a step on.
#include <math.h>

#include "common.cuh"

namespace gbmv {
namespace {

__global__ void step_begin_kernel(double* st, gbmv_step_params p) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double t = st[GBMV_ST_T];
  double h = st[GBMV_ST_H];
  if (p.hmax > 0.0 && h > p.hmax) h = p.hmax;
  const double rem = st[GBMV_ST_TF] - t;
  if (st[GBMV_ST_DONE] != 0.0 || st[GBMV_ST_STATUS] != 0.0 || !(rem > 0.0)) {
    st[GBMV_ST_DONE] = 1.0;
    st[GBMV_ST_HUSED] = 0.0;
    st[GBMV_ST_ACCEPT] = 0.0;
    return;
  }
  st[GBMV_ST_LAST] = (h >= rem) ? 1.0 : 0.0;
  st[GBMV_ST_HPROP] = h;
  st[GBMV_ST_HUSED] = (h >= rem) ? rem : h;
}

__global__ void step_end_kernel(double* st, const double* __restrict__ dsm_p, gbmv_step_params p) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (st[GBMV_ST_DONE] != 0.0) {  // nothing was attempted
    st[GBMV_ST_ACCEPT] = 0.0;
    return;
  }
  double dsm = p.fixed ? 0.0 : *dsm_p;
  if (!isfinite(dsm)) dsm = 1e10;
  const double k = (double)p.order;
  const double hu = st[GBMV_ST_HUSED];
  st[GBMV_ST_ATTEMPTS] += 1.0;
  if (dsm <= 1.0) {
    st[GBMV_ST_ACCEPT] = 1.0;
    st[GBMV_ST_STEPS] += 1.0;
    const bool last = st[GBMV_ST_LAST] != 0.0;
    st[GBMV_ST_T] = last ? st[GBMV_ST_TF] : st[GBMV_ST_T] + hu;
    if (last) st[GBMV_ST_DONE] = 1.0;
    double h;
    if (p.fixed) {
      h = st[GBMV_ST_HPROP];
    } else {
      const double e1 = fmax(p.bias * dsm, 1e-10);
      double eta = pow(e1, -p.k1 / k);
      if (p.k2 != 0.0) eta *= pow(st[GBMV_ST_E1], p.k2 / k);
      if (p.k3 != 0.0) eta *= pow(st[GBMV_ST_E2], -p.k3 / k);
      eta *= p.safety;
      eta = fmin(eta, st[GBMV_ST_FIRST] != 0.0 ? p.etamx1 : p.growth);
      if (st[GBMV_ST_NEF] > 0.0) eta = fmin(eta, 1.0);
      if (eta >= 1.0 && eta < 1.5) eta = 1.0;
      eta = fmax(eta, 0.1);
      h = hu * eta;
      if (p.hmax > 0.0 && h > p.hmax) h = p.hmax;
      st[GBMV_ST_E2] = st[GBMV_ST_E1];
      st[GBMV_ST_E1] = e1;
      // a step cut short to land on tf does not shrink the proposal for what follows
      if (last && st[GBMV_ST_HPROP] > h) h = st[GBMV_ST_HPROP];
    }
    st[GBMV_ST_H] = h;
    st[GBMV_ST_FIRST] = 0.0;
    st[GBMV_ST_NEF] = 0.0;
  } else {
    st[GBMV_ST_ACCEPT] = 0.0;
    st[GBMV_ST_FAILS] += 1.0;
    const double nef = st[GBMV_ST_NEF] + 1.0;
    st[GBMV_ST_NEF] = nef;
    if (nef >= (double)p.maxnef) {
      st[GBMV_ST_STATUS] = -1.0;  // too many error-test failures in one step
      st[GBMV_ST_DONE] = 1.0;
      return;
    }
    double eta = fmax(0.1, fmin(1.0, p.safety * pow(fmax(p.bias * dsm, 1e-10), -1.0 / k)));
    if (nef >= (double)p.small_nef) eta = fmin(eta, p.etamxf);
    st[GBMV_ST_H] = hu * eta;
  }
  if (st[GBMV_ST_ATTEMPTS] >= (double)p.max_attempts && st[GBMV_ST_DONE] == 0.0) {
    st[GBMV_ST_STATUS] = -2.0;  // attempt budget spent
    st[GBMV_ST_DONE] = 1.0;
  }
}

// y = accepted ? ynew : y over n doubles (the accepted flag read from the state)
__global__ void step_select_kernel(long n, const double* __restrict__ st, double* __restrict__ y,
                                   const double* __restrict__ ynew) {
  if (st[GBMV_ST_ACCEPT] == 0.0) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
    y[i] = ynew[i];
}

int check_params(const gbmv_step_params* p) {
  if (!p || p->order < 1 || !(p->safety > 0.0) || !(p->bias > 0.0) || !(p->growth >= 1.0) ||
      !(p->etamx1 >= 1.0) || !(p->etamxf > 0.0) || !(p->k1 > 0.0) || p->maxnef < 1 ||
      p->small_nef < 1 || p->max_attempts < 1 || !(p->hmax >= 0.0)) {
    set_error("bad step-control parameters");
    return GBMV_EINVAL;
  }
  return GBMV_OK;
}

}  // namespace
}  // namespace gbmv

using namespace gbmv;

extern "C" int gbmv_step_begin(double* d_state, const gbmv_step_params* p, void* stream) {
  if (!d_state) { set_error("null step state"); return GBMV_EINVAL; }
  if (int rc = check_params(p)) return rc;
  step_begin_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(d_state, *p);
  GBMV_LAUNCH_CHECK("step_begin_kernel");
  return GBMV_OK;
}

extern "C" int gbmv_step_end(double* d_state, const double* d_dsm, const gbmv_step_params* p,
                             void* stream) {
  if (!d_state || !d_dsm) { set_error("null step state or error norm"); return GBMV_EINVAL; }
  if (int rc = check_params(p)) return rc;
  step_end_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(d_state, d_dsm, *p);
  GBMV_LAUNCH_CHECK("step_end_kernel");
  return GBMV_OK;
}

extern "C" int gbmv_step_select(long n, const double* d_state, double* y, const double* ynew,
                                void* stream) {
  if (n <= 0 || !d_state || !y || !ynew) { set_error("bad step_select arguments"); return GBMV_EINVAL; }
  long blocks = (n + 255) / 256;
  if (blocks > 4L * kSM) blocks = 4L * kSM;
  step_select_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(n, d_state, y, ynew);
  GBMV_LAUNCH_CHECK("step_select_kernel");
  return GBMV_OK;
}
