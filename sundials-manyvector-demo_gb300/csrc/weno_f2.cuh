// Float-float (mixed) form of the WENO flux divergence (src/utilities.cpp:17-253):
//
//   prims_f2_kernel: once per cell, in FP64 exactly as the reference evaluates them per
//     stencil point -- pressure (eos), the three velocities m/rho and the sound speed
//     sqrt(gamma p / rho) -- then every field and primitive split into float pairs (hi, lo):
//     Q2[q][cell], q = rho, mx, my, mz, et, p, ux, uy, uz, c, tracers...;
//   face_flux_f2_kernel<NCHEM, DIR>: the face flux in float-float arithmetic from Q2 (no FP64
//     instruction on the common path), the two Lax-Friedrichs sides of every reconstruction
//     evaluated together on the paired FP32 instructions (df64x2.cuh); faces whose states
//     leave the float range, or touch a non-positive density (homogeneous Dirichlet ghosts),
//     are computed in FP64 from w;
//   divergence_f2: the FP64 form's divergence pass over fluxes kept as float pairs, the
//     differences in float-float, the final G - div in FP64 (weno.cu).
//
// The face-flux kernel is a template over the tracer count, the sweep direction and the weight
// variant WV (0: float-float weights everywhere; 1: FP32 weights and smoothness indicators for
// the tracer reconstructions, which are in correction form); weno_f2.cu instantiates WV = 0 and
// weno_f2_fast.cu WV = 1, so the two compile in parallel.
#pragma once

#include "common.cuh"
#include "weno_face.cuh"
#include "weno_sweep.cuh"

namespace gbmv {

constexpr int kQ2Base = 10;  // index of the first tracer in Q2

// Q2 from w, and the legal-state flags OR-ed into *d_status (weno_f2.cu)
int prims_f2(const Grid& g, const Fields& w, float2* q2, const double* tscale, int* d_status,
             cudaStream_t s);
// the WV = 1 sweep (weno_f2_fast.cu)
int feuler_f2_fast(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                   double* scratch, float2* q2, const double* tscale, int* d_status,
                   cudaStream_t s);

// Register budget (residency target, 128-thread blocks per SM; register allocation only:
// results are the same bit for bit).  WV = 1 (fewer instructions per face) runs fastest alone
// at 3 resident blocks per SM even with the register cap's spills (6.11 -> 5.63 ms per 128^3
// RHS against 2); WV = 0 at 1-2.  Beside the chemistry Newton on a second stream (255
// registers a thread) a WV = 1 sweep capped at 5 blocks per SM leaves the Newton warps room:
// the concurrent 128^3 stage measured 8.21 ms against 9.14 at 3 (Grid::sweep_shared).
constexpr int kF2FastMinB = 3;
constexpr int kF2FastSharedMinB = 5;
template <int NCHEM, int DIR, int WV, int MINB>
__global__ void __launch_bounds__(128, MINB)
    face_flux_f2_kernel(Grid g, Fields w, const float2* __restrict__ Q2,
                        float2* __restrict__ F, long nfaces) {
  const long nx = g.n[0], ny = g.n[1], n = g.ncell;
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < nfaces;
       f += (long)gridDim.x * blockDim.x) {
    long i, j, k;
    face_coords<DIR>(f, g, i, j, k);
    const long base[3] = {i, j, k};
    long cell[6];
    bool nall[6], nnorm[6];
#pragma unroll
    for (int l = 0; l < 6; ++l) {
      long p = base[DIR] - 3 + l;
      p = ghost_src(p, g.n[DIR], g.bc[2 * DIR], g.bc[2 * DIR + 1], &nall[l], &nnorm[l]);
      long q[3] = {i, j, k};
      q[DIR] = p;
      cell[l] = q[0] + nx * (q[1] + ny * q[2]);
    }
    f2 W[6][5];
    PointPrims<f2> pre;
    bool ok = true;
#pragma unroll
    for (int l = 0; l < 6; ++l) {
      // slots: rho, m_normal, m_t1, m_t2, et, p, u_normal, c
      const int src[8] = {0, 1 + DIR, DIR == 1 ? 1 : 2, DIR == 2 ? 1 : 3, 4, 5, 6 + DIR, 9};
      f2 q[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const float2 t = __ldg(Q2 + src[m] * n + cell[l]);
        q[m] = f2(t.x, t.y);
      }
      // homogeneous Dirichlet negates every conserved field (so p too; u and c unchanged);
      // reflecting negates the normal momentum (so the normal velocity)
      if (nall[l]) {
#pragma unroll
        for (int m = 0; m < 6; ++m) q[m] = -q[m];
      }
      if (nnorm[l]) {
        q[1] = -q[1];
        q[6] = -q[6];
      }
#pragma unroll
      for (int m = 0; m < 5; ++m) W[l][m] = q[m];
      pre.p[l] = q[5];
      pre.u[l] = q[6];
      pre.c[l] = q[7];
      ok = ok && (q[0].hi > 0.f);
#pragma unroll
      for (int m = 0; m < 6; ++m) ok = ok && (fabsf(q[m].hi) < 1e15f);
    }
    FaceState<f2> S;
    f2 o[5];
    if (ok) {
      // characteristic fields keep float-float weights in every mixed form: the reference's
      // eigenbasis (conditioning ~1/c^2) amplifies weight rounding in the back-projection
      fluid_face_flux_f2v(W, g.gamma, S, o, pre);
    } else {  // FP64, exactly the FP64 form's arithmetic
      double Wd[6][5];
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        double q[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) q[v] = __ldg(w.f[v] + cell[l]);
        if (nall[l]) {
#pragma unroll
          for (int v = 0; v < 5; ++v) q[v] = -q[v];
        }
        if (nnorm[l]) q[1 + DIR] = -q[1 + DIR];
        Wd[l][0] = q[0];
        Wd[l][1] = q[1 + DIR];
        Wd[l][2] = (DIR == 1) ? q[1] : q[2];
        Wd[l][3] = (DIR == 2) ? q[1] : q[3];
        Wd[l][4] = q[4];
      }
      FaceState<double> S64;
      double out[5];
      fluid_face_flux<double>(Wd, g.gamma, S64, out);
#pragma unroll
      for (int v = 0; v < 5; ++v) o[v] = f2_from_double(out[v]);
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        S.hp[l] = f2_from_double(S64.hp[l]);
        S.hm[l] = f2_from_double(S64.hm[l]);
      }
    }
    // fluxes stay float pairs: the divergence pass differences them in float-float
    const f2 o1 = o[1], oD = o[1 + DIR];
    o[1] = oD;
    o[1 + DIR] = o1;
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v * nfaces + f] = make_float2(o[v].hi, o[v].lo);
    if constexpr (MINB <= kF2FastMinB) {
      // two species per pass, two independent dependency chains (GBMV_MIXED 128^3 RHS 5.84 ->
      // 5.66 ms); under the shared register budget the extra live values spill, so that
      // budget keeps one species per pass (concurrent stage 8.46 against 8.30 ms)
      static_assert(NCHEM % 2 == 0, "tracers are reconstructed two at a time");
#pragma unroll 1
      for (int c = 0; c < NCHEM; c += 2) {
        f2 cv[6], cw[6];
#pragma unroll
        for (int l = 0; l < 6; ++l) {
          const float2 t = __ldg(Q2 + (kQ2Base + c) * n + cell[l]);
          const float2 u = __ldg(Q2 + (kQ2Base + c + 1) * n + cell[l]);
          cv[l] = nall[l] ? f2(-t.x, -t.y) : f2(t.x, t.y);
          cw[l] = nall[l] ? f2(-u.x, -u.y) : f2(u.x, u.y);
        }
        f2 r, q;
        tracer_face_flux_f2v_x2<WV>(S, cv, cw, r, q);
        F[(5 + c) * nfaces + f] = make_float2(r.hi, r.lo);
        F[(6 + c) * nfaces + f] = make_float2(q.hi, q.lo);
      }
    } else {
#pragma unroll 1
      for (int c = 0; c < NCHEM; ++c) {
        f2 cv[6];
#pragma unroll
        for (int l = 0; l < 6; ++l) {
          const float2 t = __ldg(Q2 + (kQ2Base + c) * n + cell[l]);
          cv[l] = nall[l] ? f2(-t.x, -t.y) : f2(t.x, t.y);
        }
        const f2 r = tracer_face_flux_f2v<WV>(S, cv);
        F[(5 + c) * nfaces + f] = make_float2(r.hi, r.lo);
      }
    }
  }
}

// the three face sweeps of one register budget
template <int NCHEM, int WV, int MINB>
int sweeps_f2(const Grid& g, const Fields& w, const float2* q2, float2* const (&F)[3],
              const long (&nf)[3], cudaStream_t s) {
  {
    ProfScope ps("face_flux", s);
    const int t = sweep_threads(g, nf[0], 128);
    face_flux_f2_kernel<NCHEM, 0, WV, MINB><<<sweep_blocks(nf[0], t), t, 0, s>>>(g, w, q2, F[0],
                                                                                  nf[0]);
    GBMV_LAUNCH_CHECK("face_flux_f2_kernel<x>");
  }
  {
    ProfScope ps("face_flux", s);
    const int t = sweep_threads(g, nf[1], 128);
    face_flux_f2_kernel<NCHEM, 1, WV, MINB><<<sweep_blocks(nf[1], t), t, 0, s>>>(g, w, q2, F[1],
                                                                                  nf[1]);
    GBMV_LAUNCH_CHECK("face_flux_f2_kernel<y>");
  }
  {
    ProfScope ps("face_flux", s);
    const int t = sweep_threads(g, nf[2], 128);
    face_flux_f2_kernel<NCHEM, 2, WV, MINB><<<sweep_blocks(nf[2], t), t, 0, s>>>(g, w, q2, F[2],
                                                                                  nf[2]);
    GBMV_LAUNCH_CHECK("face_flux_f2_kernel<z>");
  }
  return GBMV_OK;
}

template <int NCHEM, int WV>
int launch_f2(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
              double* scratch, float2* q2, const double* tscale, int* d_status, cudaStream_t s) {
  long nf[3];
  face_counts(g, nf);
  float2* const F2 = reinterpret_cast<float2*>(scratch);  // 8 bytes per flux, as a double
  float2* const F[3] = {F2, F2 + (long)(5 + NCHEM) * nf[0],
                        F2 + (long)(5 + NCHEM) * (nf[0] + nf[1])};
  int rc = prims_f2(g, w, q2, tscale, d_status, s);
  if (rc != GBMV_OK) return rc;
  if constexpr (WV == 1) {
    rc = g.sweep_shared ? sweeps_f2<NCHEM, WV, kF2FastSharedMinB>(g, w, q2, F, nf, s)
                        : sweeps_f2<NCHEM, WV, kF2FastMinB>(g, w, q2, F, nf, s);
  } else {
    rc = sweeps_f2<NCHEM, WV, 1>(g, w, q2, F, nf, s);
  }
  if (rc != GBMV_OK) return rc;
  return divergence_f2(g, wdot, F, G, s);
}

template <int WV>
int feuler_f2_wv(const Grid& g, const Fields& w, const Fields& wdot, const ForceTerm& G,
                 double* scratch, float2* q2, const double* tscale, int* d_status,
                 cudaStream_t s) {
  switch (g.nchem) {
    case 0: return launch_f2<0, WV>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 2: return launch_f2<2, WV>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 4: return launch_f2<4, WV>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 6: return launch_f2<6, WV>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    case 10: return launch_f2<10, WV>(g, w, wdot, G, scratch, q2, tscale, d_status, s);
    default: set_error("nchem=%d not compiled (0,2,4,6,10)", g.nchem); return GBMV_EUNSUPPORTED;
  }
}

}  // namespace gbmv
