// Derivatives of the WENO flux divergence (the FP64 form of fEuler, src/utilities.cpp:17-253):
//
//   JVP  jv = (d fEuler / d w) dw : forward mode -- the face flux evaluated on dual numbers
//        (value, tangent), the same templated code as the FP64 form, so the tangent is the
//        exact linearisation of what the FP64 kernel computes; then the (linear) divergence.
// The external forcing is constant in w, so it has no derivative.  Kinks (max over the
// stencil of |u| + c, |u|, the positivity guard of sqrt) take the branch the forward pass took.
#include "common.cuh"
#include "weno.cuh"
#include "weno_face.cuh"
#include "weno_sweep.cuh"

namespace gbmv {

// ------------------------------------------------------------------ dual numbers (JVP)

struct Dual {
  double v, d;
  Dual() = default;
  __host__ __device__ constexpr Dual(double x) : v(x), d(0.0) {}
  __host__ __device__ constexpr Dual(double x, double y) : v(x), d(y) {}
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) {
  return Dual(a.v * b.v, a.v * b.d + a.d * b.v);
}
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ bool operator<(Dual a, Dual b) { return a.v < b.v; }
__device__ __forceinline__ bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
__device__ __forceinline__ Dual num_from(double x, Dual*) { return Dual(x); }
__device__ __forceinline__ Dual num_sqrt(Dual x) {
  const double s = sqrt(x.v);
  return Dual(s, x.d / (2.0 * s));
}
__device__ __forceinline__ Dual num_fabs(Dual x) { return x.v < 0.0 ? -x : x; }
__device__ __forceinline__ Dual num_fma(Dual a, Dual b, Dual c) {
  return Dual(fma(a.v, b.v, c.v), a.v * b.d + a.d * b.v + c.d);
}
// the FP64 weight combination (product form, one division) on duals
__device__ __forceinline__ Dual weno_combine(Dual bA, Dual bB, Dual bC, Dual qA, Dual qB, Dual qC,
                                             Dual dA, Dual dB, Dual dC) {
  const Dual eps(1e-6);
  Dual aA = eps + bA, aB = eps + bB, aC = eps + bC;
  aA = aA * aA;
  aB = aB * aB;
  aC = aC * aC;
  const Dual tA = dA * (aB * aC), tB = dB * (aA * aC), tC = dC * (aA * aB);
  return (tA * qA + tB * qB + tC * qC) / (tA + tB + tC);
}
template <bool Plus>
__device__ __forceinline__ Dual weno_safe(Dual f0, Dual f1, Dual f2_, Dual f3, Dual f4) {
  return weno_side<Plus>(f0, f1, f2_, f3, f4);
}

// ------------------------------------------------------------------ JVP

template <int NCHEM, int DIR>
__global__ void __launch_bounds__(128) face_flux_jvp_kernel(Grid g, Fields w, Fields dw,
                                                            double* __restrict__ dF, long nfaces) {
  Dual* tag = nullptr;
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < nfaces;
       f += (long)gridDim.x * blockDim.x) {
    long cell[6], ijk[3];
    bool nall[6], nnorm[6];
    stencil<DIR>(g, f, cell, nall, nnorm, ijk);
    Dual W[6][5];
#pragma unroll
    for (int l = 0; l < 6; ++l) {
      double a[5], b[5];
      load_point<DIR>(w, cell[l], nall[l], nnorm[l], a);
      load_point<DIR>(dw, cell[l], nall[l], nnorm[l], b);
#pragma unroll
      for (int v = 0; v < 5; ++v) W[l][v] = Dual(a[v], b[v]);
    }
    FaceState<Dual> S;
    Dual out[5];
    fluid_face_flux<Dual>(W, g.gamma, S, out);
    double o[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) o[v] = out[v].d;
    const double o1 = o[1];
    o[1] = o[1 + DIR];
    o[1 + DIR] = o1;
#pragma unroll
    for (int v = 0; v < 5; ++v) dF[v * nfaces + f] = o[v];
#pragma unroll 1
    for (int c = 0; c < NCHEM; ++c) {
      Dual cv[6];
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        const double x = __ldg(w.f[5] + c + (long)NCHEM * cell[l]);
        const double dx = __ldg(dw.f[5] + c + (long)NCHEM * cell[l]);
        cv[l] = nall[l] ? Dual(-x, -dx) : Dual(x, dx);
      }
      dF[(5 + c) * nfaces + f] = tracer_face_flux<Dual>(S, cv).d;
    }
    (void)tag;
  }
}

// jv = -sum_d (dF_{d,+} - dF_{d,-}) / d_d
template <int NCHEM>
__global__ void __launch_bounds__(256) divergence_lin_kernel(Grid g, Fields out,
                                                             const double* __restrict__ Fx,
                                                             const double* __restrict__ Fy,
                                                             const double* __restrict__ Fz) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const long nfx = (nx + 1) * ny * nz, nfy = nx * (ny + 1) * nz, nfz = nx * ny * (nz + 1);
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < g.ncell;
       c += (long)gridDim.x * blockDim.x) {
    long i, j, k;
    split3(c, nx, ny, i, j, k);
    const long fx = i + (nx + 1) * (j + ny * k);
    const long fy = i + nx * (j + (ny + 1) * k);
    const long fz = c;
#pragma unroll
    for (int v = 0; v < 5 + NCHEM; ++v) {
      const double div = (Fx[v * nfx + fx + 1] - Fx[v * nfx + fx]) * g.inv_d[0] +
                         (Fy[v * nfy + fy + nx] - Fy[v * nfy + fy]) * g.inv_d[1] +
                         (Fz[v * nfz + fz + nx * ny] - Fz[v * nfz + fz]) * g.inv_d[2];
      double* dst = (v < 5) ? (out.f[v] + c) : (out.f[5] + (v - 5) + (long)NCHEM * c);
      *dst = -div;
    }
  }
}

// ------------------------------------------------------------------ launcher

template <int NCHEM>
static int jvp_t(const Grid& g, const Fields& w, const Fields& dw, const Fields& out,
                 double* scratch, cudaStream_t s) {
  long nf[3];
  face_counts(g, nf);
  double* F[3] = {scratch, scratch + (long)(5 + NCHEM) * nf[0],
                  scratch + (long)(5 + NCHEM) * (nf[0] + nf[1])};
  ProfScope ps("jvp", s);
  face_flux_jvp_kernel<NCHEM, 0><<<sweep_blocks(nf[0], 128), 128, 0, s>>>(g, w, dw, F[0], nf[0]);
  GBMV_LAUNCH_CHECK("face_flux_jvp_kernel<x>");
  face_flux_jvp_kernel<NCHEM, 1><<<sweep_blocks(nf[1], 128), 128, 0, s>>>(g, w, dw, F[1], nf[1]);
  GBMV_LAUNCH_CHECK("face_flux_jvp_kernel<y>");
  face_flux_jvp_kernel<NCHEM, 2><<<sweep_blocks(nf[2], 128), 128, 0, s>>>(g, w, dw, F[2], nf[2]);
  GBMV_LAUNCH_CHECK("face_flux_jvp_kernel<z>");
  divergence_lin_kernel<NCHEM><<<sweep_blocks(g.ncell, 256), 256, 0, s>>>(g, out, F[0], F[1], F[2]);
  GBMV_LAUNCH_CHECK("divergence_lin_kernel");
  return GBMV_OK;
}

int feuler_jvp(const Grid& g, const Fields& w, const Fields& dw, const Fields& out,
               double* scratch, cudaStream_t s) {
  switch (g.nchem) {
    case 0: return jvp_t<0>(g, w, dw, out, scratch, s);
    case 2: return jvp_t<2>(g, w, dw, out, scratch, s);
    case 4: return jvp_t<4>(g, w, dw, out, scratch, s);
    case 6: return jvp_t<6>(g, w, dw, out, scratch, s);
    case 10: return jvp_t<10>(g, w, dw, out, scratch, s);
    default: return GBMV_EUNSUPPORTED;
  }
}

}  // namespace gbmv
