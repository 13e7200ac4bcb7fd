// Throughput probe for the roofline denominators that no driver-side measurement provides:
// the FP64 (and FP32) fused multiply-add rate of the SIMT pipes.  Each thread runs 8
// independent FMA chains for a fixed number of iterations; flops = 2 * FMAs.
#include "common.cuh"
#include "df64.cuh"

namespace gbmv {

template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
#pragma unroll 1
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == (T)-12345.678) out[0] = s;  // keeps the chains live; never true for these inputs
}

template <typename T>
static int probe(double* flops_per_s, int blocks_per_sm) {
  T* out = nullptr;
  GBMV_CUDA_TRY(cudaMalloc(&out, sizeof(T)));
  cudaEvent_t e0, e1;
  GBMV_CUDA_TRY(cudaEventCreate(&e0));
  GBMV_CUDA_TRY(cudaEventCreate(&e1));
  int dev = 0, nsm = kSM;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = nsm * blocks_per_sm, threads = 256;
  const int iters = sizeof(T) == 8 ? 256 : 4096;
  const T a = (T)0.999999, b = (T)1e-7;
  fma_probe_kernel<T><<<blocks, threads>>>(out, 4, a, b);  // warm-up
  GBMV_LAUNCH_CHECK("fma_probe_kernel");
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    fma_probe_kernel<T><<<blocks, threads>>>(out, iters, a, b);
    cudaEventRecord(e1);
    GBMV_CUDA_TRY(cudaEventSynchronize(e1));
    count_launch();
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  const double fmas = (double)blocks * threads * iters * 16.0 * 8.0;
  *flops_per_s = 2.0 * fmas / (best * 1e-3);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return GBMV_OK;
}

// Self-check of the integer-instruction conversions of df64.cuh against the hardware
// round-to-nearest conversions: for every input double, f32_of_f64, f64_of_f32 (of the
// hardware float), f2_split and f2_to_double (of the hardware pair) must give the same bits.
__global__ void __launch_bounds__(256) convert_check_kernel(const double* __restrict__ in,
                                                            long n,
                                                            unsigned long long* __restrict__ bad) {
  unsigned long long mine = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const double d = in[i];
    const float hw = __double2float_rn(d);
    mine += __float_as_uint(f32_of_f64(d)) != __float_as_uint(hw);
    mine += __double_as_longlong(f64_of_f32(hw)) != __double_as_longlong((double)hw);
    const f2 a = f2_split(d), b = f2_from_double(d);
    mine += __float_as_uint(a.hi) != __float_as_uint(b.hi);
    mine += __float_as_uint(a.lo) != __float_as_uint(b.lo);
    mine += __double_as_longlong(f2_to_double(b)) != __double_as_longlong(b.to_double());
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, off);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(bad, mine);
}

}  // namespace gbmv

extern "C" int gbmv_diag_fma_rate(int fp64, double* flops_per_s) {
  if (!flops_per_s) return GBMV_EINVAL;
  return fp64 ? gbmv::probe<double>(flops_per_s, 8) : gbmv::probe<float>(flops_per_s, 8);
}

extern "C" int gbmv_diag_convert_check(const double* d_in, long n, unsigned long long* mismatches,
                                       void* stream) {
  using namespace gbmv;
  if (!d_in || n < 0 || !mismatches) return GBMV_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  auto ok = [](cudaError_t e, const char* where) {
    return e == cudaSuccess ? GBMV_OK : check_cuda(e, where);
  };
  unsigned long long* d_bad = nullptr;
  GBMV_CUDA_TRY(cudaMalloc(&d_bad, sizeof(unsigned long long)));
  int rc = ok(cudaMemsetAsync(d_bad, 0, sizeof(unsigned long long), s), "convert check memset");
  if (rc == GBMV_OK) {
    long b = (n + 255) / 256;
    if (b > (long)kSM * 8) b = (long)kSM * 8;
    if (b < 1) b = 1;
    convert_check_kernel<<<(int)b, 256, 0, s>>>(d_in, n, d_bad);
    count_launch();
    rc = ok(cudaGetLastError(), "convert_check_kernel");
  }
  if (rc == GBMV_OK)
    rc = ok(cudaMemcpyAsync(mismatches, d_bad, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, s), "convert check copy");
  if (rc == GBMV_OK) rc = ok(cudaStreamSynchronize(s), "convert check sync");
  cudaFree(d_bad);
  return rc;
}
