// gbmv_feuler_noalloc: the FP64 flux divergence for callers that must not allocate device
// memory (see include/gbmv.h).  Its face-flux scratch and status word live in file-scope
// __device__ arrays of fixed size instead of the cudaMalloc'ed buffers of a gbmv_hydro handle.
#include <mutex>

#include "weno.cuh"

namespace gbmv {
namespace {

// 64 MiB of flux scratch: enough for (5+nchem) * (face count of the three directions)
// doubles, e.g. a 56^3 grid at NVAR=15 or an 82^3 grid at NVAR=5.  This file has no kernel
// of its own and is a module of its own, so under CUDA's lazy module loading (the default)
// the memory is committed on a device when the first call there looks the arrays up, and
// stays committed until the process exits.
constexpr size_t kNoAllocScratchDoubles = size_t(8) << 20;

__device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];
__device__ __align__(256) int g_noalloc_status[64];  // element 0 is the legal-state mask

constexpr int kMaxDevices = 64;

struct DeviceAddrs {
  double* scratch = nullptr;
  int* status = nullptr;
  bool ready = false;
};

std::mutex g_addr_mu;
DeviceAddrs g_addr[kMaxDevices];

// In host code the array names above are host-side stand-ins, not device addresses: passing
// them to a kernel would fault.  Once per device, with that device current, look the real
// addresses up with cudaGetSymbolAddress (which also loads this module and commits its 64 MiB
// on that device) and keep them.
int device_addresses(DeviceAddrs* out) {
  int dev = 0;
  GBMV_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal %d out of range for the no-allocation entry point", dev);
    return GBMV_EINVAL;
  }
  std::lock_guard<std::mutex> lk(g_addr_mu);
  DeviceAddrs& a = g_addr[dev];
  if (!a.ready) {
    void* p = nullptr;
    GBMV_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    a.scratch = static_cast<double*>(p);
    GBMV_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_status));
    a.status = static_cast<int*>(p);
    a.ready = true;
  }
  *out = a;
  return GBMV_OK;
}

}  // namespace
}  // namespace gbmv

using namespace gbmv;

extern "C" int gbmv_feuler_noalloc(const gbmv_grid* grid, const double* force_host, double t,
                                   const double* const* w, double* const* wdot, void* stream) {
  (void)t;
  // the same checks, return codes and messages as gbmv_hydro_create
  int rc = check_grid(grid);
  if (rc) return rc;
  const Grid g = make_grid(*grid);
  const size_t need = feuler_fp64_scratch_doubles(g);
  if (need > kNoAllocScratchDoubles) {
    set_error("gbmv_feuler_noalloc: grid needs %zu scratch doubles, the fixed array holds %zu "
              "(use gbmv_hydro_create + gbmv_feuler for larger grids)",
              need, kNoAllocScratchDoubles);
    return GBMV_EINVAL;
  }
  bool fields = w && wdot;
  for (int v = 0; fields && v < 5; ++v) fields = w[v] && wdot[v];
  if (fields && g.nchem) fields = w[5] && wdot[5];
  if (!fields) {
    set_error("gbmv_feuler_noalloc: null field pointer");
    return GBMV_EINVAL;
  }

  DeviceAddrs a;
  rc = device_addresses(&a);
  if (rc) return rc;

  Fields W, Wd;
  for (int v = 0; v < 6; ++v) {
    W.f[v] = (v < 5 || g.nchem) ? const_cast<double*>(w[v]) : nullptr;
    Wd.f[v] = (v < 5 || g.nchem) ? wdot[v] : nullptr;
  }
  ForceTerm G;
  for (int v = 0; v < 16; ++v) G.c[v] = (force_host && v < 5 + g.nchem) ? force_host[v] : 0.0;
  G.in_wdot = 0;

  cudaStream_t s = (cudaStream_t)stream;
  // the status word is shared by every call and keeps the last call's value: clear it
  GBMV_CUDA_TRY(cudaMemsetAsync(a.status, 0, sizeof(int), s));
  rc = feuler_fp64(g, W, Wd, G, a.scratch, a.status, s);
  if (rc) return rc;
  int st = 0;
  GBMV_CUDA_TRY(cudaMemcpyAsync(&st, a.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBMV_CUDA_TRY(cudaStreamSynchronize(s));
  if (st) {
    set_error("illegal state (mask %d: 1 density, 2 energy, 4 pressure)", st);
    return GBMV_ILLEGAL_STATE;
  }
  return GBMV_OK;
}
