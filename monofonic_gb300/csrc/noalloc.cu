// White-noise fill for callers that must not allocate device memory.
//
// Some host codes cannot let a library call cudaMalloc: an N-body code that
// generates its initial conditions in situ and has already reserved all of
// HBM through its own pool allocator, or an application running under a
// device-memory cap enforced by its scheduler.  Such a caller allocates the
// output field itself and passes it in; the one piece of device scratch the
// noise kernel needs beyond its input and output -- the device copy of the
// NGenIC per-column seed table it reads -- lives here in a file-scope
// __device__ array of fixed size (4 MiB, grids up to 1024^3).
//
// When the array becomes resident: CUDA loads this file's module (the array
// and this file's kernels) on first use, and under the default lazy module
// loading that first use would otherwise be the entry point's first call --
// an allocation inside the call that promises none.  mfx_engine_create
// therefore loads the module on its device (noalloc_prepare below: it looks up
// the array's address with cudaGetSymbolAddress, with that device current,
// and loads both kernel instantiations); from then on the array stays resident
// until the process exits.  Create the engine before reserving the rest of
// HBM, and before any stream capture.
//
// The entry point allocates nothing: no cudaMalloc, no cudaFree, no library
// routine that allocates.  It leaves the caller's current device as it found
// it.  All calls share the one array, so calls whose work overlaps on the GPU
// race on it: issue them on one stream, or wait for one before starting the
// next.  The array keeps the previous call's table; each call overwrites the
// N*N entries it uses and the kernel writes every element of the output, so
// nothing has to start at zero.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/mfx.h"
#include "common.h"
#include "kernels.cuh"

namespace mfx {
namespace {

constexpr uint32_t kNoAllocMaxGrid = MFX_NOALLOC_MAX_NGRID;

// device copy of the seed table of the current call
static __device__ __align__(256) uint32_t g_noalloc_seed_table[size_t(kNoAllocMaxGrid) * kNoAllocMaxGrid];

std::mutex g_mu;
uint32_t *g_addr[64] = {};  // per-device address of g_noalloc_seed_table

// Resolves the array's device address on `dev` (which must be current) and
// loads this file's kernels, so that the module is resident before the entry
// point's first call.
int resolve_scratch(int dev) {
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_seed_table);
  if (e != cudaSuccess)
    return set_error(MFX_ECUDA, "cudaGetSymbolAddress(no-allocation scratch) on device %d: %s", dev,
                     cudaGetErrorString(e));
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, k_noise_phi1<double>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_noise_phi1<float>);
  if (e != cudaSuccess)
    return set_error(MFX_ECUDA, "loading the no-allocation noise kernels on device %d: %s", dev,
                     cudaGetErrorString(e));
  g_addr[dev] = static_cast<uint32_t *>(p);
  return MFX_OK;
}

int scratch_address(int dev, uint32_t **out) {
  if (dev < 0 || dev >= 64) return set_error(MFX_EINVAL, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    const int rc = resolve_scratch(dev);
    if (rc != MFX_OK) return rc;
  }
  *out = g_addr[dev];
  return MFX_OK;
}

// Makes `dev` current for the scope and gives the caller's current device back
// on every return path.
struct DeviceScope {
  int saved = -1;
  cudaError_t set(int dev) {
    cudaError_t e = cudaGetDevice(&saved);
    if (e != cudaSuccess) {
      saved = -1;
      return e;
    }
    return saved == dev ? cudaSuccess : cudaSetDevice(dev);
  }
  ~DeviceScope() {
    if (saved >= 0) cudaSetDevice(saved);
  }
};

}  // namespace

int noalloc_prepare(int dev) {
  if (dev < 0 || dev >= 64) return set_error(MFX_EINVAL, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_mu);
  return resolve_scratch(dev);  // re-resolved per engine: a reset device gets a new context
}

}  // namespace mfx

using namespace mfx;

extern "C" int mfx_noise_fill_noalloc(mfx_engine *eng, uint32_t ngrid, double boxlen, const uint32_t *seed_table,
                                      int raw, int fixing, int inversion, int precision, void *out_device,
                                      void *stream) {
  if (!eng || !seed_table || !out_device) return set_error(MFX_EINVAL, "null argument");
  if (ngrid < 8 || ngrid % 4 != 0) return set_error(MFX_EINVAL, "ngrid must be a multiple of 4 and >= 8 (got %u)", ngrid);
  if (ngrid > kNoAllocMaxGrid)
    return set_error(MFX_EINVAL, "ngrid %u exceeds the allocation-free limit of %u (seed scratch is %u^2 entries)",
                     ngrid, kNoAllocMaxGrid, kNoAllocMaxGrid);
  if (!(boxlen > 0)) return set_error(MFX_EINVAL, "boxlen must be positive");
  if (precision != MFX_FP64 && precision != MFX_FP32C) return set_error(MFX_EINVAL, "bad precision");
  const int dev = engine_device(eng);
  DeviceScope scope;
  cudaError_t e = scope.set(dev);
  if (e != cudaSuccess) return set_error(MFX_ECUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  uint32_t *seeds = nullptr;
  int rc = scratch_address(dev, &seeds);
  if (rc != MFX_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  e = cudaMemcpyAsync(seeds, seed_table, size_t(ngrid) * ngrid * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return set_error(MFX_ECUDA, "seed table upload: %s", cudaGetErrorString(e));
  NoiseArgs a;
  a.seeds = seeds;
  a.amp = nullptr;
  a.amp_len = 0;
  a.N = int(ngrid);
  a.mode = raw ? 0 : 1;
  a.fixing = fixing;
  const double volfac = std::pow(boxlen / ngrid / 2.0 / M_PI, 1.5);
  a.norm = (inversion ? -1.0 : 1.0) / volfac;
  a.out_scale = 1.0;
  const int cols = int(ngrid * ngrid);
  if (precision == MFX_FP64)
    k_noise_phi1<double><<<(cols + 127) / 128, 128, 0, st>>>(a, static_cast<double2 *>(out_device));
  else
    k_noise_phi1<float><<<(cols + 127) / 128, 128, 0, st>>>(a, static_cast<float2 *>(out_device));
  e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(MFX_ECUDA, "noise kernel launch: %s", cudaGetErrorString(e));
  return MFX_OK;
}
