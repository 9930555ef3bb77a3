// demag_static.cu -- device memory for mmc_demag_apply_static().
//
// The spectrum scratch of that entry point is this file-scope array, part of
// the library's device image: the CUDA runtime reserves it on a device when it
// loads this module there, so the entry point itself allocates nothing.  Its
// size is MMC_DEMAG_STATIC_SCRATCH_BYTES (include/mmc.h).  Every call on a
// device shares the one array.
#include <mutex>

#include "mmc.h"
#include "mmc_internal.h"

namespace mmc {

static __device__ __align__(256) unsigned char g_demag_static_scratch[MMC_DEMAG_STATIC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};
}  // namespace

// Address of the array on `device`, which must be the current device.  The
// first call per device looks it up (this loads the module there); later calls
// return the cached address.
cudaError_t demag_static_scratch(int device, void** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_demag_static_scratch);
    if (e != cudaSuccess) return e;
    g_addr[device] = p;
  }
  *out = g_addr[device];
  return cudaSuccess;
}

}  // namespace mmc
