// eff_loss_grad_static: the loss/gradient step with its scratch in a fixed,
// library-owned device array instead of a caller-provided workspace.
//
// Who needs it: a caller that binds the reference's objective/gradient
// interface (cnvinv_objfun / cnvinv_gradfun, olaGPU.py:756-811) passes only
// the image, the PSFs, the observation and the outputs -- that interface has
// no place for a workspace pointer -- and may run where device allocation is
// not allowed (a host program that reserves all device memory up front, or a
// stream-ordered pipeline where cudaMalloc's implicit device synchronisation
// is not acceptable).  This entry point calls no allocator at all.
//
// The scratch is one file-scope __device__ array of kStaticScratchBytes
// (16 MiB), so every GPU that loads the library holds that much memory until
// the process exits.  Host code cannot use the array's name as a device
// address, so the first call on each device looks the address up with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture begins, and do not use the entry point
// on a device after cudaDeviceReset of that device (the module is loaded
// again and the cached address may be stale).  All calls share the array and
// it keeps the last call's contents: the step clears what must start at zero
// (the forward output and the loss) itself, and two calls whose GPU work
// overlaps (different streams, different host threads) race on it.
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "eff_internal.h"
#include "../../include/vmbd_eff.h"

namespace {

constexpr size_t kStaticScratchBytes = size_t(16) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (looked up once).
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return eff::set_error(EFF_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return eff::set_error(EFF_ERR_UNSUPPORTED, "device ordinal too large");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p)
      return eff::set_error(EFF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return EFF_OK;
}

}  // namespace

extern "C" {

size_t eff_static_scratch_bytes(void) { return kStaticScratchBytes; }

int eff_loss_grad_static(const EffPlan* plan, const float* x, const float* f, const float* y_obs,
                         double* loss, float* gx, float* gf, int batch, void* stream) {
  if (!plan) return eff::set_error(EFF_ERR_INVALID, "null plan");
  if (batch < 1) return eff::set_error(EFF_ERR_INVALID, "batch must be >= 1");
  // the scratch address is looked up on the current device, the plan's
  // tables live on the plan's device: they must be the same device
  if (int s = eff::check_plan_device(plan)) return s;
  const size_t need = eff_loss_grad_workspace_bytes(plan, batch);
  if (need > kStaticScratchBytes)
    return eff::set_error(EFF_ERR_UNSUPPORTED,
                          "eff_loss_grad_static: this geometry and batch need " + std::to_string(need) +
                              " bytes of scratch, more than the library's static " +
                              std::to_string(kStaticScratchBytes) +
                              "-byte array; use eff_loss_grad with a workspace");
  void* scratch = nullptr;
  if (int s = scratch_address(&scratch)) return s;
  return eff_loss_grad(plan, x, f, y_obs, loss, gx, gf, scratch, kStaticScratchBytes, batch, stream);
}

}  // extern "C"
