// kf_noalloc.cu — a fit entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code running under a host framework
// that owns all device memory through its own pool (online trigger and
// reconstruction farms, inference servers), plugins whose host forbids
// foreign allocations, and latency-bound loops where cudaMalloc's implicit
// device synchronisation or a mid-run out-of-memory failure is not
// acceptable.  kf_fit_batch_noalloc serves them: the caller passes inputs and
// outputs as for kf_fit_batch, and the smoother workspace comes from a static
// device array of kNoAllocScratchBytes that every GPU loading this library
// holds until the process exits.

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/gb300kf.h"

namespace {

constexpr size_t kNoAllocScratchBytes = KF_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// The shared scratch.  In host code `g_scratch` names a host-side stand-in,
// not the device array: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_scratch[kNoAllocScratchBytes];

std::mutex g_mutex;
void *g_scratchAddr[kMaxDevices] = {};
unsigned long long g_scratchCtx[kMaxDevices] = {}; // context id the address belongs to

thread_local char g_msg[512] = "";

// The current context's process-unique id (cuCtxGetId), reached through the
// runtime's driver entry-point query so that the library needs no link
// against the driver library; 0 when unavailable.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

unsigned long long currentContextId() {
  static CtxGetCurrentFn getCurrent = nullptr;
  static CtxGetIdFn getId = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      getCurrent = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      getId = reinterpret_cast<CtxGetIdFn>(f);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (getCurrent && getId && getCurrent(&ctx) == CUDA_SUCCESS && ctx &&
      getId(ctx, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

// Device address of g_scratch in the current device's context.  The first
// call on a device does this set-up (cudaGetSymbolAddress, which also loads
// the module into the context); it is repeated when that device's context
// has been replaced since (cudaDeviceReset), because the array then lives at
// a new address.  Without a context id it is looked up on every call.
int32_t scratchAddress(void **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    std::snprintf(g_msg, sizeof(g_msg), "cudaGetDevice: %s", cudaGetErrorString(e));
    return KF_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    std::snprintf(g_msg, sizeof(g_msg), "device ordinal %d beyond %d", dev, kMaxDevices);
    return KF_ERR_UNSUPPORTED;
  }
  const unsigned long long ctx = currentContextId();
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratchAddr[dev] || ctx == 0 || g_scratchCtx[dev] != ctx) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
      std::snprintf(g_msg, sizeof(g_msg), "cudaGetSymbolAddress(scratch): %s",
                    cudaGetErrorString(e));
      return KF_ERR_CUDA;
    }
    g_scratchAddr[dev] = p;
    g_scratchCtx[dev] = ctx;
  }
  *out = g_scratchAddr[dev];
  return KF_SUCCESS;
}

} // namespace

extern "C" {

size_t kf_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

// The message of this thread's last kf_fit_batch_noalloc call: empty after a
// success.
const char *kf_noalloc_last_error_string(void) { return g_msg; }

int32_t kf_fit_batch_noalloc(const kf_inputs_t *in, kf_outputs_t *out, const kf_config_t *cfg,
                             const kf_geometry_t *geo, const kf_field_t *field, void *stream) {
  g_msg[0] = '\0';
  if (!in || !out || !cfg || !geo || !field) {
    std::snprintf(g_msg, sizeof(g_msg), "null argument");
    return KF_ERR_INVALID_ARGUMENT;
  }
  const size_t need = kf_workspace_size(cfg, in->n_tracks, in->n_surfaces);
  if (need > kNoAllocScratchBytes) {
    std::snprintf(g_msg, sizeof(g_msg),
                  "batch needs %zu bytes of scratch (%lld tracks x %d surfaces); the "
                  "no-allocation entry point holds %zu bytes: split the batch or use "
                  "kf_fit_batch with a caller workspace",
                  need, (long long)in->n_tracks, (int)in->n_surfaces, kNoAllocScratchBytes);
    return KF_ERR_WORKSPACE_TOO_SMALL;
  }
  void *scratch = nullptr;
  const int32_t rc = scratchAddress(&scratch);
  if (rc) return rc;
  // The fit writes every scratch element before reading it, so the contents
  // left by an earlier call need no clearing.
  const int32_t fit = kf_fit_batch(in, out, cfg, geo, field, scratch, kNoAllocScratchBytes, stream);
  if (fit != KF_SUCCESS) std::snprintf(g_msg, sizeof(g_msg), "%s", kf_last_error_string());
  return fit;
}

} // extern "C"
