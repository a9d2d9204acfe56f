// iact_render_noalloc: the forward render for callers that cannot allocate
// device memory.
//
// Some callers of this library cannot call cudaMalloc (or any allocator) to
// provide the scratch buffer iact_render wants: a host application whose
// device memory is entirely owned by another framework's pool allocator, a
// plugin inside a process whose memory manager forbids foreign allocations,
// or a real-time loop -- a telescope's data-acquisition or trigger path --
// that must not allocate, or risk failing to allocate, while it observes.
// For them this entry point uses a fixed scratch array that lives in the
// library itself: a file-scope __device__ array of IACT_NOALLOC_SCRATCH_BYTES
// (16 MiB). Every GPU that loads the library holds that array until the
// process exits.
//
// Rules of use:
//   * The first call on each device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current) and caches it; make
//     that first call before any stream capture on the device. The cached
//     address belongs to the device context it was looked up in: after a
//     cudaDeviceReset the library's module is loaded again and the array may
//     move, so a process that resets a device must not call this entry point
//     on it again.
//   * Every call on a device shares the one array. The render clears what
//     must start at zero (tile counter, FP64 accumulator) and rewrites the
//     rest each call, but two calls that overlap on the GPU (different
//     streams, or host threads without ordering) race on it: serialise them.
//   * A scene, sensor and source count whose scratch exceeds the array is
//     rejected with IACT_E_UNSUPPORTED before any work is queued.
//   * The call itself allocates nothing: no cudaMalloc, cudaFree or
//     allocating library routine.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "iact_internal.h"

namespace iact {
namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[IACT_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on the current device, looked up once
// per device. In host code the symbol itself is only a host-side stand-in.
int scratch_for_current_device(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return check_cuda(e, "iact_render_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return set_error(IACT_E_UNSUPPORTED, "iact_render_noalloc: device index too large");
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return check_cuda(e, "iact_render_noalloc: cudaGetSymbolAddress");
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return IACT_OK;
}

}  // namespace
}  // namespace iact

using namespace iact;

extern "C" int iact_render_noalloc(const iact_scene_t* scene, const iact_sensor_t* sensor, int32_t source_type,
                                   const float* sources, const float* values, int32_t n_sources, int32_t mode,
                                   float* out, const iact_opts_t* opts, void* stream) {
  int rc = validate_scene(scene);
  if (rc) return rc;
  rc = validate_sensor(sensor);
  if (rc) return rc;
  if (mode != IACT_MODE_IMAGE && mode != IACT_MODE_RESPONSE)
    return set_error(IACT_E_INVALID, "mode must be IACT_MODE_IMAGE or IACT_MODE_RESPONSE");
  if (n_sources < 0) return set_error(IACT_E_INVALID, "negative source count");
  const size_t need = workspace_for(scene, sensor, n_sources, mode).total;
  if (need > (size_t)IACT_NOALLOC_SCRATCH_BYTES)
    return set_error(IACT_E_UNSUPPORTED, "iact_render_noalloc: this render needs " + std::to_string(need) +
                                             " bytes of scratch, more than the fixed " +
                                             std::to_string((size_t)IACT_NOALLOC_SCRATCH_BYTES) +
                                             "; use iact_render with a caller workspace");
  void* scratch = nullptr;
  rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  return iact_render(scene, sensor, source_type, sources, values, n_sources, mode, out, scratch,
                     (size_t)IACT_NOALLOC_SCRATCH_BYTES, opts, stream);
}
