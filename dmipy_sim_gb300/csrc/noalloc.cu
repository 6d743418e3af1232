// dmsim_walk_noalloc: the walk for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc for the walk's workspace.  An XLA custom
// call (the runtime dmipy-sim's own users sit on) receives only the buffers XLA hands it, with the
// rest of the GPU typically preallocated by XLA's pool; a plug-in running under a host
// framework's fixed device-memory budget is in the same position.  For them this entry point
// takes only the inputs and outputs and runs the ordinary walk with its scratch (the re-laid-out
// waveform and the per-block FP64 partial sums) in one file-scope device array of
// DMSIM_NOALLOC_SCRATCH_BYTES bytes.
//
// Properties a caller must know:
//   * The array is part of the library image: every GPU that loads the library holds it until
//     the process exits.
//   * The first call on a device, with that device current, looks up the array's device address
//     (cudaGetSymbolAddress) once; make that first call before any stream capture.
//   * That address is kept for the life of the process.  A cudaDeviceReset (or any other reset
//     of the device's primary context) unloads the library's device image and invalidates it:
//     a process that resets a device must not call this entry point on that device again.
//   * Every call shares the one array and the array keeps the last call's contents.  Nothing in
//     it needs to start at zero (each launch writes every byte it later reads), but calls whose
//     work overlaps on the GPU race on it: serialise them (one stream, or events).
//   * Configurations whose workspace exceeds the array are rejected with DMSIM_ETOOBIG before any
//     launch; nothing here calls cudaMalloc, cudaFree or an allocating library routine.
#include <cuda_runtime.h>

#include <mutex>

#include "dmsim.h"

namespace dmsim {
int set_error(int code, const char* msg);
}

namespace {

constexpr int kMaxDevices = 64;

// Host code must not use this name as a device address: outside device code it is only a
// host-side stand-in.  The device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[DMSIM_NOALLOC_SCRATCH_BYTES];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

int scratch_for_current_device(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess)
    return dmsim::set_error(DMSIM_ECUDA, "walk_noalloc: cudaGetDevice failed");
  if (dev < 0 || dev >= kMaxDevices)
    return dmsim::set_error(DMSIM_EINVAL, "walk_noalloc: device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
      return dmsim::set_error(DMSIM_ECUDA,
                              "walk_noalloc: cudaGetSymbolAddress of the scratch array failed");
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return DMSIM_OK;
}

}  // namespace

extern "C" int dmsim_walk_noalloc(const dmsim_walk_params* p, const dmsim_geometry* g,
                                  const dmsim_walk_outputs* o, void* stream) {
  const size_t need = dmsim_walk_workspace_bytes(p, g);
  if (need == 0) return DMSIM_EINVAL;  // the planner has set the error message
  if (need > (size_t)DMSIM_NOALLOC_SCRATCH_BYTES)
    return dmsim::set_error(DMSIM_ETOOBIG,
                            "walk_noalloc: this walk needs more scratch than the built-in "
                            "DMSIM_NOALLOC_SCRATCH_BYTES array holds; call dmsim_walk with a "
                            "caller-allocated workspace instead");
  void* scratch = nullptr;
  const int rc = scratch_for_current_device(&scratch);
  if (rc != DMSIM_OK) return rc;
  return dmsim_walk(p, g, o, scratch, (size_t)DMSIM_NOALLOC_SCRATCH_BYTES, stream);
}
