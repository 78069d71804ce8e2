// rain_ice_noalloc.cu — ice3gb_rain_ice_noalloc: the rain_ice step without any
// device allocation.
//
// ice3gb_rain_ice takes its scratch (a work counter, the maximum pass key and
// one pass key per grid point) from cudaMallocAsync on every call.  Some hosts
// cannot allocate device memory from inside their physics call: a model that
// hands the GPU's memory to its own pool allocator at start-up (a further
// allocation can then fail at any step, long after initialisation), or a
// deployment that caps device memory outside the library.  This
// entry point serves them with a scratch array that is part of the loaded
// library itself: a file-scope __device__ array of four control words, then
// ICE3GB_NOALLOC_MAX_POINTS pass keys and as many processing-order words (the
// regime sort of the points, as in ice3gb_rain_ice): 32 MiB + 16 B, which
// every GPU that loads the library holds until the process exits.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side stand-in), so the device address is looked up with
// cudaGetSymbolAddress once per device, with that device current, on the
// first call made on it; that first call should therefore come before any
// stream capture.  All calls share the one array: the control words are
// cleared on the stream at the start of every call (the pass keys and the
// order words of the call's points are all rewritten by its kernels), and
// calls whose work overlaps on the GPU — on different streams, or from
// different host threads — race on it and must be serialised by the caller.
// The cached address belongs to the CUDA context it was looked up in: a
// cudaDeviceReset between calls is not supported.
#include <mutex>

#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"

int ice3gb_internal_rain_ice_with_scratch(void *handle, int nij, int nk, double dt,
                                          const Ice3gbRainIceOptions *opt, const Ice3gbRainIceFields *f,
                                          unsigned int *scratch, long scratch_points, void *stream);
int ice3gb_internal_cuda_fail(void *handle, cudaError_t e, const char *where);

// Four control words (work counter, maximum pass key, two spare), one pass
// key per grid point, one processing-order word per grid point.
static __device__ __align__(256) unsigned int g_rain_ice_scratch[4 + 2 * (size_t)ICE3GB_NOALLOC_MAX_POINTS];

namespace {

constexpr int kMaxDevices = 64;

std::mutex g_mu;
unsigned int *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of g_rain_ice_scratch on the current device (looked up once
// per device).  Returns nullptr and sets *err on failure.
unsigned int *scratch_address(cudaError_t *err)
{
  int dev = -1;
  *err = cudaGetDevice(&dev);
  if (*err != cudaSuccess) return nullptr;
  if (dev < 0 || dev >= kMaxDevices) {
    *err = cudaErrorInvalidDevice;
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    *err = cudaGetSymbolAddress(&p, g_rain_ice_scratch);
    if (*err != cudaSuccess) return nullptr;
    g_scratch_addr[dev] = static_cast<unsigned int *>(p);
  }
  return g_scratch_addr[dev];
}

}  // namespace

extern "C" int ice3gb_rain_ice_noalloc(void *handle, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                                       const Ice3gbRainIceFields *f, void *stream)
{
  const long max_points = (long)ICE3GB_NOALLOC_MAX_POINTS;
  if (nij <= 0 || nk <= 0 || (long)nij * nk > max_points) {
    // shape and size are rejected (with their message) before any CUDA call
    return ice3gb_internal_rain_ice_with_scratch(handle, nij, nk, dt, opt, f, nullptr, max_points, stream);
  }
  cudaError_t e = cudaSuccess;
  unsigned int *scr = scratch_address(&e);
  if (!scr) return ice3gb_internal_cuda_fail(handle, e, "cudaGetSymbolAddress(rain_ice scratch)");
  return ice3gb_internal_rain_ice_with_scratch(handle, nij, nk, dt, opt, f, scr, max_points, stream);
}
