// crv_pulses_static: the pulse fit with its scratch in a statically sized device array instead of a caller workspace.
//
// For callers that must not allocate device memory once they run: cudaMalloc / cudaFree synchronise the whole device,
// which stalls every other stream of a process that shares the GPU between concurrent producers (an event loop with
// several modules on their own streams), and hosts bound through a plain C FFI have no caching allocator to draw a
// workspace from.  Such a caller passes only its input and output buffers; the scratch is this translation unit's
// file-scope array, one instance per device.
//
// Rules of use:
//  * The scratch holds at most CRV_PULSES_STATIC_MAX_BYTES (64 MiB).  A call whose workspace need
//    (crv_pulses_workspace(p, nw, nsamples)) is larger returns CRV_ERR_TOO_LARGE and launches nothing.
//  * Every call looks up the array's device address for the current device (cudaGetSymbolAddress, a host-side
//    lookup that launches nothing).  The first lookup on a device also loads this module there (under lazy module
//    loading, the default since CUDA 12.2, that is when the 64 MiB are reserved; with eager loading every device the
//    library is used on reserves them when the library loads), so make the first call on each device before any
//    stream capture.  Looking the address up per call, instead of caching it, keeps the entry point correct after a
//    device reset or a re-created primary context, where the module is loaded again and the array may move.
//  * Nothing in the scratch has to start at zero: every word a call reads is written earlier by the same call, and
//    the call clears its own counters.  The status block must start at zero, as for every entry point.
//  * One scratch per device: two calls in flight on the same device at once (different streams or host threads)
//    overwrite each other's scratch and both results are undefined.  Serialise them (one stream, or the caller's lock
//    plus stream ordering).
//  * No allocation happens inside the call as long as the launch profiler (crv_profile) is off.
#include <cuda_runtime.h>

#include "../../include/crvgpu.h"

namespace {

__device__ __align__(256) unsigned char g_pulse_scratch[CRV_PULSES_STATIC_MAX_BYTES];

// Device address of the scratch on the current device (looked up on every call; see above).
int scratch_for_current_device(void** out) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_pulse_scratch) != cudaSuccess || !p) return CRV_ERR_CUDA;
  *out = p;
  return CRV_OK;
}

}  // namespace

extern "C" int crv_pulses_static(const CrvParams* p, int64_t nw, int64_t nsamples, const int64_t* off,
                                 const int32_t* n, const int64_t* start_tdc, const double* ped_db, const double* area,
                                 const double* height, const int16_t* adc16, const int64_t* adc64, int32_t max_pulses,
                                 CrvPulses* out, int64_t out_cap, int64_t* n_out_dev, uint8_t* wf_near, void* stream,
                                 CrvStatus* status_dev) {
  int64_t need = crv_pulses_workspace(p, nw, nsamples);
  if (need < 0) return CRV_ERR_ARG;
  if (need > (int64_t)CRV_PULSES_STATIC_MAX_BYTES) return CRV_ERR_TOO_LARGE;
  void* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != CRV_OK) return rc;
  return crv_pulses(p, nw, nsamples, off, n, start_tdc, ped_db, area, height, adc16, adc64, max_pulses, out, out_cap,
                    n_out_dev, wf_near, scratch, (int64_t)CRV_PULSES_STATIC_MAX_BYTES, stream, status_dev);
}
