// Seeded volume synthesis into a caller-owned device buffer without any
// device allocation.
//
// gbvr_synth_volume and gbvr_load_synthetic upload the generator's per-axis
// blob tables into device memory they allocate for the call.  Callers that
// cannot allocate device memory at the point of the call use this variant:
//  * a host application that owns the GPU memory budget and hands the
//    library only pre-allocated buffers;
//  * code issuing work between other streams' kernels, where cudaFree (and
//    often cudaMalloc) synchronises the whole device and stalls them.
// The tables live in a file-scope device array of fixed size instead, which
// every GPU that loads this library holds until the process exits.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/gbvr.h"
#include "abi_guard.h"
#include "gbvr_internal.h"
#include "synth_tables.h"

namespace gbvr {
int set_error(int code, const std::string& msg);
}

using namespace gbvr;

// Capacity of the shared table scratch, in floats (1 MiB).
static constexpr long long kSynthScratchFloats = GBVR_NOALLOC_SYNTH_MAX_FLOATS;

static __device__ __align__(256) float g_synth_scratch[kSynthScratchFloats];

namespace {

std::mutex g_mu;
constexpr int kMaxDevices = 64;
struct DeviceSetup {
  float* scratch = nullptr;     // device address of g_synth_scratch on this device
  cudaEvent_t copied = nullptr; // recorded after the last table copy queued on this device
  bool pending = false;         // a copy from g_tables_host may still be reading it
};
DeviceSetup g_dev[kMaxDevices];
// Host staging for the tables: static, so the call allocates no host heap
// either.  Guarded by g_mu; refilled only after the copy that last read it
// has completed (its event).
float g_tables_host[kSynthScratchFloats];

}  // namespace

extern "C" int gbvr_dev_synth_volume_noalloc(const gbvr_synth_params* p, void* dev_out, size_t bytes, void* stream) {
  GBVR_ABI_TRY
  if (!p || !dev_out) return set_error(GBVR_EINVAL, "null argument");
  long long need = 0;
  size_t out_bytes = 0;
  int rc = check_synth_params(p, true, &need, &out_bytes);
  if (rc != GBVR_OK) return rc;
  if (need > kSynthScratchFloats)
    return set_error(GBVR_EINVAL, "the generator tables need " + std::to_string(need) +
                                      " floats; the no-allocation entry point holds at most " +
                                      std::to_string(kSynthScratchFloats) +
                                      " (nblobs x (1 + X + Y + Z) + X + Y + Z)");
  if (bytes < out_bytes) return set_error(GBVR_EINVAL, "output buffer too small");
  cudaStream_t s = (cudaStream_t)stream;
  // a captured copy would read the static host tables when the graph is
  // replayed, by then holding another call's parameters
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cap);
  if (e != cudaSuccess) return set_error(GBVR_ECUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e));
  if (cap != cudaStreamCaptureStatusNone)
    return set_error(GBVR_EINVAL, "gbvr_dev_synth_volume_noalloc cannot be called while its stream is being captured");
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(GBVR_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error(GBVR_EINVAL, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  DeviceSetup& ds = g_dev[dev];
  if (!ds.scratch) {
    // Set-up, once per device, with that device current: resolve the device
    // address of the scratch array (the first call on a device also loads
    // the library's device code there) and create the copy event.
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_synth_scratch);
    if (e != cudaSuccess) return set_error(GBVR_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    cudaEvent_t ev = nullptr;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return set_error(GBVR_ECUDA, std::string("cudaEventCreate: ") + cudaGetErrorString(e));
    ds.copied = ev;
    ds.scratch = (float*)ptr;
  }
  float* dt = ds.scratch;
  if (need > 0) {
    // the previous table copy (on any device) must have read the host staging
    for (int d = 0; d < kMaxDevices; ++d)
      if (g_dev[d].pending) {
        e = cudaEventSynchronize(g_dev[d].copied);
        if (e != cudaSuccess) return set_error(GBVR_ECUDA, std::string("cudaEventSynchronize: ") + cudaGetErrorString(e));
        g_dev[d].pending = false;
      }
    fill_blob_tables(*p, g_tables_host);
    e = cudaMemcpyAsync(dt, g_tables_host, sizeof(float) * (size_t)need, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return set_error(GBVR_ECUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    e = cudaEventRecord(ds.copied, s);
    if (e != cudaSuccess) return set_error(GBVR_ECUDA, std::string("cudaEventRecord: ") + cudaGetErrorString(e));
    ds.pending = true;
  }
  const long long X = p->dims[0], Y = p->dims[1], Z = p->dims[2];
  const int nb = p->nblobs;
  const bool bg = p->bg_freq > 0;
  float* bgt = dt + nb + (long long)nb * (X + Y + Z);
  BlobTablesDev td{nb, dt, dt + nb, dt + nb + (long long)nb * X, dt + nb + (long long)nb * (X + Y),
                   bg ? bgt : nullptr, bg ? bgt + X : nullptr, bg ? bgt + X + Y : nullptr,
                   p->bg_level, p->bg_amp, p->scale, p->noise_amp, p->noise_kind, p->vmax, p->seed};
  const long long d[3] = {X, Y, Z};
  e = launch_synth_blobs(td, d, p->dtype, dev_out, s);
  if (e != cudaSuccess) return set_error(GBVR_ECUDA, std::string("synth launch: ") + cudaGetErrorString(e));
  return GBVR_OK;
  GBVR_ABI_CATCH
}
