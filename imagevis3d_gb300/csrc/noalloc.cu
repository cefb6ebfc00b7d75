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

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/gbvr.h"
#include "abi_guard.h"
#include "gbvr_internal.h"

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
float* g_scratch_dev[kMaxDevices] = {nullptr};  // device address of g_synth_scratch, per device
// Host staging for the tables: static, so the call allocates no host heap
// either.  Guarded by g_mu.
float g_tables_host[kSynthScratchFloats];

void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[0] = n0; c[1] = (uint32_t)p1; c[2] = n2; c[3] = (uint32_t)p0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// The generator's tables, the same draws and the same double-precision math
// as the allocating entry points, written into `t` as
// amp[nb] | ex[nb X] | ey[nb Y] | ez[nb Z] | bgx[X] | bgy[Y] | bgz[Z].
void fill_tables(const gbvr_synth_params& p, float* t) {
  const uint32_t k0 = p.seed, k1 = 0x70617261u;
  const int nb = p.nblobs;
  const long long d[3] = {p.dims[0], p.dims[1], p.dims[2]};
  float* amp = t;
  float* tab[3] = {t + nb, t + nb + (long long)nb * d[0], t + nb + (long long)nb * (d[0] + d[1])};
  for (int k = 0; k < nb; ++k) {
    uint32_t c0[4] = {(uint32_t)k, 0u, 0x626c6f62u, 0u}, c1[4] = {(uint32_t)k, 1u, 0x626c6f62u, 0u};
    philox(c0, k0, k1);
    philox(c1, k0, k1);
    double cen[3];
    for (int a = 0; a < 3; ++a) cen[a] = (double)(c0[a] >> 8) / 16777216.0 * (double)d[a];
    double sig = p.sigma_lo + (double)(c1[0] >> 8) / 16777216.0 * ((double)p.sigma_hi - p.sigma_lo);
    double am = p.amp_lo + (double)(c1[1] >> 8) / 16777216.0 * ((double)p.amp_hi - p.amp_lo);
    amp[k] = (float)am;
    for (int a = 0; a < 3; ++a)
      for (long long i = 0; i < d[a]; ++i) {
        double dd = (double)i - cen[a];
        tab[a][(long long)k * d[a] + i] = (float)std::exp(-(dd * dd) / (2.0 * sig * sig));
      }
  }
  if (p.bg_freq > 0) {
    uint32_t c[4] = {0xffffffffu, 2u, 0x626c6f62u, 0u};
    philox(c, k0, k1);
    float* bg = t + nb + (long long)nb * (d[0] + d[1] + d[2]);
    for (int a = 0; a < 3; ++a) {
      double ph = (double)(c[a] >> 8) / 16777216.0;
      for (long long i = 0; i < d[a]; ++i)
        bg[i] = (float)std::cos(2.0 * M_PI * ((double)p.bg_freq * ((double)i + 0.5) / (double)d[a] + ph));
      bg += d[a];
    }
  }
}

}  // namespace

extern "C" int gbvr_dev_synth_volume_noalloc(const gbvr_synth_params* p, void* dev_out, size_t bytes, void* stream) {
  GBVR_ABI_TRY
  if (!p || !dev_out) return set_error(GBVR_EINVAL, "null argument");
  if (p->dims[0] <= 0 || p->dims[1] <= 0 || p->dims[2] <= 0 || p->dtype < 0 || p->dtype > 2 || p->nblobs < 0)
    return set_error(GBVR_EINVAL, "bad synthetic parameters");
  const long long X = p->dims[0], Y = p->dims[1], Z = p->dims[2];
  const long long need = (long long)p->nblobs * (1 + X + Y + Z) + (p->bg_freq > 0 ? X + Y + Z : 0);
  if (need > kSynthScratchFloats)
    return set_error(GBVR_EINVAL, "the generator tables need " + std::to_string(need) +
                                      " floats; the no-allocation entry point holds at most " +
                                      std::to_string(kSynthScratchFloats) +
                                      " (nblobs x (1 + X + Y + Z) + X + Y + Z)");
  const size_t out_bytes = (size_t)X * Y * Z * dtype_size(p->dtype);
  if (bytes < out_bytes) return set_error(GBVR_EINVAL, "output buffer too small");
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(GBVR_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error(GBVR_EINVAL, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_dev[dev]) {
    // Set-up, once per device, with that device current: resolve the device
    // address of the scratch array (the first call on a device also loads
    // the library's device code there).
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_synth_scratch);
    if (e != cudaSuccess) return set_error(GBVR_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_dev[dev] = (float*)ptr;
  }
  float* dt = g_scratch_dev[dev];
  if (need > 0) {
    fill_tables(*p, g_tables_host);
    // from pageable memory: returns once the source has been staged, so the
    // static host tables may be refilled by the next call
    e = cudaMemcpyAsync(dt, g_tables_host, sizeof(float) * (size_t)need, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return set_error(GBVR_ECUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
  }
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
