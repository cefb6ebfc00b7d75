// Host runtime behind the C ABI of include/gbvr.h: dataset build and
// residency (brick pool + page table), render state, paint (plain per view or
// one persistent batch replayed as a CUDA graph), readback and statistics.
//
// The renderer object mirrors the state Tuvok's AbstrRenderer keeps behind
// the Lua calls of LuaScripts/BatchRenderer.lua:22-41 and the setters of
// ImageVis3D/UI/RenderWindow.h:77-314.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <climits>
#include <cstddef>
#include <stdexcept>
#include <cstdlib>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/gbvr.h"
#include "abi_guard.h"
#include "gbvr_internal.h"
#include "deflate.h"
#include "brick_order.h"
#include "lz4.h"
#include "synth_tables.h"
#include "uvf.h"

#include <thread>

namespace gbvr {
bool write_image(const std::string& path, const unsigned char* rgba, int w, int h, bool alpha);
}

using namespace gbvr;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& m) {
  g_err = m;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? GBVR_ENOMEM : GBVR_ECUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define CUDA_TRY(x)                                  \
  do {                                               \
    cudaError_t e_ = (x);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #x); \
  } while (0)

#define TRY(x)                 \
  do {                         \
    int rc_ = (x);             \
    if (rc_ != GBVR_OK) return rc_; \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void swap(DevBuf& o) {
    std::swap(p, o.p);
    std::swap(n, o.n);
  }
  cudaError_t alloc(size_t bytes) {
    if (bytes <= n && p) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e == cudaSuccess) n = bytes;
    else p = nullptr;
    return e;
  }
  template <typename T>
  T* as() const { return (T*)p; }
};

// Host-side failure injection for the error-path tests: the environment
// variable GBVR_FAULT_INJECT names one failure site -- "pinned_alloc" (every
// page-locked allocation fails as if host memory were exhausted) or
// "server_launch" (the serving worker's batch launch throws).  Unset in
// normal use; nothing on the GPU is made to fail.
bool fault_injected(const char* site) {
  const char* v = std::getenv("GBVR_FAULT_INJECT");
  return v && std::strcmp(v, site) == 0;
}

cudaError_t host_alloc_pinned(void** p, size_t bytes) {
  if (fault_injected("pinned_alloc")) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMallocHost(p, bytes);
}

struct PinnedBuf {
  void* p = nullptr;
  size_t n = 0;
  ~PinnedBuf() { if (p) cudaFreeHost(p); }
  void swap(PinnedBuf& o) {
    std::swap(p, o.p);
    std::swap(n, o.n);
  }
  cudaError_t alloc(size_t bytes) {
    if (bytes <= n && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    cudaError_t e = host_alloc_pinned(&p, bytes ? bytes : 16);
    if (e == cudaSuccess) n = bytes;
    return e;
  }
};

// ---------------------------------------------------------------------------
// 4x4 helpers (row-major, column vectors), double precision on the host.
// ---------------------------------------------------------------------------
void mat_mul(const double* a, const double* b, double* o) {
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += a[4 * r + k] * b[4 * k + c];
      o[4 * r + c] = s;
    }
}

bool mat_inv(const double* m, double* inv) {
  double a[4][8];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? m[4 * r + c] : (c - 4 == r ? 1.0 : 0.0);
  for (int c = 0; c < 4; ++c) {
    int piv = c;
    for (int r = c + 1; r < 4; ++r)
      if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
    if (std::fabs(a[piv][c]) < 1e-300) return false;
    if (piv != c)
      for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
    double d = a[c][c];
    for (int k = 0; k < 8; ++k) a[c][k] /= d;
    for (int r = 0; r < 4; ++r) {
      if (r == c) continue;
      double f = a[r][c];
      if (f == 0) continue;
      for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
    }
  }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) inv[4 * r + c] = a[r][c + 4];
  return true;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 on the host (same stream as the device generator).
// ---------------------------------------------------------------------------
void philox_host(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[0] = n0; c[1] = (uint32_t)p1; c[2] = n2; c[3] = (uint32_t)p0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// Per-axis blob / background tables of a synthetic volume (host math, double,
// rounded to float): the device kernel then combines them in a fixed float32
// order.  One flat array (fill_blob_tables), split here into the uploads.
struct BlobTablesHost {
  std::vector<float> amp, ex, ey, ez, bgx, bgy, bgz;
};

void make_blob_tables(const gbvr_synth_params& p, BlobTablesHost& t) {
  const size_t nb = (size_t)p.nblobs, X = (size_t)p.dims[0], Y = (size_t)p.dims[1], Z = (size_t)p.dims[2];
  const size_t bg = p.bg_freq > 0 ? X + Y + Z : 0;
  std::vector<float> flat(nb * (1 + X + Y + Z) + bg);
  fill_blob_tables(p, flat.data());
  const float* q = flat.data();
  auto take = [&](std::vector<float>& v, size_t n) {
    v.assign(q, q + n);
    q += n;
  };
  take(t.amp, nb);
  take(t.ex, nb * X);
  take(t.ey, nb * Y);
  take(t.ez, nb * Z);
  if (bg) {
    take(t.bgx, X);
    take(t.bgy, Y);
    take(t.bgz, Z);
  }
}

// ---------------------------------------------------------------------------
// Dataset: the brick pool and its page table (one LOD pyramid).
// ---------------------------------------------------------------------------
struct Level {
  long long dims[3];
  int nb[3];
  int interior;
  int brick_base;
  int nbricks;
  int nc[3];                          // macro-cell grid
  int cell_shift = 2;                 // macro-cell edge = 1 << cell_shift voxels
  std::shared_ptr<DevBuf> cells;      // float2 min/max per macro-cell
  int nsc[3] = {0, 0, 0};             // super-cell grid (4^3 macro-cells each)
  std::shared_ptr<DevBuf> smax;       // float: largest cell maximum per super-cell (MIP skipping)
};

// The super-cell maxima of a level whose macro-cell min/max is complete.
int build_supercells(Level& L, cudaStream_t s) {
  constexpr int E = 1 << SUPERCELL_SHIFT;
  for (int a = 0; a < 3; ++a) L.nsc[a] = (L.nc[a] + E - 1) / E;
  L.smax = std::make_shared<DevBuf>();
  CUDA_TRY(L.smax->alloc(sizeof(float) * (size_t)L.nsc[0] * L.nsc[1] * L.nsc[2]));
  CUDA_TRY(launch_supercell_max(L.cells->as<float2>(), L.nc, L.smax->as<float>(), L.nsc, s));
  return GBVR_OK;
}

// macro-cell edge (voxels) for empty-space skipping inside bricks, and the
// cap of the empty-cell distance field
constexpr int CELL_SHIFT = 2;
constexpr int CELL_DIST_CAP = 16;

struct Dataset {
  bool loaded = false;
  int dtype = DT_U8;
  long long dims[3] = {0, 0, 0};
  double aspect[3] = {1, 1, 1};
  int brick = 256, ghost = 2;
  int layouts = 1;
  unsigned long long copy_stride = 0;  // elements between layout copies
  std::vector<Level> levels;
  std::vector<BrickInfo> bricks;
  DevBuf pool, d_bricks;
  uint64_t stored_bytes = 0;
  double gmin = 0, gmax = 0;
  int bit_width = 8;
  std::vector<uint64_t> hist1d;
  long long merge = 1;
  std::vector<uint64_t> hist2d;
  float max_grad = 0.f;
  std::vector<cudaArray_t> arrays;
  std::vector<cudaTextureObject_t> texs;
  std::string raster_id = "GB300 volume raster";
  gbvr_build_stats build{};  // the last in-core build's phase times and bytes
  // Out of core: every brick lives in page-locked host memory (host_store,
  // element offsets host_off); the device pool is a cache of nslots
  // fixed-size slots, and BrickInfo.offset points at a brick's slot while
  // it is resident.
  bool ooc = false;
  PinnedBuf host_store;
  std::vector<unsigned long long> host_off;
  // Compressed store (brick_params.compression = 3, LZ4): brick b's chunks
  // (LZ_CHUNK raw bytes each, the last one shorter) lie back to back from
  // byte host_coff[b]; chunk_size[chunk_first[b] + k] is chunk k's compressed
  // size (bit 31: stored uncompressed).  Paged bricks are decoded on the
  // device from d_stage into their slots.
  // The compressed store is a list of page-locked segments (a brick's run
  // lies in one): segment host_cseg[b], byte host_coff[b].
  int compression = 0;
  int brick_order = 0;            // host store: order of each level's bricks (0 scanline, 1 Morton, 2 Hilbert, 3 random)
  std::vector<int> store_order;   // the bricks in host-store order, level by level
  std::vector<void*> seg_p;
  std::vector<size_t> seg_used;
  std::vector<int> host_cseg;
  std::vector<unsigned long long> host_coff;
  std::vector<unsigned> chunk_first, chunk_size;
  uint64_t raw_store_bytes = 0, comp_store_bytes = 0;
  DevBuf d_stage, d_chunks, d_lz_err;
  const uint8_t* comp_run(size_t b) const { return (const uint8_t*)seg_p[host_cseg[b]] + host_coff[b]; }
  size_t slot_elems = 0;
  int nslots = 0;
  std::vector<int> slot_of;                  // per brick, -1 = not resident
  std::vector<int> slot_brick;               // per slot, -1 = free
  std::vector<unsigned long long> slot_used; // frame of last use, per slot
  unsigned long long frame = 0;

  void release() {
    for (auto t : texs) cudaDestroyTextureObject(t);
    for (auto a : arrays) cudaFreeArray(a);
    texs.clear();
    arrays.clear();
    build = gbvr_build_stats{};
    pool.release();
    d_bricks.release();
    if (host_store.p) cudaFreeHost(host_store.p);
    host_store.p = nullptr;
    host_store.n = 0;
    ooc = false;
    host_off.clear();
    compression = 0;
    for (void* q : seg_p) cudaFreeHost(q);
    seg_p.clear();
    seg_used.clear();
    host_cseg.clear();
    comp_store_bytes = 0;
    host_coff.clear();
    chunk_first.clear();
    chunk_size.clear();
    raw_store_bytes = 0;
    d_stage.release();
    d_chunks.release();
    d_lz_err.release();
    slot_of.clear();
    slot_brick.clear();
    slot_used.clear();
    nslots = 0;
    levels.clear();
    bricks.clear();
    hist1d.clear();
    hist2d.clear();
    loaded = false;
  }
  ~Dataset() { release(); }
};

// LOD and brick-grid rules: the level count halves (ceil) until the largest
// axis fits one brick interior (brick - 2 ghost), as UVFReader/DataSource.h:521-529
// halves the raster until it fits; the oracle states the same rules.
int lod_dims(const long long dims[3], int brick, int ghost, int max_lods, std::vector<std::array<long long, 3>>& out) {
  long long I = brick - 2 * ghost;
  long long n[3] = {dims[0], dims[1], dims[2]};
  out.clear();
  for (;;) {
    out.push_back({n[0], n[1], n[2]});
    long long mx = std::max(n[0], std::max(n[1], n[2]));
    if (mx <= I || out.size() == 16) break;
    if (max_lods > 0 && (int)out.size() >= max_lods) break;
    for (int a = 0; a < 3; ++a) n[a] = (n[a] + 1) / 2;
  }
  return (int)out.size();
}

size_t elem_align(int dtype) { return 256 / dtype_size(dtype); }

void plan_level(const long long dims[3], int brick, int ghost, int level, Level& L, std::vector<BrickInfo>& bricks,
                unsigned long long& cursor, int dtype) {
  long long I = brick - 2 * ghost;
  long long mx = std::max(dims[0], std::max(dims[1], dims[2]));
  bool single = mx <= I;
  for (int a = 0; a < 3; ++a) {
    L.dims[a] = dims[a];
    L.nb[a] = single ? 1 : (int)((dims[a] + I - 1) / I);
  }
  L.interior = single ? (int)std::max<long long>(mx, 1) : (int)I;
  L.brick_base = (int)bricks.size();
  L.nbricks = L.nb[0] * L.nb[1] * L.nb[2];
  for (int bz = 0; bz < L.nb[2]; ++bz)
    for (int by = 0; by < L.nb[1]; ++by)
      for (int bx = 0; bx < L.nb[0]; ++bx) {
        BrickInfo b;
        memset(&b, 0, sizeof(b));
        int bc[3] = {bx, by, bz};
        int o[3], s[3], lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
          // interior [ilo, ihi); stored box = interior + `ghost` voxels on
          // every face (replicated edge voxels outside the level)
          long long ilo = (long long)bc[a] * L.interior, ihi = std::min<long long>(ilo + L.interior, dims[a]);
          o[a] = (int)(ilo - ghost);
          s[a] = (int)(ihi - ilo + 2 * ghost);
          lo[a] = bc[a] == 0 ? -1 : (int)ilo;
          hi[a] = (int)ihi;
        }
        b.ox = o[0]; b.oy = o[1]; b.oz = o[2];
        b.sx = s[0]; b.sy = s[1]; b.sz = s[2];
        b.lox = lo[0]; b.loy = lo[1]; b.loz = lo[2];
        b.hix = hi[0]; b.hiy = hi[1]; b.hiz = hi[2];
        b.level = level;
        b.offset = cursor;
        // room for the 4x4x4-blocked copy too (stored dims rounded up to 4)
        unsigned long long n = (unsigned long long)((s[0] + 3) & ~3) * ((s[1] + 3) & ~3) * ((s[2] + 3) & ~3);
        const unsigned long long al = elem_align(dtype);
        cursor += (n + al - 1) / al * al;
        bricks.push_back(b);
      }
}

int build_textures(Dataset& ds, cudaStream_t s) {
  cudaChannelFormatDesc cd;
  if (ds.dtype == DT_U8) cd = cudaCreateChannelDesc<unsigned char>();
  else if (ds.dtype == DT_U16) cd = cudaCreateChannelDesc<unsigned short>();
  else cd = cudaCreateChannelDesc<float>();
  const size_t es = dtype_size(ds.dtype);
  for (BrickInfo& b : ds.bricks) {
    cudaArray_t arr;
    CUDA_TRY(cudaMalloc3DArray(&arr, &cd, make_cudaExtent(b.sx, b.sy, b.sz)));
    ds.arrays.push_back(arr);
    cudaMemcpy3DParms cp = {};
    cp.srcPtr = make_cudaPitchedPtr((char*)ds.pool.p + b.offset * es, (size_t)b.sx * es, b.sx, b.sy);
    cp.dstArray = arr;
    cp.extent = make_cudaExtent(b.sx, b.sy, b.sz);
    cp.kind = cudaMemcpyDeviceToDevice;
    CUDA_TRY(cudaMemcpy3DAsync(&cp, s));
    cudaResourceDesc rd = {};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td = {};
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = ds.dtype == DT_F32 ? cudaReadModeElementType : cudaReadModeNormalizedFloat;
    td.normalizedCoords = 0;
    cudaTextureObject_t t;
    CUDA_TRY(cudaCreateTextureObject(&t, &rd, &td, nullptr));
    ds.texs.push_back(t);
    b.tex = (unsigned long long)t;
  }
  CUDA_TRY(cudaMemcpyAsync(ds.d_bricks.p, ds.bricks.data(), sizeof(BrickInfo) * ds.bricks.size(), cudaMemcpyHostToDevice, s));
  return GBVR_OK;
}

// GPU UVF build: LOD pyramid, bricks with ghosts, per-brick min/max, 1D and
// 2D histograms.  d_level0 (device, flat, x fastest) is consumed.
// Device time of one build phase: events recorded right before and after
// its launches on the build stream; read once the build has synchronised.
struct PhaseTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  double* acc;
  explicit PhaseTimer(double* out) : acc(out) {}
  ~PhaseTimer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
  cudaError_t start(cudaStream_t s) {
    cudaError_t e = a ? cudaSuccess : cudaEventCreate(&a);
    if (e == cudaSuccess && !b) e = cudaEventCreate(&b);
    return e == cudaSuccess ? cudaEventRecord(a, s) : e;
  }
  cudaError_t stop(cudaStream_t s) { return cudaEventRecord(b, s); }
  // after a synchronisation of the stream (a phase never started adds 0)
  cudaError_t add() {
    if (!a) return cudaSuccess;
    float ms = 0.f;
    cudaError_t e = cudaEventElapsedTime(&ms, a, b);
    if (e == cudaSuccess) *acc += ms;
    return e;
  }
};

int build_dataset(Dataset& ds, DevBuf& d_level0, int dtype, const long long dims[3], const gbvr_brick_params* bp,
                  cudaStream_t s) {
  ds.release();
  gbvr_build_stats& bs = ds.build;
  bs = gbvr_build_stats{};
  PhaseTimer t_pyr(&bs.pyramid_ms), t_cells(&bs.cells_ms), t_bricks(&bs.bricks_ms), t_mm(&bs.minmax_ms),
      t_h1(&bs.hist1d_ms), t_h2(&bs.hist2d_ms);
  ds.dtype = dtype;
  for (int a = 0; a < 3; ++a) ds.dims[a] = dims[a];
  ds.brick = bp && bp->brick_size > 0 ? bp->brick_size : 256;
  ds.ghost = bp && bp->overlap >= 0 ? bp->overlap : 2;
  if (bp && bp->brick_size == 0 && bp->overlap == 0) ds.ghost = 2;
  if (ds.ghost < 2) return fail(GBVR_EINVAL, "overlap must be >= 2 (gradients need two ghost voxels)");
  if (ds.brick - 2 * ds.ghost < 8) return fail(GBVR_EINVAL, "brick_size too small for the overlap");
  if (ds.brick > 2048) return fail(GBVR_EOVERSIZED, "brick_size exceeds the 2048 voxel limit");
  for (int a = 0; a < 3; ++a) ds.aspect[a] = (bp && bp->aspect[a] > 0) ? bp->aspect[a] : 1.0;
  std::vector<std::array<long long, 3>> ld;
  lod_dims(dims, ds.brick, ds.ghost, bp ? bp->max_lods : 0, ld);
  const size_t es = dtype_size(dtype);
  // level volumes
  std::vector<std::unique_ptr<DevBuf>> lv;
  lv.emplace_back(new DevBuf());
  std::swap(lv[0]->p, d_level0.p);
  std::swap(lv[0]->n, d_level0.n);
  auto level_bytes = [&](size_t l) { return (uint64_t)ld[l][0] * ld[l][1] * ld[l][2] * es; };
  for (size_t l = 1; l < ld.size(); ++l) {
    lv.emplace_back(new DevBuf());
    CUDA_TRY(lv[l]->alloc((size_t)level_bytes(l)));
  }
  CUDA_TRY(t_pyr.start(s));
  for (size_t l = 1; l < ld.size(); ++l) {
    long long pd[3] = {ld[l - 1][0], ld[l - 1][1], ld[l - 1][2]};
    CUDA_TRY(launch_downsample(lv[l - 1]->p, dtype, pd, lv[l]->p, s));
    bs.pyramid_bytes += level_bytes(l - 1) + level_bytes(l);
  }
  CUDA_TRY(t_pyr.stop(s));
  // page table
  unsigned long long cursor = 0;
  for (size_t l = 0; l < ld.size(); ++l) {
    Level L;
    long long d[3] = {ld[l][0], ld[l][1], ld[l][2]};
    plan_level(d, ds.brick, ds.ghost, (int)l, L, ds.bricks, cursor, dtype);
    ds.levels.push_back(L);
  }
  ds.stored_bytes = 0;
  for (auto& b : ds.bricks) ds.stored_bytes += (uint64_t)b.sx * b.sy * b.sz * es;
  // layout copies: 1 = x-fastest only; 3 = + y- and z-fastest; 4 = + 4^3-blocked;
  // 5 = + 4^3 blocks that also hold their +1 neighbours (5^3 voxels in 128
  // elements: twice the room of the blocked copy, which each brick's share of
  // the cursor already rounds to 4^3 blocks); 6 = + both blocked copies
  ds.layouts = (bp && bp->layouts >= 3 && bp->layouts <= 6) ? bp->layouts : 1;
  ds.copy_stride = cursor;
  const int ncopies = ds.layouts == 6 ? 4 : ds.layouts == 5 ? 3 : ds.layouts == 4 ? 2 : ds.layouts;
  CUDA_TRY(ds.pool.alloc(cursor * es * ncopies));
  // the gather reduces each brick's min/max into these
  for (BrickInfo& b : ds.bricks) {
    b.vmin = INFINITY;
    b.vmax = -INFINITY;
  }
  CUDA_TRY(ds.d_bricks.alloc(sizeof(BrickInfo) * ds.bricks.size()));
  CUDA_TRY(cudaMemcpyAsync(ds.d_bricks.p, ds.bricks.data(), sizeof(BrickInfo) * ds.bricks.size(), cudaMemcpyHostToDevice, s));
  for (size_t l = 0; l < ld.size(); ++l) {
    Level& L = ds.levels[l];
    L.cell_shift = CELL_SHIFT;
    for (int a = 0; a < 3; ++a) L.nc[a] = (int)((ld[l][a] + (1 << CELL_SHIFT) - 1) >> CELL_SHIFT);
    L.cells = std::make_shared<DevBuf>();
    CUDA_TRY(L.cells->alloc(sizeof(float2) * (size_t)L.nc[0] * L.nc[1] * L.nc[2]));
    L.smax = std::make_shared<DevBuf>();
    for (int a = 0; a < 3; ++a) L.nsc[a] = (L.nc[a] + (1 << SUPERCELL_SHIFT) - 1) >> SUPERCELL_SHIFT;
    CUDA_TRY(L.smax->alloc(sizeof(float) * (size_t)L.nsc[0] * L.nsc[1] * L.nsc[2]));
  }
  // macro-cell min/max (and the MIP super-cells) of every level
  CUDA_TRY(t_cells.start(s));
  for (size_t l = 0; l < ld.size(); ++l) {
    Level& L = ds.levels[l];
    long long d[3] = {ld[l][0], ld[l][1], ld[l][2]};
    CUDA_TRY(launch_cell_minmax(lv[l]->p, dtype, d, CELL_SHIFT, L.nc, L.cells->as<float2>(), s));
    CUDA_TRY(launch_supercell_max(L.cells->as<float2>(), L.nc, L.smax->as<float>(), L.nsc, s));
    bs.cells_bytes += level_bytes(l);
  }
  CUDA_TRY(t_cells.stop(s));
  // bricks (interior + ghosts) of every level, per layout copy
  CUDA_TRY(t_bricks.start(s));
  for (size_t l = 0; l < ld.size(); ++l) {
    Level& L = ds.levels[l];
    long long d[3] = {ld[l][0], ld[l][1], ld[l][2]};
    uint64_t stored = 0;
    for (int i = 0; i < L.nbricks; ++i) {
      const BrickInfo& b = ds.bricks[L.brick_base + i];
      stored += (uint64_t)b.sx * b.sy * b.sz * es;
    }
    // the x-fastest copy (0), the blocked copy (1) when there is one, and
    // the bricks' min/max in one pass over the level
    int max_sz = 1;
    for (int i = 0; i < L.nbricks; ++i) max_sz = std::max(max_sz, ds.bricks[L.brick_base + i].sz);
    const bool blocked = ds.layouts == 4 || ds.layouts == 6;
    CUDA_TRY(launch_gather_fused(lv[l]->p, dtype, d, ds.d_bricks.as<BrickInfo>() + L.brick_base, L.nbricks, max_sz,
                                 ds.pool.p, blocked ? (char*)ds.pool.p + (size_t)cursor * es : nullptr, s));
    bs.bricks_bytes += level_bytes(l) + stored * (blocked ? 2 : 1);
    // the other copies: (copy, layout) 1 and 2 y- and z-fastest, 4
    // overlapped blocks (two copies' room)
    std::vector<std::pair<int, int>> copies;
    if (ds.layouts == 3) copies = {{1, 1}, {2, 2}};
    else if (ds.layouts == 5) copies = {{1, 4}};
    else if (ds.layouts == 6) copies = {{2, 4}};
    for (const auto& cp : copies) {
      CUDA_TRY(launch_gather_bricks(lv[l]->p, dtype, d, ds.d_bricks.as<BrickInfo>() + L.brick_base, L.nbricks,
                                    (char*)ds.pool.p + (size_t)cp.first * cursor * es, cp.second, s));
      bs.bricks_bytes += level_bytes(l) + stored * (cp.second == 4 ? 2 : 1);
    }
  }
  CUDA_TRY(t_bricks.stop(s));
  // per-brick min/max: reduced by the gather above
  bs.minmax_bytes = 0;
  CUDA_TRY(cudaMemcpyAsync(ds.bricks.data(), ds.d_bricks.p, sizeof(BrickInfo) * ds.bricks.size(), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  ds.gmin = INFINITY;
  ds.gmax = -INFINITY;
  for (int i = 0; i < ds.levels[0].nbricks; ++i) {
    ds.gmin = std::min(ds.gmin, (double)ds.bricks[i].vmin);
    ds.gmax = std::max(ds.gmax, (double)ds.bricks[i].vmax);
  }
  // histograms of LOD 0 (integer data)
  const long long n0 = dims[0] * dims[1] * dims[2];
  if (dtype != DT_F32) {
    int nbins = (int)ds.gmax + 1;
    DevBuf dh;
    CUDA_TRY(dh.alloc(sizeof(uint64_t) * nbins));
    CUDA_TRY(cudaMemsetAsync(dh.p, 0, sizeof(uint64_t) * nbins, s));
    CUDA_TRY(t_h1.start(s));
    CUDA_TRY(launch_hist1d(lv[0]->p, dtype, n0, dh.as<unsigned long long>(), nbins, s));
    CUDA_TRY(t_h1.stop(s));
    bs.hist1d_bytes = level_bytes(0);
    std::vector<uint64_t> full(nbins);
    CUDA_TRY(cudaMemcpyAsync(full.data(), dh.p, sizeof(uint64_t) * nbins, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    long long size = nbins;
    while (size > 1 && full[size - 1] == 0) --size;
    ds.merge = (size + 4095) / 4096;
    if (ds.merge < 1) ds.merge = 1;
    long long outsize = (size + ds.merge - 1) / ds.merge;
    ds.hist1d.assign(outsize, 0);
    for (long long i = 0; i < size; ++i) ds.hist1d[i / ds.merge] += full[i];
    // 2D
    DevBuf d2, dsc;
    const size_t n2 = (size_t)outsize * 256;
    CUDA_TRY(d2.alloc(sizeof(uint64_t) * n2));
    CUDA_TRY(dsc.alloc(sizeof(Hist2DScratch)));
    CUDA_TRY(cudaMemsetAsync(d2.p, 0, sizeof(uint64_t) * n2, s));
    CUDA_TRY(t_h2.start(s));
    // ds.gmax is the level's largest voxel (the bricks' maxima)
    CUDA_TRY(launch_hist2d(lv[0]->p, dtype, dims, ds.gmax, outsize, ds.merge, d2.as<unsigned long long>(),
                           dsc.as<Hist2DScratch>(), s, dtype == DT_U16 && ds.gmax < 16384.0));
    CUDA_TRY(t_h2.stop(s));
    // two passes over the level (the largest squared gradient, then the bins);
    // the f64 pass between them revisits only the voxels attaining it
    bs.hist2d_bytes = 2 * level_bytes(0);
    ds.hist2d.resize(n2);
    Hist2DScratch hs;
    CUDA_TRY(cudaMemcpyAsync(ds.hist2d.data(), d2.p, sizeof(uint64_t) * n2, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(&hs, dsc.p, sizeof(hs), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    double g;
    memcpy(&g, &hs.gmax_bits, 8);
    ds.max_grad = (float)g;
    ds.bit_width = dtype == DT_U8 ? 8 : 16;
    CUDA_TRY(t_h1.add());
    CUDA_TRY(t_h2.add());
  } else {
    ds.bit_width = 32;
  }
  CUDA_TRY(t_pyr.add());
  CUDA_TRY(t_cells.add());
  CUDA_TRY(t_bricks.add());
  CUDA_TRY(t_mm.add());
  bs.total_ms = bs.pyramid_ms + bs.cells_ms + bs.bricks_ms + bs.minmax_ms + bs.hist1d_ms + bs.hist2d_ms;
  bs.total_bytes = bs.pyramid_bytes + bs.cells_bytes + bs.bricks_bytes + bs.minmax_bytes + bs.hist1d_bytes +
                   bs.hist2d_bytes;
  bs.level0_bytes = level_bytes(0);
  bs.lod_count = (int32_t)ld.size();
  bs.layout_copies = ds.layouts == 6 ? 3 : ds.layouts >= 4 ? 2 : ds.layouts;
  if (bp && bp->build_texture) TRY(build_textures(ds, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  ds.loaded = true;
  return GBVR_OK;
}


// ---------------------------------------------------------------------------
// Out-of-core build.  The finest level is generated on the device in z-slabs
// of S = 2^(levels-1) planes; every level keeps a window of its planes in
// device memory.  From each window the build emits, as soon as their planes
// are present: complete brick layers (interior + ghosts, the same bricks as
// the in-core build) into the page-locked host store, macro-cell layers
// (min/max) into the level's cell grid, and pairs of planes averaged into the
// next level's window.  Planes no window still needs are dropped.  Device
// memory is O(plane area x brick size), independent of the volume depth.
// ---------------------------------------------------------------------------
constexpr int OOC_CELL_SHIFT = 3;
// raw bytes per compressed chunk of a brick (one LZ4 block): small enough that
// a paged frame gives the decoder thousands of warps
constexpr size_t LZ_CHUNK = 16384;
// the host store's LZ4 encoder: hash-chain depth and the shortest match taken
constexpr int kStoreLz4Chain = 16, kStoreLz4MinMatch = 8;

int build_ooc_synth(Dataset& ds, const gbvr_synth_params* p, const gbvr_brick_params* bp, uint64_t pool_bytes,
                    cudaStream_t s) {
  ds.release();
  const int dtype = p->dtype;
  const size_t es = dtype_size(dtype);
  ds.dtype = dtype;
  long long dims[3] = {p->dims[0], p->dims[1], p->dims[2]};
  for (int a = 0; a < 3; ++a) ds.dims[a] = dims[a];
  ds.brick = bp && bp->brick_size > 0 ? bp->brick_size : 256;
  ds.ghost = bp && bp->overlap > 0 ? bp->overlap : 2;
  if (ds.ghost < 2) return fail(GBVR_EINVAL, "overlap must be >= 2 (gradients need two ghost voxels)");
  if (ds.brick - 2 * ds.ghost < 8) return fail(GBVR_EINVAL, "brick_size too small for the overlap");
  for (int a = 0; a < 3; ++a) ds.aspect[a] = (bp && bp->aspect[a] > 0) ? bp->aspect[a] : 1.0;
  std::vector<std::array<long long, 3>> ld;
  const int nlev = lod_dims(dims, ds.brick, ds.ghost, bp ? bp->max_lods : 0, ld);
  unsigned long long cursor = 0;
  for (int l = 0; l < nlev; ++l) {
    Level L;
    long long d[3] = {ld[l][0], ld[l][1], ld[l][2]};
    plan_level(d, ds.brick, ds.ghost, l, L, ds.bricks, cursor, dtype);
    L.cell_shift = OOC_CELL_SHIFT;
    for (int a = 0; a < 3; ++a) L.nc[a] = (int)((d[a] + (1 << OOC_CELL_SHIFT) - 1) >> OOC_CELL_SHIFT);
    L.cells = std::make_shared<DevBuf>();
    CUDA_TRY(L.cells->alloc(sizeof(float2) * (size_t)L.nc[0] * L.nc[1] * L.nc[2]));
    ds.levels.push_back(L);
  }
  const size_t nb = ds.bricks.size();
  ds.host_off.resize(nb);
  size_t max_brick = 0;
  ds.stored_bytes = 0;
  for (size_t i = 0; i < nb; ++i) {
    const BrickInfo& b = ds.bricks[i];
    ds.host_off[i] = b.offset;
    const size_t n = (size_t)b.sx * b.sy * b.sz;
    max_brick = std::max(max_brick, n);
    ds.stored_bytes += n * es;
  }
  const size_t al = elem_align(dtype);
  ds.slot_elems = (max_brick + al - 1) / al * al;
  const size_t slot_bytes = ds.slot_elems * es;
  ds.nslots = (int)std::min<uint64_t>(pool_bytes / slot_bytes, (uint64_t)nb);
  if (ds.nslots < 1) return fail(GBVR_EINVAL, "device pool smaller than one brick");
  CUDA_TRY(ds.pool.alloc((size_t)ds.nslots * slot_bytes));
  ds.slot_of.assign(nb, -1);
  ds.slot_brick.assign(ds.nslots, -1);
  ds.slot_used.assign(ds.nslots, 0);
  // the bricks' order in the host store (the converter's brick layouts)
  ds.brick_order = bp ? bp->brick_order : 0;
  ds.store_order.clear();
  for (const Level& L : ds.levels) {
    std::vector<int> perm;
    if (!brick_order(L.nb, ds.brick_order, 0x5eedull + (uint64_t)L.brick_base, perm))
      return fail(GBVR_EINVAL, "brick order must be 0 (scanline), 1 (Morton), 2 (Hilbert) or 3 (random)");
    for (int k : perm) ds.store_order.push_back(L.brick_base + k);
  }
  if (ds.brick_order) {
    // the same extents (each brick's share of the cursor), laid out in store order
    std::vector<unsigned long long> ext(nb);
    for (size_t i = 0; i < nb; ++i) ext[i] = (i + 1 < nb ? ds.host_off[i + 1] : cursor) - ds.host_off[i];
    unsigned long long at = 0;
    for (int bi : ds.store_order) {
      ds.host_off[(size_t)bi] = at;
      at += ext[(size_t)bi];
    }
  }
  for (auto& b : ds.bricks) b.offset = 0;
  ds.compression = bp ? bp->compression : 0;
  if (ds.compression != 0 && ds.compression != 1 && ds.compression != 3)
    return fail(GBVR_EINVAL, "compression must be 0 (none), 1 (zlib) or 3 (LZ4)");
  ds.raw_store_bytes = cursor * es;
  if (!ds.compression) {
    cudaError_t e = host_alloc_pinned(&ds.host_store.p, cursor * es);
    if (e != cudaSuccess) return fail(GBVR_ENOMEM, "page-locked host brick store of " + std::to_string(cursor * es) + " bytes");
    ds.host_store.n = cursor * es;
  } else {
    ds.host_coff.assign(nb, 0);
    ds.host_cseg.assign(nb, 0);
    ds.chunk_first.assign(nb, 0);
  }
  // compressed store: each layer of bricks comes to page-locked staging in
  // one copy and is compressed by host threads into page-locked segments of
  // 16 MiB .. 4 GiB (no copy of the whole store: it is built in place)
  const size_t kSeg = std::min<size_t>((size_t)1 << 32, std::max<size_t>((size_t)1 << 24, ds.raw_store_bytes / 8));
  auto seg_append = [&](const uint8_t* data, size_t n, int& seg, unsigned long long& off) -> int {
    if (ds.seg_p.empty() || ds.seg_used.back() + n > kSeg) {
      void* q = nullptr;
      if (host_alloc_pinned(&q, std::max(kSeg, n)) != cudaSuccess)
        return fail(GBVR_ENOMEM, "page-locked compressed brick store segment");
      ds.seg_p.push_back(q);
      ds.seg_used.push_back(0);
    }
    seg = (int)ds.seg_p.size() - 1;
    off = ds.seg_used.back();
    memcpy((uint8_t*)ds.seg_p.back() + off, data, n);
    ds.seg_used.back() += n;
    ds.comp_store_bytes += n;
    return GBVR_OK;
  };
  PinnedBuf h_layer;
  const unsigned nthreads = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  // generator tables
  BlobTablesHost tab;
  make_blob_tables(*p, tab);
  DevBuf amp, ex, ey, ez, bx, by, bz;
  auto up = [&](DevBuf& d, const std::vector<float>& v) -> cudaError_t {
    cudaError_t e = d.alloc(sizeof(float) * std::max<size_t>(v.size(), 1));
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(d.p, v.data(), sizeof(float) * v.size(), cudaMemcpyHostToDevice, s);
  };
  CUDA_TRY(up(amp, tab.amp));
  CUDA_TRY(up(ex, tab.ex));
  CUDA_TRY(up(ey, tab.ey));
  CUDA_TRY(up(ez, tab.ez));
  CUDA_TRY(up(bx, tab.bgx));
  CUDA_TRY(up(by, tab.bgy));
  CUDA_TRY(up(bz, tab.bgz));
  const bool bg = p->bg_freq > 0;
  BlobTablesDev td{p->nblobs, amp.as<float>(), ex.as<float>(), ey.as<float>(), ez.as<float>(),
                   bg ? bx.as<float>() : nullptr, bg ? by.as<float>() : nullptr, bg ? bz.as<float>() : nullptr,
                   p->bg_level, p->bg_amp, p->scale, p->noise_amp, p->noise_kind, p->vmax, p->seed};
  // per-level windows
  const long long I = ds.brick - 2 * ds.ghost, g = ds.ghost;
  const long long S = std::max<long long>(2, 1LL << (nlev - 1));
  struct Stage {
    DevBuf a, b;
    long long z0 = 0, n = 0, cap = 0, X = 0, Y = 0, Z = 0, ds_next = 0;
    int next_bz = 0, next_cz = 0;
    size_t plane = 0;
  };
  std::vector<Stage> st(nlev);
  size_t max_layer = 0;
  for (int l = 0; l < nlev; ++l) {
    Stage& w = st[l];
    w.X = ld[l][0];
    w.Y = ld[l][1];
    w.Z = ld[l][2];
    w.plane = (size_t)w.X * w.Y * es;
    const long long M = 1LL << OOC_CELL_SHIFT;
    w.cap = std::min<long long>(w.Z, I + 2 * g + M + 3 + std::max<long long>(S >> l, 2) + 4);
    CUDA_TRY(w.a.alloc(w.plane * w.cap));
    CUDA_TRY(w.b.alloc(w.plane * w.cap));
    max_layer = std::max(max_layer, (size_t)ds.levels[l].nb[0] * ds.levels[l].nb[1]);
  }
  DevBuf tmp, tmp_info, hist;
  CUDA_TRY(tmp.alloc(max_layer * slot_bytes));
  CUDA_TRY(tmp_info.alloc(sizeof(BrickInfo) * max_layer));
  const int nbins = dtype == DT_U8 ? 256 : 65536;
  if (dtype != DT_F32) {
    CUDA_TRY(hist.alloc(sizeof(uint64_t) * nbins));
    CUDA_TRY(cudaMemsetAsync(hist.p, 0, sizeof(uint64_t) * nbins, s));
  }
  std::vector<BrickInfo> layer;
  auto process = [&](int l) -> int {
    Stage& w = st[l];
    Level& L = ds.levels[l];
    const long long have_end = w.z0 + w.n;
    long long d3[3] = {w.X, w.Y, w.Z};
    // complete brick layers -> host store
    while (w.next_bz < L.nb[2]) {
      const long long hi = std::min<long long>((long long)w.next_bz * I + I + g, w.Z);
      if (hi > have_end) break;
      const int per = L.nb[0] * L.nb[1];
      const int first = L.brick_base + w.next_bz * per;
      layer.assign(ds.bricks.begin() + first, ds.bricks.begin() + first + per);
      for (int j = 0; j < per; ++j) layer[j].offset = (unsigned long long)j * ds.slot_elems;
      CUDA_TRY(cudaMemcpyAsync(tmp_info.p, layer.data(), sizeof(BrickInfo) * per, cudaMemcpyHostToDevice, s));
      CUDA_TRY(launch_gather_bricks_window(w.a.p, dtype, d3, w.z0, tmp_info.as<BrickInfo>(), per, tmp.p, 0, s));
      CUDA_TRY(launch_brick_minmax(tmp.p, dtype, tmp_info.as<BrickInfo>(), per, s));
      CUDA_TRY(cudaMemcpyAsync(layer.data(), tmp_info.p, sizeof(BrickInfo) * per, cudaMemcpyDeviceToHost, s));
      if (!ds.compression) {
        for (int j = 0; j < per; ++j) {
          const BrickInfo& b = ds.bricks[first + j];
          CUDA_TRY(cudaMemcpyAsync((char*)ds.host_store.p + ds.host_off[first + j] * es,
                                   (const char*)tmp.p + (size_t)j * slot_bytes, (size_t)b.sx * b.sy * b.sz * es,
                                   cudaMemcpyDeviceToHost, s));
        }
        CUDA_TRY(cudaStreamSynchronize(s));
      } else {
        CUDA_TRY(h_layer.alloc((size_t)per * slot_bytes));
        CUDA_TRY(cudaMemcpyAsync(h_layer.p, tmp.p, (size_t)per * slot_bytes, cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        // per brick its chunks (compressed, or raw when that is not smaller)
        std::vector<std::vector<uint8_t>> out(per);
        std::vector<std::vector<unsigned>> sizes(per);
        auto work = [&](unsigned t) {
          std::vector<uint8_t> buf(std::max(lz4_bound(LZ_CHUNK), zlib_bound(LZ_CHUNK)));
          for (int j = (int)t; j < per; j += (int)nthreads) {
            const BrickInfo& b = ds.bricks[first + j];
            const size_t nbytes = (size_t)b.sx * b.sy * b.sz * es;
            const uint8_t* src = (const uint8_t*)h_layer.p + (size_t)j * slot_bytes;
            for (size_t o = 0; o < nbytes; o += LZ_CHUNK) {
              const size_t rn = std::min(LZ_CHUNK, nbytes - o);
              const size_t cn = ds.compression == 1 ? zlib_compress(src + o, rn, buf.data(), buf.size(), 16)
                                                    : lz4_compress(src + o, rn, buf.data(), buf.size(),
                                                                   kStoreLz4Chain, kStoreLz4MinMatch);
              if (cn > 0 && cn < rn) {
                out[j].insert(out[j].end(), buf.data(), buf.data() + cn);
                sizes[j].push_back((unsigned)cn);
              } else {
                out[j].insert(out[j].end(), src + o, src + o + rn);
                sizes[j].push_back((unsigned)rn | 0x80000000u);
              }
            }
          }
        };
        std::vector<std::thread> pool_t;
        for (unsigned t = 1; t < nthreads; ++t) pool_t.emplace_back(work, t);
        work(0);
        for (auto& th : pool_t) th.join();
        for (int j = 0; j < per; ++j) {
          TRY(seg_append(out[j].data(), out[j].size(), ds.host_cseg[first + j], ds.host_coff[first + j]));
          ds.chunk_first[first + j] = (unsigned)ds.chunk_size.size();
          ds.chunk_size.insert(ds.chunk_size.end(), sizes[j].begin(), sizes[j].end());
        }
      }
      for (int j = 0; j < per; ++j) {
        ds.bricks[first + j].vmin = layer[j].vmin;
        ds.bricks[first + j].vmax = layer[j].vmax;
      }
      ++w.next_bz;
    }
    // complete macro-cell layers -> cell grid
    const long long M = 1LL << OOC_CELL_SHIFT;
    int cz1 = w.next_cz;
    while (cz1 < L.nc[2] && std::min<long long>(cz1 * M + M + 1, w.Z - 1) < have_end) ++cz1;
    if (cz1 > w.next_cz) {
      CUDA_TRY(launch_cell_minmax_layers(w.a.p, dtype, d3, w.z0, OOC_CELL_SHIFT, L.nc, w.next_cz, cz1,
                                         L.cells->as<float2>(), s));
      w.next_cz = cz1;
    }
    // pairs of planes -> next level
    if (l + 1 < nlev) {
      Stage& nx = st[l + 1];
      long long k1 = w.ds_next;
      while (2 * k1 < w.Z && std::min<long long>(2 * k1 + 2, w.Z) <= have_end) ++k1;
      if (k1 > w.ds_next) {
        const long long in0 = 2 * w.ds_next, in1 = std::min<long long>(2 * k1, w.Z);
        const long long m = k1 - w.ds_next;
        if (nx.n + m > nx.cap) return fail(GBVR_ECUDA, "out-of-core window overflow");
        long long dd[3] = {w.X, w.Y, in1 - in0};
        CUDA_TRY(launch_downsample((const char*)w.a.p + (in0 - w.z0) * w.plane, dtype, dd,
                                   (char*)nx.a.p + nx.n * nx.plane, s));
        nx.n += m;
        w.ds_next = k1;
      }
    }
    // drop planes no consumer needs any more
    long long keep = w.Z;
    if (w.next_bz < L.nb[2]) keep = std::min(keep, std::max<long long>((long long)w.next_bz * I - g, 0));
    if (w.next_cz < L.nc[2]) keep = std::min(keep, std::max<long long>((long long)w.next_cz * M - 1, 0));
    if (l + 1 < nlev && 2 * w.ds_next < w.Z) keep = std::min(keep, 2 * w.ds_next);
    keep = std::min(keep, have_end);
    if (keep > w.z0) {
      const long long drop = keep - w.z0;
      if (w.n - drop > 0)
        CUDA_TRY(cudaMemcpyAsync(w.b.p, (const char*)w.a.p + drop * w.plane, (w.n - drop) * w.plane,
                                 cudaMemcpyDeviceToDevice, s));
      std::swap(w.a.p, w.b.p);
      std::swap(w.a.n, w.b.n);
      w.n -= drop;
      w.z0 = keep;
    }
    return GBVR_OK;
  };
  Stage& w0 = st[0];
  for (long long z = 0; z < w0.Z; z += S) {
    const long long nz = std::min(S, w0.Z - z);
    if (w0.n + nz > w0.cap) return fail(GBVR_ECUDA, "out-of-core window overflow");
    char* dst = (char*)w0.a.p + w0.n * w0.plane;
    CUDA_TRY(launch_synth_blobs_planes(td, dims, dtype, z, nz, dst, s));
    if (dtype != DT_F32)
      CUDA_TRY(launch_hist1d(dst, dtype, nz * w0.X * w0.Y, hist.as<unsigned long long>(), nbins, s));
    w0.n += nz;
    for (int l = 0; l < nlev; ++l) TRY(process(l));
  }
  for (int l = 0; l < nlev; ++l)
    if (st[l].next_bz != ds.levels[l].nb[2] || st[l].next_cz != ds.levels[l].nc[2])
      return fail(GBVR_ECUDA, "out-of-core build did not complete level " + std::to_string(l));
  if (ds.compression && ds.brick_order) {
    // the compressed runs were appended layer by layer: lay them out again
    // in store order, so that bricks adjacent in that order are adjacent in
    // the segments
    std::vector<void*> old_p;
    std::vector<size_t> old_used;
    old_p.swap(ds.seg_p);
    old_used.swap(ds.seg_used);
    const std::vector<int> old_seg = ds.host_cseg;
    const std::vector<unsigned long long> old_off = ds.host_coff;
    ds.comp_store_bytes = 0;
    int rc = GBVR_OK;
    for (int bi : ds.store_order) {
      const BrickInfo& b = ds.bricks[(size_t)bi];
      const size_t nbytes = (size_t)b.sx * b.sy * b.sz * es;
      const unsigned nck = (unsigned)((nbytes + LZ_CHUNK - 1) / LZ_CHUNK);
      size_t run = 0;
      for (unsigned k = 0; k < nck; ++k) run += ds.chunk_size[ds.chunk_first[(size_t)bi] + k] & 0x7fffffffu;
      rc = seg_append((const uint8_t*)old_p[(size_t)old_seg[(size_t)bi]] + old_off[(size_t)bi], run,
                      ds.host_cseg[(size_t)bi], ds.host_coff[(size_t)bi]);
      if (rc != GBVR_OK) break;
    }
    for (void* q : old_p) cudaFreeHost(q);
    if (rc != GBVR_OK) return rc;
  }
  if (ds.compression) {
    if (h_layer.p) cudaFreeHost(h_layer.p);
    h_layer.p = nullptr;
    h_layer.n = 0;
    CUDA_TRY(ds.d_lz_err.alloc(sizeof(int)));
    CUDA_TRY(cudaMemsetAsync(ds.d_lz_err.p, 0, sizeof(int), s));
  }
  CUDA_TRY(ds.d_bricks.alloc(sizeof(BrickInfo) * nb));
  CUDA_TRY(cudaMemcpyAsync(ds.d_bricks.p, ds.bricks.data(), sizeof(BrickInfo) * nb, cudaMemcpyHostToDevice, s));
  ds.gmin = INFINITY;
  ds.gmax = -INFINITY;
  for (int i = 0; i < ds.levels[0].nbricks; ++i) {
    ds.gmin = std::min(ds.gmin, (double)ds.bricks[i].vmin);
    ds.gmax = std::max(ds.gmax, (double)ds.bricks[i].vmax);
  }
  if (dtype != DT_F32) {
    std::vector<uint64_t> full(nbins);
    CUDA_TRY(cudaMemcpyAsync(full.data(), hist.p, sizeof(uint64_t) * nbins, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    long long size = nbins;
    while (size > 1 && full[size - 1] == 0) --size;
    ds.merge = std::max<long long>(1, (size + 4095) / 4096);
    ds.hist1d.assign((size + ds.merge - 1) / ds.merge, 0);
    for (long long i = 0; i < size; ++i) ds.hist1d[i / ds.merge] += full[i];
    ds.bit_width = dtype == DT_U8 ? 8 : 16;
    // 2D histogram (the in-core rule, bit for bit): its three passes (Smax,
    // f64 max |grad| at Smax, binning) each regenerate the finest level in
    // z-slabs with one halo plane on each side for the z differences
    const long long outsize = (long long)ds.hist1d.size();
    const size_t n2 = (size_t)outsize * 256;
    DevBuf d2, dsc, slab;
    CUDA_TRY(d2.alloc(sizeof(uint64_t) * n2));
    CUDA_TRY(dsc.alloc(sizeof(Hist2DScratch)));
    CUDA_TRY(cudaMemsetAsync(d2.p, 0, sizeof(uint64_t) * n2, s));
    CUDA_TRY(cudaMemsetAsync(dsc.p, 0, sizeof(Hist2DScratch), s));
    const long long SZ = std::min<long long>(32, dims[2]);
    CUDA_TRY(slab.alloc(w0.plane * (size_t)(SZ + 2)));
    for (int pass = 1; pass <= 3; ++pass)
      for (long long z = 0; z < dims[2]; z += SZ) {
        const long long ze = std::min(z + SZ, dims[2]);
        const long long zlo = std::max<long long>(z - 1, 0), zhi = std::min(ze + 1, dims[2]);
        CUDA_TRY(launch_synth_blobs_planes(td, dims, dtype, zlo, zhi - zlo, slab.p, s));
        CUDA_TRY(launch_hist2d_slab(slab.p, dtype, dims, z, ze, zlo, ds.gmax, outsize, ds.merge, pass,
                                    d2.as<unsigned long long>(), dsc.as<Hist2DScratch>(), s));
      }
    ds.hist2d.resize(n2);
    Hist2DScratch hs;
    CUDA_TRY(cudaMemcpyAsync(ds.hist2d.data(), d2.p, sizeof(uint64_t) * n2, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(&hs, dsc.p, sizeof(hs), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    double gm;
    memcpy(&gm, &hs.gmax_bits, 8);
    ds.max_grad = (float)gm;
  } else {
    ds.bit_width = 32;
    ds.max_grad = 0.f;
  }
  for (Level& L : ds.levels) TRY(build_supercells(L, s));
  ds.layouts = 1;
  ds.copy_stride = 0;
  ds.ooc = true;
  CUDA_TRY(cudaStreamSynchronize(s));
  ds.loaded = true;
  return GBVR_OK;
}

// Classify one level of a dataset against a transfer function: per brick a
// skip byte (d_skip, indexed by global brick number) and per macro-cell the
// capped distance to a cell that may contribute (d_occ).  tf: RGBA rows of w
// entries, h rows.  Blocks until done (the host prefix table is temporary).
int classify_level(const Dataset& ds, int level, const std::vector<float>& tf, int w, int h, int mode, double lo,
                   double hi, float iso, DevBuf& d_tfprefix, DevBuf& d_skip, DevBuf& d_occ, DevBuf& d_occtmp,
                   cudaStream_t s) {
  const Level& L = ds.levels[level];
  CUDA_TRY(d_skip.alloc(ds.bricks.size()));
  const size_t ncell = (size_t)L.nc[0] * L.nc[1] * L.nc[2];
  CUDA_TRY(d_occ.alloc(ncell));
  // prefix count of TF columns with any non-zero alpha
  std::vector<int> pre(w + 1, 0);
  for (int x = 0; x < w; ++x) {
    int nz = 0;
    for (int y = 0; y < h && !nz; ++y) nz = tf[4 * ((size_t)y * w + x) + 3] != 0.f;
    pre[x + 1] = pre[x] + nz;
  }
  CUDA_TRY(d_tfprefix.alloc(sizeof(int) * pre.size()));
  CUDA_TRY(cudaMemcpyAsync(d_tfprefix.p, pre.data(), sizeof(int) * pre.size(), cudaMemcpyHostToDevice, s));
  const float idx_scale = (float)((w - 1) / (hi - lo));
  CUDA_TRY(launch_classify_bricks(ds.d_bricks.as<BrickInfo>() + L.brick_base, L.nbricks, d_tfprefix.as<int>(), w, mode,
                                  (float)lo, idx_scale, iso, d_skip.as<unsigned char>() + L.brick_base, s));
  CUDA_TRY(launch_classify_cells(L.cells->as<float2>(), (long long)ncell, d_tfprefix.as<int>(), w, mode, (float)lo,
                                 idx_scale, iso, d_occ.as<unsigned char>(), s));
  CUDA_TRY(d_occtmp.alloc(ncell));
  CUDA_TRY(launch_cell_distance(d_occ.as<unsigned char>(), d_occtmp.as<unsigned char>(), L.nc, CELL_DIST_CAP, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return GBVR_OK;
}


// Generate a seeded blob volume into a new device buffer (tables built on
// the host, combined on the device in a fixed float32 order).
int synth_to_device(const gbvr_synth_params* p, DevBuf& lv, cudaStream_t s) {
  TRY(check_synth_params(p, true, nullptr, nullptr));
  BlobTablesHost t;
  make_blob_tables(*p, t);
  DevBuf amp, ex, ey, ez, bx, by, bz;
  auto up = [&](DevBuf& d, const std::vector<float>& v) -> cudaError_t {
    cudaError_t e = d.alloc(sizeof(float) * std::max<size_t>(v.size(), 1));
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(d.p, v.data(), sizeof(float) * v.size(), cudaMemcpyHostToDevice, s);
  };
  CUDA_TRY(up(amp, t.amp));
  CUDA_TRY(up(ex, t.ex));
  CUDA_TRY(up(ey, t.ey));
  CUDA_TRY(up(ez, t.ez));
  CUDA_TRY(up(bx, t.bgx));
  CUDA_TRY(up(by, t.bgy));
  CUDA_TRY(up(bz, t.bgz));
  long long d[3] = {p->dims[0], p->dims[1], p->dims[2]};
  CUDA_TRY(lv.alloc((size_t)d[0] * d[1] * d[2] * dtype_size(p->dtype)));
  const bool bg = p->bg_freq > 0;
  BlobTablesDev td{p->nblobs, amp.as<float>(), ex.as<float>(), ey.as<float>(), ez.as<float>(),
                   bg ? bx.as<float>() : nullptr, bg ? by.as<float>() : nullptr, bg ? bz.as<float>() : nullptr,
                   p->bg_level, p->bg_amp, p->scale, p->noise_amp, p->noise_kind, p->vmax, p->seed};
  CUDA_TRY(launch_synth_blobs(td, d, p->dtype, lv.p, s));
  // the tables are freed on return: wait for the kernel that reads them
  CUDA_TRY(cudaStreamSynchronize(s));
  return GBVR_OK;
}

// Everything a frame needs besides its outputs.
struct FrameParams {
  const float* view;
  const float* proj;
  int width, height;
  float spv;
  int level;
  int mode, interp, sampler;
  float ert;
  float iso;
  float iso_rgb[3];
  int lighting;
  float amb[3], diff[3], spec[3], shininess, light_dir[3], bg[3];
  float bg_top[3];  // with bg: a vertical gradient when they differ
  int tile_w, empty_skip;
  const float4* tf;
  int tf_w, tf_h;
  double lo, hi;
  float grad_max;
  const unsigned char* skip;  // per brick of the dataset (all levels)
  const unsigned char* occ;   // per macro-cell of `level`
  int clip_on;
  float clip[4];
};

void fill_frame(FrameDesc& f, const Dataset& ds, const FrameParams& p) {
  memset(&f, 0, sizeof(f));
  const Level& L = ds.levels[p.level];
  f.pool = ds.pool.p;
  f.bricks = ds.d_bricks.as<BrickInfo>() + L.brick_base;
  f.skip = p.skip + L.brick_base;
  f.dtype = ds.dtype;
  f.sampler = p.sampler;
  double ext[3], mx = 0;
  for (int a = 0; a < 3; ++a) {
    ext[a] = (double)ds.dims[a] * ds.aspect[a];
    mx = std::max(mx, ext[a]);
  }
  long long maxd = 0;
  for (int a = 0; a < 3; ++a) {
    ext[a] /= mx;
    f.dims[a] = (int)L.dims[a];
    f.nb[a] = L.nb[a];
    f.vox_scale[a] = (float)((double)L.dims[a] / ext[a]);
    f.half_extent[a] = (float)(0.5 * ext[a]);
    maxd = std::max(maxd, L.dims[a]);
  }
  f.interior = L.interior;
  f.inv_interior = 1.f / (float)L.interior;
  f.tf = p.tf;
  f.tf_w = p.tf_w;
  f.tf_h = p.tf_h;
  f.mode = p.mode;
  f.interp = p.interp;
  f.value_lo = (float)p.lo;
  f.idx_scale = (float)((f.tf_w - 1) / (p.hi - p.lo));
  float gm = p.grad_max > 0 ? p.grad_max : ds.max_grad;
  if (!(gm > 0)) gm = 1.f;
  f.grad_scale = (float)((f.tf_h - 1) / ((double)gm * (p.hi - p.lo)));
  f.dt = (float)(1.0 / ((double)p.spv * (double)maxd));
  f.opacity_exp = (float)(1.0 / (double)p.spv);
  f.ert = p.ert;
  f.iso = p.iso;
  for (int k = 0; k < 3; ++k) {
    f.iso_rgb[k] = p.iso_rgb[k];
    f.amb[k] = p.amb[k];
    f.diff[k] = p.diff[k];
    f.spec[k] = p.spec[k];
    f.bg[k] = p.bg[k];
    f.bg_top[k] = p.bg_top[k];
    if (p.bg_top[k] != p.bg[k]) f.bg_grad = 1;
  }
  f.lighting = p.lighting;
  f.shininess = p.shininess;
  double V[16], P[16], M[16], Mi[16], Vi[16];
  for (int i = 0; i < 16; ++i) { V[i] = p.view[i]; P[i] = p.proj[i]; }
  mat_mul(P, V, M);
  mat_inv(M, Mi);
  mat_inv(V, Vi);
  for (int i = 0; i < 16; ++i) f.inv_vp[i] = (float)Mi[i];
  double ld[3];
  for (int rr = 0; rr < 3; ++rr)
    ld[rr] = Vi[4 * rr] * p.light_dir[0] + Vi[4 * rr + 1] * p.light_dir[1] + Vi[4 * rr + 2] * p.light_dir[2];
  double ll = std::sqrt(ld[0] * ld[0] + ld[1] * ld[1] + ld[2] * ld[2]);
  for (int k = 0; k < 3; ++k) f.light_to[k] = ll > 0 ? (float)(-ld[k] / ll) : 0.f;
  f.width = p.width;
  f.height = p.height;
  f.tile_w = p.tile_w;
  f.empty_skip = p.empty_skip;
  f.occ = p.occ;
  for (int a = 0; a < 3; ++a) f.nc[a] = L.nc[a];
  f.cell_shift = L.cell_shift;
  f.cells = L.cells ? L.cells->as<float2>() : nullptr;
  f.smax = L.smax ? L.smax->as<float>() : nullptr;
  for (int a = 0; a < 3; ++a) f.nsc[a] = L.nsc[a];
  f.level_max = -INFINITY;
  for (int i = 0; i < L.nbricks; ++i) f.level_max = std::max(f.level_max, ds.bricks[L.brick_base + i].vmax);
  f.clip_on = p.clip_on;
  for (int k = 0; k < 4; ++k) f.clip[k] = p.clip[k];
  f.tiles_x = (p.width + p.tile_w - 1) / p.tile_w;
  f.tiles_y = (p.height + 32 / p.tile_w - 1) / (32 / p.tile_w);
  f.tx0 = f.ty0 = 0;
  f.ntx = f.tiles_x;
  f.nty = f.tiles_y;
  // layout copy: the axis whose voxel-space extent along screen x is largest
  // (row 0 of the view matrix is the camera's right vector in world space)
  f.perm = 0;
  if (ds.layouts == 6) {
    // both blocked copies: isosurfaces sample the overlapped blocks (a cell's
    // voxels at fixed offsets), the other modes the compact 4^3 blocks
    f.perm = p.mode == GBVR_RM_ISOSURFACE ? 4 : 3;
  } else if (ds.layouts >= 4) {
    f.perm = ds.layouts - 1;  // blocked copy, independent of the view direction
  } else if (ds.layouts == 3) {
    double best = -1;
    for (int a = 0; a < 3; ++a) {
      double w = std::fabs((double)p.view[a] * f.vox_scale[a]);
      if (w > best) { best = w; f.perm = a; }
    }
  }
  f.copy_off = (unsigned long long)(f.perm == 4 && ds.layouts == 6 ? 2 : f.perm >= 3 ? 1 : f.perm) * ds.copy_stride;
}

}  // namespace

namespace gbvr {
int set_error(int code, const std::string& msg) { return fail(code, msg); }

int check_synth_params(const gbvr_synth_params* p, bool whole_volume, long long* table_floats, size_t* volume_bytes) {
  if (!p) return fail(GBVR_EINVAL, "null synthetic parameters");
  if (p->dims[0] <= 0 || p->dims[1] <= 0 || p->dims[2] <= 0 || p->dtype < 0 || p->dtype > 2)
    return fail(GBVR_EINVAL, "bad synthetic parameters (dims must be positive, dtype 0, 1 or 2)");
  if (p->nblobs < 0 || p->nblobs > kMaxSynthBlobs)
    return fail(GBVR_EINVAL, "nblobs must lie in [0, " + std::to_string(kMaxSynthBlobs) +
                                 "] (the generator keeps a row of blob weights in 48 KiB of shared memory)");
  const unsigned long long X = (unsigned long long)p->dims[0], Y = (unsigned long long)p->dims[1],
                           Z = (unsigned long long)p->dims[2];
  if (Y > 0x7fffffffull) return fail(GBVR_EINVAL, "dims[1] must be below 2^31 (one block per row)");
  if (whole_volume && Z > 65535) return fail(GBVR_EINVAL, "dims[2] must be at most 65535 (one block row per plane)");
  unsigned long long vox = 0, bytes = 0, axes = 0, tab = 0;
  if (__builtin_mul_overflow(X, Y, &vox) || __builtin_mul_overflow(vox, Z, &vox) ||
      __builtin_mul_overflow(vox, (unsigned long long)dtype_size(p->dtype), &bytes) || bytes > (unsigned long long)SIZE_MAX)
    return fail(GBVR_EINVAL, "the volume's byte count overflows");
  // each axis is below 2^63 and their product fits 64 bits, so at most one
  // axis exceeds 2^32 and 1 + X + Y + Z cannot wrap
  axes = 1 + X + Y + Z;
  if (__builtin_mul_overflow((unsigned long long)p->nblobs, axes, &tab) ||
      __builtin_add_overflow(tab, p->bg_freq > 0 ? X + Y + Z : 0ull, &tab) || tab > (unsigned long long)LLONG_MAX)
    return fail(GBVR_EINVAL, "the generator tables' size overflows");
  if (table_floats) *table_floats = (long long)tab;
  if (volume_bytes) *volume_bytes = (size_t)bytes;
  return GBVR_OK;
}

void fill_blob_tables(const gbvr_synth_params& p, float* t) {
  const uint32_t k0 = p.seed, k1 = 0x70617261u;
  const long long nb = p.nblobs;
  const long long dims[3] = {p.dims[0], p.dims[1], p.dims[2]};
  float* amp = t;
  float* tab[3] = {t + nb, t + nb + nb * dims[0], t + nb + nb * (dims[0] + dims[1])};
  for (long long k = 0; k < nb; ++k) {
    uint32_t c0[4] = {(uint32_t)k, 0u, 0x626c6f62u, 0u}, c1[4] = {(uint32_t)k, 1u, 0x626c6f62u, 0u};
    philox_host(c0, k0, k1);
    philox_host(c1, k0, k1);
    double cen[3];
    for (int a = 0; a < 3; ++a) cen[a] = (double)(c0[a] >> 8) / 16777216.0 * (double)dims[a];
    double sig = p.sigma_lo + (double)(c1[0] >> 8) / 16777216.0 * ((double)p.sigma_hi - p.sigma_lo);
    double am = p.amp_lo + (double)(c1[1] >> 8) / 16777216.0 * ((double)p.amp_hi - p.amp_lo);
    amp[k] = (float)am;
    for (int a = 0; a < 3; ++a)
      for (long long i = 0; i < dims[a]; ++i) {
        double dd = (double)i - cen[a];
        tab[a][k * dims[a] + i] = (float)std::exp(-(dd * dd) / (2.0 * sig * sig));
      }
  }
  if (p.bg_freq > 0) {
    uint32_t c[4] = {0xffffffffu, 2u, 0x626c6f62u, 0u};
    philox_host(c, k0, k1);
    float* bg = t + nb * (1 + dims[0] + dims[1] + dims[2]);
    for (int a = 0; a < 3; ++a) {
      double ph = (double)(c[a] >> 8) / 16777216.0;
      for (long long i = 0; i < dims[a]; ++i)
        bg[i] = (float)std::cos(2.0 * M_PI * ((double)p.bg_freq * ((double)i + 0.5) / (double)dims[a] + ph));
      bg += dims[a];
    }
  }
}
}  // namespace gbvr

// ---------------------------------------------------------------------------
// Renderer
// ---------------------------------------------------------------------------
// A 2D slice paint (gbvr_paint_slice) out of core: the bricks it needs
// instead of the views' frusta.  index: slice of the finest level.
struct SliceSel {
  int axis;
  long long index;
  bool mip;
};

struct gbvr_renderer {
  Dataset ds;
  uint32_t flags = 0;
  int width = 640, height = 480;  // BatchRenderer.lua:31-33 default context size
  int mode = GBVR_RM_1DTRANS, interp = GBVR_LINEAR, sampler = GBVR_SAMPLER_SW;
  int clip_on = 0;
  float clip[4] = {0.f, 0.f, 1.f, 0.f};
  // bounding boxes: the dataset box and the brick boxes of the rendered level
  const SliceSel* slice_sel = nullptr;  // during an out-of-core slice paint
  int bbox_global = 0, bbox_local = 0;
  float bbox_rgb[2][3] = {{1.f, 1.f, 1.f}, {0.6f, 0.6f, 0.6f}};
  DevBuf d_line_keys, d_line_segs, d_line_views, d_line_list, d_line_count;
  DevBuf d_tf_col;  // 2D TF: per value column, 1 if any gradient row has opacity
  // ClearView (isosurface mode): focus iso value and colour, lens size
  // (radius = size * min(width, height) / 2 pixels), context and border
  // scales, focus point in pixels (row 0 = top)
  int cv_on = 0;
  float cv_iso = 0.f, cv_rgb[3] = {1.f, 1.f, 1.f}, cv_size = 0.5f, cv_context = 1.f, cv_border = 1.f;
  float cv_fx = -1.f, cv_fy = -1.f;
  std::vector<float> tf1d;
  std::vector<float> tf2d;
  int tf2d_w = 0, tf2d_h = 0;
  float tf2d_grad_max = 0.f;
  bool range_set = false;
  double vlo = 0, vhi = 1;
  float iso = 0.f;
  bool iso_set = false;
  float iso_rgb[3] = {1, 1, 1};
  int lighting = 1;
  // MainWindow::UpdateColorWidget defaults (ImageVis3D.cpp:898-901): colour
  // times the alpha intensity
  float amb[3] = {0.1f, 0.1f, 0.1f}, diff[3] = {1, 1, 1}, spec[3] = {1, 1, 1};
  float light_dir[3] = {0, 0, -1};
  float shininess = 8.f;
  float spv = 1.f;
  int lod_min = 0, lod_max = 1 << 20;
  bool view_set = false;
  float view[16], proj[16];
  float bg_top[3] = {0, 0, 0}, bg_bot[3] = {0, 0, 0};
  float ert = 0.99f;
  int tile_w = TILE_W, ctas_per_sm = 0;
  int empty_skip = 2;
  int stats_level = 1;  // 0 samples, 1 + touched bricks, 2 + touched macro-cells
  // device state
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
  DevBuf d_tf, d_skip, d_fb8, d_fb32, d_frames, d_prefix, d_counter, d_samples, d_touched, d_tfprefix, d_occ;
  DevBuf d_tf_slice;  // the 1D TF for 2D slice views, whatever the render mode
  DevBuf d_cellbits, d_cellcount, d_occtmp, d_ooc_skip;
  // out-of-core paging state and the last paint's statistics
  cudaStream_t copy_stream = nullptr;
  // out-of-core paging, double-buffered for the fly-through pipeline: copy
  // start/end events, render-done events and page-locked staging for the page
  // table and skip table of each of two frames in flight
  cudaEvent_t ev_c0[2] = {nullptr, nullptr}, ev_c1[2] = {nullptr, nullptr}, ev_done[2] = {nullptr, nullptr};
  PinnedBuf h_pt[2], h_skip[2];
  std::vector<std::shared_ptr<DevBuf>> occ_lv;  // out of core: classified macro-cells per level
  std::vector<char> occ_valid;
  uint64_t last_misses = 0, last_paged = 0;
  uint64_t last_paged_comp = 0;  // compressed store: bytes copied host to device by the last paint
  uint64_t last_host_copies = 0; // out of core: host-to-device brick copies of the last paint
  float last_page_ms = 0.f;
  long long cell_words = 0;
  PinnedBuf h_frames, h_prefix;
  // Asynchronous batches use two sets of batch buffers ("slots"): the set of
  // the slot in use sits in the members above, the other one here, and
  // selecting a slot swaps them.  Per slot: its render's end and its
  // read-back's end.
  struct SlotBufs {
    DevBuf fb8, fb32, frames, prefix, counter, samples, touched, cellbits;
    PinnedBuf h_frames, h_prefix;
    int fb_views = 0, fb_w = 0, fb_h = 0;
  } other;
  int cur_slot = 0;
  cudaStream_t read_stream = nullptr;
  // a second copy stream for the other half of an asynchronous read-back
  // (two device-to-host copies in flight use two copy engines), joined back
  // into read_stream through read2_done
  cudaStream_t read_stream2 = nullptr;
  cudaEvent_t read2_done = nullptr;
  cudaEvent_t slot_rendered[2] = {nullptr, nullptr}, slot_read[2] = {nullptr, nullptr};
  bool slot_render_pending[2] = {false, false}, slot_read_pending[2] = {false, false};
  void select_slot(int slot) {
    if (slot == cur_slot) return;
    d_fb8.swap(other.fb8);
    d_fb32.swap(other.fb32);
    d_frames.swap(other.frames);
    d_prefix.swap(other.prefix);
    d_counter.swap(other.counter);
    d_samples.swap(other.samples);
    d_touched.swap(other.touched);
    d_cellbits.swap(other.cellbits);
    h_frames.swap(other.h_frames);
    h_prefix.swap(other.h_prefix);
    std::swap(fb_views, other.fb_views);
    std::swap(fb_w, other.fb_w);
    std::swap(fb_h, other.fb_h);
    cur_slot = slot;
  }
  bool tf_dirty = true, skip_dirty = true;
  int skip_level = -1;
  int fb_views = 0, fb_w = 0, fb_h = 0;
  int last_views = 0, last_level = 0;
  float last_ms = 0.f, last_kernel_ms = 0.f;
  uint64_t last_h2d = 0;
  int max_ctas_per_sm[4] = {0, 0, 0, 0}, max_ctas_per_sm_u[4] = {0, 0, 0, 0}, sm_count = 0;
  int max_ctas_per_sm_sps2 = 0;  // the batch kernel's two-samples-per-step variant
  int samples_per_step = 1;
  // graph cache for the batch launch
  struct GraphKey {
    int n, w, h, level, dtype, mode, sampler, grid, sps;
    void* fb8;
    void* fb32;
    bool operator<(const GraphKey& o) const {
      return std::tie(n, w, h, level, dtype, mode, sampler, grid, sps, fb8, fb32) <
             std::tie(o.n, o.w, o.h, o.level, o.dtype, o.mode, o.sampler, o.grid, o.sps, o.fb8, o.fb32);
    }
  };
  struct CachedGraph {
    cudaGraphExec_t exec;
    bool uniform;
    FrameDesc shared;  // the batch-uniform kernel parameter baked into the graph
  };
  std::map<GraphKey, CachedGraph> graphs;

  void drop_graphs() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.exec);
    graphs.clear();
  }
  ~gbvr_renderer() {
    drop_graphs();
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (evk0) cudaEventDestroy(evk0);
    if (evk1) cudaEventDestroy(evk1);
    for (int k = 0; k < 2; ++k) {
      if (slot_rendered[k]) cudaEventDestroy(slot_rendered[k]);
      if (slot_read[k]) cudaEventDestroy(slot_read[k]);
    }
    if (read_stream) cudaStreamDestroy(read_stream);
    if (read_stream2) cudaStreamDestroy(read_stream2);
    if (read2_done) cudaEventDestroy(read2_done);
    for (int k = 0; k < 2; ++k) {
      if (ev_c0[k]) cudaEventDestroy(ev_c0[k]);
      if (ev_c1[k]) cudaEventDestroy(ev_c1[k]);
      if (ev_done[k]) cudaEventDestroy(ev_done[k]);
    }
    if (copy_stream) cudaStreamDestroy(copy_stream);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int check_r(gbvr_renderer* r) {
  if (!r) return fail(GBVR_EINVAL, "null renderer");
  return GBVR_OK;
}
int check_loaded(gbvr_renderer* r) {
  TRY(check_r(r));
  if (!r->ds.loaded) return fail(GBVR_ESTATE, "no dataset loaded");
  return GBVR_OK;
}

int render_level(gbvr_renderer* r) {
  int n = (int)r->ds.levels.size();
  int l = std::min(std::max(r->lod_min, 0), n - 1);
  return l;
}

void default_range(gbvr_renderer* r, double& lo, double& hi) {
  if (r->range_set) { lo = r->vlo; hi = r->vhi; return; }
  const Dataset& ds = r->ds;
  if (ds.dtype == DT_F32) {
    lo = ds.gmin;
    hi = ds.gmax > ds.gmin ? ds.gmax : ds.gmin + 1;
  } else {
    lo = 0;
    hi = (double)((long long)ds.hist1d.size() * ds.merge - 1);
    if (hi <= 0) hi = 1;
  }
}

// Default TF: a linear ramp, as a freshly opened dataset gets in the reference.
// The device form of a 1D TF of w RGBA entries: per entry the entry and its
// FP32 difference to the next one (zero for the last), read by the kernels'
// tf1d.
std::vector<float> tf1d_pairs(const float* rgba, int w) {
  std::vector<float> out(8 * (size_t)w);
  for (int i = 0; i < w; ++i) {
    const int j = std::min(i + 1, w - 1);
    for (int c = 0; c < 4; ++c) {
      out[8 * (size_t)i + c] = rgba[4 * (size_t)i + c];
      out[8 * (size_t)i + 4 + c] = rgba[4 * (size_t)j + c] - rgba[4 * (size_t)i + c];
    }
  }
  return out;
}

void ensure_tf(gbvr_renderer* r) {
  if (r->tf1d.empty()) {
    int n = r->ds.hist1d.empty() ? 256 : (int)std::min<size_t>(r->ds.hist1d.size(), 4096);
    r->tf1d.resize(4 * n);
    for (int i = 0; i < n; ++i) {
      float v = n > 1 ? (float)i / (n - 1) : 1.f;
      r->tf1d[4 * i] = r->tf1d[4 * i + 1] = r->tf1d[4 * i + 2] = v;
      r->tf1d[4 * i + 3] = v;
    }
    r->tf_dirty = true;
  }
}

// The iso value that empty-space classification uses: with ClearView the
// march also looks for the focus surface, so the lower of the two.
float skip_iso(const gbvr_renderer* r) {
  return r->cv_on && r->mode == GBVR_RM_ISOSURFACE ? std::min(r->iso, r->cv_iso) : r->iso;
}

int upload_tf(gbvr_renderer* r, int level) {
  ensure_tf(r);
  const bool two = r->mode == GBVR_RM_2DTRANS;
  if (two && r->tf2d.empty()) return fail(GBVR_ESTATE, "2D transfer function not set");
  const std::vector<float>& tf = two ? r->tf2d : r->tf1d;
  if (r->tf_dirty) {
    // pageable sources: each copy returns once it is staged
    const std::vector<float> dev = two ? tf : tf1d_pairs(tf.data(), (int)(tf.size() / 4));
    CUDA_TRY(r->d_tf.alloc(sizeof(float) * dev.size()));
    CUDA_TRY(cudaMemcpyAsync(r->d_tf.p, dev.data(), sizeof(float) * dev.size(), cudaMemcpyHostToDevice, r->stream));
    if (two) {
      const int w = r->tf2d_w, h = r->tf2d_h;
      std::vector<unsigned char> live((size_t)w, 0);
      for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) live[x] |= tf[4 * ((size_t)y * w + x) + 3] != 0.f;
      CUDA_TRY(r->d_tf_col.alloc(live.size()));
      // pageable source: the copy returns once it is staged
      CUDA_TRY(cudaMemcpyAsync(r->d_tf_col.p, live.data(), live.size(), cudaMemcpyHostToDevice, r->stream));
    }
    r->tf_dirty = false;
    r->skip_dirty = true;
  }
  if (r->ds.ooc) {
    // out of core: frames of a fly-through change level, so each level keeps
    // its own classified macro-cells until the TF or mode changes
    const size_t nl = r->ds.levels.size();
    if (r->occ_lv.size() != nl) {
      r->occ_lv.clear();
      for (size_t l = 0; l < nl; ++l) r->occ_lv.push_back(std::make_shared<DevBuf>());
      r->occ_valid.assign(nl, 0);
    }
    if (r->skip_dirty) {
      r->occ_valid.assign(nl, 0);
      r->skip_dirty = false;
    }
    if (!r->occ_valid[level]) {
      double lo, hi;
      default_range(r, lo, hi);
      int w = two ? r->tf2d_w : (int)(r->tf1d.size() / 4), h = two ? r->tf2d_h : 1;
      TRY(classify_level(r->ds, level, tf, w, h, r->mode, lo, hi, skip_iso(r), r->d_tfprefix, r->d_skip, *r->occ_lv[level],
                         r->d_occtmp, r->stream));
      r->occ_valid[level] = 1;
    }
    return GBVR_OK;
  }
  if (r->skip_dirty || r->skip_level != level) {
    double lo, hi;
    default_range(r, lo, hi);
    int w = two ? r->tf2d_w : (int)(r->tf1d.size() / 4), h = two ? r->tf2d_h : 1;
    TRY(classify_level(r->ds, level, tf, w, h, r->mode, lo, hi, skip_iso(r), r->d_tfprefix, r->d_skip, r->d_occ,
                       r->d_occtmp, r->stream));
    r->skip_dirty = false;
    r->skip_level = level;
  }
  return GBVR_OK;
}

void default_camera(gbvr_renderer* r, float view[16], float proj[16]);

FrameDesc make_frame(gbvr_renderer* r, const float* view, const float* proj, int level, int vidx) {
  FrameParams p;
  memset(&p, 0, sizeof(p));
  p.view = view;
  p.proj = proj;
  p.width = r->width;
  p.height = r->height;
  p.spv = r->spv;
  p.level = level;
  p.mode = r->mode;
  p.interp = r->interp;
  p.sampler = r->sampler;
  p.ert = r->ert;
  p.iso = r->iso;
  p.lighting = r->lighting;
  p.shininess = r->shininess;
  for (int k = 0; k < 3; ++k) {
    p.iso_rgb[k] = r->iso_rgb[k];
    p.amb[k] = r->amb[k];
    p.diff[k] = r->diff[k];
    p.spec[k] = r->spec[k];
    p.light_dir[k] = r->light_dir[k];
    p.bg[k] = r->bg_bot[k];
    p.bg_top[k] = r->bg_top[k];
  }
  p.tile_w = r->tile_w;
  p.empty_skip = r->empty_skip;
  const bool two = r->mode == GBVR_RM_2DTRANS;
  p.tf = r->d_tf.as<float4>();
  p.tf_w = two ? r->tf2d_w : (int)(r->tf1d.size() / 4);
  p.tf_h = two ? r->tf2d_h : 1;
  default_range(r, p.lo, p.hi);
  p.grad_max = r->tf2d_grad_max;
  p.skip = r->d_skip.as<unsigned char>();
  p.occ = r->ds.ooc && level < (int)r->occ_lv.size() ? r->occ_lv[level]->as<unsigned char>() : r->d_occ.as<unsigned char>();
  p.clip_on = r->clip_on;
  for (int k = 0; k < 4; ++k) p.clip[k] = r->clip[k];
  if (r->ds.ooc) {
    // residency lives in the skip table: brick skipping is always on
    p.skip = r->d_ooc_skip.as<unsigned char>();
    p.empty_skip = std::max(p.empty_skip, 1);
  }
  FrameDesc f;
  fill_frame(f, r->ds, p);
  const Level& L = r->ds.levels[level];
  const size_t npix = (size_t)r->width * r->height;
  f.out_rgba8 = r->d_fb8.as<uchar4>() + (size_t)vidx * npix;
  f.out_f32 = r->d_fb32.p ? r->d_fb32.as<float4>() + (size_t)vidx * npix : nullptr;
  f.samples = r->d_samples.as<unsigned long long>() + vidx;
  f.touched = r->stats_level >= 1 ? r->d_touched.as<unsigned char>() + (size_t)vidx * L.nbricks : nullptr;
  f.cell_touched = (r->stats_level >= 2 && r->empty_skip >= 2)
                       ? r->d_cellbits.as<unsigned>() + (size_t)vidx * r->cell_words : nullptr;
  if (r->bbox_global || r->bbox_local) f.lines = r->d_line_keys.as<unsigned>() + (size_t)vidx * npix;
  memcpy(f.line_rgb, r->bbox_rgb, sizeof(f.line_rgb));
  f.tf_col_live = r->mode == GBVR_RM_2DTRANS ? r->d_tf_col.as<unsigned char>() : nullptr;
  f.cv_iso = r->cv_iso;
  memcpy(f.cv_rgb, r->cv_rgb, sizeof(f.cv_rgb));
  f.cv_context = r->cv_context;
  f.cv_border = r->cv_border;
  return f;
}

// ClearView lens pass of one frame (after its render and line pass).
int render_cv(gbvr_renderer* r, const FrameDesc& f) {
  if (!r->cv_on || r->mode != GBVR_RM_ISOSURFACE) return GBVR_OK;
  CvLens L;
  L.fx = r->cv_fx;
  L.fy = r->cv_fy;
  L.radius = r->cv_size * 0.5f * (float)std::min(r->width, r->height);
  if (!(L.radius > 0.f)) return GBVR_OK;
  L.x0 = (int)std::max(0.f, std::floor(L.fx - L.radius));
  L.y0 = (int)std::max(0.f, std::floor(L.fy - L.radius));
  L.x1 = (int)std::min((float)r->width, std::ceil(L.fx + L.radius) + 1.f);
  L.y1 = (int)std::min((float)r->height, std::ceil(L.fy + L.radius) + 1.f);
  CUDA_TRY(launch_render_cv(f, L, r->stream));
  return GBVR_OK;
}

// World-space segments of the bounding boxes at `level`: the 12 edges of the
// dataset box, and the lines of the level's brick grid (interior bounds at
// multiples of the interior size, clamped to the level) that are not edges
// of the drawn dataset box.  A brick bound b of an axis with d voxels and
// normalised extent e lies at (b / d) e - e/2.
void bbox_segments(const gbvr_renderer* r, int level, std::vector<LineSeg>& segs) {
  segs.clear();
  const Dataset& ds = r->ds;
  const Level& L = ds.levels[level];
  double ext[3], h[3], mx = 0;
  for (int a = 0; a < 3; ++a) {
    ext[a] = (double)ds.dims[a] * ds.aspect[a];
    mx = std::max(mx, ext[a]);
  }
  for (int a = 0; a < 3; ++a) {
    ext[a] /= mx;
    h[a] = 0.5 * ext[a];
  }
  auto add = [&](int a, double u, double v, int color) {
    const int b = (a + 1) % 3, c = (a + 2) % 3;
    LineSeg sg;
    memset(&sg, 0, sizeof(sg));
    sg.a[a] = -h[a];
    sg.b[a] = h[a];
    sg.a[b] = sg.b[b] = u;
    sg.a[c] = sg.b[c] = v;
    sg.color = color;
    segs.push_back(sg);
  };
  for (int a = 0; a < 3; ++a) {
    const int b = (a + 1) % 3, c = (a + 2) % 3;
    if (r->bbox_global)
      for (int k = 0; k < 4; ++k) add(a, (k & 1) ? h[b] : -h[b], (k & 2) ? h[c] : -h[c], 0);
    if (!r->bbox_local) continue;
    auto bound = [&](int ax, int j) {
      const long long bj = std::min<long long>((long long)j * L.interior, L.dims[ax]);
      return (double)bj / (double)L.dims[ax] * ext[ax] - h[ax];
    };
    for (int j = 0; j <= L.nb[b]; ++j)
      for (int k = 0; k <= L.nb[c]; ++k) {
        const bool edge = (j == 0 || j == L.nb[b]) && (k == 0 || k == L.nb[c]);
        if (edge && r->bbox_global) continue;
        add(a, bound(b, j), bound(c, k), 1);
      }
  }
}

int lines_on(const gbvr_renderer* r) { return r->bbox_global || r->bbox_local; }

// Key buffers, the list of covered pixels and its count for n frames.
int alloc_lines(gbvr_renderer* r, size_t npix, int n) {
  if (!lines_on(r)) return GBVR_OK;
  CUDA_TRY(r->d_line_keys.alloc(sizeof(unsigned) * npix * n));
  CUDA_TRY(r->d_line_list.alloc(sizeof(unsigned long long) * npix * n));
  CUDA_TRY(r->d_line_count.alloc(sizeof(unsigned)));
  CUDA_TRY(r->d_frames.alloc(sizeof(FrameDesc) * n));  // plain paints copy their descriptors here
  return GBVR_OK;
}

// Line stops and the covered-pixel list for the n frames in d_frames.
int line_stops(gbvr_renderer* r, int n) {
  if (!lines_on(r)) return GBVR_OK;
  CUDA_TRY(cudaMemsetAsync(r->d_line_count.p, 0, sizeof(unsigned), r->stream));
  CUDA_TRY(launch_line_stops(r->d_frames.as<FrameDesc>(), 0, n, r->height, r->d_line_list.as<unsigned long long>(),
                             r->d_line_count.as<unsigned>(), r->stream));
  return GBVR_OK;
}

// The same for one frame rendered by a plain launch (its descriptor is a
// kernel parameter: it is copied to d_frames[v] for the line passes); `reset`
// starts a new list.
int line_stops_one(gbvr_renderer* r, const FrameDesc& f, int v, bool reset) {
  if (!lines_on(r)) return GBVR_OK;
  CUDA_TRY(cudaMemcpyAsync(r->d_frames.as<FrameDesc>() + v, &f, sizeof(FrameDesc), cudaMemcpyHostToDevice, r->stream));
  if (reset) CUDA_TRY(cudaMemsetAsync(r->d_line_count.p, 0, sizeof(unsigned), r->stream));
  CUDA_TRY(launch_line_stops(r->d_frames.as<FrameDesc>(), v, 1, r->height, r->d_line_list.as<unsigned long long>(),
                             r->d_line_count.as<unsigned>(), r->stream));
  return GBVR_OK;
}

// Re-render the listed pixels (after the frames' render).
int render_lines(gbvr_renderer* r) {
  if (!lines_on(r)) return GBVR_OK;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  CUDA_TRY(launch_render_lines(r->ds.dtype, r->mode, r->sampler, r->d_frames.as<FrameDesc>(),
                               r->d_line_list.as<unsigned long long>(), r->d_line_count.as<unsigned>(),
                               std::max(sms, 1) * 8, r->stream));
  return GBVR_OK;
}

// Rasterise the bounding-box lines of views [0, n) into the key buffers of
// frames vidx0 .. vidx0 + n - 1 (on the render stream, before their render).
int draw_lines(gbvr_renderer* r, const gbvr_view* views, int vidx0, int n, int level) {
  if (!r->bbox_global && !r->bbox_local) return GBVR_OK;
  std::vector<LineSeg> segs;
  bbox_segments(r, level, segs);
  const size_t npix = (size_t)r->width * r->height;
  CUDA_TRY(cudaMemsetAsync(r->d_line_keys.as<unsigned>() + (size_t)vidx0 * npix, 0xff, sizeof(unsigned) * npix * n,
                           r->stream));
  if (segs.empty()) return GBVR_OK;
  std::vector<LineView> lv((size_t)n);
  for (int v = 0; v < n; ++v) {
    memcpy(lv[v].view, views[v].view, sizeof(lv[v].view));
    memcpy(lv[v].proj, views[v].proj, sizeof(lv[v].proj));
    lv[v].width = r->width;
    lv[v].height = r->height;
    lv[v].keys = r->d_line_keys.as<unsigned>() + (size_t)(vidx0 + v) * npix;
  }
  CUDA_TRY(r->d_line_segs.alloc(sizeof(LineSeg) * segs.size()));
  CUDA_TRY(r->d_line_views.alloc(sizeof(LineView) * lv.size()));
  // pageable sources: each copy returns once its source is staged
  CUDA_TRY(cudaMemcpyAsync(r->d_line_segs.p, segs.data(), sizeof(LineSeg) * segs.size(), cudaMemcpyHostToDevice,
                           r->stream));
  CUDA_TRY(cudaMemcpyAsync(r->d_line_views.p, lv.data(), sizeof(LineView) * lv.size(), cudaMemcpyHostToDevice,
                           r->stream));
  CUDA_TRY(launch_raster_lines(r->d_line_segs.as<LineSeg>(), (int)segs.size(), r->d_line_views.as<LineView>(), n,
                               r->stream));
  return GBVR_OK;
}

// The view's ray tiles whose pixels can see the volume: the rectangle around
// the projected corners of the volume box, one pixel wider on each side.  A
// pixel centre outside the projected box (the convex hull of its corners when
// all are in front of the eye) sends a ray that misses it.  With a corner at
// or behind the eye, or a box beyond the frame, the whole frame is kept or
// nothing (only the background).
void cull_tiles(FrameDesc& f, const gbvr_renderer* r, const float* view, const float* proj) {
  double V[16], P[16], M[16];
  for (int i = 0; i < 16; ++i) { V[i] = view[i]; P[i] = proj[i]; }
  mat_mul(P, V, M);
  double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
  for (int k = 0; k < 8; ++k) {
    const double c[3] = {(k & 1) ? f.half_extent[0] : -f.half_extent[0], (k & 2) ? f.half_extent[1] : -f.half_extent[1],
                         (k & 4) ? f.half_extent[2] : -f.half_extent[2]};
    double h[4];
    for (int rr = 0; rr < 4; ++rr) h[rr] = M[4 * rr] * c[0] + M[4 * rr + 1] * c[1] + M[4 * rr + 2] * c[2] + M[4 * rr + 3];
    if (!(h[3] > 1e-6)) return;  // a corner at or behind the eye: keep the whole frame
    const double px = (h[0] / h[3] + 1.0) * 0.5 * f.width - 0.5, py = (1.0 - h[1] / h[3]) * 0.5 * f.height - 0.5;
    x0 = std::min(x0, px); x1 = std::max(x1, px);
    y0 = std::min(y0, py); y1 = std::max(y1, py);
  }
  const int th = 32 / f.tile_w;
  const long long px0 = std::max<long long>(0, (long long)std::floor(x0) - 1);
  const long long px1 = std::min<long long>(f.width - 1, (long long)std::ceil(x1) + 1);
  const long long py0 = std::max<long long>(0, (long long)std::floor(y0) - 1);
  const long long py1 = std::min<long long>(f.height - 1, (long long)std::ceil(y1) + 1);
  if (px0 > px1 || py0 > py1) {
    f.ntx = f.nty = 0;  // the volume is outside the frame
    return;
  }
  f.tx0 = (int)(px0 / f.tile_w);
  f.ty0 = (int)(py0 / th);
  f.ntx = (int)(px1 / f.tile_w) - f.tx0 + 1;
  f.nty = (int)(py1 / th) - f.ty0 + 1;
  (void)r;
}

// Cached graphs bake in device and pinned pointers: drop them whenever a
// buffer they reference moves.
struct PtrSnapshot {
  void* p[10];
  explicit PtrSnapshot(const gbvr_renderer* r)
      : p{r->d_fb8.p, r->d_fb32.p, r->d_frames.p, r->d_prefix.p, r->d_counter.p,
          r->d_samples.p, r->d_touched.p, r->h_frames.p, r->h_prefix.p, r->d_skip.p} {}
  bool operator!=(const PtrSnapshot& o) const { return memcmp(p, o.p, sizeof(p)) != 0; }
};

// Out of core, compressed store: the compressed runs of the paged bricks
// (brick, slot) to the device staging, then one decode of all their chunks
// into the slots, both on the copy stream.  comp_bytes: bytes copied.
int page_compressed(gbvr_renderer* r, std::vector<std::pair<int, int>>& paged, uint64_t& comp_bytes) {
  Dataset& ds = r->ds;
  const size_t es = dtype_size(ds.dtype);
  // in store order, so that bricks adjacent in the store go in one copy
  std::sort(paged.begin(), paged.end(), [&](const std::pair<int, int>& x, const std::pair<int, int>& y) {
    const int sx = ds.host_cseg[(size_t)x.first], sy = ds.host_cseg[(size_t)y.first];
    return sx != sy ? sx < sy : ds.host_coff[(size_t)x.first] < ds.host_coff[(size_t)y.first];
  });
  // compressed runs to the device staging, then one decode of all their
  // chunks into the slots (both on the copy stream)
  std::vector<Lz4Chunk> jobs;
  std::vector<size_t> run(paged.size());
  size_t total = 0;
  for (size_t q = 0; q < paged.size(); ++q) {
    const int bidx = paged[q].first;
    const BrickInfo& b = ds.bricks[bidx];
    const size_t nbytes = (size_t)b.sx * b.sy * b.sz * es;
    const unsigned c0 = ds.chunk_first[bidx], nc = (unsigned)((nbytes + LZ_CHUNK - 1) / LZ_CHUNK);
    size_t cb = 0;
    for (unsigned k = 0; k < nc; ++k) {
      const unsigned cs = ds.chunk_size[c0 + k];
      Lz4Chunk ch;
      ch.src = total + cb;
      ch.dst = (unsigned long long)paged[q].second * ds.slot_elems * es + (unsigned long long)k * LZ_CHUNK;
      ch.comp = cs;
      ch.raw = (unsigned)std::min(LZ_CHUNK, nbytes - (size_t)k * LZ_CHUNK);
      jobs.push_back(ch);
      cb += cs & 0x7fffffffu;
    }
    run[q] = cb;
    total += cb;
  }
  CUDA_TRY(ds.d_stage.alloc(std::max<size_t>(total, 16)));
  CUDA_TRY(ds.d_chunks.alloc(sizeof(Lz4Chunk) * jobs.size()));
  // bricks page in store order: one copy per stretch of adjacent runs
  size_t at = 0, cp_at = 0, cp_n = 0;
  const uint8_t* cp_src = nullptr;
  for (size_t q = 0; q < paged.size(); ++q) {
    const uint8_t* h = ds.comp_run(paged[q].first);
    if (cp_n && h == cp_src + cp_n) {
      cp_n += run[q];
    } else {
      if (cp_n) {
        CUDA_TRY(cudaMemcpyAsync((char*)ds.d_stage.p + cp_at, cp_src, cp_n, cudaMemcpyHostToDevice, r->copy_stream));
        ++r->last_host_copies;
      }
      cp_src = h;
      cp_at = at;
      cp_n = run[q];
    }
    at += run[q];
  }
  if (cp_n) {
    CUDA_TRY(cudaMemcpyAsync((char*)ds.d_stage.p + cp_at, cp_src, cp_n, cudaMemcpyHostToDevice, r->copy_stream));
    ++r->last_host_copies;
  }
  // pageable source: the copy returns once it is staged
  CUDA_TRY(cudaMemcpyAsync(ds.d_chunks.p, jobs.data(), sizeof(Lz4Chunk) * jobs.size(), cudaMemcpyHostToDevice,
                           r->copy_stream));
  if (ds.compression == 1)
    CUDA_TRY(launch_inflate(ds.d_stage.p, ds.pool.p, ds.d_chunks.as<Lz4Chunk>(), (int)jobs.size(),
                            ds.d_lz_err.as<int>(), r->copy_stream));
  else
    CUDA_TRY(launch_lz4_decode(ds.d_stage.p, ds.pool.p, ds.d_chunks.as<Lz4Chunk>(), (int)jobs.size(),
                               ds.d_lz_err.as<int>(), r->copy_stream));
  comp_bytes = total;
  return GBVR_OK;
}

// Out-of-core paging for the views of one paint: pick the finest level (from
// the LOD limit down) whose bricks that may contribute and intersect a view
// frustum fit the device slots, upload the missing ones on the copy stream
// (evicting least-recently-used bricks the frame does not need), and build
// the frame's skip table: a brick is skipped when it is empty under the TF or
// not resident.  Bricks needed at the requested level but not resident when
// the paint began count as misses.
//
// Nothing here waits for the GPU: the copies go to the copy stream between
// the events ev_c0/ev_c1[stage], the render stream waits for them and then
// takes the level's page table and the skip table from the page-locked
// staging of `stage`.  A frame still rendering keeps its slots: `protect` is
// its stamp (0: none), and if the new frame cannot be placed without them the
// copies wait on the GPU for `protect_done` (that frame's end) before they
// overwrite anything.  The staging of `stage` must be free (its previous
// uploads complete) when this is called.
int ooc_page(gbvr_renderer* r, const gbvr_view* views, int n, int& level, uint64_t protect, cudaEvent_t protect_done,
             int stage, uint64_t* misses_out, uint64_t* bytes_out, const SliceSel* slice = nullptr) {
  Dataset& ds = r->ds;
  ensure_tf(r);
  // a slice is classified with the 1D TF, whatever the render mode
  const bool two = r->mode == GBVR_RM_2DTRANS && !slice;
  if (two && r->tf2d.empty()) return fail(GBVR_ESTATE, "2D transfer function not set");
  const std::vector<float>& tf = two ? r->tf2d : r->tf1d;
  const int w = two ? r->tf2d_w : (int)(r->tf1d.size() / 4), h = two ? r->tf2d_h : 1;
  std::vector<int> pre(w + 1, 0);
  for (int x = 0; x < w; ++x) {
    int nz = 0;
    for (int y = 0; y < h && !nz; ++y) nz = tf[4 * ((size_t)y * w + x) + 3] != 0.f;
    pre[x + 1] = pre[x] + nz;
  }
  double vlo, vhi;
  default_range(r, vlo, vhi);
  const float idx_scale = (float)((w - 1) / (vhi - vlo)), lo_f = (float)vlo;
  auto nonempty = [&](const BrickInfo& b) {
    if (slice && slice->mip) return true;  // the column maximum needs every brick
    if (!slice && r->mode == GBVR_RM_ISOSURFACE) return b.vmax >= skip_iso(r);
    if (!slice && r->mode == GBVR_RM_MIP) return true;
    float ilo = std::min(std::max((b.vmin - lo_f) * idx_scale, 0.f), (float)(w - 1));
    float ihi = std::min(std::max((b.vmax - lo_f) * idx_scale, 0.f), (float)(w - 1));
    int a0 = std::max((int)std::floor(ilo) - 1, 0), a1 = std::min((int)std::floor(ihi) + 2, w - 1);
    return pre[a1 + 1] - pre[a0] > 0;
  };
  // view-projection matrices of the paint
  std::vector<std::array<double, 16>> mats(n);
  for (int v = 0; v < n; ++v) {
    double V[16], P[16];
    for (int i = 0; i < 16; ++i) { V[i] = views[v].view[i]; P[i] = views[v].proj[i]; }
    mat_mul(P, V, mats[v].data());
  }
  double ext[3], mx = 0;
  for (int a = 0; a < 3; ++a) { ext[a] = (double)ds.dims[a] * ds.aspect[a]; mx = std::max(mx, ext[a]); }
  for (int a = 0; a < 3; ++a) ext[a] /= mx;
  // conservative: the brick's interior grown by one voxel, all 8 corners
  // outside one clip plane of every view means no ray of the paint samples it.
  // Rays start on the near plane and run to the volume's far side, so the
  // far plane does not cull.
  auto visible = [&](const Level& L, const BrickInfo& b) {
    const int lo[3] = {b.lox, b.loy, b.loz}, hi[3] = {b.hix, b.hiy, b.hiz};
    if (slice) {
      if (slice->mip) return true;
      // the brick holding the slice's cell (one cell either side for
      // rounding): the sampler reads the footprint from that brick
      const int a = slice->axis;
      const double wpos = ((double)slice->index + 0.5) / (double)ds.dims[a];
      const long long cell = (long long)std::floor(wpos * (double)L.dims[a] - 0.5);
      return lo[a] <= cell + 1 && cell - 1 < hi[a];
    }
    double c[8][4];
    for (int k = 0; k < 8; ++k)
      for (int a = 0; a < 3; ++a) {
        const double vx = (k >> a) & 1 ? hi[a] + 1.0 : lo[a] - 1.0;
        c[k][a] = (vx + 0.5) / (double)L.dims[a] * ext[a] - 0.5 * ext[a];
      }
    for (int v = 0; v < n; ++v) {
      const double* M = mats[v].data();
      bool out = false;
      for (int plane = 0; plane < 6 && !out; ++plane) {
        if (plane == 4) continue;  // far
        const int axis = plane >> 1;
        const double sgn = (plane & 1) ? -1.0 : 1.0;
        bool all = true;
        for (int k = 0; k < 8 && all; ++k) {
          double cl[4];
          for (int rr = 0; rr < 4; ++rr)
            cl[rr] = M[4 * rr] * c[k][0] + M[4 * rr + 1] * c[k][1] + M[4 * rr + 2] * c[k][2] + M[4 * rr + 3];
          all = sgn * cl[axis] > cl[3];  // outside this side of the clip volume
        }
        out = all;
      }
      if (!out) return true;
    }
    return false;
  };
  const int nlev = (int)ds.levels.size();
  const int target = level;
  std::vector<int> needed;
  uint64_t misses = 0;
  for (int l = target; l < nlev; ++l) {
    const Level& L = ds.levels[l];
    needed.clear();
    for (int i = 0; i < L.nbricks; ++i) {
      const BrickInfo& b = ds.bricks[L.brick_base + i];
      if (nonempty(b) && visible(L, b)) needed.push_back(L.brick_base + i);
    }
    if (l == target)
      for (int bidx : needed) misses += ds.slot_of[bidx] < 0;
    level = l;
    if ((int)needed.size() <= ds.nslots) break;
  }
  if ((int)needed.size() > ds.nslots) needed.resize(ds.nslots);  // coarsest level still too large
  ++ds.frame;
  std::vector<char> want(ds.bricks.size(), 0);
  for (int bidx : needed) {
    want[bidx] = 1;
    if (ds.slot_of[bidx] >= 0) ds.slot_used[ds.slot_of[bidx]] = ds.frame;
  }
  // victims: free slots first, then least recently used unwanted bricks; the
  // slots of a frame still rendering only if the new frame needs the room
  size_t missing = 0;
  for (int bidx : needed) missing += ds.slot_of[bidx] < 0;
  std::vector<int> victims;
  bool wait_protected = false;
  for (int pass = 0; pass < 2; ++pass) {
    const bool guard = protect != 0 && pass == 0;
    victims.clear();
    for (int sl = 0; sl < ds.nslots; ++sl)
      if (ds.slot_brick[sl] < 0 || (!want[ds.slot_brick[sl]] && !(guard && ds.slot_used[sl] == protect)))
        victims.push_back(sl);
    if (victims.size() >= missing || !guard) break;
    // no room without the frame still rendering: its slots become victims
    // and the copies wait for it on the GPU (the host keeps going)
    wait_protected = protect_done != nullptr;
  }
  std::sort(victims.begin(), victims.end(), [&](int x, int y) {
    const bool fx = ds.slot_brick[x] < 0, fy = ds.slot_brick[y] < 0;
    if (fx != fy) return fx;
    return ds.slot_used[x] < ds.slot_used[y];
  });
  const size_t es = dtype_size(ds.dtype);
  size_t vi = 0;
  uint64_t bytes = 0;
  if (!protect) {
    // slots are overwritten only after every earlier paint has read them
    CUDA_TRY(cudaEventRecord(r->ev_c0[stage], r->stream));
    CUDA_TRY(cudaStreamWaitEvent(r->copy_stream, r->ev_c0[stage], 0));
  } else if (wait_protected) {
    CUDA_TRY(cudaStreamWaitEvent(r->copy_stream, protect_done, 0));
  }
  CUDA_TRY(cudaEventRecord(r->ev_c0[stage], r->copy_stream));
  std::vector<std::pair<int, int>> paged;  // compressed store: (brick, slot) to decode
  for (int bidx : needed) {
    if (ds.slot_of[bidx] >= 0) continue;
    if (vi >= victims.size()) break;
    const int sl = victims[vi++];
    if (ds.slot_brick[sl] >= 0) ds.slot_of[ds.slot_brick[sl]] = -1;
    ds.slot_brick[sl] = bidx;
    ds.slot_of[bidx] = sl;
    ds.slot_used[sl] = ds.frame;
    const BrickInfo& b = ds.bricks[bidx];
    const size_t nbytes = (size_t)b.sx * b.sy * b.sz * es;
    if (ds.compression) {
      paged.emplace_back(bidx, sl);
    } else {
      CUDA_TRY(cudaMemcpyAsync((char*)ds.pool.p + (size_t)sl * ds.slot_elems * es,
                               (const char*)ds.host_store.p + ds.host_off[bidx] * es, nbytes, cudaMemcpyHostToDevice,
                               r->copy_stream));
      ++r->last_host_copies;
    }
    bytes += nbytes;
  }
  uint64_t comp_bytes = 0;
  if (!paged.empty()) {
    // a failure below leaves these bricks undecoded: they go back to not
    // resident (their slots free), so a later paint pages them again
    auto rollback = [&]() {
      for (const auto& pr : paged) {
        ds.slot_of[pr.first] = -1;
        ds.slot_brick[pr.second] = -1;
      }
    };
    const int rc = page_compressed(r, paged, comp_bytes);
    if (rc != GBVR_OK) {
      rollback();
      return rc;
    }
  }
  r->last_paged_comp += comp_bytes;
  CUDA_TRY(cudaEventRecord(r->ev_c1[stage], r->copy_stream));
  CUDA_TRY(cudaStreamWaitEvent(r->stream, r->ev_c1[stage], 0));
  // page table of the rendered level and its skip table, staged in page-locked
  // memory so the uploads queue behind the renders already on the stream
  const Level& L = ds.levels[level];
  CUDA_TRY(r->h_pt[stage].alloc(sizeof(BrickInfo) * ds.bricks.size()));
  CUDA_TRY(r->h_skip[stage].alloc(ds.bricks.size()));
  BrickInfo* pt = (BrickInfo*)r->h_pt[stage].p;
  unsigned char* skip = (unsigned char*)r->h_skip[stage].p;
  memset(skip, 1, ds.bricks.size());
  for (int i = 0; i < L.nbricks; ++i) {
    BrickInfo& b = ds.bricks[L.brick_base + i];
    const int sl = ds.slot_of[L.brick_base + i];
    b.offset = sl >= 0 ? (unsigned long long)sl * ds.slot_elems : 0;
    pt[i] = b;
    skip[L.brick_base + i] = (sl >= 0 && nonempty(b)) ? 0 : 1;
  }
  CUDA_TRY(cudaMemcpyAsync(ds.d_bricks.as<BrickInfo>() + L.brick_base, pt, sizeof(BrickInfo) * L.nbricks,
                           cudaMemcpyHostToDevice, r->stream));
  CUDA_TRY(r->d_ooc_skip.alloc(ds.bricks.size()));
  CUDA_TRY(cudaMemcpyAsync(r->d_ooc_skip.p, skip, ds.bricks.size(), cudaMemcpyHostToDevice, r->stream));
  if (misses_out) *misses_out = misses;
  if (bytes_out) *bytes_out = bytes;
  return GBVR_OK;
}

int ooc_streams(gbvr_renderer* r) {
  if (!r->copy_stream) {
    CUDA_TRY(cudaStreamCreateWithFlags(&r->copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      CUDA_TRY(cudaEventCreate(&r->ev_c0[k]));
      CUDA_TRY(cudaEventCreate(&r->ev_c1[k]));
      CUDA_TRY(cudaEventCreate(&r->ev_done[k]));
    }
  }
  return GBVR_OK;
}

// Out of core with a compressed store: a chunk the device decoder found
// malformed (the store is written by this library's compressors, so only a
// corrupted store does this) fails the paint.
int check_decode(gbvr_renderer* r) {
  if (!r->ds.ooc || !r->ds.compression) return GBVR_OK;
  int e = 0;
  CUDA_TRY(cudaMemcpy(&e, r->ds.d_lz_err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) return fail(GBVR_EFORMAT, "corrupt compressed brick in the out-of-core store");
  return GBVR_OK;
}

int prepare(gbvr_renderer* r, int nviews, int& level, const gbvr_view* views) {
  TRY(check_loaded(r));
  if (nviews <= 0) return fail(GBVR_EINVAL, "view count must be positive");
  level = render_level(r);
  if (r->ds.ooc) {
    TRY(ooc_streams(r));
    std::vector<gbvr_view> vs;
    if (!views) {
      gbvr_view v;
      if (r->view_set) {
        memcpy(v.view, r->view, sizeof(v.view));
        memcpy(v.proj, r->proj, sizeof(v.proj));
      } else {
        default_camera(r, v.view, v.proj);
      }
      vs.push_back(v);
      views = vs.data();
    }
    // every earlier paint has finished (paints are synchronous): no slot is in use
    r->last_paged_comp = 0;
    r->last_host_copies = 0;
    TRY(ooc_page(r, views, views == vs.data() ? 1 : nviews, level, 0, nullptr, 0, &r->last_misses, &r->last_paged,
                 r->slice_sel));
    CUDA_TRY(cudaEventSynchronize(r->ev_c1[0]));
    TRY(check_decode(r));
    CUDA_TRY(cudaEventElapsedTime(&r->last_page_ms, r->ev_c0[0], r->ev_c1[0]));
    r->drop_graphs();  // the page table changes between paints
  }
  const size_t npix = (size_t)r->width * r->height;
  if (r->fb_views < nviews || r->fb_w != r->width || r->fb_h != r->height) {
    CUDA_TRY(r->d_fb8.alloc(npix * 4 * nviews));
    if (r->flags & 1u) CUDA_TRY(r->d_fb32.alloc(npix * 16 * nviews));
    r->fb_views = nviews;
    r->fb_w = r->width;
    r->fb_h = r->height;
    r->drop_graphs();
  }
  CUDA_TRY(r->d_samples.alloc(sizeof(unsigned long long) * nviews));
  CUDA_TRY(r->d_touched.alloc((size_t)nviews * r->ds.levels[level].nbricks));
  TRY(alloc_lines(r, npix, nviews));
  {
    const Level& L = r->ds.levels[level];
    r->cell_words = ((long long)L.nc[0] * L.nc[1] * L.nc[2] + 31) / 32;
    if (r->stats_level >= 2) {
      CUDA_TRY(r->d_cellbits.alloc(sizeof(unsigned) * r->cell_words * nviews));
      CUDA_TRY(r->d_cellcount.alloc(sizeof(unsigned long long) * nviews));
    }
  }
  TRY(upload_tf(r, level));
  return GBVR_OK;
}

// The synchronous calls first let queued asynchronous work finish, so they
// never overwrite framebuffers a read-back still copies.
int settle_async(gbvr_renderer* r) {
  if (!r->read_stream) return GBVR_OK;
  if (r->slot_render_pending[0] || r->slot_render_pending[1] || r->slot_read_pending[0] || r->slot_read_pending[1]) {
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->read_stream));
    for (int k = 0; k < 2; ++k) r->slot_render_pending[k] = r->slot_read_pending[k] = false;
  }
  return GBVR_OK;
}

int finish(gbvr_renderer* r, int nviews, int level) {
  CUDA_TRY(cudaEventSynchronize(r->ev1));
  CUDA_TRY(cudaEventElapsedTime(&r->last_ms, r->ev0, r->ev1));
  CUDA_TRY(cudaEventElapsedTime(&r->last_kernel_ms, r->evk0, r->evk1));
  r->last_views = nviews;
  r->last_level = level;
  return GBVR_OK;
}

int paint_plain(gbvr_renderer* r, const gbvr_view* views, int n) {
  int level;
  TRY(prepare(r, n, level, views));
  CUDA_TRY(cudaMemsetAsync(r->d_samples.p, 0, sizeof(unsigned long long) * n, r->stream));
  CUDA_TRY(cudaMemsetAsync(r->d_touched.p, 0, (size_t)n * r->ds.levels[level].nbricks, r->stream));
  if (r->stats_level >= 2) CUDA_TRY(cudaMemsetAsync(r->d_cellbits.p, 0, sizeof(unsigned) * r->cell_words * n, r->stream));
  CUDA_TRY(cudaEventRecord(r->ev0, r->stream));
  gbvr_view cur;
  if (!views) {
    if (r->view_set) {
      memcpy(cur.view, r->view, sizeof(cur.view));
      memcpy(cur.proj, r->proj, sizeof(cur.proj));
    } else {
      default_camera(r, cur.view, cur.proj);
    }
  }
  TRY(draw_lines(r, views ? views : &cur, 0, n, level));
  CUDA_TRY(cudaEventRecord(r->evk0, r->stream));
  for (int v = 0; v < n; ++v) {
    const float *vw = views ? views[v].view : cur.view, *pj = views ? views[v].proj : cur.proj;
    FrameDesc f = make_frame(r, vw, pj, level, v);
    cull_tiles(f, r, vw, pj);
    TRY(line_stops_one(r, f, v, v == 0));
    CUDA_TRY(launch_fill_outside_one(f, r->stream));
    CUDA_TRY(launch_render_plain(f, r->stream));
    if (!lines_on(r)) TRY(render_cv(r, f));
  }
  TRY(render_lines(r));
  if (lines_on(r))
    for (int v = 0; v < n; ++v) {
      const float *vw = views ? views[v].view : cur.view, *pj = views ? views[v].proj : cur.proj;
      TRY(render_cv(r, make_frame(r, vw, pj, level, v)));
    }
  CUDA_TRY(cudaEventRecord(r->evk1, r->stream));
  CUDA_TRY(cudaEventRecord(r->ev1, r->stream));
  r->last_h2d = 0;  // descriptors travel as kernel parameters
  return finish(r, n, level);
}

// 2D slice view into framebuffer 0 (see k_render_slice).
int paint_slice(gbvr_renderer* r, int axis, int64_t index, int flip_x, int flip_y, int use_mip) {
  TRY(check_loaded(r));
  const Dataset& ds = r->ds;
  if (axis < 0 || axis > 2) return fail(GBVR_EINVAL, "slice axis must be 0, 1 or 2");
  if (index < 0 || index >= ds.dims[axis]) return fail(GBVR_EINVAL, "slice index outside the volume");
  int level;
  {
    // out of core, the slice's bricks are paged in (every brick for MIP;
    // a coarser level when they do not fit the device slots)
    const SliceSel sel{axis, (long long)index, use_mip != 0};
    r->slice_sel = &sel;
    const int rc = prepare(r, 1, level, nullptr);
    r->slice_sel = nullptr;
    TRY(rc);
  }
  ensure_tf(r);
  const std::vector<float> slice_tf = tf1d_pairs(r->tf1d.data(), (int)(r->tf1d.size() / 4));
  CUDA_TRY(r->d_tf_slice.alloc(sizeof(float) * slice_tf.size()));
  CUDA_TRY(cudaMemcpyAsync(r->d_tf_slice.p, slice_tf.data(), sizeof(float) * slice_tf.size(), cudaMemcpyHostToDevice,
                           r->stream));
  float dv[16], dp[16];
  default_camera(r, dv, dp);
  FrameDesc f = make_frame(r, dv, dp, level, 0);
  double lo, hi;
  default_range(r, lo, hi);
  f.tf = r->d_tf_slice.as<float4>();
  f.tf_w = (int)(r->tf1d.size() / 4);
  f.idx_scale = (float)((f.tf_w - 1) / (hi - lo));
  f.interp = r->interp;
  const Level& L = ds.levels[level];
  double ext[3], mx = 0;
  for (int a = 0; a < 3; ++a) { ext[a] = (double)ds.dims[a] * ds.aspect[a]; mx = std::max(mx, ext[a]); }
  for (int a = 0; a < 3; ++a) ext[a] /= mx;
  const int ua = axis == 0 ? 1 : 0, va = axis == 2 ? 1 : 2;
  SliceDesc sd;
  sd.axis = axis;
  // the slice's world position (centre of voxel `index` of the finest level) on the rendered level
  const double w = ((double)index + 0.5) / (double)ds.dims[axis] * ext[axis];
  sd.coord = (float)(w * (double)L.dims[axis] / ext[axis] - 0.5);
  const double sc = std::min((double)r->width / ext[ua], (double)r->height / ext[va]);
  sd.inv_s = (float)(1.0 / sc);
  sd.half_w = 0.5f * (float)r->width;
  sd.half_h = 0.5f * (float)r->height;
  sd.ext_u = (float)ext[ua];
  sd.ext_v = (float)ext[va];
  sd.scale_u = (float)((double)L.dims[ua] / ext[ua]);
  sd.scale_v = (float)((double)L.dims[va] / ext[va]);
  sd.flip_x = flip_x ? 1 : 0;
  sd.flip_y = flip_y ? 1 : 0;
  sd.mip = use_mip ? 1 : 0;
  sd.use_skip = ds.ooc ? 1 : 0;
  CUDA_TRY(cudaMemsetAsync(r->d_samples.p, 0, sizeof(unsigned long long), r->stream));
  CUDA_TRY(cudaEventRecord(r->ev0, r->stream));
  CUDA_TRY(cudaEventRecord(r->evk0, r->stream));
  CUDA_TRY(launch_render_slice(f, sd, r->stream));
  CUDA_TRY(cudaEventRecord(r->evk1, r->stream));
  CUDA_TRY(cudaEventRecord(r->ev1, r->stream));
  r->last_h2d = sizeof(float) * r->tf1d.size();
  return finish(r, 1, level);
}

// A sequence of frames (a fly-through) into framebuffers 0..n-1.  Out of
// core the frames form a pipeline: while frame i renders, the host picks
// frame i + 1's level and bricks and their copies run on the copy stream;
// frame i's slots are kept until it is done, and at most two frames are in
// flight (frame i is paged only after frame i - 2 has finished, which frees
// its staging and its slots).  Each frame renders with the per-view kernel
// at its own level.  In core the frames simply render one after the other.
// capture (optional): frame i's RGBA8 pixels are copied to capture + i *
// width * height * 4 on the read stream once frame i is done.
int paint_path(gbvr_renderer* r, const gbvr_view* views, int n, int32_t* lod_out, uint64_t* miss_out,
               uint64_t* paged_out, uint8_t* capture = nullptr, size_t capture_bytes = 0) {
  TRY(check_loaded(r));
  if (n <= 0 || !views) return fail(GBVR_EINVAL, "bad view list");
  const size_t frame_bytes = (size_t)r->width * r->height * 4;
  if (capture && capture_bytes < frame_bytes * n) return fail(GBVR_EINVAL, "capture buffer too small");
  if (capture && !r->read_stream) CUDA_TRY(cudaStreamCreateWithFlags(&r->read_stream, cudaStreamNonBlocking));
  Dataset& ds = r->ds;
  if (!ds.ooc) {
    TRY(paint_plain(r, views, n));
    for (int i = 0; i < n; ++i) {
      if (lod_out) lod_out[i] = r->last_level;
      if (miss_out) miss_out[i] = 0;
      if (paged_out) paged_out[i] = 0;
    }
    if (capture) {
      CUDA_TRY(cudaMemcpyAsync(capture, r->d_fb8.p, frame_bytes * n, cudaMemcpyDeviceToHost, r->stream));
      CUDA_TRY(cudaStreamSynchronize(r->stream));
    }
    return GBVR_OK;
  }
  TRY(ooc_streams(r));
  r->last_paged_comp = 0;
  r->last_host_copies = 0;
  const size_t npix = (size_t)r->width * r->height;
  if (r->fb_views < n || r->fb_w != r->width || r->fb_h != r->height) {
    CUDA_TRY(r->d_fb8.alloc(npix * 4 * n));
    if (r->flags & 1u) CUDA_TRY(r->d_fb32.alloc(npix * 16 * n));
    r->fb_views = n;
    r->fb_w = r->width;
    r->fb_h = r->height;
    r->drop_graphs();
  }
  const int nb0 = ds.levels[0].nbricks;  // the finest level has the most bricks
  CUDA_TRY(r->d_samples.alloc(sizeof(unsigned long long) * n));
  CUDA_TRY(r->d_touched.alloc((size_t)n * nb0));
  TRY(alloc_lines(r, npix, n));
  CUDA_TRY(cudaMemsetAsync(r->d_samples.p, 0, sizeof(unsigned long long) * n, r->stream));
  CUDA_TRY(cudaMemsetAsync(r->d_touched.p, 0, (size_t)n * nb0, r->stream));
  r->drop_graphs();
  uint64_t stamp[2] = {0, 0};
  uint64_t tot_miss = 0, tot_paged = 0;
  float tot_page_ms = 0.f;
  int level = 0;
  auto page_time = [&](int st) -> int {
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, r->ev_c0[st], r->ev_c1[st]));
    tot_page_ms += ms;
    return GBVR_OK;
  };
  CUDA_TRY(cudaEventRecord(r->ev0, r->stream));
  CUDA_TRY(cudaEventRecord(r->evk0, r->stream));
  for (int i = 0; i < n; ++i) {
    const int st = i & 1;
    if (i >= 2) {
      CUDA_TRY(cudaEventSynchronize(r->ev_done[st]));  // frame i - 2 is done
      TRY(page_time(st));
    }
    level = render_level(r);
    uint64_t miss = 0, bytes = 0;
    const uint64_t protect = i >= 1 ? stamp[st ^ 1] : 0;
    TRY(ooc_page(r, views + i, 1, level, protect, i >= 1 ? r->ev_done[st ^ 1] : nullptr, st, &miss, &bytes));
    stamp[st] = ds.frame;
    TRY(upload_tf(r, level));
    FrameDesc f = make_frame(r, views[i].view, views[i].proj, level, i);
    f.touched = r->stats_level >= 1 ? r->d_touched.as<unsigned char>() + (size_t)i * nb0 : nullptr;
    f.cell_touched = nullptr;
    cull_tiles(f, r, views[i].view, views[i].proj);
    TRY(draw_lines(r, views + i, i, 1, level));
    TRY(line_stops_one(r, f, i, true));
    CUDA_TRY(launch_fill_outside_one(f, r->stream));
    CUDA_TRY(launch_render_plain(f, r->stream));
    TRY(render_lines(r));  // while the frame's bricks are resident
    TRY(render_cv(r, f));
    CUDA_TRY(cudaEventRecord(r->ev_done[st], r->stream));
    if (capture) {
      // the frame's framebuffer is written once per path: no later frame reuses it
      CUDA_TRY(cudaStreamWaitEvent(r->read_stream, r->ev_done[st], 0));
      CUDA_TRY(cudaMemcpyAsync(capture + frame_bytes * i, (const char*)r->d_fb8.p + frame_bytes * i, frame_bytes,
                               cudaMemcpyDeviceToHost, r->read_stream));
    }
    if (lod_out) lod_out[i] = level;
    if (miss_out) miss_out[i] = miss;
    if (paged_out) paged_out[i] = bytes;
    tot_miss += miss;
    tot_paged += bytes;
  }
  CUDA_TRY(cudaEventRecord(r->evk1, r->stream));
  CUDA_TRY(cudaEventRecord(r->ev1, r->stream));
  CUDA_TRY(cudaEventSynchronize(r->ev1));
  if (capture) CUDA_TRY(cudaStreamSynchronize(r->read_stream));
  for (int i = std::max(0, n - 2); i < n; ++i) TRY(page_time(i & 1));
  r->last_misses = tot_miss;
  r->last_paged = tot_paged;
  r->last_page_ms = tot_page_ms;
  TRY(check_decode(r));
  r->last_h2d = 0;
  return finish(r, n, level);
}

// async: the step of a pipeline (gbvr_paint_batch_async): returns once the
// work is queued; the staging of the slot is reused only after the slot's
// previous render has consumed it, and the framebuffers only after their
// previous read-back.
int paint_batch(gbvr_renderer* r, const gbvr_view* views, int n, bool async = false) {
  int level;
  const int slot = r->cur_slot;
  if (async && r->slot_read_pending[slot]) CUDA_TRY(cudaStreamWaitEvent(r->stream, r->slot_read[slot], 0));
  const PtrSnapshot before(r);
  TRY(prepare(r, n, level, views));
  CUDA_TRY(r->h_frames.alloc(sizeof(FrameDesc) * n));
  CUDA_TRY(r->h_prefix.alloc(sizeof(int) * (n + 1)));
  CUDA_TRY(r->d_frames.alloc(sizeof(FrameDesc) * n));
  CUDA_TRY(r->d_prefix.alloc(sizeof(int) * (n + 1)));
  CUDA_TRY(r->d_counter.alloc(sizeof(int)));
  // the previous replay may still read the pinned staging buffers
  if (async) {
    if (r->slot_render_pending[slot]) CUDA_TRY(cudaEventSynchronize(r->slot_rendered[slot]));
  } else {
    CUDA_TRY(cudaStreamSynchronize(r->stream));
  }
  FrameDesc* hf = (FrameDesc*)r->h_frames.p;
  int* hp = (int*)r->h_prefix.p;
  long long total = 0;
  for (int v = 0; v < n; ++v) {
    hf[v] = make_frame(r, views[v].view, views[v].proj, level, v);
    cull_tiles(hf[v], r, views[v].view, views[v].proj);
    hp[v] = (int)total;
    total += (long long)hf[v].ntx * hf[v].nty;
    // work items are 32-bit (the atomic counter runs up to total + grid)
    if (total > (long long)INT32_MAX - (1 << 24)) return fail(GBVR_EINVAL, "batch too large: split it");
  }
  hp[n] = (int)total;
  if (PtrSnapshot(r) != before) r->drop_graphs();
  if (!r->sm_count) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&r->sm_count, cudaDevAttrMultiProcessorCount, dev);
    for (int m = 0; m < 4; ++m) {
      r->max_ctas_per_sm[m] = std::max(1, persistent_grid_size(dev, m) / std::max(r->sm_count, 1));
      r->max_ctas_per_sm_u[m] = std::max(1, persistent_grid_size_uniform(dev, m) / std::max(r->sm_count, 1));
    }
    r->max_ctas_per_sm_sps2 = persistent_ctas_per_sm_sps2();
  }
  // Views of one renderer batch share everything but camera, outputs and
  // counters, unless they sample different brick layout copies: then the
  // shared part goes to the kernel as a parameter.
  bool uniform = true;
  for (int v = 1; v < n; ++v)
    if (hf[v].perm != hf[0].perm || hf[v].copy_off != hf[0].copy_off) uniform = false;
  FrameDesc shared = hf[0];
  if (uniform) {
    // per-view parts, read from each view's own descriptor
    memset(shared.inv_vp, 0, sizeof(shared.inv_vp));
    memset(shared.light_to, 0, sizeof(shared.light_to));
    shared.tx0 = shared.ty0 = shared.ntx = shared.nty = 0;
    shared.out_rgba8 = nullptr;
    shared.out_f32 = nullptr;
    shared.samples = nullptr;
    shared.lines = nullptr;
    shared.touched_stride = shared.touched ? r->ds.levels[level].nbricks : 0;
    shared.cell_touched_stride = shared.cell_touched ? r->cell_words : 0;
  }
  const int sps = uniform && r->mode == GBVR_RM_1DTRANS && r->sampler == GBVR_SAMPLER_SW ? r->samples_per_step : 1;
  const int max_per_sm = sps >= 2 ? r->max_ctas_per_sm_sps2
                                  : (uniform ? r->max_ctas_per_sm_u[r->mode] : r->max_ctas_per_sm[r->mode]);
  const int per_sm = r->ctas_per_sm > 0 ? std::min(r->ctas_per_sm, max_per_sm) : max_per_sm;
  const int grid = r->sm_count * per_sm;
  if (n == 1) {
    // a single view (gbvr_paint): a direct launch; its descriptor changes
    // with every dataset, TF and size, which would re-capture a graph each time
    CUDA_TRY(cudaEventRecord(r->ev0, r->stream));
    TRY(draw_lines(r, views, 0, 1, level));
    CUDA_TRY(cudaMemcpyAsync(r->d_frames.p, r->h_frames.p, sizeof(FrameDesc), cudaMemcpyHostToDevice, r->stream));
    CUDA_TRY(cudaMemcpyAsync(r->d_prefix.p, r->h_prefix.p, sizeof(int) * 2, cudaMemcpyHostToDevice, r->stream));
    CUDA_TRY(cudaMemsetAsync(r->d_counter.p, 0, sizeof(int), r->stream));
    CUDA_TRY(cudaMemsetAsync(r->d_samples.p, 0, sizeof(unsigned long long), r->stream));
    CUDA_TRY(cudaMemsetAsync(r->d_touched.p, 0, (size_t)r->ds.levels[level].nbricks, r->stream));
    if (r->stats_level >= 2) CUDA_TRY(cudaMemsetAsync(r->d_cellbits.p, 0, sizeof(unsigned) * r->cell_words, r->stream));
    TRY(line_stops(r, 1));
    CUDA_TRY(launch_fill_outside(r->d_frames.as<FrameDesc>(), 1, r->height, r->stream));
    CUDA_TRY(cudaEventRecord(r->evk0, r->stream));  // kernel time: the raycast alone
    cudaError_t le =
        uniform ? launch_render_persistent_uniform(r->ds.dtype, r->mode, r->sampler, shared, r->d_frames.as<FrameDesc>(),
                                                   1, r->d_prefix.as<int>(), r->d_counter.as<int>(), grid, r->stream,
                                                   sps)
                : launch_render_persistent_typed(r->ds.dtype, r->mode, r->sampler, r->d_frames.as<FrameDesc>(), 1,
                                                 r->d_prefix.as<int>(), r->d_counter.as<int>(), grid, r->stream);
    if (le != cudaSuccess) return cuda_fail(le, "persistent launch");
    TRY(render_lines(r));
    TRY(render_cv(r, hf[0]));
    CUDA_TRY(cudaEventRecord(r->evk1, r->stream));
    CUDA_TRY(cudaEventRecord(r->ev1, r->stream));
    r->last_h2d = sizeof(FrameDesc) + sizeof(int) * 2;
    return finish(r, 1, level);
  }
  gbvr_renderer::GraphKey key{n,    r->width, r->height, level,       r->ds.dtype, r->mode,
                              r->sampler, grid,  sps,     r->d_fb8.p, r->d_fb32.p};
  auto it = r->graphs.find(key);
  if (it != r->graphs.end() &&
      (it->second.uniform != uniform || (uniform && memcmp(&it->second.shared, &shared, sizeof(FrameDesc)) != 0))) {
    cudaGraphExecDestroy(it->second.exec);  // the baked-in parameter changed
    r->graphs.erase(it);
    it = r->graphs.end();
  }
  if (it == r->graphs.end()) {
    // The graph holds the persistent launch; descriptor uploads and counter
    // resets are plain stream operations before it, so the kernel-only
    // events can bracket the graph launch.
    cudaGraph_t g;
    (void)cudaGetLastError();
    CUDA_TRY(cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t le =
        uniform ? launch_render_persistent_uniform(r->ds.dtype, r->mode, r->sampler, shared, r->d_frames.as<FrameDesc>(),
                                                   n, r->d_prefix.as<int>(), r->d_counter.as<int>(), grid, r->stream,
                                                   sps)
                : launch_render_persistent_typed(r->ds.dtype, r->mode, r->sampler, r->d_frames.as<FrameDesc>(), n,
                                                 r->d_prefix.as<int>(), r->d_counter.as<int>(), grid, r->stream);
    cudaError_t ce = cudaStreamEndCapture(r->stream, &g);
    if (le != cudaSuccess) return cuda_fail(le, "persistent launch capture");
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    cudaGraphExec_t ge;
    cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate");
    it = r->graphs.emplace(key, gbvr_renderer::CachedGraph{ge, uniform, shared}).first;
  }
  CUDA_TRY(cudaEventRecord(r->ev0, r->stream));
  TRY(draw_lines(r, views, 0, n, level));
  CUDA_TRY(cudaMemcpyAsync(r->d_frames.p, r->h_frames.p, sizeof(FrameDesc) * n, cudaMemcpyHostToDevice, r->stream));
  CUDA_TRY(cudaMemcpyAsync(r->d_prefix.p, r->h_prefix.p, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, r->stream));
  CUDA_TRY(cudaMemsetAsync(r->d_counter.p, 0, sizeof(int), r->stream));
  CUDA_TRY(cudaMemsetAsync(r->d_samples.p, 0, sizeof(unsigned long long) * n, r->stream));
  CUDA_TRY(cudaMemsetAsync(r->d_touched.p, 0, (size_t)n * r->ds.levels[level].nbricks, r->stream));
  if (r->stats_level >= 2) CUDA_TRY(cudaMemsetAsync(r->d_cellbits.p, 0, sizeof(unsigned) * r->cell_words * n, r->stream));
  TRY(line_stops(r, n));
  CUDA_TRY(launch_fill_outside(r->d_frames.as<FrameDesc>(), n, r->height, r->stream));
  CUDA_TRY(cudaEventRecord(r->evk0, r->stream));  // kernel time: the raycast alone
  CUDA_TRY(cudaGraphLaunch(it->second.exec, r->stream));
  TRY(render_lines(r));
  for (int v = 0; v < n; ++v) TRY(render_cv(r, hf[v]));
  CUDA_TRY(cudaEventRecord(r->evk1, r->stream));
  CUDA_TRY(cudaEventRecord(r->ev1, r->stream));
  r->last_h2d = sizeof(FrameDesc) * n + sizeof(int) * (n + 1);
  if (async) {
    CUDA_TRY(cudaEventRecord(r->slot_rendered[slot], r->stream));
    r->slot_render_pending[slot] = true;
    r->last_views = n;
    r->last_level = level;
    return GBVR_OK;
  }
  return finish(r, n, level);
}

void look_at(const double eye[3], const double c[3], const double up[3], double* m) {
  double f[3] = {c[0] - eye[0], c[1] - eye[1], c[2] - eye[2]};
  double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  for (double& x : f) x /= fl;
  double s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
  double sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
  for (double& x : s) x /= sl;
  double u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
  double rows[3][3] = {{s[0], s[1], s[2]}, {u[0], u[1], u[2]}, {-f[0], -f[1], -f[2]}};
  for (int r = 0; r < 3; ++r) {
    for (int k = 0; k < 3; ++k) m[4 * r + k] = rows[r][k];
    m[4 * r + 3] = -(rows[r][0] * eye[0] + rows[r][1] * eye[1] + rows[r][2] * eye[2]);
  }
  m[12] = m[13] = m[14] = 0;
  m[15] = 1;
}

void perspective(double fovy_deg, double aspect, double zn, double zf, double* m) {
  double t = 1.0 / std::tan(fovy_deg * M_PI / 360.0);
  for (int i = 0; i < 16; ++i) m[i] = 0;
  m[0] = t / aspect;
  m[5] = t;
  m[10] = (zf + zn) / (zn - zf);
  m[11] = 2 * zf * zn / (zn - zf);
  m[14] = -1;
}

void orbit(double az_deg, double el_deg, double radius, double fov, int w, int h, float* view, float* proj) {
  double az = az_deg * M_PI / 180.0, el = el_deg * M_PI / 180.0;
  double eye[3] = {radius * std::cos(el) * std::sin(az), radius * std::sin(el), radius * std::cos(el) * std::cos(az)};
  double c[3] = {0, 0, 0}, up[3] = {0, 1, 0};
  double V[16], P[16];
  look_at(eye, c, up, V);
  perspective(fov, (double)w / h, std::max(0.01, radius - 2.0), radius + 2.0, P);
  for (int i = 0; i < 16; ++i) { view[i] = (float)V[i]; proj[i] = (float)P[i]; }
}

void default_camera(gbvr_renderer* r, float view[16], float proj[16]) {
  // 45 degree field of view, orbit radius 2.5 x the (unit-normalised) box diagonal
  orbit(0.0, 0.0, 2.5 * std::sqrt(3.0), 45.0, r->width, r->height, view, proj);
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int gbvr_last_error(char* buf, size_t size) {
  GBVR_ABI_TRY
  if (!buf || size == 0) return GBVR_EINVAL;
  size_t n = std::min(size - 1, g_err.size());
  memcpy(buf, g_err.data(), n);
  buf[n] = 0;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_device_info(int* sm_count, size_t* free_bytes, size_t* total_bytes) {
  GBVR_ABI_TRY
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if (sm_count) CUDA_TRY(cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev));
  size_t f = 0, t = 0;
  CUDA_TRY(cudaMemGetInfo(&f, &t));
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_create(int renderer_type, uint32_t flags, gbvr_renderer** out) {
  GBVR_ABI_TRY
  if (!out) return fail(GBVR_EINVAL, "null output handle");
  *out = nullptr;
  if (renderer_type != GBVR_CUDA_RAYCASTER)
    return fail(GBVR_EINVAL, "this library implements only GBVR_CUDA_RAYCASTER (type 9)");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(GBVR_ECUDA, "no CUDA device available");
  std::unique_ptr<gbvr_renderer> r(new gbvr_renderer());
  r->flags = flags;
  CUDA_TRY(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
  CUDA_TRY(cudaEventCreate(&r->ev0));
  CUDA_TRY(cudaEventCreate(&r->ev1));
  CUDA_TRY(cudaEventCreate(&r->evk0));
  CUDA_TRY(cudaEventCreate(&r->evk1));
  *out = r.release();
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_destroy(gbvr_renderer* r) {
  GBVR_ABI_TRY
  if (!r) return GBVR_OK;
  if (r->stream) cudaStreamSynchronize(r->stream);
  delete r;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_load_volume(gbvr_renderer* r, const void* host, const int64_t dims[3], int dtype, const gbvr_brick_params* bp) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!host || !dims || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return fail(GBVR_EINVAL, "bad volume");
  if (dtype < 0 || dtype > 2) return fail(GBVR_EINVAL, "bad dtype");
  long long d[3] = {dims[0], dims[1], dims[2]};
  const size_t bytes = (size_t)d[0] * d[1] * d[2] * dtype_size(dtype);
  DevBuf lv;
  CUDA_TRY(lv.alloc(bytes));
  CUDA_TRY(cudaMemcpyAsync(lv.p, host, bytes, cudaMemcpyHostToDevice, r->stream));
  r->drop_graphs();
  r->skip_dirty = true;
  r->tf_dirty = true;
  TRY(build_dataset(r->ds, lv, dtype, d, bp, r->stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_load_synthetic(gbvr_renderer* r, const gbvr_synth_params* p, const gbvr_brick_params* bp) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  DevBuf lv;
  TRY(synth_to_device(p, lv, r->stream));
  r->drop_graphs();
  r->skip_dirty = true;
  r->tf_dirty = true;
  long long d[3] = {p->dims[0], p->dims[1], p->dims[2]};
  TRY(build_dataset(r->ds, lv, p->dtype, d, bp, r->stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_synth_volume(const gbvr_synth_params* p, void* host_out, size_t bytes) {
  GBVR_ABI_TRY
  if (!p || !host_out) return fail(GBVR_EINVAL, "null argument");
  size_t need = 0;
  TRY(check_synth_params(p, true, nullptr, &need));
  if (bytes < need) return fail(GBVR_EINVAL, "output buffer too small");
  gbvr_renderer tmp;
  CUDA_TRY(cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking));
  BlobTablesHost t;
  make_blob_tables(*p, t);
  DevBuf amp, ex, ey, ez, bx, by, bz, lv;
  auto up = [&](DevBuf& d, const std::vector<float>& v) -> cudaError_t {
    cudaError_t e = d.alloc(sizeof(float) * std::max<size_t>(v.size(), 1));
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(d.p, v.data(), sizeof(float) * v.size(), cudaMemcpyHostToDevice, tmp.stream);
  };
  CUDA_TRY(up(amp, t.amp));
  CUDA_TRY(up(ex, t.ex));
  CUDA_TRY(up(ey, t.ey));
  CUDA_TRY(up(ez, t.ez));
  CUDA_TRY(up(bx, t.bgx));
  CUDA_TRY(up(by, t.bgy));
  CUDA_TRY(up(bz, t.bgz));
  CUDA_TRY(lv.alloc(need));
  BlobTablesDev td{p->nblobs, amp.as<float>(), ex.as<float>(), ey.as<float>(), ez.as<float>(),
                   p->bg_freq > 0 ? bx.as<float>() : nullptr, p->bg_freq > 0 ? by.as<float>() : nullptr,
                   p->bg_freq > 0 ? bz.as<float>() : nullptr, p->bg_level, p->bg_amp, p->scale, p->noise_amp,
                   p->noise_kind, p->vmax, p->seed};
  long long d[3] = {p->dims[0], p->dims[1], p->dims[2]};
  CUDA_TRY(launch_synth_blobs(td, d, p->dtype, lv.p, tmp.stream));
  CUDA_TRY(cudaMemcpyAsync(host_out, lv.p, need, cudaMemcpyDeviceToHost, tmp.stream));
  CUDA_TRY(cudaStreamSynchronize(tmp.stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

static int check_fbm(const gbvr_fbm_params* p) {
  if (!p || p->dims[0] <= 0 || p->dims[1] <= 0 || p->dims[2] <= 0 || p->dtype < 0 || p->dtype > 2 ||
      p->octaves < 1 || p->octaves > 12 || p->base_period < 1 || (long long)p->base_period << (p->octaves - 1) > 65535 ||
      !(p->threshold < 1.0f))
    return fail(GBVR_EINVAL, "bad fractal-volume parameters");
  return GBVR_OK;
}

int gbvr_synth_fbm_volume(const gbvr_fbm_params* p, void* host_out, size_t bytes) {
  GBVR_ABI_TRY
  TRY(check_fbm(p));
  if (!host_out) return fail(GBVR_EINVAL, "null output");
  const size_t need = (size_t)p->dims[0] * p->dims[1] * p->dims[2] * dtype_size(p->dtype);
  if (bytes < need) return fail(GBVR_EINVAL, "output buffer too small");
  gbvr_renderer tmp;
  CUDA_TRY(cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking));
  DevBuf lv;
  CUDA_TRY(lv.alloc(need));
  long long d[3] = {p->dims[0], p->dims[1], p->dims[2]};
  CUDA_TRY(launch_synth_fbm(d, p->dtype, p->seed, p->octaves, p->base_period, p->threshold, p->vmax, lv.p, tmp.stream));
  CUDA_TRY(cudaMemcpyAsync(host_out, lv.p, need, cudaMemcpyDeviceToHost, tmp.stream));
  CUDA_TRY(cudaStreamSynchronize(tmp.stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_load_synthetic_fbm(gbvr_renderer* r, const gbvr_fbm_params* p, const gbvr_brick_params* bp) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  TRY(check_fbm(p));
  long long d[3] = {p->dims[0], p->dims[1], p->dims[2]};
  DevBuf lv;
  CUDA_TRY(lv.alloc((size_t)d[0] * d[1] * d[2] * dtype_size(p->dtype)));
  CUDA_TRY(launch_synth_fbm(d, p->dtype, p->seed, p->octaves, p->base_period, p->threshold, p->vmax, lv.p, r->stream));
  r->drop_graphs();
  r->skip_dirty = true;
  r->tf_dirty = true;
  TRY(build_dataset(r->ds, lv, p->dtype, d, bp, r->stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_load_synthetic_ooc(gbvr_renderer* r, const gbvr_synth_params* p, const gbvr_brick_params* bp,
                            uint64_t device_pool_bytes) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  TRY(check_synth_params(p, false, nullptr, nullptr));
  r->drop_graphs();
  r->skip_dirty = true;
  r->tf_dirty = true;
  TRY(build_ooc_synth(r->ds, p, bp, device_pool_bytes, r->stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_load_uvf(gbvr_renderer* r, const char* path, int verify, const gbvr_brick_params* bp) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!path) return fail(GBVR_EINVAL, "null path");
  UvfFile uf;
  std::string msg;
  int rc = uvf_read(path, verify != 0, uf, msg);
  if (rc) return fail(rc, msg);
  const UvfRaster& ra = uf.raster;
  int dtype;
  if (ra.is_float) dtype = DT_F32;
  else if (ra.bit_size == 8 && !ra.is_signed) dtype = DT_U8;
  else if (ra.bit_size == 16 && !ra.is_signed) dtype = DT_U16;
  else return fail(GBVR_EFORMAT, "unsupported raster element type");
  uint64_t lods = 1;
  for (uint64_t c : ra.lod_counts) lods = std::max(lods, c);
  if (lods != 1) return fail(GBVR_EFORMAT, "multi-LOD raster blocks are rebuilt from LOD 0: store LOD 0 only");
  const size_t bytes = (size_t)ra.dims[0] * ra.dims[1] * ra.dims[2] * dtype_size(dtype);
  std::vector<unsigned char> host(bytes);
  rc = uvf_read_voxels(path, uf, host.data(), bytes, msg);
  if (rc) return fail(rc, msg);
  gbvr_brick_params p = {};
  if (bp) p = *bp;
  if (p.brick_size <= 0) p.brick_size = (int)ra.brick_size[0];
  if (p.overlap <= 0) p.overlap = std::max(2, (int)(ra.overlap[0] / 2));
  for (int a = 0; a < 3; ++a)
    if (p.aspect[a] <= 0) p.aspect[a] = ra.transform[5 * a] > 0 ? ra.transform[5 * a] : 1.0;
  int64_t dims[3] = {(int64_t)ra.dims[0], (int64_t)ra.dims[1], (int64_t)ra.dims[2]};
  TRY(gbvr_load_volume(r, host.data(), dims, dtype, &p));
  r->ds.raster_id = ra.id;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_get_build_stats(gbvr_renderer* r, gbvr_build_stats* out) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  if (!out) return fail(GBVR_EINVAL, "null output");
  if (r->ds.ooc) return fail(GBVR_ESTATE, "build statistics are kept for in-core builds only");
  *out = r->ds.build;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_get_dataset_info(gbvr_renderer* r, gbvr_dataset_info* info) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  if (!info) return fail(GBVR_EINVAL, "null info");
  memset(info, 0, sizeof(*info));
  const Dataset& ds = r->ds;
  for (int a = 0; a < 3; ++a) info->dims[a] = ds.dims[a];
  info->dtype = ds.dtype;
  info->bit_width = ds.bit_width;
  info->range[0] = ds.gmin;
  info->range[1] = ds.gmax;
  info->lod_count = (int)ds.levels.size();
  info->brick_size = ds.brick;
  info->overlap = ds.ghost;
  for (size_t l = 0; l < ds.levels.size() && l < 16; ++l)
    for (int a = 0; a < 3; ++a) {
      info->lod_dims[l][a] = ds.levels[l].dims[a];
      info->lod_bricks[l][a] = ds.levels[l].nb[a];
    }
  info->total_bricks = (int64_t)ds.bricks.size();
  info->device_bytes = ds.ooc ? (uint64_t)ds.nslots * ds.slot_elems * dtype_size(ds.dtype) : ds.stored_bytes;
  info->host_bytes = ds.ooc ? (ds.compression ? ds.comp_store_bytes : ds.stored_bytes) : 0;
  info->device_slots = ds.ooc ? ds.nslots : 0;
  info->compression = ds.ooc ? ds.compression : 0;
  info->host_raw_bytes = ds.ooc ? ds.stored_bytes : 0;
  info->hist1d_size = (int)ds.hist1d.size();
  info->hist2d_max_grad = ds.max_grad;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_get_hist1d(gbvr_renderer* r, uint64_t* out, size_t n) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  if (!out || n < r->ds.hist1d.size()) return fail(GBVR_EINVAL, "histogram buffer too small");
  memcpy(out, r->ds.hist1d.data(), sizeof(uint64_t) * r->ds.hist1d.size());
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_get_hist2d(gbvr_renderer* r, uint64_t* out, size_t nx, size_t ny, float* max_grad) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  if (!out || nx * ny < r->ds.hist2d.size() || ny != 256) return fail(GBVR_EINVAL, "histogram buffer too small");
  memcpy(out, r->ds.hist2d.data(), sizeof(uint64_t) * r->ds.hist2d.size());
  if (max_grad) *max_grad = r->ds.max_grad;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_get_brick_minmax(gbvr_renderer* r, int lod, double* out, size_t nbricks) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  if (lod < 0 || lod >= (int)r->ds.levels.size()) return fail(GBVR_EINVAL, "bad lod");
  const Level& L = r->ds.levels[lod];
  if (!out || nbricks < (size_t)L.nbricks) return fail(GBVR_EINVAL, "buffer too small");
  for (int i = 0; i < L.nbricks; ++i) {
    out[2 * i] = r->ds.bricks[L.brick_base + i].vmin;
    out[2 * i + 1] = r->ds.bricks[L.brick_base + i].vmax;
  }
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_get_cell_minmax(gbvr_renderer* r, int lod, float* out, size_t ncells, int32_t nc[3], int32_t* cell_edge) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  TRY(settle_async(r));
  if (lod < 0 || lod >= (int)r->ds.levels.size()) return fail(GBVR_EINVAL, "bad lod");
  const Level& L = r->ds.levels[lod];
  const size_t n = (size_t)L.nc[0] * L.nc[1] * L.nc[2];
  if (nc)
    for (int a = 0; a < 3; ++a) nc[a] = L.nc[a];
  if (cell_edge) *cell_edge = 1 << L.cell_shift;
  if (!out) return GBVR_OK;
  if (ncells < n || !L.cells) return fail(GBVR_EINVAL, "buffer too small");
  CUDA_TRY(cudaMemcpy(out, L.cells->p, n * sizeof(float2), cudaMemcpyDeviceToHost));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_get_brick(gbvr_renderer* r, int lod, const int32_t brick[3], void* out, size_t bytes, int64_t origin[3],
                   int64_t stored_dims[3]) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  if (lod < 0 || lod >= (int)r->ds.levels.size() || !brick) return fail(GBVR_EINVAL, "bad lod");
  const Level& L = r->ds.levels[lod];
  for (int a = 0; a < 3; ++a)
    if (brick[a] < 0 || brick[a] >= L.nb[a]) return fail(GBVR_EINVAL, "brick index out of range");
  const BrickInfo& b = r->ds.bricks[L.brick_base + (brick[2] * L.nb[1] + brick[1]) * L.nb[0] + brick[0]];
  const size_t es = dtype_size(r->ds.dtype);
  const size_t need = (size_t)b.sx * b.sy * b.sz * es;
  if (origin) { origin[0] = b.ox; origin[1] = b.oy; origin[2] = b.oz; }
  if (stored_dims) { stored_dims[0] = b.sx; stored_dims[1] = b.sy; stored_dims[2] = b.sz; }
  if (!out) return GBVR_OK;
  if (bytes < need) return fail(GBVR_EINVAL, "brick buffer too small");
  if (r->ds.ooc && r->ds.compression) {
    // decode the brick's chunks on the host
    const size_t bidx = &b - r->ds.bricks.data();
    const uint8_t* src = r->ds.comp_run(bidx);
    for (size_t k = 0, o = 0; o < need; ++k, o += LZ_CHUNK) {
      const unsigned cs = r->ds.chunk_size[r->ds.chunk_first[bidx] + k];
      const size_t rn = std::min(LZ_CHUNK, need - o), cn = cs & 0x7fffffffu;
      if (cs & 0x80000000u) memcpy((uint8_t*)out + o, src, rn);
      else if (!(r->ds.compression == 1 ? zlib_decompress(src, cn, (uint8_t*)out + o, rn)
                                        : lz4_decompress(src, cn, (uint8_t*)out + o, rn)))
        return fail(GBVR_EFORMAT, "corrupt compressed brick");
      src += cn;
    }
    return GBVR_OK;
  }
  if (r->ds.ooc) {
    memcpy(out, (const char*)r->ds.host_store.p + r->ds.host_off[&b - r->ds.bricks.data()] * es, need);
    return GBVR_OK;
  }
  CUDA_TRY(cudaMemcpy(out, (const char*)r->ds.pool.p + b.offset * es, need, cudaMemcpyDeviceToHost));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_resize(gbvr_renderer* r, int width, int height) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (width <= 0 || height <= 0 || width > 16384 || height > 16384) return fail(GBVR_EINVAL, "bad framebuffer size");
  r->width = width;
  r->height = height;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_render_mode(gbvr_renderer* r, int mode) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (mode < 0 || mode > 3) return fail(GBVR_EINVAL, "bad render mode");
  if (mode != r->mode) { r->tf_dirty = true; r->skip_dirty = true; }
  r->mode = mode;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_paint_path(gbvr_renderer* r, const gbvr_view* views, int n, int32_t* lod, uint64_t* misses,
                    uint64_t* bytes_paged) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  TRY(settle_async(r));
  return paint_path(r, views, n, lod, misses, bytes_paged);
  GBVR_ABI_CATCH
}

int gbvr_paint_path_capture(gbvr_renderer* r, const gbvr_view* views, int n, int32_t* lod, uint64_t* misses,
                            uint64_t* bytes_paged, uint8_t* rgba8, size_t bytes) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!rgba8) return fail(GBVR_EINVAL, "null capture buffer");
  TRY(settle_async(r));
  return paint_path(r, views, n, lod, misses, bytes_paged, rgba8, bytes);
  GBVR_ABI_CATCH
}

int gbvr_paint_slice(gbvr_renderer* r, int axis, int64_t index, int flip_x, int flip_y, int use_mip) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  TRY(settle_async(r));
  return paint_slice(r, axis, index, flip_x, flip_y, use_mip);
  GBVR_ABI_CATCH
}

int gbvr_set_clip_plane(gbvr_renderer* r, int enabled, const float plane[4]) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (enabled) {
    if (!plane) return fail(GBVR_EINVAL, "null plane");
    for (int k = 0; k < 4; ++k)
      if (!std::isfinite(plane[k])) return fail(GBVR_EINVAL, "plane coefficients must be finite");
    for (int k = 0; k < 4; ++k) r->clip[k] = plane[k];
  }
  r->clip_on = enabled ? 1 : 0;
  r->drop_graphs();
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_tf1d(gbvr_renderer* r, const float* rgba, int n) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!rgba || n < 2 || n > 65536) return fail(GBVR_EINVAL, "1D transfer function needs 2..65536 entries");
  r->tf1d.assign(rgba, rgba + 4 * (size_t)n);
  r->tf_dirty = true;
  r->skip_dirty = true;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_tf2d(gbvr_renderer* r, const float* rgba, int w, int h, float max_grad) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!rgba || w < 2 || h < 2 || w > 4096 || h > 4096) return fail(GBVR_EINVAL, "bad 2D transfer function size");
  r->tf2d.assign(rgba, rgba + 4 * (size_t)w * h);
  r->tf2d_w = w;
  r->tf2d_h = h;
  r->tf2d_grad_max = max_grad;
  r->tf_dirty = true;
  r->skip_dirty = true;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_value_range(gbvr_renderer* r, double lo, double hi) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!(hi > lo)) return fail(GBVR_EINVAL, "value range must have hi > lo");
  r->range_set = true;
  r->vlo = lo;
  r->vhi = hi;
  r->skip_dirty = true;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_iso(gbvr_renderer* r, float value, const float rgb[3]) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  r->iso = value;
  r->iso_set = true;
  if (rgb) for (int k = 0; k < 3; ++k) r->iso_rgb[k] = rgb[k];
  r->skip_dirty = true;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_iso_relative(gbvr_renderer* r, float fraction, const float rgb[3]) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  double lo, hi;
  default_range(r, lo, hi);
  const float f = std::min(std::max(fraction, 0.f), 1.f);
  return gbvr_set_iso(r, f * (float)(long long)hi, rgb);
  GBVR_ABI_CATCH
}

int gbvr_set_blend_precision(gbvr_renderer* r, int bits) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (bits != 8 && bits != 16 && bits != 32) return fail(GBVR_EINVAL, "blend precision must be 8, 16 or 32 bits");
  return GBVR_OK;  // compositing is FP32 for every setting
  GBVR_ABI_CATCH
}

int gbvr_set_lighting(gbvr_renderer* r, int enabled, const float amb[4], const float diff[4], const float spec[4],
                      const float dir[3]) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  r->lighting = enabled != 0;
  for (int k = 0; k < 3; ++k) {
    if (amb) r->amb[k] = amb[k] * amb[3];
    if (diff) r->diff[k] = diff[k] * diff[3];
    if (spec) r->spec[k] = spec[k] * spec[3];
    if (dir) r->light_dir[k] = dir[k];
  }
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_sample_rate(gbvr_renderer* r, float spv) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!(spv >= 0.05f && spv <= 64.f)) return fail(GBVR_EINVAL, "samples per voxel must be in [0.05, 64]");
  r->spv = spv;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_interpolant(gbvr_renderer* r, int interp) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (interp != GBVR_NEAREST && interp != GBVR_LINEAR) return fail(GBVR_EINVAL, "bad interpolant");
  r->interp = interp;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_sampler(gbvr_renderer* r, int sampler) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (sampler != GBVR_SAMPLER_SW && sampler != GBVR_SAMPLER_TEX) return fail(GBVR_EINVAL, "bad sampler");
  if (sampler == GBVR_SAMPLER_TEX && r->ds.loaded && (r->ds.texs.empty() || r->ds.ooc))
    return fail(GBVR_ESTATE, "dataset was loaded without build_texture");
  r->sampler = sampler;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_lod_limits(gbvr_renderer* r, int min_lod, int max_lod) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (min_lod < 0 || max_lod < min_lod) return fail(GBVR_EINVAL, "bad LOD limits");
  r->lod_min = min_lod;
  r->lod_max = max_lod;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_view(gbvr_renderer* r, const float view[16], const float proj[16]) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!view || !proj) return fail(GBVR_EINVAL, "null matrix");
  memcpy(r->view, view, sizeof(r->view));
  memcpy(r->proj, proj, sizeof(r->proj));
  r->view_set = true;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_background(gbvr_renderer* r, const float top[3], const float bottom[3]) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  for (int k = 0; k < 3; ++k) {
    if (top) r->bg_top[k] = top[k];
    if (bottom) r->bg_bot[k] = bottom[k];
  }
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_early_termination(gbvr_renderer* r, float alpha) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!(alpha > 0.f && alpha <= 1.0f)) return fail(GBVR_EINVAL, "termination alpha must be in (0, 1]");
  r->ert = alpha;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_launch_shape(gbvr_renderer* r, int tile_w, int ctas_per_sm) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (tile_w != 4 && tile_w != 8 && tile_w != 16 && tile_w != 32) return fail(GBVR_EINVAL, "tile_w must be 4, 8, 16 or 32");
  if (ctas_per_sm < 0 || ctas_per_sm > 64) return fail(GBVR_EINVAL, "bad ctas_per_sm");
  r->tile_w = tile_w;
  r->ctas_per_sm = ctas_per_sm;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_empty_skipping(gbvr_renderer* r, int mode) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (mode < 0 || mode > 2) return fail(GBVR_EINVAL, "empty skipping mode must be 0, 1 or 2");
  r->empty_skip = mode;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_autotune(gbvr_renderer* r, const gbvr_view* views, int n, gbvr_tune_result* out) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  if (!views || n <= 0) return fail(GBVR_EINVAL, "no tuning views");
  const int tiles[] = {4, 8, 16, 32};
  const int ctas[] = {0, 4, 6};
  float best = INFINITY, def = INFINITY;
  int bt = 8, bc = 0, count = 0;
  for (int tw : tiles)
    for (int c : ctas) {
      r->tile_w = tw;
      r->ctas_per_sm = c;
      TRY(paint_batch(r, views, n));  // warm-up (and graph instantiation)
      TRY(paint_batch(r, views, n));
      float ms = r->last_kernel_ms;
      ++count;
      if (tw == TILE_W && c == 0) def = ms;
      if (ms < best) { best = ms; bt = tw; bc = c; }
    }
  r->tile_w = bt;
  r->ctas_per_sm = bc;
  if (out) {
    out->tile_w = bt;
    out->ctas_per_sm = bc;
    out->candidates = count;
    out->best_ms = best;
    out->default_ms = def;
  }
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_samples_per_step(gbvr_renderer* r, int sps) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (sps != 1 && sps != 2 && sps != 4 && sps != 8) return fail(GBVR_EINVAL, "samples per step must be 1, 2, 4 or 8");
  r->samples_per_step = sps;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_autotune_ex(gbvr_renderer* r, const gbvr_view* views, int n, const gbvr_tune_params* tp,
                     gbvr_tune_result_ex* out) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  if (!views || n <= 0) return fail(GBVR_EINVAL, "no tuning views");
  if (r->ds.ooc) return fail(GBVR_ESTATE, "the extended autotuner rebuilds the dataset: in-core datasets only");
  TRY(settle_async(r));
  std::vector<int> bricks, spss;
  for (int i = 0; i < 4 && tp && tp->brick_sizes[i] > 0; ++i) bricks.push_back(tp->brick_sizes[i]);
  for (int i = 0; i < 4 && tp && tp->samples_per_step[i] > 0; ++i) spss.push_back(tp->samples_per_step[i]);
  for (int b : bricks)
    if (b - 2 * r->ds.ghost < 8 || b > 2048) return fail(GBVR_EINVAL, "brick size out of range");
  for (int v : spss)
    if (v != 1 && v != 2 && v != 4 && v != 8) return fail(GBVR_EINVAL, "samples per step must be 1, 2, 4 or 8");
  const int brick0 = r->ds.brick;
  if (bricks.empty()) bricks.push_back(brick0);
  if (spss.empty()) spss.push_back(r->samples_per_step);
  // the finest level, reassembled from the bricks' interiors, for the rebuilds
  DevBuf level0;
  gbvr_brick_params bp = {};
  const long long dims[3] = {r->ds.dims[0], r->ds.dims[1], r->ds.dims[2]};
  const size_t lbytes = (size_t)dims[0] * dims[1] * dims[2] * dtype_size(r->ds.dtype);
  const bool rebuild = bricks.size() > 1 || bricks[0] != brick0;
  if (rebuild) {
    const Level& L0 = r->ds.levels[0];
    CUDA_TRY(level0.alloc(lbytes));
    CUDA_TRY(launch_scatter_interiors(r->ds.pool.p, r->ds.dtype, r->ds.d_bricks.as<BrickInfo>() + L0.brick_base,
                                      L0.nbricks, dims, level0.p, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    bp.overlap = r->ds.ghost;
    bp.layouts = r->ds.layouts;
    bp.build_texture = r->ds.texs.empty() ? 0 : 1;
    for (int a = 0; a < 3; ++a) bp.aspect[a] = r->ds.aspect[a];
  }
  auto build_at = [&](int b) -> int {
    if (r->ds.brick == b && r->ds.loaded) return GBVR_OK;
    DevBuf lv;
    CUDA_TRY(lv.alloc(lbytes));
    CUDA_TRY(cudaMemcpyAsync(lv.p, level0.p, lbytes, cudaMemcpyDeviceToDevice, r->stream));
    bp.brick_size = b;
    r->drop_graphs();
    r->skip_dirty = true;
    r->tf_dirty = true;
    r->occ_valid.clear();
    return build_dataset(r->ds, lv, r->ds.dtype, dims, &bp, r->stream);
  };
  const int tiles[] = {4, 8, 16, 32};
  const int ctas[] = {0, 4, 6};
  float best = INFINITY, def = INFINITY, worst = 0.f;
  int bt = TILE_W, bc = 0, bb = brick0, bs = 1, count = 0;
  // the current brick size first, so the default combination is measured on it
  std::stable_partition(bricks.begin(), bricks.end(), [&](int b) { return b == brick0; });
  for (int b : bricks) {
    TRY(build_at(b));
    for (int v : spss)
      for (int tw : tiles)
        for (int c : ctas) {
          r->samples_per_step = v;
          r->tile_w = tw;
          r->ctas_per_sm = c;
          TRY(paint_batch(r, views, n));  // warm-up (and graph instantiation)
          TRY(paint_batch(r, views, n));
          const float ms = r->last_kernel_ms;
          ++count;
          if (b == brick0 && v == 1 && tw == TILE_W && c == 0) def = ms;
          worst = std::max(worst, ms);
          if (ms < best) {
            best = ms;
            bt = tw;
            bc = c;
            bb = b;
            bs = v;
          }
        }
  }
  TRY(build_at(bb));
  r->tile_w = bt;
  r->ctas_per_sm = bc;
  r->samples_per_step = bs;
  if (out) {
    out->tile_w = bt;
    out->ctas_per_sm = bc;
    out->brick_size = bb;
    out->samples_per_step = bs;
    out->candidates = count;
    out->best_ms = best;
    out->default_ms = def;
    out->worst_ms = worst;
  }
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_paint(gbvr_renderer* r) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  TRY(settle_async(r));
  // One view: the per-view kernel.  A one-view persistent launch measured no
  // faster (1063 vs 1109 frames/s at 1920x1080): a single frame's time is set
  // by its slowest ray tiles, which only other views' work can hide.
  return paint_plain(r, nullptr, 1);
  GBVR_ABI_CATCH
}

int gbvr_paint_batch_async(gbvr_renderer* r, const gbvr_view* views, int n, int slot) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  if (!views || n <= 0) return fail(GBVR_EINVAL, "bad view list");
  if (slot < 0 || slot > 1) return fail(GBVR_EINVAL, "slot must be 0 or 1");
  if (r->ds.ooc) return fail(GBVR_ESTATE, "asynchronous batches need an in-core dataset");
  // each resource on its own: a captured path may have made the read stream
  if (!r->read_stream) CUDA_TRY(cudaStreamCreateWithFlags(&r->read_stream, cudaStreamNonBlocking));
  if (!r->read_stream2) CUDA_TRY(cudaStreamCreateWithFlags(&r->read_stream2, cudaStreamNonBlocking));
  if (!r->read2_done) CUDA_TRY(cudaEventCreateWithFlags(&r->read2_done, cudaEventDisableTiming));
  for (int k = 0; k < 2; ++k) {
    if (!r->slot_rendered[k]) CUDA_TRY(cudaEventCreateWithFlags(&r->slot_rendered[k], cudaEventDisableTiming));
    if (!r->slot_read[k]) CUDA_TRY(cudaEventCreateWithFlags(&r->slot_read[k], cudaEventDisableTiming));
  }
  r->select_slot(slot);
  return paint_batch(r, views, n, true);
  GBVR_ABI_CATCH
}

int gbvr_read_framebuffers_async(gbvr_renderer* r, int slot, int first, int n, void* host, size_t bytes) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (slot < 0 || slot > 1 || !r->read_stream || !r->read2_done || !r->slot_render_pending[slot])
    return fail(GBVR_ESTATE, "no asynchronous batch rendered into that slot");
  const bool cur = slot == r->cur_slot;
  const int w = cur ? r->fb_w : r->other.fb_w, h = cur ? r->fb_h : r->other.fb_h;
  const int views = cur ? r->fb_views : r->other.fb_views;
  const void* fb = cur ? r->d_fb8.p : r->other.fb8.p;
  const size_t per = (size_t)w * h * 4;
  if (first < 0 || n <= 0 || first + n > views) return fail(GBVR_EINVAL, "view range out of range");
  if (!host || bytes < per * n) return fail(GBVR_EINVAL, "host buffer too small");
  CUDA_TRY(cudaStreamWaitEvent(r->read_stream, r->slot_rendered[slot], 0));
  const int n2 = (r->read_stream2 && n >= 2) ? n / 2 : 0;  // frames on the second stream
  if (n2 > 0) {
    CUDA_TRY(cudaStreamWaitEvent(r->read_stream2, r->slot_rendered[slot], 0));
    CUDA_TRY(cudaMemcpyAsync((char*)host + per * (n - n2), (const char*)fb + per * (first + n - n2), per * n2,
                             cudaMemcpyDeviceToHost, r->read_stream2));
    CUDA_TRY(cudaEventRecord(r->read2_done, r->read_stream2));
  }
  CUDA_TRY(cudaMemcpyAsync(host, (const char*)fb + per * first, per * (n - n2), cudaMemcpyDeviceToHost,
                           r->read_stream));
  if (n2 > 0) CUDA_TRY(cudaStreamWaitEvent(r->read_stream, r->read2_done, 0));
  CUDA_TRY(cudaEventRecord(r->slot_read[slot], r->read_stream));
  r->slot_read_pending[slot] = true;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_clearview(gbvr_renderer* r, int enabled, float iso, const float rgb[3], float size, float context_scale,
                       float border_scale, float focus_x, float focus_y) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  TRY(settle_async(r));
  if (enabled && !(size > 0.f)) return fail(GBVR_EINVAL, "lens size must be positive");
  r->cv_on = enabled ? 1 : 0;
  r->cv_iso = iso;
  if (rgb) for (int k = 0; k < 3; ++k) r->cv_rgb[k] = rgb[k];
  r->cv_size = size;
  r->cv_context = context_scale;
  r->cv_border = border_scale;
  r->cv_fx = focus_x;
  r->cv_fy = focus_y;
  r->skip_dirty = true;  // classification uses the lower iso value while on
  r->drop_graphs();
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_bboxes(gbvr_renderer* r, int global, int local, const float global_rgb[3], const float local_rgb[3]) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  TRY(settle_async(r));
  r->bbox_global = global ? 1 : 0;
  r->bbox_local = local ? 1 : 0;
  for (int k = 0; k < 3; ++k) {
    if (global_rgb) r->bbox_rgb[0][k] = global_rgb[k];
    if (local_rgb) r->bbox_rgb[1][k] = local_rgb[k];
  }
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_wait_read(gbvr_renderer* r, int slot) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (slot < 0 || slot > 1) return fail(GBVR_EINVAL, "slot must be 0 or 1");
  if (!r->read_stream || !r->slot_read_pending[slot]) return GBVR_OK;
  // read-backs share one stream: the slot's last event covers all of them
  CUDA_TRY(cudaEventSynchronize(r->slot_read[slot]));
  r->slot_read_pending[slot] = false;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_wait_async(gbvr_renderer* r) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  CUDA_TRY(cudaStreamSynchronize(r->stream));
  if (r->read_stream) CUDA_TRY(cudaStreamSynchronize(r->read_stream));
  for (int k = 0; k < 2; ++k) r->slot_render_pending[k] = r->slot_read_pending[k] = false;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_paint_views(gbvr_renderer* r, const gbvr_view* views, int n) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  TRY(settle_async(r));
  if (!views) return fail(GBVR_EINVAL, "null views");
  return paint_plain(r, views, n);
  GBVR_ABI_CATCH
}

int gbvr_paint_batch(gbvr_renderer* r, const gbvr_view* views, int n) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  TRY(settle_async(r));
  if (!views) return fail(GBVR_EINVAL, "null views");
  return paint_batch(r, views, n);
  GBVR_ABI_CATCH
}

int gbvr_read_framebuffer(gbvr_renderer* r, int view, uint8_t* rgba8, size_t bytes) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  TRY(settle_async(r));
  const size_t need = (size_t)r->fb_w * r->fb_h * 4;
  if (view < 0 || view >= r->last_views) return fail(GBVR_EINVAL, "view index out of range");
  if (!rgba8 || bytes < need) return fail(GBVR_EINVAL, "framebuffer buffer too small");
  CUDA_TRY(cudaMemcpyAsync(rgba8, (const char*)r->d_fb8.p + need * view, need, cudaMemcpyDeviceToHost, r->stream));
  CUDA_TRY(cudaStreamSynchronize(r->stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_read_framebuffers(gbvr_renderer* r, int first, int n, uint8_t* rgba8, size_t bytes) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  TRY(settle_async(r));
  const size_t per = (size_t)r->fb_w * r->fb_h * 4;
  if (first < 0 || n <= 0 || first + n > r->last_views) return fail(GBVR_EINVAL, "view range out of range");
  if (!rgba8 || bytes < per * n) return fail(GBVR_EINVAL, "framebuffer buffer too small");
  CUDA_TRY(cudaMemcpyAsync(rgba8, (const char*)r->d_fb8.p + per * first, per * n, cudaMemcpyDeviceToHost, r->stream));
  CUDA_TRY(cudaStreamSynchronize(r->stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_read_framebuffer_f32(gbvr_renderer* r, int view, float* rgba, size_t bytes) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  TRY(settle_async(r));
  if (!r->d_fb32.p) return fail(GBVR_ESTATE, "renderer was created without the float framebuffer flag (1)");
  const size_t need = (size_t)r->fb_w * r->fb_h * 16;
  if (view < 0 || view >= r->last_views) return fail(GBVR_EINVAL, "view index out of range");
  if (!rgba || bytes < need) return fail(GBVR_EINVAL, "framebuffer buffer too small");
  CUDA_TRY(cudaMemcpyAsync(rgba, (const char*)r->d_fb32.p + need * view, need, cudaMemcpyDeviceToHost, r->stream));
  CUDA_TRY(cudaStreamSynchronize(r->stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_capture_single_frame(gbvr_renderer* r, const char* path, int preserve_transparency) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!path) return fail(GBVR_EINVAL, "null path");
  if (r->last_views < 1) return fail(GBVR_ESTATE, "nothing painted yet");
  std::vector<uint8_t> px((size_t)r->fb_w * r->fb_h * 4);
  TRY(gbvr_read_framebuffer(r, 0, px.data(), px.size()));
  if (!write_image(path, px.data(), r->fb_w, r->fb_h, preserve_transparency != 0))
    return fail(GBVR_EIO, std::string("cannot write ") + path);
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_capture_view(gbvr_renderer* r, int view, const char* path, int preserve_transparency) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!path) return fail(GBVR_EINVAL, "null path");
  if (view < 0 || view >= r->last_views) return fail(GBVR_EINVAL, "view index out of range");
  std::vector<uint8_t> px((size_t)r->fb_w * r->fb_h * 4);
  TRY(gbvr_read_framebuffer(r, view, px.data(), px.size()));
  if (!write_image(path, px.data(), r->fb_w, r->fb_h, preserve_transparency != 0))
    return fail(GBVR_EIO, std::string("cannot write ") + path);
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_get_stats(gbvr_renderer* r, gbvr_stats* out) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (!out) return fail(GBVR_EINVAL, "null stats");
  memset(out, 0, sizeof(*out));
  out->frames = (uint64_t)r->last_views;
  out->lod = r->last_level;
  out->subframes = 1;
  out->gpu_ms = r->last_ms;
  out->kernel_ms = r->last_kernel_ms;
  out->h2d_bytes = r->last_h2d + (r->ds.compression ? r->last_paged_comp : r->last_paged);
  out->brick_misses = r->last_misses;
  out->bytes_paged = r->last_paged;
  out->bytes_paged_compressed = r->last_paged_comp;
  out->host_copies = r->last_host_copies;
  out->page_ms = r->last_page_ms;
  if (r->last_views < 1 || !r->ds.loaded) return GBVR_OK;
  const int n = r->last_views;
  const Level& L = r->ds.levels[r->last_level];
  std::vector<unsigned long long> s(n);
  std::vector<unsigned char> t((size_t)n * L.nbricks), skip(L.nbricks);
  CUDA_TRY(cudaMemcpyAsync(s.data(), r->d_samples.p, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, r->stream));
  CUDA_TRY(cudaMemcpyAsync(t.data(), r->d_touched.p, t.size(), cudaMemcpyDeviceToHost, r->stream));
  CUDA_TRY(cudaMemcpyAsync(skip.data(), r->d_skip.as<unsigned char>() + L.brick_base, L.nbricks, cudaMemcpyDeviceToHost, r->stream));
  CUDA_TRY(cudaStreamSynchronize(r->stream));
  const size_t es = dtype_size(r->ds.dtype);
  for (int v = 0; v < n; ++v) {
    out->samples += s[v];
    for (int b = 0; b < L.nbricks; ++b)
      if (t[(size_t)v * L.nbricks + b]) {
        const BrickInfo& bi = r->ds.bricks[L.brick_base + b];
        out->bricks_touched++;
        out->brick_bytes += (uint64_t)bi.sx * bi.sy * bi.sz * es;
      }
  }
  for (int b = 0; b < L.nbricks; ++b) out->bricks_skipped += skip[b];
  if (r->stats_level >= 2 && r->empty_skip >= 2 && r->d_cellbits.p) {
    std::vector<unsigned long long> cc(n);
    CUDA_TRY(cudaMemsetAsync(r->d_cellcount.p, 0, sizeof(unsigned long long) * n, r->stream));
    CUDA_TRY(launch_count_bits(r->d_cellbits.as<unsigned>(), r->cell_words, n, r->d_cellcount.as<unsigned long long>(),
                               r->stream));
    CUDA_TRY(cudaMemcpyAsync(cc.data(), r->d_cellcount.p, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    const uint64_t cell_vox = (uint64_t)1 << (3 * L.cell_shift);
    for (int v = 0; v < n; ++v) {
      out->cells_touched += cc[v];
      out->cell_bytes += cc[v] * cell_vox * es;
    }
  }
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_stats_level(gbvr_renderer* r, int level) {
  GBVR_ABI_TRY
  TRY(check_r(r));
  if (level < 0 || level > 2) return fail(GBVR_EINVAL, "stats level must be 0, 1 or 2");
  r->stats_level = level;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_write_uvf(gbvr_renderer* r, const char* path) {
  GBVR_ABI_TRY
  TRY(check_loaded(r));
  if (!path) return fail(GBVR_EINVAL, "null path");
  if (r->ds.ooc) return fail(GBVR_EINVAL, "out-of-core datasets are not written back as one raster");
  const Dataset& ds = r->ds;
  // LOD 0 re-assembled from its bricks' interiors
  const size_t es = dtype_size(ds.dtype);
  const size_t bytes = (size_t)ds.dims[0] * ds.dims[1] * ds.dims[2] * es;
  std::vector<unsigned char> vol(bytes);
  const Level& L = ds.levels[0];
  std::vector<unsigned char> tmp;
  for (int i = 0; i < L.nbricks; ++i) {
    const BrickInfo& b = ds.bricks[L.brick_base + i];
    tmp.resize((size_t)b.sx * b.sy * b.sz * es);
    CUDA_TRY(cudaMemcpy(tmp.data(), (const char*)ds.pool.p + b.offset * es, tmp.size(), cudaMemcpyDeviceToHost));
    int lo[3] = {std::max(b.lox, 0), std::max(b.loy, 0), std::max(b.loz, 0)};
    int hi[3] = {b.hix, b.hiy, b.hiz};
    for (int z = lo[2]; z < hi[2]; ++z)
      for (int y = lo[1]; y < hi[1]; ++y)
        memcpy(&vol[(((size_t)z * ds.dims[1] + y) * ds.dims[0] + lo[0]) * es],
               &tmp[(((size_t)(z - b.oz) * b.sy + (y - b.oy)) * b.sx + (lo[0] - b.ox)) * es], (size_t)(hi[0] - lo[0]) * es);
  }
  UvfWriteSpec s;
  s.raster.id = ds.raster_id;
  for (int a = 0; a < 3; ++a) {
    s.raster.dims[a] = (uint64_t)ds.dims[a];
    s.raster.brick_size[a] = (uint64_t)ds.brick;
    s.raster.overlap[a] = (uint64_t)(2 * ds.ghost);
  }
  for (int i = 0; i < 16; ++i) s.raster.transform[i] = (i % 5 == 0) ? 1.0 : 0.0;
  for (int a = 0; a < 3; ++a) s.raster.transform[5 * a] = ds.aspect[a];
  s.raster.lod_counts = {1};
  s.raster.bit_size = ds.dtype == DT_U8 ? 8 : ds.dtype == DT_U16 ? 16 : 32;
  s.raster.mantissa = ds.dtype == DT_F32 ? 23 : s.raster.bit_size;
  s.raster.is_signed = ds.dtype == DT_F32;
  s.voxels = vol.data();
  s.voxel_bytes = bytes;
  s.hist1d = ds.hist1d;
  s.hist2d = ds.hist2d;
  s.hist2d_nx = ds.hist1d.size();
  s.hist2d_ny = ds.hist2d.empty() ? 0 : 256;
  s.hist2d_max_grad = ds.max_grad;
  // MaxMinDataBlock(1): one entry per stored brick of LOD 0, gradients not
  // computed (DataSource.h:467-469; c60.uvf stores -DBL_MAX / +DBL_MAX)
  for (int i = 0; i < L.nbricks; ++i) {
    const BrickInfo& b = ds.bricks[L.brick_base + i];
    s.minmax.push_back({(double)b.vmin, (double)b.vmax, -1.7976931348623157e308, 1.7976931348623157e308});
  }
  std::string msg;
  int rc = uvf_write(path, s, msg);
  if (rc) return fail(rc, msg);
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_build_uvf(const void* host, const int64_t dims[3], int dtype, const gbvr_brick_params* bp, const char* out_path) {
  GBVR_ABI_TRY
  gbvr_renderer* r = nullptr;
  TRY(gbvr_create(GBVR_CUDA_RAYCASTER, 0, &r));
  std::unique_ptr<gbvr_renderer> hold(r);
  TRY(gbvr_load_volume(r, host, dims, dtype, bp));
  return gbvr_write_uvf(r, out_path);
  GBVR_ABI_CATCH
}

static_assert(sizeof(gbvr_zchunk) == sizeof(Lz4Chunk) && offsetof(gbvr_zchunk, comp) == offsetof(Lz4Chunk, comp),
              "gbvr_zchunk is the decoders' chunk record");

int gbvr_dev_zlib_decode(const void* dev_src, void* dev_dst, const gbvr_zchunk* dev_chunks, int n, int* dev_err,
                         void* stream) {
  GBVR_ABI_TRY
  if (n < 0 || (n > 0 && (!dev_src || !dev_dst || !dev_chunks || !dev_err))) return fail(GBVR_EINVAL, "bad arguments");
  CUDA_TRY(launch_inflate(dev_src, dev_dst, reinterpret_cast<const Lz4Chunk*>(dev_chunks), n, dev_err,
                          (cudaStream_t)stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_dev_lz4_decode(const void* dev_src, void* dev_dst, const gbvr_zchunk* dev_chunks, int n, int* dev_err,
                        void* stream) {
  GBVR_ABI_TRY
  if (n < 0 || (n > 0 && (!dev_src || !dev_dst || !dev_chunks || !dev_err))) return fail(GBVR_EINVAL, "bad arguments");
  CUDA_TRY(launch_lz4_decode(dev_src, dev_dst, reinterpret_cast<const Lz4Chunk*>(dev_chunks), n, dev_err,
                             (cudaStream_t)stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_dev_hist1d(const void* dev_vol, int dtype, int64_t n, uint64_t* dev_hist, int nbins, void* stream) {
  GBVR_ABI_TRY
  if (!dev_vol || !dev_hist || n < 0 || nbins <= 0) return fail(GBVR_EINVAL, "bad argument");
  CUDA_TRY(launch_hist1d(dev_vol, dtype, n, (unsigned long long*)dev_hist, nbins, (cudaStream_t)stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_dev_hist2d(const void* dev_vol, int dtype, const int64_t dims[3], double max_scalar, int64_t nx,
                    int64_t merge, uint64_t* dev_hist, float* max_grad, void* stream) {
  GBVR_ABI_TRY
  if (!dev_vol || !dev_hist || !dims || nx <= 0 || merge <= 0) return fail(GBVR_EINVAL, "bad argument");
  DevBuf sc;
  CUDA_TRY(sc.alloc(sizeof(Hist2DScratch)));
  long long d[3] = {dims[0], dims[1], dims[2]};
  CUDA_TRY(launch_hist2d(dev_vol, dtype, d, max_scalar, nx, merge, (unsigned long long*)dev_hist, sc.as<Hist2DScratch>(),
                         (cudaStream_t)stream));
  Hist2DScratch hs;
  CUDA_TRY(cudaMemcpyAsync(&hs, sc.p, sizeof(hs), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  double g;
  memcpy(&g, &hs.gmax_bits, 8);
  if (max_grad) *max_grad = (float)g;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_dev_downsample(const void* dev_in, int dtype, const int64_t dims[3], void* dev_out, void* stream) {
  GBVR_ABI_TRY
  if (!dev_in || !dev_out || !dims) return fail(GBVR_EINVAL, "bad argument");
  long long d[3] = {dims[0], dims[1], dims[2]};
  CUDA_TRY(launch_downsample(dev_in, dtype, d, dev_out, (cudaStream_t)stream));
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_look_at_camera(const float eye[3], const float ref[3], const float up[3], float fov_deg, float znear,
                        float zfar, int width, int height, float view[16], float proj[16]) {
  GBVR_ABI_TRY
  if (!eye || !ref || !up || !view || !proj || width <= 0 || height <= 0 || !(znear > 0) || !(zfar > znear))
    return fail(GBVR_EINVAL, "bad camera");
  double e[3] = {eye[0], eye[1], eye[2]}, c[3] = {ref[0], ref[1], ref[2]}, u[3] = {up[0], up[1], up[2]};
  const double f[3] = {c[0] - e[0], c[1] - e[1], c[2] - e[2]};
  const double x[3] = {f[1] * u[2] - f[2] * u[1], f[2] * u[0] - f[0] * u[2], f[0] * u[1] - f[1] * u[0]};
  if (!(x[0] * x[0] + x[1] * x[1] + x[2] * x[2] > 0)) return fail(GBVR_EINVAL, "camera direction parallel to up");
  double V[16], P[16];
  look_at(e, c, u, V);
  perspective(fov_deg, (double)width / height, znear, zfar, P);
  for (int i = 0; i < 16; ++i) { view[i] = (float)V[i]; proj[i] = (float)P[i]; }
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_orbit_camera(float azimuth_deg, float elevation_deg, float radius, float fov_deg, int width, int height,
                      float view[16], float proj[16]) {
  GBVR_ABI_TRY
  if (!view || !proj || width <= 0 || height <= 0 || !(radius > 0)) return fail(GBVR_EINVAL, "bad camera");
  orbit(azimuth_deg, elevation_deg, radius, fov_deg, width, height, view, proj);
  return GBVR_OK;
  GBVR_ABI_CATCH
}

}  // extern "C"

// ===========================================================================
// Serving loop: many datasets and transfer functions, requests from any
// thread, continuous batching into graph-replayed persistent launches.
//
// A worker thread owns the GPU side and keeps up to `slots` batches in
// flight, each on its own stream.  Whenever a slot is free and requests are
// pending it assembles a batch and launches it at once, so a batch starts
// while earlier ones still run and its ray tiles take the SMs their tails
// leave idle.  A batch takes pending requests in arrival order until it holds
// max_batch of them or its framebuffer share (fb_budget_bytes / slots) is
// full.  Its requests are grouped by (voxel type, mode) -- group index
// dtype * 4 + mode -- and each group is one persistent launch
// (k_render_persistent_g) whose frames, count and tile prefix come from a
// device table, so the launches of a slot are captured once per set of
// groups and replayed.  Each group has its own launch shape (tile width, CTAs
// per SM; gbvr_server_autotune).  A host function queued behind a slot's
// read-back wakes the worker when it is done (no polling).
//
// Admission by memory: with device_pool_bytes > 0 every dataset's brick pool
// is copied to page-locked host memory when it is added and made resident on
// demand: a request whose dataset is not resident is admitted once the pool
// fits the budget, evicting idle datasets (no batch in flight uses them)
// least recently used first; the upload runs on the batch's stream ahead of
// its kernels, and later batches on other streams wait for it by event.
// Requests behind one that must wait are not held up.  Every ray is computed
// independently of its batch, so a request's image is the same alone and in
// any mix.
// ===========================================================================
#include <chrono>
#include <condition_variable>
#include <deque>
#include <list>
#include <map>
#include <thread>
#include <unordered_map>

namespace {

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

constexpr int kServerGroups = 12;     // 3 voxel types x 4 render modes
constexpr int kMaxServerSlots = 8;
constexpr int kEventRing = 64;        // per-batch kernel-span events, reused every kEventRing batches

struct ServerTf {
  int dataset = 0;
  int mode = GBVR_RM_1DTRANS, w = 0, h = 1, level = 0;
  std::vector<float> host;
  DevBuf d_tf, d_prefix, d_skip, d_occ, d_occtmp;
  double lo = 0, hi = 1;
  float grad_max = 0.f, iso = 0.f, iso_rgb[3] = {1, 1, 1};
};

struct ServerDataset {
  std::unique_ptr<Dataset> ds;
  size_t pool_bytes = 0;
  bool resident = true;
  bool async_pool = false;        // the device pool came from cudaMallocAsync
  PinnedBuf host_pool;            // page-locked copy of the pool (under a memory budget)
  int inflight = 0;               // batches in flight that use it
  uint64_t last_use = 0;          // sequence number of the last batch that used it
  cudaEvent_t uploaded = nullptr; // recorded behind its last upload
  bool ever_uploaded = false;
};

struct ServerRequest {
  gbvr_request req;
  uint64_t ticket = 0;
  double t_submit = 0, t_launch = 0, t_done = 0;
  int status = 1;  // 1 pending, 0 done, < 0 error
  int batch_size = 0;
  uint64_t batch = 0;
  double gpu_ms = 0;
};

struct GroupShape {
  int tile_w = TILE_W;
  int ctas_per_sm = 0;  // 0 = as many as fit
};

struct BatchSlot {
  gbvr_server* server = nullptr;
  int index = 0;
  cudaStream_t stream = nullptr;
  DevBuf d_frames, d_prefix, d_counter, d_samples, d_fb, d_groups;
  PinnedBuf h_frames, h_prefix, h_fb, h_groups;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<ServerRequest*> reqs;
  std::vector<size_t> fb_off;
  // per request, taken under the server's mutex (the worker then reads no
  // server container): its dataset, TF preset and group (dtype * 4 + mode)
  std::vector<const Dataset*> req_ds;
  std::vector<const ServerTf*> req_tf;
  std::vector<int> req_gi;
  std::vector<int> datasets;      // distinct datasets of the batch
  std::vector<ServerDataset*> dsets;  // ... and their records (upload events)
  size_t fb_used = 0;
  bool busy = false;
  bool done = false;              // set by the host function behind the batch
  uint64_t seq = 0;
  unsigned shape_version = 0;
  std::map<unsigned, cudaGraphExec_t> graphs;  // by set of groups present (bit gi)
};

}  // namespace

struct gbvr_server {
  gbvr_server_params params;
  int device = 0;
  int sm_count = 0, max_ctas[4] = {1, 1, 1, 1};
  int nslots = 3;
  cudaStream_t stream = nullptr;          // dataset builds, TF classification
  cudaStream_t capture_stream = nullptr;  // graph capture only
  std::vector<std::unique_ptr<ServerDataset>> datasets;
  std::vector<std::unique_ptr<ServerTf>> tfs;
  std::vector<std::unique_ptr<BatchSlot>> slots;
  GroupShape shape[kServerGroups];
  unsigned shape_version = 1;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<ServerRequest*> pending;
  std::unordered_map<uint64_t, std::unique_ptr<ServerRequest>> reqs;
  uint64_t next_ticket = 1, next_batch = 1;
  bool stop = false;
  bool blocked = false;   // the pending requests cannot be admitted until something changes
  bool tuning = false;    // the autotuner owns the slots
  std::string worker_error;
  std::thread worker;
  size_t resident_bytes = 0;
  // kernel spans per batch (ring by sequence number) for the overlap count
  cudaEvent_t k0[kEventRing] = {}, k1[kEventRing] = {};
  bool span_done[kEventRing] = {};
  uint64_t span_seq[kEventRing] = {};
  // statistics since the last reset
  std::vector<double> latencies;
  uint64_t submitted = 0, completed = 0, batches = 0, batched_requests = 0;
  uint64_t overlap_checked = 0, overlapped = 0, uploads = 0, evictions = 0, upload_bytes = 0;
  double t_first = -1, t_last = 0;

  ~gbvr_server() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    for (auto& sl : slots) {
      if (sl->stream) cudaStreamSynchronize(sl->stream);
      for (auto& g : sl->graphs) cudaGraphExecDestroy(g.second);
      if (sl->ev0) cudaEventDestroy(sl->ev0);
      if (sl->ev1) cudaEventDestroy(sl->ev1);
    }
    for (auto& d : datasets) {
      if (d->async_pool && d->ds->pool.p) {
        cudaFreeAsync(d->ds->pool.p, stream);
        d->ds->pool.p = nullptr;
        d->ds->pool.n = 0;
      }
      if (d->uploaded) cudaEventDestroy(d->uploaded);
    }
    if (stream) cudaStreamSynchronize(stream);
    for (int i = 0; i < kEventRing; ++i) {
      if (k0[i]) cudaEventDestroy(k0[i]);
      if (k1[i]) cudaEventDestroy(k1[i]);
    }
    for (auto& sl : slots)
      if (sl->stream) cudaStreamDestroy(sl->stream);
    if (capture_stream) cudaStreamDestroy(capture_stream);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int group_of(const gbvr_server* s, const ServerRequest* q) {
  return s->datasets[q->req.dataset]->ds->dtype * 4 + s->tfs[q->req.tf]->mode;
}

int group_grid(const gbvr_server* s, int gi, const GroupShape& sh) {
  const int m = gi & 3;
  const int ctas = sh.ctas_per_sm > 0 ? std::min(sh.ctas_per_sm, s->max_ctas[m]) : s->max_ctas[m];
  return s->sm_count * std::max(1, ctas);
}

// Host function queued behind a slot's read-back: the slot may be retired.
void CUDART_CB slot_done_cb(void* arg) {
  BatchSlot* sl = static_cast<BatchSlot*>(arg);
  gbvr_server* s = sl->server;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    sl->done = true;
  }
  s->cv_work.notify_all();
}

// Evict idle datasets (least recently used first, none of `keep`) until
// `need` more bytes fit the budget; then allocate and upload the pool of D on
// stream st.  Worker thread, mutex held.  Returns false when it cannot fit now.
bool make_resident(gbvr_server* s, ServerDataset& D, cudaStream_t st, const std::vector<int>& keep, int& rc) {
  rc = GBVR_OK;
  const size_t budget = s->params.device_pool_bytes;
  while (s->resident_bytes + D.pool_bytes > budget) {
    ServerDataset* victim = nullptr;
    for (size_t i = 0; i < s->datasets.size(); ++i) {
      ServerDataset& c = *s->datasets[i];
      if (!c.resident || c.inflight > 0 || &c == &D) continue;
      if (std::find(keep.begin(), keep.end(), (int)i) != keep.end()) continue;
      if (!victim || c.last_use < victim->last_use) victim = &c;
    }
    if (!victim) return false;
    // stream-ordered: no batch in flight reads it, and no device-wide synchronisation
    cudaError_t e = cudaFreeAsync(victim->ds->pool.p, st);
    if (e != cudaSuccess) { rc = cuda_fail(e, "cudaFreeAsync"); return false; }
    victim->ds->pool.p = nullptr;
    victim->ds->pool.n = 0;
    victim->resident = false;
    s->resident_bytes -= victim->pool_bytes;
    ++s->evictions;
  }
  void* p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, D.pool_bytes, st);
  if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMallocAsync (brick pool)"); return false; }
  e = cudaMemcpyAsync(p, D.host_pool.p, D.pool_bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaEventRecord(D.uploaded, st);
  if (e != cudaSuccess) {
    cudaFreeAsync(p, st);
    rc = cuda_fail(e, "brick pool upload");
    return false;
  }
  D.ds->pool.p = p;
  D.ds->pool.n = D.pool_bytes;
  D.async_pool = true;
  D.resident = true;
  D.ever_uploaded = true;
  s->resident_bytes += D.pool_bytes;
  ++s->uploads;
  s->upload_bytes += D.pool_bytes;
  return true;
}

// Queue the batch of `slot` on its stream: descriptors, background fill, one
// persistent launch per group present (captured once per set of groups and
// replayed; `force` launches every group with one shape directly instead, for
// the autotuner), the read-back and the completion host function.  Worker
// thread (or the autotuner), mutex released.  gpu_spans: record the kernel
// span events of the batch's ring entry.
int launch_batch(gbvr_server* s, BatchSlot& slot, const GroupShape* force, bool gpu_spans) {
  const int n = (int)slot.reqs.size();
  if (!force && fault_injected("server_launch")) throw std::runtime_error("injected failure of a batch launch");
  const int mb = std::max(s->params.max_batch, n);
  CUDA_TRY(slot.d_frames.alloc(sizeof(FrameDesc) * mb));
  CUDA_TRY(slot.d_prefix.alloc(sizeof(int) * (mb + kServerGroups)));
  CUDA_TRY(slot.d_counter.alloc(sizeof(int) * kServerGroups));
  CUDA_TRY(slot.d_samples.alloc(sizeof(unsigned long long) * mb));
  CUDA_TRY(slot.d_groups.alloc(sizeof(LaunchGroup) * kServerGroups));
  CUDA_TRY(slot.h_frames.alloc(sizeof(FrameDesc) * mb));
  CUDA_TRY(slot.h_prefix.alloc(sizeof(int) * (mb + kServerGroups)));
  CUDA_TRY(slot.h_groups.alloc(sizeof(LaunchGroup) * kServerGroups));
  FrameDesc* hf = (FrameDesc*)slot.h_frames.p;
  int* hp = (int*)slot.h_prefix.p;
  LaunchGroup* hg = (LaunchGroup*)slot.h_groups.p;
  for (int g = 0; g < kServerGroups; ++g) hg[g] = LaunchGroup{0, 0, 0, 0};
  unsigned mask = 0;
  int pcur = 0, max_h = 0, cur = -1, total = 0;
  for (int i = 0; i < n; ++i) {
    const ServerRequest* q = slot.reqs[i];
    const Dataset& ds = *slot.req_ds[i];
    const ServerTf& t = *slot.req_tf[i];
    const int gi = slot.req_gi[i];
    const GroupShape& sh = force ? *force : s->shape[gi];
    FrameParams p;
    memset(&p, 0, sizeof(p));
    p.view = q->req.view;
    p.proj = q->req.proj;
    p.width = q->req.width;
    p.height = q->req.height;
    p.spv = q->req.samples_per_voxel > 0 ? q->req.samples_per_voxel : 1.f;
    p.level = t.level;
    p.mode = t.mode;
    p.interp = GBVR_LINEAR;
    p.sampler = GBVR_SAMPLER_SW;
    p.ert = 0.99f;
    p.iso = t.iso;
    p.lighting = 1;
    p.shininess = 8.f;
    for (int k = 0; k < 3; ++k) {
      p.iso_rgb[k] = t.iso_rgb[k];
      p.amb[k] = 0.1f;
      p.diff[k] = 1.f;
      p.spec[k] = 1.f;
      p.light_dir[k] = k == 2 ? -1.f : 0.f;
      p.bg[k] = 0.f;
      p.bg_top[k] = 0.f;
    }
    p.tile_w = sh.tile_w;
    p.empty_skip = 2;
    p.tf = t.d_tf.as<float4>();
    p.tf_w = t.w;
    p.tf_h = t.h;
    p.lo = t.lo;
    p.hi = t.hi;
    p.grad_max = t.grad_max;
    p.skip = t.d_skip.as<unsigned char>();
    p.occ = t.d_occ.as<unsigned char>();
    fill_frame(hf[i], ds, p);
    hf[i].out_rgba8 = (uchar4*)((char*)slot.d_fb.p + slot.fb_off[i]);
    hf[i].samples = slot.d_samples.as<unsigned long long>() + i;
    cull_tiles(hf[i], nullptr, p.view, p.proj);
    max_h = std::max(max_h, p.height);
    if (gi != cur) {
      if (cur >= 0) {
        hp[pcur++] = total;  // closing entry of the previous group
      }
      cur = gi;
      mask |= 1u << gi;
      hg[gi] = LaunchGroup{i, 0, pcur, 0};
      total = 0;
    }
    hp[pcur++] = total;
    total += hf[i].ntx * hf[i].nty;
    ++hg[gi].count;
  }
  if (cur >= 0) hp[pcur++] = total;
  cudaStream_t st = slot.stream;
  // the batch's pools: uploads queued on other streams finish first
  for (const ServerDataset* D : slot.dsets)
    if (D->ever_uploaded) CUDA_TRY(cudaStreamWaitEvent(st, D->uploaded, 0));
  CUDA_TRY(cudaEventRecord(slot.ev0, st));
  CUDA_TRY(cudaMemcpyAsync(slot.d_frames.p, hf, sizeof(FrameDesc) * n, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(slot.d_prefix.p, hp, sizeof(int) * pcur, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(slot.d_groups.p, hg, sizeof(LaunchGroup) * kServerGroups, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(slot.d_counter.p, 0, sizeof(int) * kServerGroups, st));
  CUDA_TRY(cudaMemsetAsync(slot.d_samples.p, 0, sizeof(unsigned long long) * n, st));
  // background outside each request's tile rectangle (frames differ in size:
  // the grid covers the tallest, each block checks its own frame's rows)
  CUDA_TRY(launch_fill_outside(slot.d_frames.as<FrameDesc>(), n, max_h, st));
  const int ring = (int)(slot.seq % kEventRing);
  if (gpu_spans) CUDA_TRY(cudaEventRecord(s->k0[ring], st));
  auto launch_groups = [&](cudaStream_t ls) -> int {
    for (int gi = 0; gi < kServerGroups; ++gi) {
      if (!(mask >> gi & 1)) continue;
      const GroupShape& sh = force ? *force : s->shape[gi];
      CUDA_TRY(launch_render_persistent_group(gi >> 2, gi & 3, slot.d_frames.as<FrameDesc>(),
                                              slot.d_groups.as<LaunchGroup>(), gi, slot.d_prefix.as<int>(),
                                              slot.d_counter.as<int>(), group_grid(s, gi, sh), ls));
    }
    return GBVR_OK;
  };
  if (force) {
    TRY(launch_groups(st));
  } else {
    if (slot.shape_version != s->shape_version) {
      for (auto& g : slot.graphs) cudaGraphExecDestroy(g.second);
      slot.graphs.clear();
      slot.shape_version = s->shape_version;
    }
    auto it = slot.graphs.find(mask);
    if (it == slot.graphs.end()) {
      CUDA_TRY(cudaStreamBeginCapture(s->capture_stream, cudaStreamCaptureModeThreadLocal));
      const int rc = launch_groups(s->capture_stream);
      cudaGraph_t g = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(s->capture_stream, &g);
      if (rc != GBVR_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      CUDA_TRY(ce);
      cudaGraphExec_t ge = nullptr;
      const cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      CUDA_TRY(ie);
      it = slot.graphs.emplace(mask, ge).first;
    }
    CUDA_TRY(cudaGraphLaunch(it->second, st));
  }
  if (gpu_spans) CUDA_TRY(cudaEventRecord(s->k1[ring], st));
  CUDA_TRY(cudaMemcpyAsync(slot.h_fb.p, slot.d_fb.p, slot.fb_used, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaEventRecord(slot.ev1, st));
  CUDA_TRY(cudaLaunchHostFunc(st, slot_done_cb, &slot));
  return GBVR_OK;
}

// Compare the kernel spans of batches a < b (consecutive sequence numbers,
// both complete): overlapped when b's kernels started before a's ended.
void count_overlap(gbvr_server* s, uint64_t a) {
  const int ra = (int)(a % kEventRing), rb = (int)((a + 1) % kEventRing);
  if (!s->span_done[ra] || !s->span_done[rb] || s->span_seq[ra] != a || s->span_seq[rb] != a + 1) return;
  float to_b = 0.f, span_a = 0.f;
  if (cudaEventElapsedTime(&to_b, s->k0[ra], s->k0[rb]) != cudaSuccess) return;
  if (cudaEventElapsedTime(&span_a, s->k0[ra], s->k1[ra]) != cudaSuccess) return;
  ++s->overlap_checked;
  if (to_b < span_a) ++s->overlapped;
}

// Retire a finished slot: pixels to the callers' buffers, statistics.
// Worker thread, mutex held on entry and exit.
void retire(gbvr_server* s, BatchSlot& slot, std::unique_lock<std::mutex>& lk) {
  const cudaError_t e = cudaEventQuery(slot.ev1);
  float ms = 0.f;
  lk.unlock();
  if (e == cudaSuccess) {
    cudaEventElapsedTime(&ms, slot.ev0, slot.ev1);
    for (size_t i = 0; i < slot.reqs.size(); ++i) {
      const ServerRequest* q = slot.reqs[i];
      memcpy(q->req.out_rgba8, (const char*)slot.h_fb.p + slot.fb_off[i], (size_t)q->req.width * q->req.height * 4);
    }
  }
  lk.lock();
  const double t = now_ms();
  for (ServerRequest* q : slot.reqs) {
    q->status = e == cudaSuccess ? GBVR_OK : GBVR_ECUDA;
    q->t_done = t;
    q->gpu_ms = ms;
    if (e == cudaSuccess) {
      s->latencies.push_back(t - q->t_submit);
      ++s->completed;
      s->t_last = t;
    }
  }
  if (e != cudaSuccess) s->worker_error = cudaGetErrorString(e);
  for (int d : slot.datasets) {
    --s->datasets[d]->inflight;
    s->datasets[d]->last_use = std::max(s->datasets[d]->last_use, slot.seq);
  }
  const int ring = (int)(slot.seq % kEventRing);
  s->span_done[ring] = e == cudaSuccess;
  s->span_seq[ring] = slot.seq;
  if (slot.seq > 1) count_overlap(s, slot.seq - 1);
  count_overlap(s, slot.seq);
  ++s->batches;
  s->batched_requests += slot.reqs.size();
  slot.busy = false;
  slot.done = false;
  slot.reqs.clear();
  slot.datasets.clear();
  s->blocked = false;
  s->cv_done.notify_all();
}

// Order the batch's requests by group (each group one contiguous run of
// frames) and take the per-request pointers the launch reads.  Mutex held.
void snapshot_batch(gbvr_server* s, BatchSlot& slot) {
  const int n = (int)slot.reqs.size();
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return group_of(s, slot.reqs[x]) < group_of(s, slot.reqs[y]); });
  std::vector<ServerRequest*> sorted(n);
  std::vector<size_t> offs(n);
  for (int i = 0; i < n; ++i) {
    sorted[i] = slot.reqs[order[i]];
    offs[i] = slot.fb_off[order[i]];
  }
  slot.reqs.swap(sorted);
  slot.fb_off.swap(offs);
  slot.req_ds.resize(n);
  slot.req_tf.resize(n);
  slot.req_gi.resize(n);
  for (int i = 0; i < n; ++i) {
    const ServerRequest* q = slot.reqs[i];
    slot.req_ds[i] = s->datasets[q->req.dataset]->ds.get();
    slot.req_tf[i] = s->tfs[q->req.tf].get();
    slot.req_gi[i] = group_of(s, q);
  }
  slot.dsets.clear();
  for (int d : slot.datasets) slot.dsets.push_back(s->datasets[d].get());
}

// Fill `slot` from the pending requests (arrival order; a request whose
// dataset cannot be made resident now is passed over and stays pending).
// Worker thread, mutex held.  Returns the status of an upload failure.
int assemble(gbvr_server* s, BatchSlot& slot) {
  slot.reqs.clear();
  slot.fb_off.clear();
  slot.datasets.clear();
  const size_t slot_budget = s->params.fb_budget_bytes / s->nslots;
  size_t used = 0;
  for (auto it = s->pending.begin(); it != s->pending.end() && (int)slot.reqs.size() < s->params.max_batch;) {
    ServerRequest* q = *it;
    const size_t aligned = ((size_t)q->req.width * q->req.height * 4 + 255) & ~(size_t)255;
    if (used + aligned > slot_budget) break;  // the framebuffer share is full: the rest wait
    const int d = q->req.dataset;
    ServerDataset& D = *s->datasets[d];
    if (!D.resident) {
      int rc = GBVR_OK;
      if (!make_resident(s, D, slot.stream, slot.datasets, rc)) {
        if (rc != GBVR_OK) return rc;
        ++it;  // waits until its pool fits
        continue;
      }
    }
    it = s->pending.erase(it);
    if (std::find(slot.datasets.begin(), slot.datasets.end(), d) == slot.datasets.end()) slot.datasets.push_back(d);
    slot.reqs.push_back(q);
    slot.fb_off.push_back(used);
    used += aligned;
  }
  slot.fb_used = used;
  snapshot_batch(s, slot);
  return GBVR_OK;
}

void server_worker(gbvr_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  auto any_busy = [&] {
    for (auto& sl : s->slots)
      if (sl->busy) return true;
    return false;
  };
  auto ready = [&] {
    if (s->stop) return true;
    for (auto& sl : s->slots) {
      if (sl->busy && sl->done) return true;
      if (!sl->busy && !s->pending.empty() && !s->blocked && !s->tuning) return true;
    }
    return false;
  };
  for (;;) {
    s->cv_work.wait(lk, ready);
    if (s->stop && s->pending.empty() && !any_busy()) break;
    for (auto& sl : s->slots)
      if (sl->busy && sl->done) retire(s, *sl, lk);
    for (auto& slp : s->slots) {
      BatchSlot& slot = *slp;
      if (slot.busy || s->pending.empty() || s->tuning || s->blocked) continue;
      int rc = assemble(s, slot);
      if (rc == GBVR_OK && slot.reqs.empty()) {
        s->blocked = true;  // nothing admissible until a batch retires or a request arrives
        continue;
      }
      slot.busy = true;
      slot.done = false;
      slot.seq = s->next_batch++;
      const double t = now_ms();
      for (ServerRequest* q : slot.reqs) {
        q->t_launch = t;
        q->batch = slot.seq;
        q->batch_size = (int)slot.reqs.size();
      }
      for (int d : slot.datasets) ++s->datasets[d]->inflight;
      if (rc == GBVR_OK) {
        lk.unlock();
        try {  // the worker thread must not end on an exception: the batch fails instead
          rc = launch_batch(s, slot, nullptr, true);
        } catch (const std::bad_alloc&) {
          rc = fail(GBVR_ENOMEM, "out of host memory");
        } catch (const std::exception& e) {
          rc = fail(GBVR_EINVAL, e.what());
        }
        lk.lock();
      }
      if (rc != GBVR_OK) {
        // the batch never reached the GPU (or only its uploads did): fail its requests
        if (slot.stream) {
          lk.unlock();
          cudaStreamSynchronize(slot.stream);
          lk.lock();
        }
        s->worker_error = g_err;
        for (ServerRequest* q : slot.reqs) {
          q->status = rc;
          q->t_done = now_ms();
        }
        for (int d : slot.datasets) --s->datasets[d]->inflight;
        slot.reqs.clear();
        slot.datasets.clear();
        slot.busy = false;
        slot.done = false;
        s->cv_done.notify_all();
      }
    }
  }
}

int check_s(gbvr_server* s) {
  if (!s) return fail(GBVR_EINVAL, "null server");
  return GBVR_OK;
}

int server_add_dataset(gbvr_server* s, DevBuf& lv, int dtype, const long long d[3], const gbvr_brick_params* bp,
                       int* id) {
  std::unique_ptr<ServerDataset> sd(new ServerDataset());
  sd->ds.reset(new Dataset());
  gbvr_brick_params b = {};
  if (bp) b = *bp;
  if (b.layouts == 0) b.layouts = 4;
  b.build_texture = 0;  // the serving launches sample in software
  TRY(build_dataset(*sd->ds, lv, dtype, d, &b, s->stream));
  sd->pool_bytes = sd->ds->pool.n;
  CUDA_TRY(cudaEventCreateWithFlags(&sd->uploaded, cudaEventDisableTiming));
  if (s->params.device_pool_bytes > 0) {
    if (sd->pool_bytes > s->params.device_pool_bytes)
      return fail(GBVR_EINVAL, "the dataset's brick pool (" + std::to_string(sd->pool_bytes) +
                                   " bytes) exceeds the server's device_pool_bytes");
    // a page-locked copy of the pool; it is made resident when a request needs it
    CUDA_TRY(sd->host_pool.alloc(sd->pool_bytes));
    CUDA_TRY(cudaMemcpyAsync(sd->host_pool.p, sd->ds->pool.p, sd->pool_bytes, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    sd->ds->pool.release();
    sd->resident = false;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (sd->resident) s->resident_bytes += sd->pool_bytes;
  s->datasets.push_back(std::move(sd));
  if (id) *id = (int)s->datasets.size() - 1;
  return GBVR_OK;
}

// Wait until no batch is in flight and keep the worker from launching
// (autotuner); mutex held on entry and exit.
void pause_worker(gbvr_server* s, std::unique_lock<std::mutex>& lk) {
  s->tuning = true;
  for (;;) {
    bool busy = false;
    for (auto& sl : s->slots) busy = busy || sl->busy;
    if (!busy) break;
    s->cv_done.wait(lk);
  }
}

}  // namespace

extern "C" {

int gbvr_server_create(const gbvr_server_params* params, gbvr_server** out) {
  GBVR_ABI_TRY
  if (!out) return fail(GBVR_EINVAL, "null output handle");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(GBVR_ECUDA, "no CUDA device available");
  std::unique_ptr<gbvr_server> s(new gbvr_server());
  gbvr_server_params p = {};
  if (params) p = *params;
  if (p.max_batch <= 0) p.max_batch = 64;
  if (p.max_batch > 4096) return fail(GBVR_EINVAL, "max_batch above 4096");
  if (p.tile_w == 0) p.tile_w = TILE_W;
  if (p.tile_w != 4 && p.tile_w != 8 && p.tile_w != 16 && p.tile_w != 32) return fail(GBVR_EINVAL, "bad tile_w");
  if (p.fb_budget_bytes == 0) p.fb_budget_bytes = (uint64_t)2 << 30;
  if (p.slots == 0) p.slots = 3;
  if (p.slots < 1 || p.slots > kMaxServerSlots) return fail(GBVR_EINVAL, "slots must lie in [1, 8]");
  s->params = p;
  s->nslots = p.slots;
  for (auto& g : s->shape) g.tile_w = p.tile_w;
  CUDA_TRY(cudaGetDevice(&s->device));
  CUDA_TRY(cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device));
  for (int m = 0; m < 4; ++m) s->max_ctas[m] = persistent_group_ctas_per_sm(m);
  CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  CUDA_TRY(cudaStreamCreateWithFlags(&s->capture_stream, cudaStreamNonBlocking));
  for (int i = 0; i < kEventRing; ++i) {
    CUDA_TRY(cudaEventCreate(&s->k0[i]));
    CUDA_TRY(cudaEventCreate(&s->k1[i]));
  }
  for (int i = 0; i < s->nslots; ++i) {
    std::unique_ptr<BatchSlot> sl(new BatchSlot());
    sl->server = s.get();
    sl->index = i;
    CUDA_TRY(cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreate(&sl->ev0));
    CUDA_TRY(cudaEventCreate(&sl->ev1));
    CUDA_TRY(sl->d_fb.alloc(p.fb_budget_bytes / s->nslots));
    CUDA_TRY(sl->h_fb.alloc(p.fb_budget_bytes / s->nslots));
    s->slots.push_back(std::move(sl));
  }
  gbvr_server* raw = s.get();
  s->worker = std::thread(server_worker, raw);
  *out = s.release();
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_server_destroy(gbvr_server* s) {
  GBVR_ABI_TRY
  delete s;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_server_add_volume(gbvr_server* s, const void* host, const int64_t dims[3], int dtype,
                           const gbvr_brick_params* bp, int* id) {
  GBVR_ABI_TRY
  TRY(check_s(s));
  if (!host || !dims || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0 || dtype < 0 || dtype > 2)
    return fail(GBVR_EINVAL, "bad volume");
  long long d[3] = {dims[0], dims[1], dims[2]};
  unsigned long long bytes = 0;
  if (__builtin_mul_overflow((unsigned long long)d[0], (unsigned long long)d[1], &bytes) ||
      __builtin_mul_overflow(bytes, (unsigned long long)d[2], &bytes) ||
      __builtin_mul_overflow(bytes, (unsigned long long)dtype_size(dtype), &bytes))
    return fail(GBVR_EINVAL, "the volume's byte count overflows");
  DevBuf lv;
  CUDA_TRY(lv.alloc((size_t)bytes));
  CUDA_TRY(cudaMemcpyAsync(lv.p, host, (size_t)bytes, cudaMemcpyHostToDevice, s->stream));
  return server_add_dataset(s, lv, dtype, d, bp, id);
  GBVR_ABI_CATCH
}

int gbvr_server_add_synthetic(gbvr_server* s, const gbvr_synth_params* p, const gbvr_brick_params* bp, int* id) {
  GBVR_ABI_TRY
  TRY(check_s(s));
  DevBuf lv;
  TRY(synth_to_device(p, lv, s->stream));
  long long d[3] = {p->dims[0], p->dims[1], p->dims[2]};
  return server_add_dataset(s, lv, p->dtype, d, bp, id);
  GBVR_ABI_CATCH
}

int gbvr_server_add_tf(gbvr_server* s, int dataset, int mode, const float* rgba, int w, int h, float grad_max,
                       float iso, const float iso_rgb[3], double lo, double hi, int* tf_id) {
  GBVR_ABI_TRY
  TRY(check_s(s));
  const Dataset* dsp = nullptr;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (dataset < 0 || dataset >= (int)s->datasets.size()) return fail(GBVR_EINVAL, "bad dataset id");
    dsp = s->datasets[dataset]->ds.get();
  }
  if (mode < 0 || mode > 3) return fail(GBVR_EINVAL, "bad render mode");
  if (mode == GBVR_RM_1DTRANS || mode == GBVR_RM_MIP) h = 1;
  if (mode == GBVR_RM_ISOSURFACE) {
    static const float dummy[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (!rgba) { rgba = dummy; w = 2; h = 1; }
  }
  if (!rgba || w < 2 || h < 1 || w > 65536 || h > 4096) return fail(GBVR_EINVAL, "bad transfer function size");
  const Dataset& ds = *dsp;
  std::unique_ptr<ServerTf> t(new ServerTf());
  t->dataset = dataset;
  t->mode = mode;
  t->w = w;
  t->h = h;
  t->host.assign(rgba, rgba + 4 * (size_t)w * h);
  t->grad_max = grad_max;
  t->iso = iso;
  if (iso_rgb) for (int k = 0; k < 3; ++k) t->iso_rgb[k] = iso_rgb[k];
  if (hi > lo) {
    t->lo = lo;
    t->hi = hi;
  } else if (ds.dtype == DT_F32) {
    t->lo = ds.gmin;
    t->hi = ds.gmax > ds.gmin ? ds.gmax : ds.gmin + 1;
  } else {
    t->lo = 0;
    t->hi = std::max(1.0, (double)((long long)ds.hist1d.size() * ds.merge - 1));
  }
  const std::vector<float> dev = mode == GBVR_RM_2DTRANS ? t->host : tf1d_pairs(t->host.data(), w);
  CUDA_TRY(t->d_tf.alloc(sizeof(float) * dev.size()));
  CUDA_TRY(cudaMemcpyAsync(t->d_tf.p, dev.data(), sizeof(float) * dev.size(), cudaMemcpyHostToDevice, s->stream));
  // classification reads the per-level macro-cell grids, which stay resident
  TRY(classify_level(ds, t->level, t->host, w, h, mode, t->lo, t->hi, t->iso, t->d_prefix, t->d_skip, t->d_occ,
                     t->d_occtmp, s->stream));
  std::lock_guard<std::mutex> lk(s->mu);
  s->tfs.push_back(std::move(t));
  if (tf_id) *tf_id = (int)s->tfs.size() - 1;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_server_submit(gbvr_server* s, const gbvr_request* req, uint64_t* ticket) {
  GBVR_ABI_TRY
  TRY(check_s(s));
  if (!req || !req->out_rgba8 || req->width <= 0 || req->height <= 0 || req->width > 16384 || req->height > 16384)
    return fail(GBVR_EINVAL, "bad request");
  const size_t fb = ((size_t)req->width * req->height * 4 + 255) & ~(size_t)255;
  std::unique_ptr<ServerRequest> q(new ServerRequest());
  q->req = *req;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (req->dataset < 0 || req->dataset >= (int)s->datasets.size() || req->tf < 0 || req->tf >= (int)s->tfs.size() ||
        s->tfs[req->tf]->dataset != req->dataset)
      return fail(GBVR_EINVAL, "request names an unknown dataset or a transfer function of another dataset");
    if (fb > s->params.fb_budget_bytes / s->nslots)
      return fail(GBVR_EINVAL, "the request's framebuffer exceeds a batch slot's share of fb_budget_bytes");
    q->ticket = s->next_ticket++;
    q->t_submit = now_ms();
    if (s->t_first < 0) s->t_first = q->t_submit;
    ++s->submitted;
    if (ticket) *ticket = q->ticket;
    s->pending.push_back(q.get());
    s->reqs.emplace(q->ticket, std::move(q));
    s->blocked = false;
  }
  s->cv_work.notify_all();
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_server_wait(gbvr_server* s, uint64_t ticket, double timeout_s, gbvr_request_result* out) {
  GBVR_ABI_TRY
  TRY(check_s(s));
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return fail(GBVR_EINVAL, "unknown ticket");
  ServerRequest* q = it->second.get();
  auto done = [&] { return q->status != 1; };
  if (timeout_s > 0) {
    if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
      return fail(GBVR_ETIMEOUT, "request not finished within the timeout");
  } else {
    s->cv_done.wait(lk, done);
  }
  if (out) {
    out->status = q->status;
    out->batch_size = q->batch_size;
    out->batch = q->batch;
    out->latency_ms = q->t_done - q->t_submit;
    out->queue_ms = q->t_launch > 0 ? q->t_launch - q->t_submit : 0;
    out->gpu_ms = q->gpu_ms;
  }
  const int st = q->status;
  s->reqs.erase(it);
  if (st != GBVR_OK) return fail(st, s->worker_error.empty() ? "request failed" : s->worker_error);
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_server_get_stats(gbvr_server* s, gbvr_server_stats* out) {
  GBVR_ABI_TRY
  TRY(check_s(s));
  if (!out) return fail(GBVR_EINVAL, "null stats");
  std::lock_guard<std::mutex> lk(s->mu);
  memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->batches = s->batches;
  out->mean_batch = s->batches ? (double)s->batched_requests / s->batches : 0;
  std::vector<double> l = s->latencies;
  std::sort(l.begin(), l.end());
  if (!l.empty()) {
    auto pct = [&](double q) { return l[std::min(l.size() - 1, (size_t)std::floor(q * (l.size() - 1) + 0.5))]; };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    out->max_ms = l.back();
  }
  if (s->completed && s->t_last > s->t_first) out->frames_per_s = s->completed / ((s->t_last - s->t_first) / 1000.0);
  out->overlap_checked = s->overlap_checked;
  out->overlapped = s->overlapped;
  out->uploads = s->uploads;
  out->evictions = s->evictions;
  out->upload_bytes = s->upload_bytes;
  out->resident_bytes = s->resident_bytes;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_server_reset_stats(gbvr_server* s) {
  GBVR_ABI_TRY
  TRY(check_s(s));
  std::lock_guard<std::mutex> lk(s->mu);
  s->latencies.clear();
  s->submitted = s->completed = s->batches = s->batched_requests = 0;
  s->overlap_checked = s->overlapped = s->uploads = s->evictions = s->upload_bytes = 0;
  s->t_first = -1;
  s->t_last = 0;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_server_autotune(gbvr_server* s, int width, int height, int n, gbvr_server_tune* out, int cap, int* n_out) {
  GBVR_ABI_TRY
  TRY(check_s(s));
  if (width <= 0 || height <= 0 || n <= 0 || n > s->params.max_batch || (cap > 0 && !out))
    return fail(GBVR_EINVAL, "bad tuning batch (width, height > 0; 0 < n <= max_batch)");
  const size_t fb = ((size_t)width * height * 4 + 255) & ~(size_t)255;
  if (fb * n > s->params.fb_budget_bytes / s->nslots)
    return fail(GBVR_EINVAL, "the tuning batch exceeds a batch slot's framebuffer share");
  std::unique_lock<std::mutex> lk(s->mu);
  pause_worker(s, lk);
  BatchSlot& slot = *s->slots[0];
  // per group: one dataset (the first of the group that fits the memory
  // budget) and its presets in turn
  struct Plan { int gi, dataset; std::vector<int> tfs; };
  std::vector<Plan> plans;
  for (int gi = 0; gi < kServerGroups; ++gi) {
    Plan pl{gi, -1, {}};
    for (size_t t = 0; t < s->tfs.size(); ++t) {
      const ServerTf& tf = *s->tfs[t];
      const ServerDataset& D = *s->datasets[tf.dataset];
      if (D.ds->dtype * 4 + tf.mode != gi) continue;
      if (pl.dataset < 0) pl.dataset = tf.dataset;
      if (tf.dataset == pl.dataset) pl.tfs.push_back((int)t);
    }
    if (pl.dataset >= 0) plans.push_back(pl);
  }
  int rc = GBVR_OK;
  int count = 0;
  std::vector<uint8_t> sink(fb);
  std::vector<ServerRequest> fake(n);
  const int tiles[] = {4, 8, 16};
  for (const Plan& pl : plans) {
    ServerDataset& D = *s->datasets[pl.dataset];
    slot.datasets.assign(1, pl.dataset);
    if (!D.resident && !make_resident(s, D, slot.stream, slot.datasets, rc)) {
      if (rc != GBVR_OK) break;
      continue;  // does not fit next to the pinned datasets: keep its default shape
    }
    ++D.inflight;
    for (int i = 0; i < n; ++i) {
      ServerRequest& q = fake[i];
      memset(&q.req, 0, sizeof(q.req));
      q.req.dataset = pl.dataset;
      q.req.tf = pl.tfs[i % pl.tfs.size()];
      q.req.width = width;
      q.req.height = height;
      q.req.samples_per_voxel = 1.f;
      q.req.out_rgba8 = sink.data();
      orbit(360.0 * i / n, 25.0 * std::sin(0.7 * i), 2.5 * std::sqrt(3.0), 45.0, width, height, q.req.view,
            q.req.proj);
    }
    slot.reqs.clear();
    slot.fb_off.clear();
    for (int i = 0; i < n; ++i) {
      slot.reqs.push_back(&fake[i]);
      slot.fb_off.push_back((size_t)i * fb);
    }
    slot.fb_used = fb * n;
    snapshot_batch(s, slot);
    lk.unlock();
    const int m = pl.gi & 3;
    const GroupShape def{s->params.tile_w, 0};
    std::vector<GroupShape> cands;
    cands.push_back(def);
    for (int tw : tiles)
      for (int c : {s->max_ctas[m], std::max(1, s->max_ctas[m] - 2), std::max(1, s->max_ctas[m] / 2)})
        if (!(tw == def.tile_w && c == s->max_ctas[m])) cands.push_back(GroupShape{tw, c});
    float best = 1e30f, def_ms = 0.f;
    GroupShape best_shape = def;
    for (size_t ci = 0; ci < cands.size() && rc == GBVR_OK; ++ci) {
      float ms_best = 1e30f;
      for (int rep = 0; rep < 3 && rc == GBVR_OK; ++rep) {  // one warm-up, best of two
        rc = launch_batch(s, slot, &cands[ci], false);
        if (rc == GBVR_OK) {
          cudaError_t e = cudaStreamSynchronize(slot.stream);
          float ms = 0.f;
          if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, slot.ev0, slot.ev1);
          if (e != cudaSuccess) rc = cuda_fail(e, "tuning batch");
          else if (rep > 0) ms_best = std::min(ms_best, ms);
        }
      }
      if (ci == 0) def_ms = ms_best;
      if (ms_best < best) {
        best = ms_best;
        best_shape = cands[ci];
      }
    }
    lk.lock();
    --D.inflight;
    if (rc != GBVR_OK) break;
    s->shape[pl.gi] = best_shape;
    if (out && count < cap) {
      gbvr_server_tune& r = out[count];
      r.dtype = pl.gi >> 2;
      r.mode = m;
      r.tile_w = best_shape.tile_w;
      r.ctas_per_sm = best_shape.ctas_per_sm > 0 ? best_shape.ctas_per_sm : s->max_ctas[m];
      r.candidates = (int)cands.size();
      r.best_ms = best;
      r.default_ms = def_ms;
    }
    ++count;
  }
  slot.reqs.clear();
  slot.datasets.clear();
  slot.dsets.clear();
  slot.done = false;
  ++s->shape_version;  // the slots re-capture their graphs with the new shapes
  s->tuning = false;
  lk.unlock();
  s->cv_work.notify_all();
  if (n_out) *n_out = std::min(count, cap);
  return rc;
  GBVR_ABI_CATCH
}

}  // extern "C"
