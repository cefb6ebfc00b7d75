// UVF build kernels: seeded volume synthesis, 2x2x2 LOD averaging, brick
// gather with ghost voxels, per-brick min/max, 1D and 2D histograms.
//
// These replace the CPU loops behind the reference's UVF build sequence
// (UVFReader/DataSource.h:475-616: FlatDataToBrickedLOD with
// CombineAverage<T,1> and SimpleMaxMin<T,1>, Histogram1DDataBlock::Compute /
// Compress(4096), Histogram2DDataBlock::Compute).  Every kernel here is
// integer-exact (or a fixed float32 operation order with round-to-nearest
// intrinsics), so results are bit-identical to the CPU restatement.
#include <algorithm>
#include <type_traits>
#include <cstdint>

#include "gbvr_internal.h"

namespace gbvr {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11), the counter-based generator used for
// all seeded draws; identical on host and device.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
    uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

__device__ __forceinline__ float blob_noise(const BlobTablesDev& t, unsigned long long idx) {
  if (t.noise_kind == 1) {
    uint32_t c[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 0x6e6f6973u, 0u};
    philox(c, t.seed, 0x766f6c21u);
    float u = __fmul_rn((float)(c[0] >> 8), 1.0f / 16777216.0f);
    float n = __fmul_rn(u, __fmul_rn(2.0f, t.noise_amp));
    return __fsub_rn(n, t.noise_amp);
  }
  if (t.noise_kind == 2) {
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      uint32_t c[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 0x6e6f6973u, (uint32_t)k};
      philox(c, t.seed, 0x766f6c21u);
      s += (c[0] >> 16) + (c[1] >> 16) + (c[2] >> 16) + (c[3] >> 16);
    }
    float z = __fmul_rn((float)s, 1.0f / 65536.0f);
    z = __fsub_rn(z, 6.0f);
    return __fmul_rn(z, t.noise_amp);
  }
  return 0.0f;
}

// One CTA per (y, z) row; blob weights of the row staged in shared memory.
template <typename T>
__global__ void k_synth_blobs(BlobTablesDev t, long long X, long long Y, long long Z, long long z0,
                              T* __restrict__ out) {
  extern __shared__ float w_row[];
  // this CTA's row: global z = z0 + blockIdx.y; out holds planes from z0 on
  const long long y = blockIdx.x, z = z0 + blockIdx.y;
  for (int k = threadIdx.x; k < t.nblobs; k += blockDim.x) {
    float w = __fmul_rn(t.amp[k], t.ez[(long long)k * Z + z]);
    w_row[k] = __fmul_rn(w, t.ey[(long long)k * Y + y]);
  }
  float bgyz = 0.f;
  if (t.bgx) bgyz = t.bgy[y];
  __syncthreads();
  for (long long x = threadIdx.x; x < X; x += blockDim.x) {
    float acc = 0.0f;
    if (t.bgx) {
      float b = __fmul_rn(t.bgx[x], bgyz);
      b = __fmul_rn(b, t.bgz[z]);
      b = __fmul_rn(b, t.bg_amp);
      acc = __fadd_rn(t.bg_level, b);
    }
    for (int k = 0; k < t.nblobs; ++k) acc = __fadd_rn(acc, __fmul_rn(w_row[k], __ldg(t.ex + (long long)k * X + x)));
    float v = __fmul_rn(acc, t.scale);
    const long long idx = (z * Y + y) * X + x;  // global voxel index (seeds the noise)
    const long long o = ((z - z0) * Y + y) * X + x;
    v = __fadd_rn(v, blob_noise(t, (unsigned long long)idx));
    if (sizeof(T) == 4) {
      out[o] = (T)v;
    } else {
      float r = rintf(v);
      r = fminf(fmaxf(r, 0.0f), t.vmax);
      out[o] = (T)r;
    }
  }
}

cudaError_t launch_synth_blobs_planes(const BlobTablesDev& t, const long long dims[3], int dtype, long long z0,
                                      long long nz, void* out, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nz <= 0) return cudaSuccess;
  dim3 grid((unsigned)dims[1], (unsigned)nz);
  int threads = dims[0] >= 256 ? 256 : 128;
  size_t smem = sizeof(float) * (t.nblobs > 0 ? t.nblobs : 1);
  if (dtype == DT_U8) k_synth_blobs<uint8_t><<<grid, threads, smem, s>>>(t, dims[0], dims[1], dims[2], z0, (uint8_t*)out);
  else if (dtype == DT_U16) k_synth_blobs<uint16_t><<<grid, threads, smem, s>>>(t, dims[0], dims[1], dims[2], z0, (uint16_t*)out);
  else k_synth_blobs<float><<<grid, threads, smem, s>>>(t, dims[0], dims[1], dims[2], z0, (float*)out);
  return cudaGetLastError();
}

cudaError_t launch_synth_blobs(const BlobTablesDev& t, const long long dims[3], int dtype, void* out, cudaStream_t s) {
  return launch_synth_blobs_planes(t, dims, dtype, 0, dims[2], out, s);
}

// ---------------------------------------------------------------------------
// 2x2x2 LOD averaging (DataSource.h:551,563 CombineAverage<T,1>): the mean of
// the children that exist, floor for integers, float(sum/count) with a double
// sum for float32.  One thread per output voxel; x fastest for coalescing.
// ---------------------------------------------------------------------------
// two x-adjacent 8- or 16-bit voxels (the first at an even index of a row of
// even length, so the pair is aligned) summed from one load
__device__ __forceinline__ unsigned pair_sum(const uint8_t* p) {
  const unsigned w = __ldg(reinterpret_cast<const unsigned short*>(p));
  return (w & 0xffu) + (w >> 8);
}
__device__ __forceinline__ unsigned pair_sum(const uint16_t* p) {
  const unsigned w = __ldg(reinterpret_cast<const unsigned*>(p));
  return (w & 0xffffu) + (w >> 16);
}
__device__ __forceinline__ unsigned pair_sum(const float*) { return 0u; }

template <typename T>
__global__ void k_downsample(const T* __restrict__ in, long long X, long long Y, long long Z, T* __restrict__ out,
                             long long OX, long long OY, long long OZ) {
  // pairs: rows of even length from an aligned base, so every even x starts
  // an aligned pair
  const bool pairs = sizeof(T) < 4 && (X & 1) == 0 && (reinterpret_cast<uintptr_t>(in) % (2 * sizeof(T))) == 0;
  for (long long row = blockIdx.x; row < OY * OZ; row += gridDim.x) {
    const long long z = row / OY, y = row - z * OY;
    const long long y0 = 2 * y, z0 = 2 * z;
    const int ny = (y0 + 1 < Y) ? 2 : 1, nz = (z0 + 1 < Z) ? 2 : 1;
    for (long long x = threadIdx.x; x < OX; x += blockDim.x) {
      const long long x0 = 2 * x;
      const int nx = (x0 + 1 < X) ? 2 : 1;
      const long long o = row * OX + x;
      if (sizeof(T) == 4) {
        double sum = 0.0;
        for (int dz = 0; dz < nz; ++dz)
          for (int dy = 0; dy < ny; ++dy)
            for (int dx = 0; dx < nx; ++dx) sum += (double)__ldg(in + ((z0 + dz) * Y + (y0 + dy)) * X + x0 + dx);
        out[o] = (T)(float)(sum / (double)(nx * ny * nz));
      } else if (pairs && nx == 2 && ny == 2 && nz == 2) {
        // all 8 children: the x pairs in one load each, the mean by a shift
        const T* p = in + (z0 * Y + y0) * X + x0;
        const unsigned sum = pair_sum(p) + pair_sum(p + X) + pair_sum(p + X * Y) + pair_sum(p + X * Y + X);
        out[o] = (T)(sum >> 3);
      } else {
        unsigned sum = 0;
        for (int dz = 0; dz < nz; ++dz)
          for (int dy = 0; dy < ny; ++dy)
            for (int dx = 0; dx < nx; ++dx) sum += (unsigned)__ldg(in + ((z0 + dz) * Y + (y0 + dy)) * X + x0 + dx);
        out[o] = (T)(sum / (unsigned)(nx * ny * nz));
      }
    }
  }
}

static int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 152LL * 64) b = 152LL * 64;
  return (int)(b < 1 ? 1 : b);
}

// ---------------------------------------------------------------------------
// Seeded fractal (fBm) volume: octaves of periodic value noise with
// lowbias32-hashed lattice values (C. Wellons, 2018), smoothstep trilinear
// weights, weight 2^-o per octave; normalised, thresholded, scaled.  Each
// step is one round-to-nearest float32 operation in the order of the CPU
// restatement, so both produce the same bits.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t lowbias32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ float fbm_lat(uint32_t i, uint32_t j, uint32_t k, uint32_t P, uint32_t salt) {
  return __fmul_rn((float)(lowbias32(((k * P + j) * P + i) ^ salt) >> 8), 1.0f / 16777216.0f);
}

__device__ __forceinline__ float fbm_lerp(float a, float b, float t) {
  return __fadd_rn(a, __fmul_rn(__fsub_rn(b, a), t));
}

template <typename T>
__global__ void k_synth_fbm(long long X, long long Y, long long Z, uint32_t seed, int octaves, int base_period,
                            float thr, float vmax, T* __restrict__ out) {
  const long long dims[3] = {X, Y, Z};
  const float inv = __fdiv_rn(1.0f, __fsub_rn(1.0f, thr));
  for (long long row = blockIdx.x; row < Y * Z; row += gridDim.x)
  for (long long x = threadIdx.x; x < X; x += blockDim.x) {
    const long long z = row / Y, y = row - z * Y;
    const long long idx = row * X + x;
    const long long c[3] = {x, y, z};
    float acc = 0.0f, norm = 0.0f, amp = 1.0f;
    for (int o = 0; o < octaves; ++o) {
      const uint32_t P = (uint32_t)base_period << o;
      const uint32_t salt = seed + 0x9E3779B9u * (uint32_t)(o + 1);
      uint32_t i0[3], i1[3];
      float s[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float scale = __fdiv_rn((float)P, (float)dims[a]);
        const float u = __fmul_rn(__fadd_rn((float)c[a], 0.5f), scale);
        const float f = floorf(u);
        const float t = __fsub_rn(u, f);
        s[a] = __fmul_rn(__fmul_rn(t, t), __fsub_rn(3.0f, __fadd_rn(t, t)));
        const uint32_t ii = (uint32_t)(long long)f % P;
        i0[a] = ii;
        i1[a] = (ii + 1) % P;
      }
      const float c00 = fbm_lerp(fbm_lat(i0[0], i0[1], i0[2], P, salt), fbm_lat(i1[0], i0[1], i0[2], P, salt), s[0]);
      const float c10 = fbm_lerp(fbm_lat(i0[0], i1[1], i0[2], P, salt), fbm_lat(i1[0], i1[1], i0[2], P, salt), s[0]);
      const float c01 = fbm_lerp(fbm_lat(i0[0], i0[1], i1[2], P, salt), fbm_lat(i1[0], i0[1], i1[2], P, salt), s[0]);
      const float c11 = fbm_lerp(fbm_lat(i0[0], i1[1], i1[2], P, salt), fbm_lat(i1[0], i1[1], i1[2], P, salt), s[0]);
      const float v = fbm_lerp(fbm_lerp(c00, c10, s[1]), fbm_lerp(c01, c11, s[1]), s[2]);
      acc = __fadd_rn(acc, __fmul_rn(amp, v));
      norm = __fadd_rn(norm, amp);
      amp = __fmul_rn(amp, 0.5f);
    }
    float v = __fdiv_rn(acc, norm);
    v = __fmul_rn(__fsub_rn(v, thr), inv);
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    v = __fmul_rn(v, vmax);
    if (sizeof(T) == 4) out[idx] = (T)v;
    else out[idx] = (T)rintf(v);
  }
}

cudaError_t launch_synth_fbm(const long long dims[3], int dtype, uint32_t seed, int octaves, int base_period,
                             float thr, float vmax, void* out, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  const long long rows = dims[1] * dims[2];
  int threads = dims[0] >= 256 ? 256 : 128;
  int blocks = (int)(rows < 152LL * 256 ? rows : 152LL * 256);
  if (dtype == DT_U8)
    k_synth_fbm<uint8_t><<<blocks, threads, 0, s>>>(dims[0], dims[1], dims[2], seed, octaves, base_period, thr, vmax, (uint8_t*)out);
  else if (dtype == DT_U16)
    k_synth_fbm<uint16_t><<<blocks, threads, 0, s>>>(dims[0], dims[1], dims[2], seed, octaves, base_period, thr, vmax, (uint16_t*)out);
  else
    k_synth_fbm<float><<<blocks, threads, 0, s>>>(dims[0], dims[1], dims[2], seed, octaves, base_period, thr, vmax, (float*)out);
  return cudaGetLastError();
}


cudaError_t launch_downsample(const void* in, int dtype, const long long dims[3], void* out, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  long long OX = (dims[0] + 1) / 2, OY = (dims[1] + 1) / 2, OZ = (dims[2] + 1) / 2;
  int threads = OX >= 256 ? 256 : 128;
  int blocks = (int)(OY * OZ < 152LL * 64 ? OY * OZ : 152LL * 64);
  if (dtype == DT_U8)
    k_downsample<uint8_t><<<blocks, threads, 0, s>>>((const uint8_t*)in, dims[0], dims[1], dims[2], (uint8_t*)out, OX, OY, OZ);
  else if (dtype == DT_U16)
    k_downsample<uint16_t><<<blocks, threads, 0, s>>>((const uint16_t*)in, dims[0], dims[1], dims[2], (uint16_t*)out, OX, OY, OZ);
  else
    k_downsample<float><<<blocks, threads, 0, s>>>((const float*)in, dims[0], dims[1], dims[2], (float*)out, OX, OY, OZ);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Brick gather: copy each brick's stored box (interior + ghosts) out of the
// flat level into its pool slot.  One CTA per (brick, z-slice) row block;
// x fastest so both sides are coalesced.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_gather(const T* __restrict__ level, long long X, long long Y, long long Z, long long vz0,
                         const BrickInfo* __restrict__ bricks, T* __restrict__ pool, int perm) {
  // level holds planes vz0.. of the level (0: the whole level)
  const BrickInfo b = bricks[blockIdx.y];
  const long long plane = (long long)b.sx * b.sy;
  // destination strides of x, y, z in this layout copy (perm 3: 4^3 blocks,
  // each 64 voxels contiguous with x fastest, blocks in x, y, z order)
  long long s0 = 0, s1 = 0, s2 = 0;
  if (perm == 0) { s0 = 1; s1 = b.sx; s2 = (long long)b.sx * b.sy; }
  else if (perm == 1) { s1 = 1; s2 = b.sy; s0 = (long long)b.sy * b.sz; }
  else if (perm == 2) { s2 = 1; s0 = b.sz; s1 = (long long)b.sz * b.sx; }
  const long long nbx = (b.sx + 3) >> 2, nby = (b.sy + 3) >> 2;
  (void)plane;
  for (int zs = blockIdx.x; zs < b.sz; zs += gridDim.x) {
    const long long z = min(max((long long)b.oz + zs, 0LL), Z - 1);
    for (long long r = 0; r < b.sy; ++r)
    for (long long xs = threadIdx.x; xs < b.sx; xs += blockDim.x) {
      // ghosts outside the level replicate its edge voxels
      const long long y = min(max((long long)b.oy + r, 0LL), Y - 1);
      const long long x = min(max((long long)b.ox + xs, 0LL), X - 1);
      long long di;
      if (perm == 3)
        di = ((((long long)(zs >> 2) * nby + (r >> 2)) * nbx + (xs >> 2)) << 6) + ((zs & 3) << 4) + ((r & 3) << 2) + (xs & 3);
      else
        di = xs * s0 + r * s1 + zs * s2;
      pool[b.offset + di] = __ldg(level + ((z - vz0) * Y + y) * X + x);
    }
  }
}

// Brick gather into overlapped 4^3 blocks (layout copy 4): block (bx, by, bz)
// of a brick's stored box holds the 5^3 voxels 4 b + (0..4) per axis, x
// fastest, in 128 elements (the last 3 zero), blocks in x, y, z order, the
// brick's blocks at twice its offset of the x-fastest copy.  Voxel 4 of a
// block repeats voxel 0 of the next one, so every trilinear footprint of a
// cell in the block lies in the block; the footprint of a cell inside the
// stored box never reaches past it, and slots past the box hold its edge.
// One warp per destination block (its 128 elements, 4 per lane, written in
// order); a lane's slots, and so their offsets inside a block, are the same
// for every block.
template <typename T>
__global__ void __launch_bounds__(256) k_gather_ov(const T* __restrict__ level, long long X, long long Y, long long Z,
                                                   long long vz0, const BrickInfo* __restrict__ bricks,
                                                   T* __restrict__ pool) {
  const BrickInfo b = bricks[blockIdx.y];
  const int nbx = (b.sx + 3) >> 2, nby = (b.sy + 3) >> 2, nbz = (b.sz + 3) >> 2;
  const int nblk = nbx * nby * nbz;
  T* dst = pool + 2 * (long long)b.offset;
  const int lane = threadIdx.x & 31;
  int si[4], sj[4], sk[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int slot = lane + 32 * q;
    si[q] = slot % 5;
    sj[q] = (slot / 5) % 5;
    sk[q] = slot / 25;  // 5 for the 3 padding slots
  }
  const int warps = (int)(blockDim.x >> 5);
  for (int blk = (int)blockIdx.x * warps + (int)(threadIdx.x >> 5); blk < nblk; blk += (int)gridDim.x * warps) {
    const int bx = blk % nbx, t = blk / nbx, by = t % nby, bz = t / nby;
    T* d = dst + ((long long)blk << 7);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int slot = lane + 32 * q;
      T val = T(0);
      if (slot < 125) {
        // ghosts outside the level replicate its edge voxels
        const int xs = min(4 * bx + si[q], b.sx - 1), ys = min(4 * by + sj[q], b.sy - 1),
                  zs = min(4 * bz + sk[q], b.sz - 1);
        const long long x = min(max((long long)b.ox + xs, 0LL), X - 1);
        const long long y = min(max((long long)b.oy + ys, 0LL), Y - 1);
        const long long z = min(max((long long)b.oz + zs, 0LL), Z - 1);
        val = __ldg(level + ((z - vz0) * Y + y) * X + x);
      }
      d[slot] = val;
    }
  }
}

// The inverse of k_gather for the x-fastest copy: every brick's interior
// voxels (its [max(lo, 0), min(hi, dims)) box) back into the flat level.  The
// interiors tile the level, so every voxel is written once.  One block per
// brick, plane by plane.
template <typename T>
__global__ void k_scatter_interiors(const T* __restrict__ pool, const BrickInfo* __restrict__ bricks, long long X,
                                    long long Y, long long Z, T* __restrict__ level) {
  const BrickInfo b = bricks[blockIdx.x];
  const long long x0 = max(b.lox, 0), x1 = min((long long)b.hix, X);
  const long long y0 = max(b.loy, 0), y1 = min((long long)b.hiy, Y);
  const long long z0 = max(b.loz, 0), z1 = min((long long)b.hiz, Z);
  const long long nx = x1 - x0;
  for (long long z = z0 + blockIdx.y; z < z1; z += gridDim.y)
    for (long long y = y0; y < y1; ++y)
      for (long long i = threadIdx.x; i < nx; i += blockDim.x) {
        const long long x = x0 + i;
        const long long src = ((z - b.oz) * b.sy + (y - b.oy)) * b.sx + (x - b.ox);
        level[(z * Y + y) * X + x] = __ldg(pool + b.offset + src);
      }
}

cudaError_t launch_scatter_interiors(const void* pool, int dtype, const BrickInfo* bricks, int nbricks,
                                     const long long dims[3], void* level, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nbricks <= 0) return cudaSuccess;
  dim3 grid((unsigned)nbricks, 16);
  if (dtype == DT_U8)
    k_scatter_interiors<uint8_t><<<grid, 256, 0, s>>>((const uint8_t*)pool, bricks, dims[0], dims[1], dims[2],
                                                      (uint8_t*)level);
  else if (dtype == DT_U16)
    k_scatter_interiors<uint16_t><<<grid, 256, 0, s>>>((const uint16_t*)pool, bricks, dims[0], dims[1], dims[2],
                                                       (uint16_t*)level);
  else
    k_scatter_interiors<float><<<grid, 256, 0, s>>>((const float*)pool, bricks, dims[0], dims[1], dims[2],
                                                    (float*)level);
  return cudaGetLastError();
}

cudaError_t launch_gather_bricks_window(const void* level, int dtype, const long long dims[3], long long vz0,
                                        const BrickInfo* bricks_dev, int nbricks, void* pool, int perm,
                                        cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nbricks <= 0) return cudaSuccess;
  dim3 grid((unsigned)(dims[2] < 256 ? dims[2] : 256), (unsigned)nbricks);
  int threads = 256;
  if (perm == 4) {
    if (dtype == DT_U8)
      k_gather_ov<uint8_t><<<grid, threads, 0, s>>>((const uint8_t*)level, dims[0], dims[1], dims[2], vz0, bricks_dev,
                                                    (uint8_t*)pool);
    else if (dtype == DT_U16)
      k_gather_ov<uint16_t><<<grid, threads, 0, s>>>((const uint16_t*)level, dims[0], dims[1], dims[2], vz0,
                                                     bricks_dev, (uint16_t*)pool);
    else
      k_gather_ov<float><<<grid, threads, 0, s>>>((const float*)level, dims[0], dims[1], dims[2], vz0, bricks_dev,
                                                  (float*)pool);
    return cudaGetLastError();
  }
  if (dtype == DT_U8)
    k_gather<uint8_t><<<grid, threads, 0, s>>>((const uint8_t*)level, dims[0], dims[1], dims[2], vz0, bricks_dev, (uint8_t*)pool, perm);
  else if (dtype == DT_U16)
    k_gather<uint16_t><<<grid, threads, 0, s>>>((const uint16_t*)level, dims[0], dims[1], dims[2], vz0, bricks_dev, (uint16_t*)pool, perm);
  else
    k_gather<float><<<grid, threads, 0, s>>>((const float*)level, dims[0], dims[1], dims[2], vz0, bricks_dev, (float*)pool, perm);
  return cudaGetLastError();
}

cudaError_t launch_gather_bricks(const void* level, int dtype, const long long dims[3], const BrickInfo* bricks_dev,
                                 int nbricks, void* pool, int perm, cudaStream_t s) {
  return launch_gather_bricks_window(level, dtype, dims, 0, bricks_dev, nbricks, pool, perm, s);
}

// ---------------------------------------------------------------------------
// Brick gather of the in-core build in one pass over the level: every brick's
// stored box into the x-fastest copy and, with `blocked`, into the 4x4x4-
// blocked copy, and the brick's min/max over those voxels (ghosts included),
// reduced per CTA and combined with float atomics.  A CTA of 8 warps takes
// z-slices of one brick; a warp takes rows, its lanes consecutive x, so the
// level is read and the x-fastest copy written in whole rows.  vmin / vmax of
// every brick must be +inf / -inf on entry.
// ---------------------------------------------------------------------------
// Float min / max through integer atomics: non-negative floats order as
// their bit patterns read as signed ints, negative floats in reverse as
// unsigned ints.
__device__ __forceinline__ void atomic_min_float(float* a, float v) {
  if (v >= 0.f) atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
  else atomicMax(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_float(float* a, float v) {
  if (v >= 0.f) atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));
  else atomicMin(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}

constexpr int GATHER_WARPS = 8;

// Tiles of 4 rows x 4 voxels: two loads of voxel pairs per row, one store
// of 4 voxels per row into each copy; in the blocked copy the tile is one
// z-slice of a 4^3 block, contiguous, so its sectors are written whole by
// one thread.  Pair / Quad: 2 and 4 voxels as one word.
template <typename T> struct GatherVec;
template <> struct GatherVec<uint8_t> {
  using Pair = unsigned short;
  using Quad = unsigned;
  __device__ static Quad quad(Pair a, Pair b) { return (unsigned)a | ((unsigned)b << 16); }
  __device__ static Quad make4(uint8_t a, uint8_t b, uint8_t c, uint8_t d) {
    return (unsigned)a | ((unsigned)b << 8) | ((unsigned)c << 16) | ((unsigned)d << 24);
  }
  // packed per-byte min / max
  __device__ static void acc(Quad q, unsigned& mn, unsigned& mx) { mn = __vminu4(mn, q); mx = __vmaxu4(mx, q); }
  __device__ static void fold(unsigned mn, unsigned mx, float& fmn, float& fmx) {
    for (int i = 0; i < 4; ++i) {
      fmn = fminf(fmn, (float)((mn >> (8 * i)) & 0xffu));
      fmx = fmaxf(fmx, (float)((mx >> (8 * i)) & 0xffu));
    }
  }
};
template <> struct GatherVec<uint16_t> {
  using Pair = unsigned;
  using Quad = uint2;
  __device__ static Quad quad(Pair a, Pair b) { return make_uint2(a, b); }
  __device__ static Quad make4(uint16_t a, uint16_t b, uint16_t c, uint16_t d) {
    return make_uint2((unsigned)a | ((unsigned)b << 16), (unsigned)c | ((unsigned)d << 16));
  }
  __device__ static void acc(Quad q, unsigned& mn, unsigned& mx) {
    mn = __vminu2(mn, __vminu2(q.x, q.y));
    mx = __vmaxu2(mx, __vmaxu2(q.x, q.y));
  }
  __device__ static void fold(unsigned mn, unsigned mx, float& fmn, float& fmx) {
    fmn = fminf(fmn, (float)min(mn & 0xffffu, mn >> 16));
    fmx = fmaxf(fmx, (float)max(mx & 0xffffu, mx >> 16));
  }
};
template <> struct GatherVec<float> {
  using Pair = float2;
  using Quad = float4;
  __device__ static Quad quad(Pair a, Pair b) { return make_float4(a.x, a.y, b.x, b.y); }
  __device__ static Quad make4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }
  // min / max kept in the float accumulators directly (NaN voxels passed over)
  __device__ static void acc(Quad q, float& mn, float& mx) {
    mn = fminf(fminf(mn, q.x), fminf(q.y, fminf(q.z, q.w)));
    mx = fmaxf(fmaxf(mx, q.x), fmaxf(q.y, fmaxf(q.z, q.w)));
  }
};

template <typename T, bool BLOCKED>
__global__ void __launch_bounds__(32 * GATHER_WARPS) k_gather_fused(const T* __restrict__ level, long long X,
                                                                    long long Y, long long Z,
                                                                    BrickInfo* __restrict__ bricks,
                                                                    T* __restrict__ pool0, T* __restrict__ pool1) {
  BrickInfo* bp = bricks + blockIdx.y;
  const int ox = bp->ox, oy = bp->oy, oz = bp->oz, sx = bp->sx, sy = bp->sy, sz = bp->sz;
  const long long off = (long long)bp->offset;
  const int nbx = (sx + 3) >> 2, nby = (sy + 3) >> 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float mn = INFINITY, mx = -INFINITY;
  using V = GatherVec<T>;
  // the tiled path needs voxel pairs at even level x (X, ox even, aligned
  // rows) and 4-voxel stores at multiples of 4 elements in both copies
  const bool tiled = (X % 2 == 0) && (ox % 2 == 0) && (sx % 4 == 0) &&
                     reinterpret_cast<uintptr_t>(level) % (2 * sizeof(T)) == 0 &&
                     reinterpret_cast<uintptr_t>(pool0 + off) % (4 * sizeof(T)) == 0 &&
                     (!BLOCKED || reinterpret_cast<uintptr_t>(pool1 + off) % (4 * sizeof(T)) == 0);
  const int row_start = tiled ? (sy & ~3) : 0;  // rows below it go by tiles
  // blocked copy at 16-byte boundaries: a slice (16 voxels at a multiple of
  // 16 elements from the brick's start) goes out in 16-byte stores
  const bool wide1 = BLOCKED && reinterpret_cast<uintptr_t>(pool1 + off) % 16 == 0;
  if (tiled) {
    using Acc = typename std::conditional<std::is_same<T, float>::value, float, unsigned>::type;
    Acc pmn, pmx;
    if constexpr (std::is_same<T, float>::value) { pmn = INFINITY; pmx = -INFINITY; }
    else { pmn = 0xffffffffu; pmx = 0u; }
    const int nq = sx >> 2;
    for (int zs = blockIdx.x; zs < sz; zs += gridDim.x) {
      const long long z = min(max((long long)oz + zs, 0LL), Z - 1);
      for (int band = warp; 4 * band < row_start; band += GATHER_WARPS) {
        const int r0 = 4 * band;
        const T* src[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) src[k] = level + (z * Y + min(max((long long)oy + r0 + k, 0LL), Y - 1)) * X;
        T* d0 = pool0 + off + ((long long)zs * sy + r0) * sx;
        T* d1 = BLOCKED ? pool1 + off + ((((long long)(zs >> 2) * nby + band) * nbx) << 6) + ((zs & 3) << 4) : nullptr;
        for (int q = lane; q < nq; q += 32) {
          const long long x = (long long)ox + 4 * q;
          typename V::Quad t[4];
          if (x >= 0 && x + 3 < X) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const typename V::Pair* pp = reinterpret_cast<const typename V::Pair*>(src[k] + x);
              t[k] = V::quad(__ldg(pp), __ldg(pp + 1));
            }
          } else {
            // ghosts outside the level replicate its edge voxels
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              auto at = [&](int i) { return __ldg(src[k] + min(max(x + i, 0LL), X - 1)); };
              t[k] = V::make4(at(0), at(1), at(2), at(3));
            }
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            *reinterpret_cast<typename V::Quad*>(d0 + (long long)k * sx + 4 * q) = t[k];
            V::acc(t[k], pmn, pmx);
          }
          if (BLOCKED) {
            // the block's z-slice: 16 contiguous voxels, in 16-byte stores
            // where the copy is aligned for them
            T* ds = d1 + ((long long)q << 6);
            if constexpr (sizeof(T) == 1) {
              if (wide1) *reinterpret_cast<uint4*>(ds) = make_uint4(t[0], t[1], t[2], t[3]);
              else
#pragma unroll
                for (int k = 0; k < 4; ++k) *reinterpret_cast<typename V::Quad*>(ds + (k << 2)) = t[k];
            } else if constexpr (sizeof(T) == 2) {
              if (wide1) {
                reinterpret_cast<uint4*>(ds)[0] = make_uint4(t[0].x, t[0].y, t[1].x, t[1].y);
                reinterpret_cast<uint4*>(ds)[1] = make_uint4(t[2].x, t[2].y, t[3].x, t[3].y);
              } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) *reinterpret_cast<typename V::Quad*>(ds + (k << 2)) = t[k];
              }
            } else {
#pragma unroll
              for (int k = 0; k < 4; ++k) *reinterpret_cast<typename V::Quad*>(ds + (k << 2)) = t[k];
            }
          }
        }
      }
    }
    if constexpr (std::is_same<T, float>::value) {
      mn = pmn;
      mx = pmx;
    } else {
      V::fold(pmn, pmx, mn, mx);
    }
  }
  for (int zs = blockIdx.x; zs < sz; zs += gridDim.x) {
    const long long z = min(max((long long)oz + zs, 0LL), Z - 1);
    for (int r = row_start + warp; r < sy; r += GATHER_WARPS) {
      // ghosts outside the level replicate its edge voxels
      const long long y = min(max((long long)oy + r, 0LL), Y - 1);
      const T* src = level + (z * Y + y) * X;
      T* d0 = pool0 + off + ((long long)zs * sy + r) * sx;
      T* d1 = BLOCKED ? pool1 + off + ((((long long)(zs >> 2) * nby + (r >> 2)) * nbx) << 6) + ((zs & 3) << 4) +
                            ((r & 3) << 2)
                      : nullptr;
#pragma unroll 4
      for (int xs = lane; xs < sx; xs += 32) {
        const long long x = min(max((long long)ox + xs, 0LL), X - 1);
        const T v = __ldg(src + x);
        d0[xs] = v;
        if (BLOCKED) d1[((xs >> 2) << 6) + (xs & 3)] = v;
        const float f = (float)v;
        mn = fminf(mn, f);
        mx = fmaxf(mx, f);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  __shared__ float smn[GATHER_WARPS], smx[GATHER_WARPS];
  if (lane == 0) { smn[warp] = mn; smx[warp] = mx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < GATHER_WARPS; ++w) {
      mn = fminf(mn, smn[w]);
      mx = fmaxf(mx, smx[w]);
    }
    if (mn <= mx) {  // the CTA saw at least one voxel
      atomic_min_float(&bp->vmin, mn);
      atomic_max_float(&bp->vmax, mx);
    }
  }
}

cudaError_t launch_gather_fused(const void* level, int dtype, const long long dims[3], BrickInfo* bricks_dev,
                                int nbricks, int max_sz, void* pool0, void* pool1, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nbricks <= 0) return cudaSuccess;
  dim3 grid((unsigned)std::max(1, std::min(max_sz, 64)), (unsigned)nbricks);
  const int threads = 32 * GATHER_WARPS;
#define GBVR_GATHER(TT)                                                                                         \
  if (pool1)                                                                                                     \
    k_gather_fused<TT, true><<<grid, threads, 0, s>>>((const TT*)level, dims[0], dims[1], dims[2], bricks_dev,  \
                                                      (TT*)pool0, (TT*)pool1);                                   \
  else                                                                                                           \
    k_gather_fused<TT, false><<<grid, threads, 0, s>>>((const TT*)level, dims[0], dims[1], dims[2], bricks_dev, \
                                                       (TT*)pool0, nullptr);
  if (dtype == DT_U8) { GBVR_GATHER(uint8_t) }
  else if (dtype == DT_U16) { GBVR_GATHER(uint16_t) }
  else { GBVR_GATHER(float) }
#undef GBVR_GATHER
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Per-brick min/max over the stored voxels (ghosts included: the renderer's
// empty-space test needs the range of every voxel a sample can touch).
// One CTA per brick.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_brick_minmax(const T* __restrict__ pool, BrickInfo* __restrict__ bricks) {
  BrickInfo& b = bricks[blockIdx.x];
  const T* p = pool + b.offset;
  const long long n = (long long)b.sx * b.sy * b.sz;
  float mn = INFINITY, mx = -INFINITY;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    float v = (float)__ldg(p + i);
    mn = fminf(mn, v);
    mx = fmaxf(mx, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  __shared__ float smn[32], smx[32];
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { smn[w] = mn; smx[w] = mx; }
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
    mn = l < nw ? smn[l] : INFINITY;
    mx = l < nw ? smx[l] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) {
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (l == 0) { b.vmin = mn; b.vmax = mx; }
  }
}

cudaError_t launch_brick_minmax(const void* pool, int dtype, BrickInfo* bricks_dev, int nbricks, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nbricks <= 0) return cudaSuccess;
  if (dtype == DT_U8) k_brick_minmax<uint8_t><<<nbricks, 1024, 0, s>>>((const uint8_t*)pool, bricks_dev);
  else if (dtype == DT_U16) k_brick_minmax<uint16_t><<<nbricks, 1024, 0, s>>>((const uint16_t*)pool, bricks_dev);
  else k_brick_minmax<float><<<nbricks, 1024, 0, s>>>((const float*)pool, bricks_dev);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Macro-cell min/max for empty-space skipping inside bricks: one thread per
// cell, over the (M + 3)^3 voxels [c M - 1, c M + M + 1] around the
// footprints of its samples (the finer grid of the reference's
// GridLeaper-style acceleration).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_cell_minmax(const T* __restrict__ v, long long X, long long Y, long long Z, long long vz0, int sh,
                              int ncx, int ncy, int cz0, int cz1, float2* __restrict__ out) {
  // v holds planes vz0 .. of the level; cells of layers [cz0, cz1) are written
  const long long n = (long long)ncx * ncy * (cz1 - cz0);
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
    const long long cx = j % ncx, t = j / ncx, cy = t % ncy, cz = cz0 + t / ncy;
    // one voxel of margin beyond the footprint [c M, c M + M] on each side:
    // the walk skips empty cells by their estimated exit, and a sample that
    // rounding puts in a neighbouring cell is at most that far outside
    const long long x0 = max((cx << sh) - 1, 0LL), y0 = max((cy << sh) - 1, 0LL), z0 = max((cz << sh) - 1, 0LL);
    const long long x1 = min((cx << sh) + (1LL << sh) + 1, X - 1), y1 = min((cy << sh) + (1LL << sh) + 1, Y - 1),
                    z1 = min((cz << sh) + (1LL << sh) + 1, Z - 1);
    float mn = INFINITY, mx = -INFINITY;
    for (long long z = z0; z <= z1; ++z)
      for (long long y = y0; y <= y1; ++y) {
        const T* row = v + ((z - vz0) * Y + y) * X;
        for (long long x = x0; x <= x1; ++x) {
          float a = (float)__ldg(row + x);
          mn = fminf(mn, a);
          mx = fmaxf(mx, a);
        }
      }
    out[((long long)cz * ncy + cy) * ncx + cx] = make_float2(mn, mx);
  }
}

// The same ranges for 4^3 cells (shift 2) from a shared-memory tile: a CTA
// takes CX x 4 x 2 cells (CX = 15 for 8- and 16-bit voxels, 7 for float, so
// a tile row of 4 CX + 3 voxels fills whole warps), loads the voxels their
// ranges cover row by row (edge-replicated where the level ends, which
// leaves every range as the clamped one), and reduces along x (7 voxels per
// cell and row), then y, then z, keeping the partial minima and maxima as
// voxel values.  Each voxel is read from memory about 1.6 times instead of
// 5.4, with one 64-bit row address per row.
template <typename T> struct CellTile {
  static constexpr int CX = 15;  // 16-bit voxels: rows of 63 voxels, two warp-wide loads or one of words
  __device__ static T mn(T a, T b) { return a < b ? a : b; }
  __device__ static T mx(T a, T b) { return a > b ? a : b; }
};
// 8-bit voxels: rows of 127 voxels, so the halo is a smaller share
template <> struct CellTile<uint8_t> {
  static constexpr int CX = 31;
  __device__ static uint8_t mn(uint8_t a, uint8_t b) { return a < b ? a : b; }
  __device__ static uint8_t mx(uint8_t a, uint8_t b) { return a > b ? a : b; }
};
// float: fminf / fmaxf from +inf / -inf, as k_cell_minmax (NaN voxels are
// passed over)
template <> struct CellTile<float> {
  static constexpr int CX = 7;
  __device__ static float mn(float a, float b) { return fminf(a, b); }
  __device__ static float mx(float a, float b) { return fmaxf(a, b); }
};
constexpr int CT_Y = 4, CT_Z = 2;
constexpr int CV_Y = 4 * CT_Y + 3, CV_Z = 4 * CT_Z + 3;

template <typename T>
__global__ void __launch_bounds__(256) k_cell_minmax_tiled(const T* __restrict__ v, long long X, long long Y,
                                                           long long Z, long long vz0, int ncx, int ncy, int cz0,
                                                           int cz1, int tiles_x, int tiles_y, float2* __restrict__ out) {
  constexpr int CX = CellTile<T>::CX, VX = 4 * CX + 3;
  __shared__ T tile[CV_Z][CV_Y][VX];
  __shared__ T rmn[CV_Z][CV_Y][CX], rmx[CV_Z][CV_Y][CX];
  __shared__ T qmn[CV_Z][CT_Y][CX], qmx[CV_Z][CT_Y][CX];
  const int tx = blockIdx.x % tiles_x, ty = (blockIdx.x / tiles_x) % tiles_y, tz = blockIdx.x / (tiles_x * tiles_y);
  const int cx0 = tx * CX, cy0 = ty * CT_Y, cz0t = cz0 + tz * CT_Z;
  const long long vx0 = 4LL * cx0 - 1, vy0 = 4LL * cy0 - 1, vzz0 = 4LL * cz0t - 1;
  // planes the requested layers' ranges cover (the window holds them); a
  // tile reaching past the last layer reads clamped planes for cells it does
  // not write
  const long long zlo = max(4LL * cz0 - 1, 0LL), zhi = min(4LL * cz1 + 1, Z - 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // four rows per step, so that several loads of a lane are in flight together
  constexpr int NXL = (VX + 31) / 32;  // loads per lane and row
  static_assert(NXL <= 4, "a tile row is at most four warps wide");
  int xcol[NXL];
#pragma unroll
  for (int q = 0; q < NXL; ++q) xcol[q] = (int)min(max(vx0 + lane + 32 * q, 0LL), X - 1);
  constexpr int ROWS = CV_Y * CV_Z;
  // 16-bit voxels of a tile inside the level, rows of 4-byte-aligned words:
  // VPL voxels per load, from the word holding voxel vx0 on (lane l loads
  // voxels a0 + VPL l ..; columns outside the tile are dropped).  For 8-bit
  // voxels the four extractions and shared stores per word cost more than
  // the loads they save (c3: 24.7 against 28.3 ms), so they load one by one.
  constexpr int VPL = sizeof(T) == 2 ? 2 : 1;
  constexpr int SHIFT = VPL == 4 ? 3 : VPL == 2 ? 1 : 0;
  constexpr int NL = (VX + SHIFT + VPL - 1) / VPL;
  const long long a0 = vx0 - SHIFT;
  const bool words = VPL > 1 && a0 >= 0 && a0 + VPL * NL <= X && X % VPL == 0 &&
                     reinterpret_cast<uintptr_t>(v) % 4 == 0;
  if (words) {
#pragma unroll 4
    for (int row = warp; row < ROWS; row += 8) {
      const int ly = row % CV_Y, lz = row / CV_Y;
      const long long y = min(max(vy0 + ly, 0LL), Y - 1), z = min(max(vzz0 + lz, zlo), zhi);
      if (lane < NL) {
        const unsigned wv = __ldg(reinterpret_cast<const unsigned*>(v + ((z - vz0) * Y + y) * X + a0) + lane);
#pragma unroll
        for (int e = 0; e < VPL; ++e) {
          const int lx = VPL * lane + e - SHIFT;
          if (lx >= 0 && lx < VX) tile[lz][ly][lx] = (T)((wv >> (e * 8 * (int)sizeof(T))) & (VPL == 4 ? 0xffu : 0xffffu));
        }
      }
    }
  } else {
#pragma unroll 4
    for (int row = warp; row < ROWS; row += 8) {
      const int ly = row % CV_Y, lz = row / CV_Y;
      const long long y = min(max(vy0 + ly, 0LL), Y - 1), z = min(max(vzz0 + lz, zlo), zhi);
      const T* src = v + ((z - vz0) * Y + y) * X;
      T val[NXL];
#pragma unroll
      for (int q = 0; q < NXL; ++q) val[q] = lane + 32 * q < VX ? __ldg(src + xcol[q]) : T(0);
#pragma unroll
      for (int q = 0; q < NXL; ++q)
        if (lane + 32 * q < VX) tile[lz][ly][lane + 32 * q] = val[q];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < CX * CV_Y * CV_Z; i += blockDim.x) {
    const int c = i % CX, r = i / CX, ly = r % CV_Y, lz = r / CV_Y;
    using C = CellTile<T>;
    T mn = std::is_same<T, float>::value ? T(INFINITY) : tile[lz][ly][4 * c];
    T mx = std::is_same<T, float>::value ? T(-INFINITY) : mn;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      const T a = tile[lz][ly][4 * c + k];
      mn = C::mn(mn, a);
      mx = C::mx(mx, a);
    }
    rmn[lz][ly][c] = mn;
    rmx[lz][ly][c] = mx;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < CX * CT_Y * CV_Z; i += blockDim.x) {
    const int c = i % CX, r = i / CX, cy = r % CT_Y, lz = r / CT_Y;
    using C = CellTile<T>;
    T mn = rmn[lz][4 * cy][c], mx = rmx[lz][4 * cy][c];
#pragma unroll
    for (int k = 1; k < 7; ++k) {
      mn = C::mn(mn, rmn[lz][4 * cy + k][c]);
      mx = C::mx(mx, rmx[lz][4 * cy + k][c]);
    }
    qmn[lz][cy][c] = mn;
    qmx[lz][cy][c] = mx;
  }
  __syncthreads();
  if (threadIdx.x < CX * CT_Y * CT_Z) {
    const int c = threadIdx.x % CX, r = threadIdx.x / CX, cy = r % CT_Y, cz = r / CT_Y;
    const int gx = cx0 + c, gy = cy0 + cy, gz = cz0t + cz;
    if (gx < ncx && gy < ncy && gz < cz1) {
      using C = CellTile<T>;
      T mn = qmn[4 * cz][cy][c], mx = qmx[4 * cz][cy][c];
#pragma unroll
      for (int k = 1; k < 7; ++k) {
        mn = C::mn(mn, qmn[4 * cz + k][cy][c]);
        mx = C::mx(mx, qmx[4 * cz + k][cy][c]);
      }
      out[((long long)gz * ncy + gy) * ncx + gx] = make_float2((float)mn, (float)mx);
    }
  }
}

cudaError_t launch_cell_minmax_layers(const void* level, int dtype, const long long dims[3], long long vz0, int sh,
                                      const int nc[3], int cz0, int cz1, float2* out, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  const long long n = (long long)nc[0] * nc[1] * (cz1 - cz0);
  if (n <= 0) return cudaSuccess;
  if (sh == 2) {
    const int cx = dtype == DT_F32 ? CellTile<float>::CX : dtype == DT_U8 ? CellTile<uint8_t>::CX
                                                                            : CellTile<uint16_t>::CX;
    const int tiles_x = (nc[0] + cx - 1) / cx, tiles_y = (nc[1] + CT_Y - 1) / CT_Y,
              tiles_z = (cz1 - cz0 + CT_Z - 1) / CT_Z;
    const long long nt = (long long)tiles_x * tiles_y * tiles_z;
    if (nt < (1LL << 31)) {
#define GBVR_CELLS(TT)                                                                                         \
  k_cell_minmax_tiled<TT><<<(unsigned)nt, 256, 0, s>>>((const TT*)level, dims[0], dims[1], dims[2], vz0, nc[0], \
                                                        nc[1], cz0, cz1, tiles_x, tiles_y, out);
      if (dtype == DT_U8) { GBVR_CELLS(uint8_t) }
      else if (dtype == DT_U16) { GBVR_CELLS(uint16_t) }
      else { GBVR_CELLS(float) }
#undef GBVR_CELLS
      return cudaGetLastError();
    }
  }
  int threads = 128;
  int blocks = grid_for(n, threads);
  if (dtype == DT_U8)
    k_cell_minmax<uint8_t><<<blocks, threads, 0, s>>>((const uint8_t*)level, dims[0], dims[1], dims[2], vz0, sh, nc[0], nc[1], cz0, cz1, out);
  else if (dtype == DT_U16)
    k_cell_minmax<uint16_t><<<blocks, threads, 0, s>>>((const uint16_t*)level, dims[0], dims[1], dims[2], vz0, sh, nc[0], nc[1], cz0, cz1, out);
  else
    k_cell_minmax<float><<<blocks, threads, 0, s>>>((const float*)level, dims[0], dims[1], dims[2], vz0, sh, nc[0], nc[1], cz0, cz1, out);
  return cudaGetLastError();
}

__global__ void k_supercell_max(const float2* __restrict__ cells, int ncx, int ncy, int ncz, float* __restrict__ out,
                                int nsx, int nsy, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sx = (int)(i % nsx);
  const long long t = i / nsx;
  const int sy = (int)(t % nsy), sz = (int)(t / nsy);
  constexpr int E = 1 << SUPERCELL_SHIFT;
  float m = -INFINITY;
  for (int z = sz * E; z < min(sz * E + E, ncz); ++z)
    for (int y = sy * E; y < min(sy * E + E, ncy); ++y)
      for (int x = sx * E; x < min(sx * E + E, ncx); ++x) m = fmaxf(m, cells[((size_t)z * ncy + y) * ncx + x].y);
  out[i] = m;
}

cudaError_t launch_supercell_max(const float2* cells, const int nc[3], float* out, const int nsc[3], cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  const long long n = (long long)nsc[0] * nsc[1] * nsc[2];
  if (n <= 0) return cudaSuccess;
  k_supercell_max<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(cells, nc[0], nc[1], nc[2], out, nsc[0], nsc[1], n);
  return cudaGetLastError();
}

cudaError_t launch_cell_minmax(const void* level, int dtype, const long long dims[3], int sh, const int nc[3],
                               float2* out, cudaStream_t s) {
  return launch_cell_minmax_layers(level, dtype, dims, 0, sh, nc, 0, nc[2], out, s);
}

// ---------------------------------------------------------------------------
// 1D histogram (Histogram1DDataBlock::Compute, DataSource.h:603): one bin per
// value.  Privatised in shared memory (u32 per CTA, flushed with u64 global
// atomics) when the value range fits; global atomics otherwise.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_hist1d_smem(const T* __restrict__ v, long long n, unsigned long long* __restrict__ hist, int nbins) {
  extern __shared__ unsigned sh[];
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  unsigned run_bin = 0xffffffffu, run = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned b = (unsigned)__ldg(v + i);
    if (b >= (unsigned)nbins) continue;
    if (b == run_bin) {
      ++run;  // runs of one value (empty space) cost no shared-memory atomic
    } else {
      if (run) atomicAdd(sh + run_bin, run);
      run_bin = b;
      run = 1;
    }
  }
  if (run) atomicAdd(sh + run_bin, run);
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (sh[i]) atomicAdd(hist + i, (unsigned long long)sh[i]);
}

// The same from 16-byte loads: a thread takes 16 consecutive bytes (8 16-bit
// or 16 8-bit values) at a time, so runs of one value along x (smooth data,
// not only empty space) cost one shared-memory atomic.  v must be 16-byte
// aligned; the last n mod (16 / sizeof(T)) values are counted one by one.
template <typename T>
__global__ void k_hist1d_vec(const T* __restrict__ v, long long n, unsigned long long* __restrict__ hist, int nbins) {
  constexpr int PER = 16 / (int)sizeof(T);
  extern __shared__ unsigned sh[];
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  unsigned run_bin = 0xffffffffu, run = 0;
  auto count = [&](unsigned b) {
    if (b >= (unsigned)nbins) return;
    if (b == run_bin) {
      ++run;
    } else {
      if (run) atomicAdd(sh + run_bin, run);
      run_bin = b;
      run = 1;
    }
  };
  const long long nv = n / PER;
  const uint4* v4 = reinterpret_cast<const uint4*>(v);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nv; i += stride) {
    const uint4 w = __ldg(v4 + i);
    const unsigned q[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (sizeof(T) == 2) {
        count(q[k] & 0xffffu);
        count(q[k] >> 16);
      } else {
        count(q[k] & 0xffu);
        count((q[k] >> 8) & 0xffu);
        count((q[k] >> 16) & 0xffu);
        count(q[k] >> 24);
      }
    }
  }
  for (long long i = nv * PER + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    count((unsigned)__ldg(v + i));
  if (run) atomicAdd(sh + run_bin, run);
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (sh[i]) atomicAdd(hist + i, (unsigned long long)sh[i]);
}

template <typename T>
__global__ void k_hist1d_global(const T* __restrict__ v, long long n, unsigned long long* __restrict__ hist, int nbins) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned b = (unsigned)__ldg(v + i);
    if (b < (unsigned)nbins) atomicAdd(hist + b, 1ULL);
  }
}

cudaError_t launch_hist1d(const void* vol, int dtype, long long n, unsigned long long* hist, int nbins, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (dtype == DT_F32) return cudaErrorInvalidValue;
  int threads = 512;
  int blocks = grid_for(n, threads);
  if (blocks > 152 * 4) blocks = 152 * 4;
  if (nbins <= 16384) {
    size_t smem = sizeof(unsigned) * nbins;
    const bool vec = ((uintptr_t)vol & 15) == 0;
    const void* fn = vec ? (dtype == DT_U8 ? (const void*)k_hist1d_vec<uint8_t> : (const void*)k_hist1d_vec<uint16_t>)
                         : (dtype == DT_U8 ? (const void*)k_hist1d_smem<uint8_t> : (const void*)k_hist1d_smem<uint16_t>);
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    if (vec) {
      if (dtype == DT_U8) k_hist1d_vec<uint8_t><<<blocks, threads, smem, s>>>((const uint8_t*)vol, n, hist, nbins);
      else k_hist1d_vec<uint16_t><<<blocks, threads, smem, s>>>((const uint16_t*)vol, n, hist, nbins);
    } else if (dtype == DT_U8) {
      k_hist1d_smem<uint8_t><<<blocks, threads, smem, s>>>((const uint8_t*)vol, n, hist, nbins);
    } else {
      k_hist1d_smem<uint16_t><<<blocks, threads, smem, s>>>((const uint16_t*)vol, n, hist, nbins);
    }
  } else {
    k_hist1d_global<uint16_t><<<blocks, threads, 0, s>>>((const uint16_t*)vol, n, hist, nbins);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// 2D histogram (Histogram2DDataBlock::Compute, DataSource.h:609-616), rule
// recovered bit-exactly from DemoData/c60.uvf and stated as an f64 formula:
//   f = voxel / maxScalar; g_a = central difference / 2 inside, one-sided
//   first difference on borders; |g| = sqrt((gx^2 + gy^2) + gz^2);
//   y-bin = floor(|g| / max|g| * 255).
// Evaluating that in f64 for every voxel is slow on this part, so the kernel
// works in exact integers: with D_a = v[i+1] - v[i-1] inside and
// 2 (v[1] - v[0]) on borders, |g| = sqrt(S) / (2 maxScalar) with
// S = Dx^2 + Dy^2 + Dz^2, and the exact bin is the largest k with
// k^2 Smax <= 65025 S.  The f64 formula can only land on a different integer
// when 65025 S - k^2 Smax is within f64 rounding of zero; since that
// difference is an integer and |r - k| >= 1 / (511 Smax) whenever it is
// non-zero, which exceeds the f64 error bound (~2e-13 at r <= 255) for every
// 8- or 16-bit volume, only exact ties (65025 S == k^2 Smax) are evaluated
// with the f64 formula itself, using __d*_rn intrinsics in the same order.
// Pass 1 finds Smax and the f64 max |g| over the voxels attaining it;
// pass 2 bins.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void int_diffs(const T* __restrict__ v, long long X, long long Y, long long Z, long long x,
                                          long long y, long long z, long long i, int D[3]) {
  const long long sx = 1, sy = X, sz = X * Y;
  const long long c[3] = {x, y, z}, n[3] = {X, Y, Z}, st[3] = {sx, sy, sz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (n[a] == 1) D[a] = 0;
    else if (c[a] == 0) D[a] = 2 * ((int)__ldg(v + i + st[a]) - (int)__ldg(v + i));
    else if (c[a] == n[a] - 1) D[a] = 2 * ((int)__ldg(v + i) - (int)__ldg(v + i - st[a]));
    else D[a] = (int)__ldg(v + i + st[a]) - (int)__ldg(v + i - st[a]);
  }
}

// The f64 formula for one voxel, operation for operation.  Called only for
// exact ties and the voxels attaining Smax: kept out of line so the common
// path does not carry its registers.
template <typename T>
__device__ __noinline__ double grad_f64(const T* __restrict__ v, long long X, long long Y, long long Z, long long x, long long y,
                           long long z, long long i, double c) {
  const long long c3[3] = {x, y, z}, n[3] = {X, Y, Z}, st[3] = {1, X, X * Y};
  double g[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (n[a] == 1) { g[a] = 0.0; continue; }
    if (c3[a] == 0) g[a] = __dsub_rn(__ddiv_rn((double)__ldg(v + i + st[a]), c), __ddiv_rn((double)__ldg(v + i), c));
    else if (c3[a] == n[a] - 1) g[a] = __dsub_rn(__ddiv_rn((double)__ldg(v + i), c), __ddiv_rn((double)__ldg(v + i - st[a]), c));
    else g[a] = __ddiv_rn(__dsub_rn(__ddiv_rn((double)__ldg(v + i + st[a]), c), __ddiv_rn((double)__ldg(v + i - st[a]), c)), 2.0);
  }
  double s = __dmul_rn(g[0], g[0]);
  s = __dadd_rn(s, __dmul_rn(g[1], g[1]));
  s = __dadd_rn(s, __dmul_rn(g[2], g[2]));
  return __dsqrt_rn(s);
}

// The gradient row of a voxel: floor(255 sqrt(S / Smax)) for 0 < S <= Smax,
// exactly.  The FP32 estimate is within 2e-4 of the real value (S and Smax
// below 2^36 converted with relative error 2^-24, a rounded reciprocal and
// product, rsqrtf within 2 ulp, times 255), so when its fraction lies more
// than 1/256 from an integer its floor is the answer; otherwise (and for the
// top row) the exact integer tests decide: the largest k with
// k^2 Smax <= 65025 S.  tie: k^2 Smax == 65025 S, the real value is the
// integer k and the f64 formula decides between k and k - 1.
template <typename U>
__device__ __forceinline__ int h2_row(U S, unsigned long long smax, float inv_smax, bool& tie) {
  const float q = (float)S * inv_smax;
  const float est = 255.f * (q * rsqrtf(q));
  const float fl = floorf(est);
  const float fr = est - fl;
  int k = (int)fl;
  tie = false;
  if (fr > 1.f / 256.f && fr < 255.f / 256.f && k < 255) return k;
  const unsigned long long lhs = 65025ULL * (unsigned long long)S;
  if (k > 255) k = 255;
  while (k < 255 && (unsigned long long)(k + 1) * (k + 1) * smax <= lhs) ++k;
  while (k > 0 && (unsigned long long)k * k * smax > lhs) --k;
  tie = (unsigned long long)k * k * smax == lhs;
  return k;
}

// The three passes walk the volume row by row (one CTA per z-slab of rows,
// threads along x) so no voxel pays for a 64-bit division of its index.
// They cover the planes [zb, ze) of a Z-plane volume of which `v` holds the
// planes from zlo on (a slab of a volume streamed in z: the planes zb - 1
// and ze, where they exist, must be present for the z differences); the
// whole volume is zb = zlo = 0, ze = Z.
template <typename T>
__global__ void k_hist2d_pass1(const T* __restrict__ v, long long X, long long Y, long long Z, long long zb,
                               long long ze, long long zlo, Hist2DScratch* sc) {
  unsigned long long smax = 0;
  for (long long row = blockIdx.x; row < Y * (ze - zb); row += gridDim.x) {
    const long long zr = row / Y, y = row - zr * Y, z = zb + zr;
    for (long long x = threadIdx.x; x < X; x += blockDim.x) {
      const long long i = ((z - zlo) * Y + y) * X + x;
      int D[3];
      int_diffs(v, X, Y, Z, x, y, z, i, D);
      const unsigned long long S =
          (unsigned long long)((long long)D[0] * D[0] + (long long)D[1] * D[1] + (long long)D[2] * D[2]);
      smax = S > smax ? S : smax;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long t = __shfl_xor_sync(0xffffffffu, smax, o);
    smax = t > smax ? t : smax;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(&sc->smax, smax);
}

// f64 max |g| over the voxels with S == Smax (positive doubles order like
// their bit patterns).
template <typename T>
__global__ void k_hist2d_pass1b(const T* __restrict__ v, long long X, long long Y, long long Z, long long zb,
                                long long ze, long long zlo, double c, Hist2DScratch* sc) {
  const unsigned long long smax = sc->smax;
  if (smax == 0) return;
  for (long long row = blockIdx.x; row < Y * (ze - zb); row += gridDim.x) {
    const long long zr = row / Y, y = row - zr * Y, z = zb + zr;
    for (long long x = threadIdx.x; x < X; x += blockDim.x) {
      const long long i = ((z - zlo) * Y + y) * X + x;
      int D[3];
      int_diffs(v, X, Y, Z, x, y, z, i, D);
      const unsigned long long S =
          (unsigned long long)((long long)D[0] * D[0] + (long long)D[1] * D[1] + (long long)D[2] * D[2]);
      if (S == smax) {
        const double g = grad_f64(v, X, Y, Z, x, y, z, i, c);
        atomicMax(&sc->gmax_bits, (unsigned long long)__double_as_longlong(g));
      }
    }
  }
}

template <typename T>
__global__ void k_hist2d_pass2(const T* __restrict__ v, long long X, long long Y, long long Z, long long zb,
                               long long ze, long long zlo, double c, long long nx, long long merge,
                               unsigned long long* __restrict__ hist, const Hist2DScratch* sc) {
  const unsigned long long smax = sc->smax;
  const double gmax = __longlong_as_double((long long)sc->gmax_bits);
  const float smax_f = (float)smax;
  const float inv_smax = 1.f / smax_f;  // the estimate below needs to be within one bin only
  const bool merge1 = merge == 1;
  // values are below 2^16, so any merge above 2^16 bins like 2^16
  const unsigned merge32 = (unsigned)(merge < 1 ? 1 : merge > 65536 ? 65536 : merge);
  unsigned long long run_bin = ~0ULL, run = 0;
  for (long long row = blockIdx.x; row < Y * (ze - zb); row += gridDim.x) {
    const long long zr = row / Y, y = row - zr * Y, z = zb + zr;
    for (long long x = threadIdx.x; x < X; x += blockDim.x) {
      const long long i = ((z - zlo) * Y + y) * X + x;
      int D[3];
      int_diffs(v, X, Y, Z, x, y, z, i, D);
      const unsigned long long S =
          (unsigned long long)((long long)D[0] * D[0] + (long long)D[1] * D[1] + (long long)D[2] * D[2]);
      int k = 0;
      if (smax > 0 && S > 0) {
        const unsigned long long lhs = 65025ULL * S;
        // FP32 estimate (within one of the exact bin: S, Smax < 2^36), then
        // settled by the exact integer tests; FP64 arithmetic is slow on this
        // part and stays confined to ties
        (void)lhs;
        bool tie;
        k = h2_row(S, smax, inv_smax, tie);
        if (tie) {
          // exact tie: the f64 formula decides between k and k - 1
          const double g = grad_f64(v, X, Y, Z, x, y, z, i, c);
          const double r = __dmul_rn(__ddiv_rn(g, gmax), 255.0);
          k = (int)floor(r);
          if (k > 255) k = 255;
        }
      }
      const unsigned val = (unsigned)__ldg(v + i);
      long long bx = merge1 ? val : val / merge32;
      if (bx >= nx) bx = nx - 1;
      // run-length accumulation per thread: empty space puts almost every
      // voxel in one bin, and one atomic per voxel on one address serialises
      const unsigned long long bin = (unsigned long long)(bx * 256 + k);
      if (bin == run_bin) {
        ++run;
      } else {
        if (run) atomicAdd(hist + run_bin, run);
        run_bin = bin;
        run = 1;
      }
    }
  }
  if (run) atomicAdd(hist + run_bin, run);
}

// ---- vectorised z-march: rows whose length is a multiple of 4 voxels ----
// Each thread owns a column of 4 consecutive voxels (x0 .. x0 + 3 of row y)
// and walks it along z, keeping the planes z - 1, z, z + 1 of the column in
// registers: per step one 4-voxel load of the next plane, one of each of the
// rows y - 1 and y + 1, and two scalar loads for the x neighbours.  The
// border rules (one-sided difference x 2 on the faces) are the multipliers
// my / mz.  Same integer differences as int_diffs.
// 4 consecutive voxels of a row as raw words: one 32-bit word for 8-bit
// voxels, two for 16-bit ones (the column walker keeps its planes packed so
// that the neighbour rows of the next plane fit in registers too).
template <typename T> struct Packed4;
template <> struct Packed4<uint8_t> {
  using W = unsigned;
  __device__ static W load(const uint8_t* p) { return __ldg(reinterpret_cast<const unsigned*>(p)); }
  __device__ static int at(W w, int j) { return (int)((w >> (8 * j)) & 0xffu); }
};
template <> struct Packed4<uint16_t> {
  using W = uint2;
  __device__ static W load(const uint16_t* p) { return __ldg(reinterpret_cast<const uint2*>(p)); }
  __device__ static int at(W w, int j) { return (int)(((j < 2 ? w.x : w.y) >> (16 * (j & 1))) & 0xffffu); }
};

// Squared-difference sums: below 2^20 for 8-bit voxels (32-bit arithmetic),
// up to 3 (2 x 65535)^2 for 16-bit ones (64-bit), or, NARROW, below
// 3 (2 x 16383)^2 < 2^32 for 16-bit volumes whose values stay below 16384
// (12-bit data; the caller knows the volume's maximum): 32-bit again.
template <typename T, bool NARROW = false> struct SumT { using U = unsigned long long; };
template <bool NARROW> struct SumT<uint8_t, NARROW> { using U = unsigned; };
template <> struct SumT<uint16_t, true> { using U = unsigned; };

// A 4-voxel column walked along z: packed planes, the neighbour rows of
// plane z + 1 loaded in step(z), a full step before they are used (c3's 2D
// histogram 39.4 -> 33.4 ms; for 16-bit voxels, with the binning pass at
// 640 threads and 96 registers, c2's 9.40 -> 8.86 ms).
template <typename T>
struct ColumnAhead {
  using P = Packed4<T>;
  using W = typename P::W;
  const T* base;  // voxel (x0, y, 0)
  long long plane;
  int X, Z, x0, ym, yp, my;
  W prv, cur, nxt;  // planes z - 1, z, z + 1 of the 4 voxels
  W na, nb;         // rows y - 1 and y + 1 of plane z, loaded a plane ahead
  int nxl, nxr;     // voxels x0 - 1 and x0 + 4 of plane z, likewise
  __device__ __forceinline__ void load_neighbours(int z) {
    const T* row = base + z * plane;
    na = P::load(row + ym);
    nb = P::load(row + yp);
    nxl = x0 > 0 ? (int)__ldg(row - 1) : 0;
    nxr = x0 + 4 < X ? (int)__ldg(row + 4) : 0;
  }
  __device__ __forceinline__ ColumnAhead(const T* v, int X_, int Y, int Z_, int x0_, int y) {
    X = X_; Z = Z_; x0 = x0_;
    plane = (long long)X * Y;
    base = v + (long long)y * X + x0;
    if (Y == 1) { ym = yp = 0; my = 0; }
    else if (y == 0) { ym = 0; yp = X; my = 2; }
    else if (y == Y - 1) { ym = -X; yp = 0; my = 2; }
    else { ym = -X; yp = X; my = 1; }
    cur = P::load(base);
    nxt = Z > 1 ? P::load(base + plane) : cur;
    prv = cur;
    load_neighbours(0);
  }
  // voxel j of plane z (after step(z - 1))
  __device__ __forceinline__ int val(int j) const { return P::at(cur, j); }
  // S = Dx^2 + Dy^2 + Dz^2 of the 4 voxels at plane z (their values in cur),
  // in U: unsigned arithmetic modulo 2^bits, exact while the sum fits
  template <typename U>
  __device__ __forceinline__ void diffs(int z, U S[4]) const {
    int c[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) c[j] = P::at(cur, j);
    int dx[4];
    dx[0] = x0 == 0 ? 2 * (c[1] - c[0]) : c[1] - nxl;
    dx[1] = c[2] - c[0];
    dx[2] = c[3] - c[1];
    dx[3] = x0 + 4 == X ? 2 * (c[3] - c[2]) : nxr - c[2];
    const int mz = Z == 1 ? 0 : ((z == 0 || z == Z - 1) ? 2 : 1);
    const W zm = z == 0 ? cur : prv;
    const W zp = z == Z - 1 ? cur : nxt;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const U ux = (U)dx[j], uy = (U)(my * (P::at(nb, j) - P::at(na, j))),
              uz = (U)(mz * (P::at(zp, j) - P::at(zm, j)));
      S[j] = ux * ux + uy * uy + uz * uz;
    }
  }
  // move to plane z + 1: its neighbour rows and the plane after it are
  // loaded now, a full step before they are used
  __device__ __forceinline__ void step(int z) {
    prv = cur;
    cur = nxt;
    if (z + 2 < Z) nxt = P::load(base + (z + 2) * plane);
    if (z + 1 < Z) load_neighbours(z + 1);
  }
};

// Pass 1: the largest S.  One thread per 4-voxel column (all of z), which
// also records where its column attains its own largest S (the first
// COL_KEEP voxels as 4 z + j, and how many there are), so that the f64 pass
// revisits only those voxels.
constexpr int COL_KEEP = 3;
struct ColMax {
  unsigned long long s;
  unsigned cnt;
  unsigned pos[COL_KEEP];
};

template <typename T, bool NARROW>
__global__ void __launch_bounds__(256) k_h2v_max(const T* __restrict__ v, int X, int Y, int Z, Hist2DScratch* sc,
                                                 ColMax* __restrict__ cols) {
  const int cpr = X >> 2;
  const long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  using U = typename SumT<T, NARROW>::U;
  U smax = 0;
  if (col < (long long)cpr * Y) {
    const int y = (int)(col / cpr), x0 = 4 * (int)(col - (long long)y * cpr);
    ColumnAhead<T> c(v, X, Y, Z, x0, y);
    unsigned cnt = 0, pos[COL_KEEP] = {0u, 0u, 0u};
    for (int z = 0; z < Z; ++z) {
      U S[4];
      c.diffs(z, S);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (S[j] > smax) {
          smax = S[j];
          cnt = 0;
        }
        if (S[j] == smax && smax > 0) {
#pragma unroll
          for (int q = 0; q < COL_KEEP; ++q)
            if (cnt == (unsigned)q) pos[q] = 4u * (unsigned)z + (unsigned)j;
          ++cnt;
        }
      }
      c.step(z);
    }
    ColMax r;
    r.s = (unsigned long long)smax;
    r.cnt = cnt;
#pragma unroll
    for (int q = 0; q < COL_KEEP; ++q) r.pos[q] = pos[q];
    cols[col] = r;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const U t = __shfl_xor_sync(0xffffffffu, smax, o);
    smax = t > smax ? t : smax;
  }
  if ((threadIdx.x & 31) == 0 && smax) atomicMax(&sc->smax, (unsigned long long)smax);
}

// Pass 1b: the f64 |g| over the voxels attaining Smax, one thread per
// column record: the recorded voxels, or the whole column again when it
// attains Smax at more voxels than were recorded.
template <typename T, bool NARROW>
__global__ void __launch_bounds__(256) k_h2v_gmax(const T* __restrict__ v, int X, int Y, int Z, double c,
                                                  Hist2DScratch* sc, const ColMax* __restrict__ cols) {
  const unsigned long long smax = sc->smax;
  if (smax == 0) return;
  const int cpr = X >> 2;
  const long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= (long long)cpr * Y) return;
  const ColMax r = cols[col];
  if (r.s != smax) return;
  const int y = (int)(col / cpr), x0 = 4 * (int)(col - (long long)y * cpr);
  if (r.cnt <= (unsigned)COL_KEEP) {
    for (unsigned q = 0; q < r.cnt; ++q) {
      const int z = (int)(r.pos[q] >> 2), j = (int)(r.pos[q] & 3u);
      const double g = grad_f64(v, X, Y, Z, x0 + j, y, z, ((long long)z * Y + y) * X + x0 + j, c);
      atomicMax(&sc->gmax_bits, (unsigned long long)__double_as_longlong(g));
    }
    return;
  }
  ColumnAhead<T> cl(v, X, Y, Z, x0, y);
  for (int z = 0; z < Z; ++z) {
    typename SumT<T, NARROW>::U S[4];
    cl.diffs(z, S);
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if ((unsigned long long)S[j] == smax) {
        const double g = grad_f64(v, X, Y, Z, x0 + j, y, z, ((long long)z * Y + y) * X + x0 + j, c);
        atomicMax(&sc->gmax_bits, (unsigned long long)__double_as_longlong(g));
      }
    cl.step(z);
  }
}

// Pass 2: bins.  SMEM: each block counts the gradient rows k < kshared into
// a shared copy of that part of the histogram (two 16-bit counters per word,
// nx * kshared bins; about 48 KB so several blocks share an SM) and adds it
// to the global one every `flush_steps` z-steps, before any counter can
// reach 2^16 (flush_steps * 4 * blockDim <= 65535); higher rows, rare in
// practice, go to global memory directly.  Blocks loop over groups of
// blockDim columns.  Runs of equal bins along a thread's voxels are counted
// in registers first either way.
// WIDE: 32-bit shared counters, one per bin (one block per SM with about
// 200 KB of them: 768 threads for 8-bit data, 640 at 96 registers for 16-bit
// data), flushed only when a counter could overflow, i.e. in practice once at
// the end, instead of 16-bit pairs flushed every 63 z-steps.
template <typename T, bool SMEM, bool WIDE = false, bool NARROW = false>
__global__ void __launch_bounds__(WIDE ? (sizeof(T) == 2 ? 640 : 768) : 256, WIDE ? 1 : 3)
    k_h2v_bin(const T* __restrict__ v, int X, int Y, int Z, double c, int nx, int merge,
              unsigned long long* __restrict__ hist, const Hist2DScratch* sc, int flush_steps, int kshared) {
  extern __shared__ unsigned sh[];
  const unsigned long long smax = sc->smax;
  const double gmax = __longlong_as_double((long long)sc->gmax_bits);
  const float smax_f = (float)smax;
  const float inv_smax = 1.f / smax_f;  // the estimate below needs to be within one bin only
  const unsigned merge32 = (unsigned)merge;
  const int words = WIDE ? nx * kshared : nx * kshared / 2;  // kshared is even
  if (SMEM) {
    for (int i = threadIdx.x; i < words; i += blockDim.x) sh[i] = 0;
    __syncthreads();
  }
  unsigned run_bin = ~0u, run = 0;
  auto add = [&](unsigned bin, unsigned cnt) {
    const unsigned k = bin & 255u;
    if (SMEM && k < (unsigned)kshared) {
      const unsigned sb = (bin >> 8) * (unsigned)kshared + k;
      if (WIDE) atomicAdd(sh + sb, cnt);
      else atomicAdd(sh + (sb >> 1), cnt << ((sb & 1u) << 4));
    } else {
      atomicAdd(hist + bin, (unsigned long long)cnt);
    }
  };
  auto flush = [&]() {
    if (run) add(run_bin, run);
    run = 0;
    run_bin = ~0u;
    __syncthreads();
    for (int i = threadIdx.x; i < words; i += blockDim.x) {
      const unsigned wv = sh[i];
      if (wv) {
        if (WIDE) {
          const unsigned bx = (unsigned)i / (unsigned)kshared, k = (unsigned)i - bx * (unsigned)kshared;
          atomicAdd(hist + bx * 256u + k, (unsigned long long)wv);
        } else {
          const unsigned sb = 2u * i, bx = sb / (unsigned)kshared, k = sb - bx * (unsigned)kshared;  // k even
          if (wv & 0xffffu) atomicAdd(hist + bx * 256u + k, (unsigned long long)(wv & 0xffffu));
          if (wv >> 16) atomicAdd(hist + bx * 256u + k + 1, (unsigned long long)(wv >> 16));
        }
        sh[i] = 0;
      }
    }
    __syncthreads();
  };
  const int cpr = X >> 2;
  const long long ncols = (long long)cpr * Y;
  const long long groups = (ncols + blockDim.x - 1) / blockDim.x;
  int since = 0;
  for (long long g = blockIdx.x; g < groups; g += gridDim.x) {
    const long long col = g * blockDim.x + threadIdx.x;
    const bool active = col < ncols;
    const int y = active ? (int)(col / cpr) : 0, x0 = active ? 4 * (int)(col - (long long)y * cpr) : 0;
    ColumnAhead<T> cl(v, X, Y, Z, x0, y);  // inactive threads walk column 0 and count nothing
    for (int z = 0; z < Z; ++z) {
      if (active) {
        typename SumT<T, NARROW>::U S[4];
        cl.diffs(z, S);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          int k = 0;
          if (smax > 0 && S[j] > 0) {
            const unsigned long long lhs = 65025ULL * (unsigned long long)S[j];
            // FP32 estimate (within one of the exact bin), settled exactly
            (void)lhs;
            bool tie;
            k = h2_row(S[j], smax, inv_smax, tie);
            if (tie) {
              // exact tie: the f64 formula decides
              const double gg = grad_f64(v, X, Y, Z, x0 + j, y, z, ((long long)z * Y + y) * X + x0 + j, c);
              k = (int)floor(__dmul_rn(__ddiv_rn(gg, gmax), 255.0));
              if (k > 255) k = 255;
            }
          }
          int bx = merge32 == 1 ? cl.val(j) : (int)((unsigned)cl.val(j) / merge32);
          if (bx >= nx) bx = nx - 1;
          const unsigned bin = (unsigned)bx * 256u + (unsigned)k;
          if (bin == run_bin) {
            ++run;
          } else {
            if (run) add(run_bin, run);
            run_bin = bin;
            run = 1;
          }
        }
        cl.step(z);
      }
      if (SMEM && ++since == flush_steps) {
        flush();
        since = 0;
      }
    }
  }
  if (SMEM) {
    flush();
  } else if (run) {
    add(run_bin, run);
  }
}

// The three passes of the 4-voxel-column path.
template <typename T, bool NARROW>
static cudaError_t hist2d_vec_passes(const T* v, int X, int Y, int Z, double c, int nx, int merge,
                                     unsigned long long* hist, Hist2DScratch* scratch, ColMax* cols, long long blocks,
                                     int threads, bool smem, size_t shbytes, int grid2, int wide_threads,
                                     int flush_steps, int kshared, cudaStream_t s) {
  k_h2v_max<T, NARROW><<<(unsigned)blocks, threads, 0, s>>>(v, X, Y, Z, scratch, cols);
  k_h2v_gmax<T, NARROW><<<(unsigned)blocks, threads, 0, s>>>(v, X, Y, Z, c, scratch, cols);
  if (smem) {
    const cudaError_t e =
        cudaFuncSetAttribute(k_h2v_bin<T, true, true, NARROW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shbytes);
    if (e != cudaSuccess) return e;
    k_h2v_bin<T, true, true, NARROW><<<grid2, wide_threads, shbytes, s>>>(v, X, Y, Z, c, nx, merge, hist, scratch,
                                                                         flush_steps, kshared);
  } else {
    k_h2v_bin<T, false, false, NARROW><<<grid2, threads, 0, s>>>(v, X, Y, Z, c, nx, merge, hist, scratch, 0, 0);
  }
  return cudaGetLastError();
}

cudaError_t launch_hist2d(const void* vol, int dtype, const long long dims[3], double max_scalar, long long nx,
                          long long merge, unsigned long long* hist, Hist2DScratch* scratch, cudaStream_t s,
                          bool narrow) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (dtype == DT_F32) return cudaErrorInvalidValue;
  {
    const long long X = dims[0], Y = dims[1], Z = dims[2];
    const size_t es = dtype == DT_U8 ? 1 : 2;
    const bool vec = X >= 4 && X % 4 == 0 && X <= (1LL << 30) && Y <= (1LL << 30) && Z <= (1LL << 30) &&
                     ((uintptr_t)vol % (4 * es)) == 0 && merge >= 1 && merge <= 65536 && nx >= 1 && nx <= (1LL << 22);
    if (vec) {
      int dev = 0, sms = 152;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      const double c = max_scalar > 0 ? max_scalar : 1.0;
      const int threads = 256;
      const long long ncols = (X / 4) * Y;
      const long long blocks = (ncols + threads - 1) / threads;
      if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
      cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(Hist2DScratch), s);
      if (e != cudaSuccess) return e;
      // one record per column (stream-ordered, freed after the passes)
      ColMax* cols = nullptr;
      e = cudaMallocAsync(reinterpret_cast<void**>(&cols), (size_t)ncols * sizeof(ColMax), s);
      if (e != cudaSuccess) return e;
      // shared counters for the gradient rows k < kshared: 32 bits per bin in
      // about 200 KB for one block per SM (768 threads at 80 registers for
      // 8-bit data, 640 at 96 for 16-bit data, whose packed column walker
      // needs the registers); a block adds at most 4 * wide_threads voxels
      // per z-step, so counters flush before 2^32
      const int wide_threads = dtype == DT_U16 ? 640 : 768;
      const int kshared = (int)std::min<long long>(256, ((200 * 1024) / (4 * nx)) & ~1LL);
      const bool smem = kshared >= 2;
      const size_t shbytes = smem ? (size_t)nx * kshared * 4 : 0;
      const int flush_steps = (int)std::min<long long>(0x7fffffffLL, 0xffffffffLL / (4 * wide_threads));
      const long long wblocks = (ncols + wide_threads - 1) / wide_threads;
      const int grid2 = smem ? (int)std::min<long long>(wblocks, (long long)sms) : (int)blocks;
      const int nxi = (int)nx, mi = (int)merge, Xi = (int)X, Yi = (int)Y, Zi = (int)Z;
      if (dtype == DT_U8)
        e = hist2d_vec_passes<uint8_t, false>((const uint8_t*)vol, Xi, Yi, Zi, c, nxi, mi, hist, scratch, cols,
                                              blocks, threads, smem, shbytes, grid2, wide_threads, flush_steps,
                                              kshared, s);
      else if (narrow)
        e = hist2d_vec_passes<uint16_t, true>((const uint16_t*)vol, Xi, Yi, Zi, c, nxi, mi, hist, scratch, cols,
                                              blocks, threads, smem, shbytes, grid2, wide_threads, flush_steps,
                                              kshared, s);
      else
        e = hist2d_vec_passes<uint16_t, false>((const uint16_t*)vol, Xi, Yi, Zi, c, nxi, mi, hist, scratch, cols,
                                               blocks, threads, smem, shbytes, grid2, wide_threads, flush_steps,
                                               kshared, s);
      if (e != cudaSuccess) {
        cudaFreeAsync(cols, s);
        return e;
      }
      e = cudaGetLastError();
      const cudaError_t ef = cudaFreeAsync(cols, s);
      return e != cudaSuccess ? e : ef;
    }
  }
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (dtype == DT_F32) return cudaErrorInvalidValue;
  const long long X = dims[0], Y = dims[1], Z = dims[2];
  const double c = max_scalar > 0 ? max_scalar : 1.0;
  const int threads = X >= 256 ? 256 : 128;
  long long rows = Y * Z;
  const int blocks = (int)(rows < 152LL * 64 ? rows : 152LL * 64);
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(Hist2DScratch), s);
  if (e != cudaSuccess) return e;
  if (dtype == DT_U8) {
    const uint8_t* v = (const uint8_t*)vol;
    k_hist2d_pass1<<<blocks, threads, 0, s>>>(v, X, Y, Z, 0, Z, 0, scratch);
    k_hist2d_pass1b<<<blocks, threads, 0, s>>>(v, X, Y, Z, 0, Z, 0, c, scratch);
    k_hist2d_pass2<<<blocks, threads, 0, s>>>(v, X, Y, Z, 0, Z, 0, c, nx, merge, hist, scratch);
  } else {
    const uint16_t* v = (const uint16_t*)vol;
    k_hist2d_pass1<<<blocks, threads, 0, s>>>(v, X, Y, Z, 0, Z, 0, scratch);
    k_hist2d_pass1b<<<blocks, threads, 0, s>>>(v, X, Y, Z, 0, Z, 0, c, scratch);
    k_hist2d_pass2<<<blocks, threads, 0, s>>>(v, X, Y, Z, 0, Z, 0, c, nx, merge, hist, scratch);
  }
  return cudaGetLastError();
}

cudaError_t launch_hist2d_slab(const void* slab, int dtype, const long long dims[3], long long zb, long long ze,
                               long long zlo, double max_scalar, long long nx, long long merge, int pass,
                               unsigned long long* hist, Hist2DScratch* scratch, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (dtype == DT_F32 || pass < 1 || pass > 3) return cudaErrorInvalidValue;
  const long long X = dims[0], Y = dims[1], Z = dims[2];
  if (zb < 0 || ze > Z || zb >= ze || zlo > zb || (zb > 0 && zlo > zb - 1)) return cudaErrorInvalidValue;
  const double c = max_scalar > 0 ? max_scalar : 1.0;
  const int threads = X >= 256 ? 256 : 128;
  const long long rows = Y * (ze - zb);
  const int blocks = (int)(rows < 152LL * 64 ? rows : 152LL * 64);
  if (dtype == DT_U8) {
    const uint8_t* v = (const uint8_t*)slab;
    if (pass == 1) k_hist2d_pass1<<<blocks, threads, 0, s>>>(v, X, Y, Z, zb, ze, zlo, scratch);
    else if (pass == 2) k_hist2d_pass1b<<<blocks, threads, 0, s>>>(v, X, Y, Z, zb, ze, zlo, c, scratch);
    else k_hist2d_pass2<<<blocks, threads, 0, s>>>(v, X, Y, Z, zb, ze, zlo, c, nx, merge, hist, scratch);
  } else {
    const uint16_t* v = (const uint16_t*)slab;
    if (pass == 1) k_hist2d_pass1<<<blocks, threads, 0, s>>>(v, X, Y, Z, zb, ze, zlo, scratch);
    else if (pass == 2) k_hist2d_pass1b<<<blocks, threads, 0, s>>>(v, X, Y, Z, zb, ze, zlo, c, scratch);
    else k_hist2d_pass2<<<blocks, threads, 0, s>>>(v, X, Y, Z, zb, ze, zlo, c, nx, merge, hist, scratch);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// LZ4 block decoding of paged bricks (out-of-core store compressed with the
// codec of lz4.cpp, one block per 16 KiB chunk of a brick), one warp per
// chunk, every read and write bound checked.
//
// Window path (most sequences of brick data: no or few literals, a 2-byte
// offset, at most one length byte, i.e. 3-4 input bytes for ~30 output
// bytes): the warp loads the 32 input bytes at the parse position, and every
// lane decodes the sequence that would start at its byte.  Walking the true
// starts from lane 0 is one shuffle per sequence; the sequences that lie
// wholly in the window (up to 10) are then written together, 32 output bytes
// per step.  A lane finds the sequence of its byte from the sequences'
// output starts (a prefix sum), and takes a literal from the window, a match
// byte written by an earlier step from memory, or a match byte of the same
// step from the lane that writes it (pointer jumping, at most 5 rounds:
// sources lie before their bytes).
//
// Single-sequence path (the block's last sequence, long literal runs,
// lengths of more than one extension byte, a sequence at the window's end):
// the warp parses the header in lockstep, copies the literals, then the
// match.  With offset >= 32 a 32-byte step reads bytes written by earlier
// steps; a shorter offset repeats its pattern, so byte i of the match is
// output[start - offset + i mod offset].
//
// __syncwarp orders the lanes' writes between steps.  A malformed block sets
// *err and stops.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_lz4_decode(const unsigned char* __restrict__ stage,
                                                    unsigned char* __restrict__ pool,
                                                    const Lz4Chunk* __restrict__ chunks, int nchunks,
                                                    int* __restrict__ err) {
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nchunks) return;
  const Lz4Chunk c = chunks[w];
  const unsigned char* in = stage + c.src;
  unsigned char* out = pool + c.dst;
  const unsigned n = c.comp & 0x7fffffffu, raw = c.raw;
  if (c.comp & 0x80000000u) {  // stored uncompressed
    if (n != raw) {
      if (lane == 0) atomicOr(err, 1);
      return;
    }
    for (unsigned i = lane; i < raw; i += 32) out[i] = __ldg(in + i);
    return;
  }
  // The warp parses in lockstep from a 32-byte window of the input, one byte
  // per lane (refilled with one coalesced load when the parse leaves it):
  // header bytes come by shuffle, not by dependent loads.  wpair: the lane's
  // byte and the next one, so a 2-byte offset is one shuffle.
  unsigned wbase = 0xffffffffu, wbyte = 0, wpair = 0;
  auto refill = [&](unsigned pos) {
    wbase = pos;
    wbyte = pos + lane < n ? (unsigned)__ldg(in + pos + lane) : 0u;
    wpair = wbyte | (__shfl_down_sync(0xffffffffu, wbyte, 1) << 8);
  };
  auto byte_at = [&](unsigned pos) -> unsigned {
    if (pos < wbase || pos >= wbase + 32) refill(pos);
    return __shfl_sync(0xffffffffu, wbyte, (int)(pos - wbase));
  };
  auto pair_at = [&](unsigned pos) -> unsigned {
    if (pos < wbase || pos + 1 >= wbase + 32) refill(pos);
    return __shfl_sync(0xffffffffu, wpair, (int)(pos - wbase)) & 0xffffu;
  };
  constexpr unsigned FULL = 0xffffffffu;
  __shared__ unsigned char seq_lane_all[4][32];  // per warp: window byte of its k-th sequence
  unsigned char* seq_lane = seq_lane_all[threadIdx.x >> 5];
  unsigned ip = 0, op = 0;
  for (;;) {
    if (ip >= n) break;  // malformed: the block ended after a match
    {
      // window path: the sequence that would start at this lane's byte
      const unsigned avail = min(n - ip, 32u);
      const unsigned wb = lane < avail ? (unsigned)__ldg(in + ip + lane) : 0u;
      unsigned nl = wb >> 4, ml = wb & 15u, pos = lane + 1;
      const unsigned e1 = __shfl_sync(FULL, wb, (lane + 1) & 31);
      bool ok = true;
      if (nl == 15) {
        ok = e1 < 255;
        nl += e1;
        ++pos;
      }
      const unsigned lit_pos = pos;
      pos += nl;
      const unsigned o0 = __shfl_sync(FULL, wb, pos & 31), o1 = __shfl_sync(FULL, wb, (pos + 1) & 31);
      pos += 2;
      const unsigned e2 = __shfl_sync(FULL, wb, pos & 31);
      if (ml == 15) {
        ok = ok && e2 < 255;
        ml += e2;
        ++pos;
      }
      ml += 4;
      // wholly inside the input bytes of the window (so never the block's
      // last sequence, which has no offset)
      ok = ok && pos <= avail;
      const unsigned nxt = ok ? pos : 64u;
      unsigned starts = 0, s = 0;
      while (s < 32) {  // s is the same in every lane
        const unsigned t = __shfl_sync(FULL, nxt, s);
        if (t == 64u) break;
        starts |= 1u << s;
        s = t;  // > s
      }
      if (starts) {
        const unsigned nseq = __popc(starts);
        // ok lanes: nl <= 29, lit_pos <= 30
        const unsigned info = (o0 | (o1 << 8)) | ((nl & 31u) << 16) | ((lit_pos & 31u) << 21);
        if ((starts >> lane) & 1u) seq_lane[__popc(starts & ((1u << lane) - 1u))] = (unsigned char)lane;
        __syncwarp();
        const unsigned from = lane < nseq ? seq_lane[lane] : 0u;
        __syncwarp();
        unsigned sinfo = __shfl_sync(FULL, info, from);
        unsigned sml = __shfl_sync(FULL, ml, from);
        if (lane >= nseq) sinfo = sml = 0;
        const unsigned snl = (sinfo >> 16) & 31u, soff = sinfo & 0xffffu;
        const unsigned len = snl + sml;
        unsigned incl = len;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const unsigned y = __shfl_up_sync(FULL, incl, d);
          if (lane >= (unsigned)d) incl += y;
        }
        const unsigned excl = incl - len;  // output start of sequence `lane`, from op
        const unsigned total = __shfl_sync(FULL, incl, 31);
        // a match starts inside the output written so far; the output fits the chunk
        const bool bad = lane < nseq && (soff == 0 || soff > op + excl + snl);
        if (__any_sync(FULL, bad) || total > raw - op) break;
        for (unsigned base = 0; base < total; base += 32) {
          const unsigned q = base + lane;
          // the sequence holding byte base, then the starts inside (base, base + 32)
          const unsigned first = __popc(__ballot_sync(FULL, lane < nseq && excl <= base)) - 1u;
          const bool st = lane < nseq && excl > base && excl < base + 32;
          const unsigned M = __reduce_or_sync(FULL, st ? 1u << (excl - base) : 0u);
          const unsigned k = (first + __popc(M & ((2u << lane) - 1u))) & 31u;
          const unsigned ki = __shfl_sync(FULL, sinfo, k), ke = __shfl_sync(FULL, excl, k);
          const unsigned r = q - ke, knl = (ki >> 16) & 31u, koff = ki & 0xffffu;
          const unsigned lit = __shfl_sync(FULL, wb, ((ki >> 21) + r) & 31u);
          const bool valid = q < total;
          unsigned val = 0;
          int ptr = -1;
          if (valid) {
            if (r < knl) {
              val = lit;
            } else {
              const int src = (int)q - (int)koff;  // from op; op + src >= 0 by the check above
              if (src < (int)base) val = out[(int)op + src];
              else ptr = src - (int)base;  // a lane below this one
            }
          }
          while (__any_sync(FULL, ptr >= 0)) {
            const unsigned pv = __shfl_sync(FULL, val, ptr & 31);
            const int pp = __shfl_sync(FULL, ptr, ptr & 31);
            if (ptr >= 0) {
              if (pp < 0) {
                val = pv;
                ptr = -1;
              } else {
                ptr = pp;
              }
            }
          }
          if (valid) out[op + q] = (unsigned char)val;
          __syncwarp();
        }
        op += total;
        ip += s;
        continue;
      }
    }
    // single-sequence path
    const unsigned token = byte_at(ip++);
    unsigned nlit = token >> 4;
    bool bad = false;
    if (nlit == 15) {
      unsigned b = 255;
      while (b == 255) {
        if (ip >= n) { bad = true; break; }
        b = byte_at(ip++);
        nlit += b;
      }
    }
    if (bad || nlit > n - ip || nlit > raw - op) break;
    const unsigned lit_at = ip;
    ip += nlit;
    if (ip == n) {
      for (unsigned i = lane; i < nlit; i += 32) out[op + i] = __ldg(in + lit_at + i);
      if (op + nlit == raw) return;  // the last sequence: done
      break;
    }
    if (n - ip < 2) break;
    const unsigned off = pair_at(ip);
    ip += 2;
    unsigned mlen = token & 15;
    if (mlen == 15) {
      unsigned b = 255;
      while (b == 255) {
        if (ip >= n) { bad = true; break; }
        b = byte_at(ip++);
        mlen += b;
      }
    }
    mlen += 4;
    if (bad || off == 0 || off > op + nlit || mlen > raw - op - nlit) break;
    if (nlit + mlen <= 32) {
      // the whole sequence in one step: lane j writes its byte j.  A match
      // byte's source, nlit - off + ((j - nlit) mod off), lies before the
      // match: a literal of this step (taken from its lane) or earlier
      // output (in memory, ordered by the last __syncwarp).
      const unsigned j = lane;
      // literals inside the current window come from it by shuffle
      const bool lit_in_win = lit_at >= wbase && lit_at + nlit <= wbase + 32;
      const unsigned wl = __shfl_sync(0xffffffffu, wbyte, (int)((lit_at - wbase + j) & 31u));
      const unsigned lit = j < nlit ? (lit_in_win ? wl : (unsigned)__ldg(in + lit_at + j)) : 0u;
      int src = 0;
      if (j >= nlit) {
        int d = (int)(j - nlit);
        if (d >= (int)off) {
          // d mod off for d, off < 32: a float quotient within one of the
          // exact one, then settled
          const int q = (int)((float)d * __frcp_rn((float)off));
          d -= q * (int)off;
          if (d < 0) d += (int)off;
          else if (d >= (int)off) d -= (int)off;
        }
        src = (int)nlit - (int)off + d;
      }
      const unsigned from_lane = __shfl_sync(0xffffffffu, lit, src > 0 ? src : 0);
      if (j < nlit + mlen) {
        const unsigned v = j < nlit ? lit : (src >= 0 ? from_lane : (unsigned)out[(int)op + src]);
        out[op + j] = (unsigned char)v;
      }
      op += nlit + mlen;
      __syncwarp();
      continue;
    }
    for (unsigned i = lane; i < nlit; i += 32) out[op + i] = __ldg(in + lit_at + i);
    op += nlit;
    __syncwarp();
    if (off >= 32) {
      for (unsigned base = 0; base < mlen; base += 32) {
        const unsigned i = base + lane;
        if (i < mlen) out[op + i] = out[op - off + i];
        __syncwarp();
      }
    } else {
      // i mod off, stepped by 32 mod off
      unsigned r = lane % off;
      const unsigned step = 32 % off;
      for (unsigned i = lane; i < mlen; i += 32) {
        out[op + i] = out[op - off + r];
        r += step;
        if (r >= off) r -= off;
      }
      __syncwarp();
    }
    op += mlen;
  }
  if (lane == 0) atomicOr(err, 1);
}

cudaError_t launch_lz4_decode(const void* stage, void* pool, const Lz4Chunk* chunks, int nchunks, int* err,
                              cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nchunks <= 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((nchunks + 3) / 4);
  k_lz4_decode<<<blocks, 128, 0, s>>>((const unsigned char*)stage, (unsigned char*)pool, chunks, nchunks, err);
  return cudaGetLastError();
}


// DEFLATE's length / distance tables and the order of the code-length code
// lengths (RFC 1951 3.2.5, 3.2.7), for the device decoder
__constant__ uint16_t kLenBaseDev[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                         31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
__constant__ uint8_t kLenExtraDev[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                                         2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
__constant__ uint16_t kDistBaseDev[30] = {1,    2,    3,    4,    5,    7,     9,     13,    17,  25,
                                          33,   49,   65,   97,   129,  193,   257,   385,   513, 769,
                                          1025, 1537, 2049, 3073, 4097, 6145,  8193,  12289, 16385, 24577};
__constant__ uint8_t kDistExtraDev[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                                          6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
__constant__ uint8_t kClOrderDev[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// ---------------------------------------------------------------------------
// zlib (RFC 1950) / DEFLATE (RFC 1951) decoding of paged brick chunks: one
// warp per chunk (a zlib stream of one chunk's raw bytes, or the raw bytes
// when bit 31 of comp is set).  Lane 0 reads the bit stream: block headers,
// code lengths and symbols, writing literals itself; a match is handed to the
// whole warp, which copies it in steps of min(distance, 32) bytes with
// __syncwarp between steps (a step reads only bytes written before it).  The
// warp builds each block's decode tables together: per code a 10-bit (literal
// / length) or 8-bit (distance) direct table entry (symbol << 4 | length) for
// codes that short, canonical decoding by length for the rest.  After the last
// block the warp sums the Adler-32 of the output and checks it.  Every read
// and write is bounds-checked; a malformed chunk sets *err and stops.
// ---------------------------------------------------------------------------
namespace {

constexpr int kInfLitFast = 10, kInfDistFast = 8;
constexpr int kInfWarps = 4;

struct InflateSmem {
  uint16_t lit_fast[1 << kInfLitFast];
  uint16_t dist_fast[1 << kInfDistFast];
  uint16_t code[320];                   // canonical code of each symbol (most significant bit first)
  uint16_t lit_sym[288], dist_sym[32];  // symbols in code order
  uint16_t lit_count[16], dist_count[16];
  // literal/length lengths [0, 288), distance lengths [288, 320); while a
  // dynamic header is read, the code-length code's lengths [0, 19) and the
  // decoded HLIT + HDIST <= 316 lengths from 19 on
  uint8_t lens[19 + 316 + 1];
};

struct InflateBits {
  const unsigned char* in;
  unsigned n, pos, past;
  unsigned long long acc;
  int bits;
  __device__ void fill() {
    while (bits <= 56) {
      unsigned long long b = 0;
      if (pos < n) b = in[pos];
      else ++past;
      ++pos;
      acc |= b << bits;
      bits += 8;
    }
  }
  __device__ unsigned get(int k) {  // k <= 32
    if (k == 0) return 0;
    if (bits < k) fill();
    const unsigned v = (unsigned)(acc & ((1ull << k) - 1ull));
    acc >>= k;
    bits -= k;
    return v;
  }
  // bits beyond the input were consumed
  __device__ bool over() const { return past > 0 && (unsigned long long)bits < 8ull * past; }
};

__device__ __forceinline__ unsigned rev_bits(unsigned c, int len) { return __brev(c) >> (32 - len); }

// Count, validate (not over-subscribed), order the symbols and fill the
// direct table of one code (lane 0 counts and orders; the warp fills).
// Returns false (warp-uniform) for a malformed code.
__device__ bool inflate_table(InflateSmem& sm, const uint8_t* lens, int n, uint16_t* count, uint16_t* sym,
                              uint16_t* fast, int fast_bits, int lane) {
  int ok = 1;
  if (lane == 0) {
    for (int b = 0; b < 16; ++b) count[b] = 0;
    for (int i = 0; i < n; ++i) ++count[lens[i]];
    count[0] = 0;
    int left = 1;
    for (int b = 1; b < 16; ++b) {
      left = 2 * left - count[b];
      if (left < 0) ok = 0;
    }
    if (ok) {
      int offs[16], next[16];
      offs[1] = 0;
      for (int b = 1; b < 15; ++b) offs[b + 1] = offs[b] + count[b];
      int c = 0;
      next[0] = 0;
      for (int b = 1; b < 16; ++b) {
        c = (c + count[b - 1]) << 1;
        next[b] = c;
      }
      for (int i = 0; i < n; ++i)
        if (lens[i]) {
          sym[offs[lens[i]]++] = (uint16_t)i;
          sm.code[i] = (uint16_t)next[lens[i]]++;
        }
    }
  }
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  if (!ok) return false;
  const int size = 1 << fast_bits;
  for (int i = lane; i < size; i += 32) fast[i] = 0;
  __syncwarp();
  for (int s = lane; s < n; s += 32) {
    const int l = lens[s];
    if (l == 0 || l > fast_bits) continue;
    const unsigned r = rev_bits(sm.code[s], l);
    const uint16_t e = (uint16_t)((s << 4) | l);
    for (int k = (int)r; k < size; k += 1 << l) fast[k] = e;
  }
  __syncwarp();
  return true;
}

// One symbol (lane 0): the direct table, else canonical decoding bit by bit.
__device__ int inflate_symbol(InflateBits& br, const uint16_t* fast, int fast_bits, const uint16_t* count,
                              const uint16_t* sym) {
  if (br.bits < 15) br.fill();
  const uint16_t e = fast[br.acc & ((1u << fast_bits) - 1u)];
  if (e) {
    br.get(e & 15);
    return e >> 4;
  }
  int code = 0, first = 0, index = 0;
  for (int b = 1; b < 16; ++b) {
    code |= (int)br.get(1);
    const int c = count[b];
    if (code - first < c) return sym[index + code - first];
    index += c;
    first = (first + c) << 1;
    code <<= 1;
  }
  return -1;
}

}  // namespace

__global__ void __launch_bounds__(32 * kInfWarps) k_inflate(const unsigned char* __restrict__ stage,
                                                            unsigned char* __restrict__ pool,
                                                            const Lz4Chunk* __restrict__ chunks, int nchunks,
                                                            int* __restrict__ err) {
  __shared__ InflateSmem smem[kInfWarps];
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nchunks) return;
  InflateSmem& sm = smem[threadIdx.x >> 5];
  const Lz4Chunk c = chunks[w];
  const unsigned char* in = stage + c.src;
  unsigned char* out = pool + c.dst;
  const unsigned n = c.comp & 0x7fffffffu, raw = c.raw;
  if (c.comp & 0x80000000u) {  // stored uncompressed
    if (n != raw) {
      if (lane == 0) atomicOr(err, 1);
      return;
    }
    for (unsigned i = lane; i < raw; i += 32) out[i] = in[i];
    return;
  }
  int bad = 0;
  if (lane == 0) {
    const unsigned cmf = n >= 6 ? in[0] : 0, flg = n >= 6 ? in[1] : 0;
    bad = n < 6 || (cmf & 15) != 8 || (cmf >> 4) > 7 || (cmf * 256 + flg) % 31 != 0 || (flg & 0x20);
  }
  if (__shfl_sync(0xffffffffu, bad, 0)) {
    if (lane == 0) atomicOr(err, 1);
    return;
  }
  // the last 4 bytes (the Adler-32) are not DEFLATE input
  InflateBits br{in + 2, n - 6, 0, 0, 0ull, 0};
  unsigned o = 0;
  int last = 0;
  while (!last && !bad) {
    int type = 0;
    if (lane == 0) {
      last = (int)br.get(1);
      type = (int)br.get(2);
      if (br.over() || type == 3) bad = 1;
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    type = __shfl_sync(0xffffffffu, type, 0);
    bad = __shfl_sync(0xffffffffu, bad, 0);
    if (bad) break;
    if (type == 0) {
      // stored: to the byte boundary, LEN, NLEN, then LEN bytes (the warp copies)
      unsigned L = 0, src = 0;
      if (lane == 0) {
        br.get(br.bits & 7);
        const unsigned len = br.get(16), nlen = br.get(16);
        const bool short_in = br.over();  // before the buffer is emptied below
        // the whole bytes left in the bit buffer go back to the input
        src = br.pos - (unsigned)(br.bits >> 3);
        br.acc = 0;
        br.bits = 0;
        if (short_in || (len ^ 0xffffu) != nlen || o + len > raw || src + len > br.n) bad = 1;
        L = len;
        br.pos = src + len;
        br.past = 0;
      }
      bad = __shfl_sync(0xffffffffu, bad, 0);
      L = __shfl_sync(0xffffffffu, L, 0);
      src = __shfl_sync(0xffffffffu, src, 0);
      const unsigned o0 = __shfl_sync(0xffffffffu, o, 0);
      if (bad) break;
      for (unsigned i = lane; i < L; i += 32) out[o0 + i] = br.in[src + i];
      o = o0 + L;
      __syncwarp();
      continue;
    }
    // the block's code lengths
    if (type == 1) {
      for (int i = lane; i < 320; i += 32) sm.lens[i] = i < 288 ? (i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8) : 5;
      __syncwarp();
    } else {
      int hlit = 0, hdist = 0;
      if (lane == 0) {
        hlit = (int)br.get(5) + 257;
        hdist = (int)br.get(5) + 1;
        const int hclen = (int)br.get(4) + 4;
        if (hlit > 286 || hdist > 30) bad = 1;
        for (int i = 0; i < 19; ++i) sm.lens[i] = 0;
        for (int k = 0; k < hclen; ++k) sm.lens[kClOrderDev[k]] = (uint8_t)br.get(3);
        if (br.over()) bad = 1;
      }
      bad = __shfl_sync(0xffffffffu, bad, 0);
      __syncwarp();
      if (bad) break;
      // the code-length code (in the distance slots of the tables, rebuilt below)
      if (!inflate_table(sm, sm.lens, 19, sm.dist_count, sm.dist_sym, sm.dist_fast, kInfDistFast, lane)) {
        bad = 1;
        break;
      }
      if (lane == 0) {
        uint8_t* lens = sm.lens + 19;  // decoded lengths, moved into place afterwards
        const int total = hlit + hdist;
        for (int k = 0; k < total && !bad;) {
          const int sy = inflate_symbol(br, sm.dist_fast, kInfDistFast, sm.dist_count, sm.dist_sym);
          if (sy < 0 || br.over()) {
            bad = 1;
            break;
          }
          if (sy < 16) {
            lens[k++] = (uint8_t)sy;
          } else {
            int rep, val = 0;
            if (sy == 16) {
              if (k == 0) {
                bad = 1;
                break;
              }
              val = lens[k - 1];
              rep = 3 + (int)br.get(2);
            } else if (sy == 17) {
              rep = 3 + (int)br.get(3);
            } else {
              rep = 11 + (int)br.get(7);
            }
            if (k + rep > total) {
              bad = 1;
              break;
            }
            while (rep--) lens[k++] = (uint8_t)val;
          }
        }
        if (!bad) {
          // literal/length lengths to [0, 288), distance lengths to [288, 320)
          uint8_t tmp[32];
          for (int i = 0; i < hdist; ++i) tmp[i] = lens[hlit + i];
          for (int i = 0; i < hlit; ++i) sm.lens[i] = lens[i];  // moves down: no overlap hazard
          for (int i = hlit; i < 288; ++i) sm.lens[i] = 0;
          for (int i = 0; i < 32; ++i) sm.lens[288 + i] = i < hdist ? tmp[i] : 0;
          if (sm.lens[256] == 0) bad = 1;
        }
      }
      bad = __shfl_sync(0xffffffffu, bad, 0);
      __syncwarp();
      if (bad) break;
    }
    if (!inflate_table(sm, sm.lens, 288, sm.lit_count, sm.lit_sym, sm.lit_fast, kInfLitFast, lane) ||
        !inflate_table(sm, sm.lens + 288, 32, sm.dist_count, sm.dist_sym, sm.dist_fast, kInfDistFast, lane)) {
      bad = 1;
      break;
    }
    // symbols: lane 0 writes literals; a match goes to the warp
    for (;;) {
      int op = 0;  // 1 match, 2 end of block, 3 malformed
      unsigned L = 0, D = 0;
      if (lane == 0) {
        for (;;) {
          const int sy = inflate_symbol(br, sm.lit_fast, kInfLitFast, sm.lit_count, sm.lit_sym);
          if (sy < 0 || br.over()) {
            op = 3;
            break;
          }
          if (sy < 256) {
            if (o >= raw) {
              op = 3;
              break;
            }
            out[o++] = (unsigned char)sy;
            continue;
          }
          if (sy == 256) {
            op = 2;
            break;
          }
          const int li = sy - 257;
          if (li >= 29) {
            op = 3;
            break;
          }
          L = kLenBaseDev[li] + br.get(kLenExtraDev[li]);
          const int ds = inflate_symbol(br, sm.dist_fast, kInfDistFast, sm.dist_count, sm.dist_sym);
          if (ds < 0 || ds >= 30) {
            op = 3;
            break;
          }
          D = kDistBaseDev[ds] + br.get(kDistExtraDev[ds]);
          if (br.over() || D > o || o + L > raw) {
            op = 3;
            break;
          }
          op = 1;
          break;
        }
      }
      op = __shfl_sync(0xffffffffu, op, 0);
      if (op == 3) {
        bad = 1;
        break;
      }
      if (op == 2) break;
      L = __shfl_sync(0xffffffffu, L, 0);
      D = __shfl_sync(0xffffffffu, D, 0);
      const unsigned o0 = __shfl_sync(0xffffffffu, o, 0);
      __syncwarp();  // lane 0's literals are visible to the copy
      const unsigned step = D < 32 ? D : 32;
      for (unsigned base = 0; base < L; base += step) {
        const unsigned i = base + (unsigned)lane;
        if ((unsigned)lane < step && i < L) out[o0 + i] = out[o0 - D + i];
        __syncwarp();
      }
      o = o0 + L;
    }
  }
  bad = __shfl_sync(0xffffffffu, bad, 0);
  o = __shfl_sync(0xffffffffu, o, 0);
  if (bad || o != raw) {
    if (lane == 0) atomicOr(err, 1);
    return;
  }
  // Adler-32 of the output against the stream's, at the byte after the last block
  unsigned stored = 0;
  int ok = 1;
  if (lane == 0) {
    const unsigned used = br.pos - (unsigned)(br.bits >> 3);
    if (used + 4 > n - 2) {
      ok = 0;
    } else {
      const unsigned char* a = in + 2 + used;
      stored = ((unsigned)a[0] << 24) | ((unsigned)a[1] << 16) | ((unsigned)a[2] << 8) | a[3];
    }
  }
  __syncwarp();
  unsigned long long sa = 0, sb = 0;  // sum of bytes, sum of (raw - i) * byte
  for (unsigned i = lane; i < raw; i += 32) {
    const unsigned v = out[i];
    sa += v;
    sb += (unsigned long long)(raw - i) * v;
  }
  for (int k = 16; k > 0; k >>= 1) {
    sa += __shfl_xor_sync(0xffffffffu, sa, k);
    sb += __shfl_xor_sync(0xffffffffu, sb, k);
  }
  if (lane == 0) {
    const unsigned A = (unsigned)((1ull + sa) % 65521ull), B = (unsigned)((sb + raw) % 65521ull);
    if (!ok || ((B << 16) | A) != stored) atomicOr(err, 1);
  }
}

cudaError_t launch_inflate(const void* stage, void* pool, const Lz4Chunk* chunks, int nchunks, int* err,
                           cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nchunks <= 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((nchunks + kInfWarps - 1) / kInfWarps);
  k_inflate<<<blocks, 32 * kInfWarps, 0, s>>>((const unsigned char*)stage, (unsigned char*)pool, chunks, nchunks,
                                              err);
  return cudaGetLastError();
}

}  // namespace gbvr
