// Raycasting kernels: ray setup, bricked front-to-back walk with empty-brick
// and macro-cell skipping, SW or texture trilinear sampling, 1D / 2D transfer
// functions with opacity correction, FP32 compositing with early ray
// termination, the isosurface first-hit mode with central-difference Phong
// shading, maximum-intensity projection, and a clip plane.
//
// Replaces the fragment-shader raycaster behind Tuvok's AbstrRenderer::Paint
// (reached from LuaScripts/BatchRenderer.lua:35 `renderer.paint()` and
// ImageVis3D/UI/RenderWindow.cpp:2464).  The sampling rule is the project's
// own (Tuvok's shaders are absent): samples at t_k = t_entry + (k + 1/2) dt along the unit
// world-space ray, dt = 1 / (samples_per_voxel * max level dim), trilinear on
// cell-centred voxels with clamp-to-edge, TF index (v - lo) (N - 1) / (hi - lo)
// with linear interpolation between entries, alpha' = 1 - (1 - alpha)^(1/s),
// C += (1 - A) alpha' c, A += (1 - A) alpha', stop at A >= ert, background
// composited last.
//
// One warp renders one 8x4 ray tile.  Launch forms sharing march():
//   k_render_plain          one launch per view, one warp per tile (the drop-in
//                           per-view form of AbstrRenderer::Paint)
//   k_render_persistent     grid = SMs x resident CTAs; warps pull (view, tile)
//                           items from one atomic counter spanning every view
//                           of the batch, so views and uneven rays share the GPU
//   k_render_persistent_u   the same for batches whose views share all but the
//                           camera: the shared descriptor is a kernel parameter
// Around them: the background outside each view's projected volume
// rectangle (k_fill_outside), bounding-box lines (k_raster_lines,
// k_line_stops, k_render_lines: FP64 coverage, covered rays re-rendered),
// the ClearView lens pass (k_render_cv), 2D slice views (k_render_slice) and
// TF classification of bricks and macro-cells.
#include <type_traits>
#include <algorithm>

#include "gbvr_internal.h"

namespace gbvr {

template <typename T>
struct VoxelTraits;
template <>
struct VoxelTraits<uint8_t> {
  static constexpr float tex_scale = 255.0f;
};
template <>
struct VoxelTraits<uint16_t> {
  static constexpr float tex_scale = 65535.0f;
};
template <>
struct VoxelTraits<float> {
  static constexpr float tex_scale = 1.0f;
};

// Voxel value as float.  8- and 16-bit values are placed in the mantissa of
// 2^23 and the bias subtracted: exact, and it keeps the conversion off the
// narrow integer-to-float pipe.
__device__ __forceinline__ float ldv(const uint8_t* p) {
  return __int_as_float(0x4B000000 | (unsigned)__ldg(p)) - 8388608.0f;
}
__device__ __forceinline__ float ldv(const uint16_t* p) {
  return __int_as_float(0x4B000000 | (unsigned)__ldg(p)) - 8388608.0f;
}
__device__ __forceinline__ float ldv(const float* p) { return __ldg(p); }

// The same voxel with the bias left in (2^23 + value for 8- and 16-bit data,
// the value itself for float data), and the x lerp of two such voxels: the
// difference of two biased values is exact, so only the lerp's base needs
// the bias taken off -- the same result as lerping ldv values, one FADD
// fewer.
__device__ __forceinline__ float ldb(const uint8_t* p) { return __int_as_float(0x4B000000 | (unsigned)__ldg(p)); }
__device__ __forceinline__ float ldb(const uint16_t* p) { return __int_as_float(0x4B000000 | (unsigned)__ldg(p)); }
__device__ __forceinline__ float ldb(const float* p) { return __ldg(p); }
template <typename T>
__device__ __forceinline__ float lerp_b(float fx, float b0, float b1) {
  if constexpr (std::is_same<T, float>::value) return fmaf(fx, b1 - b0, b0);
  else return fmaf(fx, b1 - b0, b0 - 8388608.0f);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

// A brick as the sampler sees it: voxel (gx, gy, gz) of the level (a cell
// inside the brick's stored box) is element base + gx s0 + gy s1 + gz s2 of
// the pool in the frame's layout copy; the texture coordinate of its centre
// is g + t.
struct BrickView {
  long long base;    // perm 3, 4: element offset of the brick's first block
  int s0, s1, s2;    // perm 3 (4): 64 (128) * blocks per row, per slab (s1, s2)
  int ox, oy, oz;    // perm 3: stored origin
  unsigned long long tex;
  float tx, ty, tz;
  int lox, loy, loz, hix, hiy, hiz;  // interior (membership of sample cells)
};

__device__ __forceinline__ void load_brick(const FrameDesc& f, int bi, BrickView& b) {
  const BrickInfo* B = f.bricks + bi;
  const int4 w0 = __ldg(reinterpret_cast<const int4*>(B));      // offset, tex
  const int4 w1 = __ldg(reinterpret_cast<const int4*>(B) + 1);  // ox oy oz sx
  const int4 w2 = __ldg(reinterpret_cast<const int4*>(B) + 2);  // sy sz lox loy
  const int4 w3 = __ldg(reinterpret_cast<const int4*>(B) + 3);  // loz hix hiy hiz
  const long long off = (long long)(((unsigned long long)(unsigned)w0.y << 32) | (unsigned)w0.x);
  b.tex = ((unsigned long long)(unsigned)w0.w << 32) | (unsigned)w0.z;
  const int ox = w1.x, oy = w1.y, oz = w1.z, sx = w1.w, sy = w2.x, sz = w2.y;
  b.ox = ox; b.oy = oy; b.oz = oz;
  if (f.perm == 3) {
    b.s0 = 64;
    b.s1 = ((sx + 3) >> 2) << 6;
    b.s2 = b.s1 * ((sy + 3) >> 2);
    b.base = (long long)f.copy_off + off;
  } else if (f.perm == 4) {
    b.s0 = 128;
    b.s1 = ((sx + 3) >> 2) << 7;
    b.s2 = b.s1 * ((sy + 3) >> 2);
    b.base = (long long)f.copy_off + 2 * off;
  } else {
    if (f.perm == 0) { b.s0 = 1; b.s1 = sx; b.s2 = sx * sy; }
    else if (f.perm == 1) { b.s1 = 1; b.s2 = sy; b.s0 = sy * sz; }
    else { b.s2 = 1; b.s0 = sz; b.s1 = sz * sx; }
    b.base = (long long)f.copy_off + off - ((long long)ox * b.s0 + (long long)oy * b.s1 + (long long)oz * b.s2);
  }
  b.tx = 0.5f - (float)ox; b.ty = 0.5f - (float)oy; b.tz = 0.5f - (float)oz;
  b.lox = w2.z; b.loy = w2.w;
  b.loz = w3.x; b.hix = w3.y; b.hiy = w3.z; b.hiz = w3.w;
}

// A sample position split into its voxel cell (global integer floor) and
// the trilinear fractions, exactly as the CPU oracle splits it.
struct Cell {
  int x, y, z;
  float fx, fy, fz;
};

// Cell of a position, clamped to [-1, n-1]: positions computed in FP32 can
// land a rounding error outside the level; clamping keeps brick lookup and
// membership consistent (so the walk always advances) and equals the
// clamp-to-edge rule.  NaN converts to 0.
__device__ __forceinline__ int clamp_cell(float p, int n) { return clampi((int)floorf(p), -1, n - 1); }

__device__ __forceinline__ Cell make_cell(const FrameDesc& f, float px, float py, float pz) {
  Cell c;
  const float x0 = floorf(px), y0 = floorf(py), z0 = floorf(pz);
  c.fx = px - x0; c.fy = py - y0; c.fz = pz - z0;
  c.x = clampi((int)x0, -1, f.dims[0] - 1);
  c.y = clampi((int)y0, -1, f.dims[1] - 1);
  c.z = clampi((int)z0, -1, f.dims[2] - 1);
  return c;
}

// Every stored brick holds its interior plus 2 ghost voxels on every face
// (replicated edge voxels outside the level).  A cell inside the interior,
// shifted by up to one voxel per axis (gradient taps), keeps its whole
// 2x2x2 trilinear footprint inside the stored box, so no clamping is needed:
// local indices run from lo - o - 1 >= 0 to hi - o + 1 <= stored - 1.
template <typename T, int SAMPLER>
__device__ __forceinline__ float sample_cell(const FrameDesc& f, const BrickView& b, int gx, int gy, int gz, float fx,
                                             float fy, float fz) {
  if (SAMPLER == SAMPLER_TEX) {
    cudaTextureObject_t tex = (cudaTextureObject_t)b.tex;
    if (f.interp)
      return tex3D<float>(tex, ((float)gx + b.tx) + fx, ((float)gy + b.ty) + fy, ((float)gz + b.tz) + fz) *
             VoxelTraits<T>::tex_scale;
    return tex3D<float>(tex, (float)(gx + (fx >= 0.5f)) + b.tx, (float)(gy + (fy >= 0.5f)) + b.ty,
                        (float)(gz + (fz >= 0.5f)) + b.tz) * VoxelTraits<T>::tex_scale;
  }
  const T* pool = reinterpret_cast<const T*>(f.pool);
  if (f.perm == 4) {
    // 4^3 blocks that hold their +1 neighbours: voxel (lx, ly, lz) at
    // (lz & 3) 25 + (ly & 3) 5 + (lx & 3) of block l >> 2, and the cell's
    // other 7 voxels at fixed offsets from it
    int lx = gx - b.ox, ly = gy - b.oy, lz = gz - b.oz;
    if (!f.interp) {
      lx += fx >= 0.5f; ly += fy >= 0.5f; lz += fz >= 0.5f;
      return ldv(pool + (b.base + (long long)(lz >> 2) * b.s2 + (ly >> 2) * b.s1 + ((lx >> 2) << 7) +
                         ((lz & 3) * 25 + (ly & 3) * 5 + (lx & 3))));
    }
    const T* p0 = pool + (b.base + (long long)(lz >> 2) * b.s2 + (ly >> 2) * b.s1 + ((lx >> 2) << 7) +
                          ((lz & 3) * 25 + (ly & 3) * 5 + (lx & 3)));
    const float v000 = ldb(p0), v100 = ldb(p0 + 1), v010 = ldb(p0 + 5), v110 = ldb(p0 + 6);
    const float v001 = ldb(p0 + 25), v101 = ldb(p0 + 26), v011 = ldb(p0 + 30), v111 = ldb(p0 + 31);
    const float c00 = lerp_b<T>(fx, v000, v100);
    const float c10 = lerp_b<T>(fx, v010, v110);
    const float c01 = lerp_b<T>(fx, v001, v101);
    const float c11 = lerp_b<T>(fx, v011, v111);
    float c0 = fmaf(fy, c10 - c00, c00);
    float c1 = fmaf(fy, c11 - c01, c01);
    return fmaf(fz, c1 - c0, c0);
  }
  if (f.perm == 3) {
    // 4^3 blocks: voxel (lx, ly, lz) of the stored box sits in block
    // (l >> 2) at position (lz & 3) 16 + (ly & 3) 4 + (lx & 3)
    int lx = gx - b.ox, ly = gy - b.oy, lz = gz - b.oz;
    if (!f.interp) {
      lx += fx >= 0.5f; ly += fy >= 0.5f; lz += fz >= 0.5f;
      return ldv(pool + (b.base + (long long)(lz >> 2) * b.s2 + (ly >> 2) * b.s1 + ((lx >> 2) << 6) +
                         (((lz & 3) << 4) | ((ly & 3) << 2) | (lx & 3))));
    }
    const T* p0 = pool + (b.base + (long long)(lz >> 2) * b.s2 + (ly >> 2) * b.s1 + ((lx >> 2) << 6) +
                          (((lz & 3) << 4) | ((ly & 3) << 2) | (lx & 3)));
    const int dx = (lx & 3) == 3 ? 61 : 1;
    const int dy = (ly & 3) == 3 ? b.s1 - 12 : 4;
    const int dz = (lz & 3) == 3 ? b.s2 - 48 : 16;
    const T* p1 = p0 + dz;
    const float v000 = ldb(p0), v100 = ldb(p0 + dx), v010 = ldb(p0 + dy), v110 = ldb(p0 + dy + dx);
    const float v001 = ldb(p1), v101 = ldb(p1 + dx), v011 = ldb(p1 + dy), v111 = ldb(p1 + dy + dx);
    const float c00 = lerp_b<T>(fx, v000, v100);
    const float c10 = lerp_b<T>(fx, v010, v110);
    const float c01 = lerp_b<T>(fx, v001, v101);
    const float c11 = lerp_b<T>(fx, v011, v111);
    float c0 = fmaf(fy, c10 - c00, c00);
    float c1 = fmaf(fy, c11 - c01, c01);
    return fmaf(fz, c1 - c0, c0);
  }
  if (!f.interp)
    return ldv(pool + (b.base + (long long)(gz + (fz >= 0.5f)) * b.s2 + (long long)(gy + (fy >= 0.5f)) * b.s1 +
                       (long long)(gx + (fx >= 0.5f)) * b.s0));
  const T* p0 = pool + (b.base + (long long)gz * b.s2 + (long long)gy * b.s1 + (long long)gx * b.s0);
  const T* p1 = p0 + b.s2;
  const int s0 = b.s0, s1 = b.s1;
  const float v000 = ldb(p0), v100 = ldb(p0 + s0), v010 = ldb(p0 + s1), v110 = ldb(p0 + s1 + s0);
  const float v001 = ldb(p1), v101 = ldb(p1 + s0), v011 = ldb(p1 + s1), v111 = ldb(p1 + s1 + s0);
  const float c00 = lerp_b<T>(fx, v000, v100);
  const float c10 = lerp_b<T>(fx, v010, v110);
  const float c01 = lerp_b<T>(fx, v001, v101);
  const float c11 = lerp_b<T>(fx, v011, v111);
  float c0 = fmaf(fy, c10 - c00, c00);
  float c1 = fmaf(fy, c11 - c01, c01);
  return fmaf(fz, c1 - c0, c0);
}

// floor(g / interior) for 0 <= g < 2^24: a float estimate (off by at most
// one) settled with exact integer tests, cheaper than an integer division.
__device__ __forceinline__ int brick_col(const FrameDesc& f, int g, int nb) {
  if (g < 0) return 0;
  int q = (int)((float)g * f.inv_interior);
  if (q * f.interior > g) --q;
  else if ((q + 1) * f.interior <= g) ++q;
  return min(q, nb - 1);
}

__device__ __forceinline__ int brick_index(const FrameDesc& f, int gx, int gy, int gz) {
  const int bx = brick_col(f, gx, f.nb[0]), by = brick_col(f, gy, f.nb[1]), bz = brick_col(f, gz, f.nb[2]);
  return (bz * f.nb[1] + by) * f.nb[0] + bx;
}

__device__ __forceinline__ bool inside(const BrickView& b, int gx, int gy, int gz) {
  return gx >= b.lox && gx < b.hix && gy >= b.loy && gy < b.hiy && gz >= b.loz && gz < b.hiz;
}

// Sample at an arbitrary position (isosurface bisection): find its brick first.
template <typename T, int SAMPLER>
__device__ float sample_anywhere(const FrameDesc& f, float px, float py, float pz) {
  Cell c = make_cell(f, px, py, pz);
  BrickView b;
  load_brick(f, brick_index(f, c.x, c.y, c.z), b);
  return sample_cell<T, SAMPLER>(f, b, c.x, c.y, c.z, c.fx, c.fy, c.fz);
}

// Central differences of the interpolated field at h = 1 voxel (data units
// per voxel): the taps are the same fractions one cell over.
template <typename T, int SAMPLER>
__device__ __forceinline__ void gradient(const FrameDesc& f, const BrickView& b, const Cell& c, float g[3]) {
  g[0] = (sample_cell<T, SAMPLER>(f, b, c.x + 1, c.y, c.z, c.fx, c.fy, c.fz) -
          sample_cell<T, SAMPLER>(f, b, c.x - 1, c.y, c.z, c.fx, c.fy, c.fz)) * 0.5f;
  g[1] = (sample_cell<T, SAMPLER>(f, b, c.x, c.y + 1, c.z, c.fx, c.fy, c.fz) -
          sample_cell<T, SAMPLER>(f, b, c.x, c.y - 1, c.z, c.fx, c.fy, c.fz)) * 0.5f;
  g[2] = (sample_cell<T, SAMPLER>(f, b, c.x, c.y, c.z + 1, c.fx, c.fy, c.fz) -
          sample_cell<T, SAMPLER>(f, b, c.x, c.y, c.z - 1, c.fx, c.fy, c.fz)) * 0.5f;
}

// Trilinear interpolation of 8 biased voxels (ldb) in sample_cell's order of
// operations.
template <typename T>
__device__ __forceinline__ float trilin(float v000, float v100, float v010, float v110, float v001, float v101,
                                        float v011, float v111, float fx, float fy, float fz) {
  const float c00 = lerp_b<T>(fx, v000, v100);
  const float c10 = lerp_b<T>(fx, v010, v110);
  const float c01 = lerp_b<T>(fx, v001, v101);
  const float c11 = lerp_b<T>(fx, v011, v111);
  const float c0 = fmaf(fy, c10 - c00, c00);
  const float c1 = fmaf(fy, c11 - c01, c01);
  return fmaf(fz, c1 - c0, c0);
}

// A cell's value and central-difference gradient together (software
// trilinear sampler): the six gradient taps, the same fractions one cell
// over, share half their voxels with the cell's own sample, so 32 voxels are
// loaded instead of 56.  Voxel addresses are the sum of per-axis offsets of
// the coordinates -1 .. +2 around the cell; values and arithmetic are those
// of sample_cell and gradient, bit for bit.
struct Taps {
  long long base;
  int X[4], Y[4], Z[4];
};

__device__ __forceinline__ void make_taps(const FrameDesc& f, const BrickView& b, const Cell& c, Taps& t) {
  const int lx = c.x - b.ox - 1, ly = c.y - b.oy - 1, lz = c.z - b.oz - 1;
  if (f.perm == 3) {
    t.base = b.base;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int x = lx + i, y = ly + i, z = lz + i;
      t.X[i] = ((x >> 2) << 6) + (x & 3);
      t.Y[i] = (y >> 2) * b.s1 + ((y & 3) << 2);
      t.Z[i] = (z >> 2) * b.s2 + ((z & 3) << 4);
    }
  } else if (f.perm == 4) {
    t.base = b.base;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int x = lx + i, y = ly + i, z = lz + i;
      t.X[i] = ((x >> 2) << 7) + (x & 3);
      t.Y[i] = (y >> 2) * b.s1 + (y & 3) * 5;
      t.Z[i] = (z >> 2) * b.s2 + (z & 3) * 25;
    }
  } else {
    t.base = b.base + (long long)b.ox * b.s0 + (long long)b.oy * b.s1 + (long long)b.oz * b.s2;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      t.X[i] = (lx + i) * b.s0;
      t.Y[i] = (ly + i) * b.s1;
      t.Z[i] = (lz + i) * b.s2;
    }
  }
}

template <typename T>
__device__ __forceinline__ float tap(const FrameDesc& f, const Taps& t, int i, int j, int k) {
  return ldb(reinterpret_cast<const T*>(f.pool) + (t.base + (long long)(t.Z[k] + t.Y[j] + t.X[i])));
}

// m: the cell's 8 voxels, biased (ldb), in sample_cell's order (v000, v100,
// v010, v110, v001, v101, v011, v111)
template <typename T>
__device__ __forceinline__ float sample_taps(const FrameDesc& f, const Taps& t, const Cell& c, float m[8]) {
  m[0] = tap<T>(f, t, 1, 1, 1); m[1] = tap<T>(f, t, 2, 1, 1); m[2] = tap<T>(f, t, 1, 2, 1); m[3] = tap<T>(f, t, 2, 2, 1);
  m[4] = tap<T>(f, t, 1, 1, 2); m[5] = tap<T>(f, t, 2, 1, 2); m[6] = tap<T>(f, t, 1, 2, 2); m[7] = tap<T>(f, t, 2, 2, 2);
  return trilin<T>(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], c.fx, c.fy, c.fz);
}

template <typename T>
__device__ __forceinline__ void gradient_taps(const FrameDesc& f, const Taps& t, const Cell& c, const float m[8],
                                              float g[3]) {
  const float fx = c.fx, fy = c.fy, fz = c.fz;
  const float xp = trilin<T>(m[1], tap<T>(f, t, 3, 1, 1), m[3], tap<T>(f, t, 3, 2, 1), m[5], tap<T>(f, t, 3, 1, 2), m[7],
                          tap<T>(f, t, 3, 2, 2), fx, fy, fz);
  const float xm = trilin<T>(tap<T>(f, t, 0, 1, 1), m[0], tap<T>(f, t, 0, 2, 1), m[2], tap<T>(f, t, 0, 1, 2), m[4],
                          tap<T>(f, t, 0, 2, 2), m[6], fx, fy, fz);
  g[0] = (xp - xm) * 0.5f;
  const float yp = trilin<T>(m[2], m[3], tap<T>(f, t, 1, 3, 1), tap<T>(f, t, 2, 3, 1), m[6], m[7], tap<T>(f, t, 1, 3, 2),
                          tap<T>(f, t, 2, 3, 2), fx, fy, fz);
  const float ym = trilin<T>(tap<T>(f, t, 1, 0, 1), tap<T>(f, t, 2, 0, 1), m[0], m[1], tap<T>(f, t, 1, 0, 2),
                          tap<T>(f, t, 2, 0, 2), m[4], m[5], fx, fy, fz);
  g[1] = (yp - ym) * 0.5f;
  const float zp = trilin<T>(m[4], m[5], m[6], m[7], tap<T>(f, t, 1, 1, 3), tap<T>(f, t, 2, 1, 3), tap<T>(f, t, 1, 2, 3),
                          tap<T>(f, t, 2, 2, 3), fx, fy, fz);
  const float zm = trilin<T>(tap<T>(f, t, 1, 1, 0), tap<T>(f, t, 2, 1, 0), tap<T>(f, t, 1, 2, 0), tap<T>(f, t, 2, 2, 0),
                          m[0], m[1], m[2], m[3], fx, fy, fz);
  g[2] = (zp - zm) * 0.5f;
}

// Phong, directional light, two-sided: normal = -grad/|grad| turned towards
// the viewer.  g is a world-space gradient, V the unit vector to the viewer,
// L the unit vector towards the light in world space (it follows the view:
// the light is fixed in eye space).
__device__ __forceinline__ void shade(const FrameDesc& f, const float* L, const float g[3], const float V[3],
                                      const float col[3], float out[3]) {
  float gl = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
  if (!(gl > 0.f)) {
    out[0] = col[0] * f.amb[0];
    out[1] = col[1] * f.amb[1];
    out[2] = col[2] * f.amb[2];
    return;
  }
  // one correctly rounded reciprocal and three products instead of three
  // divisions
  const float rg = -__frcp_rn(gl);
  float n0 = g[0] * rg, n1 = g[1] * rg, n2 = g[2] * rg;
  if (n0 * V[0] + n1 * V[1] + n2 * V[2] < 0.f) { n0 = -n0; n1 = -n1; n2 = -n2; }
  float nl = fmaxf(0.f, n0 * L[0] + n1 * L[1] + n2 * L[2]);
  float H0 = L[0] + V[0], H1 = L[1] + V[1], H2 = L[2] + V[2];
  float hl = sqrtf(H0 * H0 + H1 * H1 + H2 * H2);
  float nh = hl > 0.f ? fmaxf(0.f, (n0 * H0 + n1 * H1 + n2 * H2) * __frcp_rn(hl)) : 0.f;
  float sp = nh > 0.f ? __powf(nh, f.shininess) : 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = col[k] * (f.amb[k] + f.diff[k] * nl) + f.spec[k] * sp;
}

// A 1D TF lives on the device as pairs (entry i, entry min(i + 1, w - 1) -
// entry i), the difference taken in FP32 on the host: the lerp reads one
// 32-byte pair and gives exactly a + fr (b - a) as computed here.
__device__ __forceinline__ float4 tf1d(const FrameDesc& f, float v) {
  float idx = fminf(fmaxf((v - f.value_lo) * f.idx_scale, 0.f), (float)(f.tf_w - 1));
  float i0f = floorf(idx);
  float fr = idx - i0f;
  const float4* p = f.tf + 2 * (int)i0f;
  float4 a = __ldg(p), d = __ldg(p + 1);
  return make_float4(fmaf(fr, d.x, a.x), fmaf(fr, d.y, a.y), fmaf(fr, d.z, a.z), fmaf(fr, d.w, a.w));
}

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t) {
  return make_float4(fmaf(t, b.x - a.x, a.x), fmaf(t, b.y - a.y, a.y), fmaf(t, b.z - a.z, a.z),
                     fmaf(t, b.w - a.w, a.w));
}

__device__ __forceinline__ float4 tf2d(const FrameDesc& f, float v, float gmag) {
  float ix = fminf(fmaxf((v - f.value_lo) * f.idx_scale, 0.f), (float)(f.tf_w - 1));
  float iy = fminf(fmaxf(gmag * f.grad_scale, 0.f), (float)(f.tf_h - 1));
  float x0f = floorf(ix), y0f = floorf(iy);
  int x0 = (int)x0f, y0 = (int)y0f;
  int x1 = min(x0 + 1, f.tf_w - 1), y1 = min(y0 + 1, f.tf_h - 1);
  float fx = ix - x0f, fy = iy - y0f;
  float4 a = __ldg(f.tf + y0 * f.tf_w + x0), b = __ldg(f.tf + y0 * f.tf_w + x1);
  float4 c = __ldg(f.tf + y1 * f.tf_w + x0), d = __ldg(f.tf + y1 * f.tf_w + x1);
  return lerp4(lerp4(a, b, fx), lerp4(c, d, fx), fy);
}

struct RaySetup {
  float ov[3], dv[3];  // voxel-centre origin and direction (per world unit of t)
  float inv[3];        // 1 / dv
  float dw[3];         // unit world direction
  float t0, t1;
  bool hit;
};

// No bounding-box line covers the pixel.
constexpr unsigned NO_LINE = 0xffffffffu;

// Per-pixel passes over whole frames (background fill, line stops): a block
// covers FILL_ROWS rows of one frame, its threads stride along each row.
constexpr int FILL_ROWS = 8;
constexpr int FILL_THREADS = 256;

__device__ __forceinline__ void setup_ray(const FrameDesc& f, int px, int py, RaySetup& r) {
  float nx = ((float)px + 0.5f) / (float)f.width * 2.f - 1.f;
  float ny = 1.f - ((float)py + 0.5f) / (float)f.height * 2.f;
  const float* M = f.inv_vp;
  float a[4], b[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float base = M[4 * i] * nx + M[4 * i + 1] * ny + M[4 * i + 3];
    a[i] = base - M[4 * i + 2];
    b[i] = base + M[4 * i + 2];
  }
  float o[3], d[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    o[i] = a[i] / a[3];
    d[i] = b[i] / b[3] - o[i];
  }
  float dl = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  float t0 = 0.f, t1 = INFINITY;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    d[i] = d[i] / dl;
    float inv = 1.f / d[i];
    float ta = (-f.half_extent[i] - o[i]) * inv;
    float tb = (f.half_extent[i] - o[i]) * inv;
    t0 = fmaxf(t0, fminf(ta, tb));
    t1 = fminf(t1, fmaxf(ta, tb));
    r.dw[i] = d[i];
    r.ov[i] = (o[i] + f.half_extent[i]) * f.vox_scale[i] - 0.5f;
    r.dv[i] = d[i] * f.vox_scale[i];
    r.inv[i] = 1.f / r.dv[i];
  }
  r.t0 = t0;
  r.t1 = t1;
  // a chord through the unit-normalised box is at most sqrt(3) long; the
  // comparison also rejects NaN rays from degenerate matrices
  r.hit = t1 > t0 && (t1 - t0) < 4.0f;
}

// The pixel is covered by a bounding-box line with key `line`: opaque
// geometry at NDC depth z, so the ray ends where it reaches that depth (the
// ray's point a + (z + 1) / 2 (b - a) in homogeneous world coordinates, with
// a, b its near and far points as in setup_ray).  Returns that ray parameter.
__device__ __forceinline__ float line_stop_t(const FrameDesc& f, int px, int py, unsigned line) {
  RaySetup r;
  setup_ray(f, px, py, r);
  const float nx = ((float)px + 0.5f) / (float)f.width * 2.f - 1.f;
  const float ny = 1.f - ((float)py + 0.5f) / (float)f.height * 2.f;
  const float* M = f.inv_vp;
  const float h = (line_ndc_z(line) + 1.f) * 0.5f;
  float a[4], g[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float base = M[4 * i] * nx + M[4 * i + 1] * ny + M[4 * i + 3];
    a[i] = base - M[4 * i + 2];
    g[i] = fmaf(h, 2.f * M[4 * i + 2], a[i]);
  }
  float ts = 0.f;
#pragma unroll
  for (int i = 0; i < 3; ++i) ts = fmaf(g[i] / g[3] - a[i] / a[3], r.dw[i], ts);
  return ts;
}

// After the lines are rasterised: each covered pixel's key becomes the ray
// parameter where its ray ends (float bits, bit 0 still the colour), and the
// pixel (frame << 32 | pixel) goes to `list`, which the line pass re-renders.
// NO_LINE (a NaN pattern) stays.
__device__ __forceinline__ void line_stops_rows(const FrameDesc& f, int frame, int row_block,
                                                unsigned long long* list, unsigned* count) {
  unsigned* keys = const_cast<unsigned*>(f.lines);
  const int y0 = row_block * FILL_ROWS;
  const int y1 = min(y0 + FILL_ROWS, f.height);
  const int lane = threadIdx.x & 31;
  for (int y = y0; y < y1; ++y)
    for (int x0 = 0; x0 < f.width; x0 += FILL_THREADS) {
      const int x = x0 + (int)threadIdx.x;
      const size_t p = (size_t)y * f.width + x;
      const unsigned k = x < f.width ? keys[p] : NO_LINE;
      const bool on = k != NO_LINE;
      if (on) keys[p] = (__float_as_uint(line_stop_t(f, x, y, k)) & ~1u) | (k & 1u);
      // one atomic per warp for its covered pixels
      const unsigned m = __ballot_sync(0xffffffffu, on);
      if (!m) continue;
      unsigned base = 0;
      if (lane == __ffs(m) - 1) base = atomicAdd(count, (unsigned)__popc(m));
      base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
      if (on) list[base + __popc(m & ((1u << lane) - 1u))] = ((unsigned long long)frame << 32) | (unsigned long long)p;
    }
}

struct Accum {
  float C0, C1, C2, A;
};

// Classify one sample and composite it front to back; returns true when the
// ray is opaque enough to stop.
template <int MODE>
__device__ __forceinline__ bool composite(const FrameDesc& f, float4 c, Accum& acc) {
  float al = c.w;
  if (f.opacity_exp != 1.f) al = 1.f - __powf(1.f - al, f.opacity_exp);
  const float w = (1.f - acc.A) * al;
  acc.C0 = fmaf(w, c.x, acc.C0);
  acc.C1 = fmaf(w, c.y, acc.C1);
  acc.C2 = fmaf(w, c.z, acc.C2);
  acc.A += w;
  return acc.A >= f.ert;
}

// CV (isosurface mode only): ClearView.  The first hit of f.iso is the
// context surface; inside the lens (cv_rho < 1: distance to the focus point
// over the lens radius) it gets opacity clamp(cv_context (1 - |n.v|) +
// cv_border rho^2, 0, 1), and the march goes on to the first hit of f.cv_iso
// (the focus surface, from the context hit's sample on), which lies behind.
// The walk along one ray, in sample-index units: K samples, the first kept
// sample k (after the clip plane), and the crossing of the plane x_i = p as
// fma(p, ka_i, kb_i) -- the k with t_k = (p - ov_i) / dv_i, the -1/2 of the
// sample centres included.  Per axis the ray leaves a box through its upper
// plane when dv_i > 0 and its lower plane otherwise; an axis the ray runs
// parallel to gives +inf.
struct Walk {
  int K, k;
  float ka[3], kb[3];
};

__device__ __forceinline__ void walk_setup(const FrameDesc& f, const RaySetup& r, Walk& w) {
  const float dt = f.dt;
  const float t0 = r.t0;
  w.K = max(0, (int)ceilf((r.t1 - t0) / dt - 0.5f));
  const float inv_dt = 1.f / dt;
  {
    const float kt = fmaf(t0, inv_dt, 0.5f);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const bool par = !(fabsf(r.dv[i]) > 1e-30f);
      w.ka[i] = par ? 0.f : r.inv[i] * inv_dt;
      w.kb[i] = par ? INFINITY : -fmaf(r.ov[i], w.ka[i], kt);
    }
  }
  w.k = 0;
  if (f.clip_on) {
    // Clip plane: keep the samples with n . p + d <= 0.  Along the ray
    // n . p + d = s0 + s1 t is monotone, so the kept samples are a prefix
    // or a suffix of [0, K): estimated from the crossing, then settled with
    // the per-sample test itself.  Sample positions do not move.
    float s0 = f.clip[3], s1 = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float o = (r.ov[i] + 0.5f) / f.vox_scale[i] - f.half_extent[i];
      s0 = fmaf(f.clip[i], o, s0);
      s1 = fmaf(f.clip[i], r.dw[i], s1);
    }
    auto keep = [&](int kk) { return fmaf(s1, fmaf((float)kk + 0.5f, dt, t0), s0) <= 0.f; };
    if (s1 > 0.f) {
      const float kf = floorf((-s0 / s1 - t0) * inv_dt - 0.5f);
      int e = kf < 0.f ? 0 : (kf >= (float)w.K ? w.K : (int)kf + 1);
      while (e > 0 && !keep(e - 1)) --e;
      while (e < w.K && keep(e)) ++e;
      w.K = e;
    } else if (s1 < 0.f) {
      const float kf = ceilf((-s0 / s1 - t0) * inv_dt - 0.5f);
      int e = kf <= 0.f ? 0 : (kf >= (float)w.K ? w.K : (int)kf);
      while (e < w.K && !keep(e)) ++e;
      while (e > 0 && keep(e - 1)) --e;
      w.k = e;
    } else if (!(s0 <= 0.f)) {
      w.K = 0;
    }
  }
}

__device__ __forceinline__ float walk_exit(const Walk& w, int ex, int ey, int ez) {
  return fminf(fminf(fmaf((float)ex, w.ka[0], w.kb[0]), fmaf((float)ey, w.ka[1], w.kb[1])),
               fmaf((float)ez, w.ka[2], w.kb[2]));
}

__device__ __forceinline__ void walk_pos(const FrameDesc& f, const RaySetup& r, int kk, float& px, float& py,
                                         float& pz) {
  const float t = fmaf((float)kk + 0.5f, f.dt, r.t0);
  px = fmaf(t, r.dv[0], r.ov[0]);
  py = fmaf(t, r.dv[1], r.ov[1]);
  pz = fmaf(t, r.dv[2], r.ov[2]);
}

// First sample index >= k0 + 1 whose cell leaves the box [lo, hi) (per axis,
// on clamped floor coordinates), or K: estimated from the box's exit planes,
// then settled by the same floor(pos) rule that assigns samples to bricks and
// cells.  Positions are monotone in k, so members form one run and only its
// ends need checking.
__device__ __forceinline__ int walk_run_end(const FrameDesc& f, const RaySetup& r, const Walk& w, int k0, int lx,
                                            int ly, int lz, int hx, int hy, int hz) {
  const float kef =
      ceilf(walk_exit(w, r.dv[0] > 0.f ? hx : lx, r.dv[1] > 0.f ? hy : ly, r.dv[2] > 0.f ? hz : lz));
  int ke = kef >= (float)w.K ? w.K : max(k0 + 1, (int)kef);
  auto in_box = [&](int kk) {
    float qx, qy, qz;
    walk_pos(f, r, kk, qx, qy, qz);
    const int cx = clamp_cell(qx, f.dims[0]), cy = clamp_cell(qy, f.dims[1]), cz = clamp_cell(qz, f.dims[2]);
    return cx >= lx && cx < hx && cy >= ly && cy < hy && cz >= lz && cz < hz;
  };
  while (ke > k0 + 1 && !in_box(ke - 1)) --ke;
  while (ke < w.K && in_box(ke)) ++ke;
  return ke;
}

// SPS (1D TF, software sampler only): samples per step of the inner loop.
// With 2, a step evaluates two consecutive samples -- both samples' voxel and
// TF loads in flight together -- and composites them in order, stopping after
// the first if it ends the ray: the same pixels as one sample per step.
// (4 and 8: march_1d_shared.)
template <typename T, int MODE, int SAMPLER, bool CV = false, int SPS = 1>
__device__ float4 march(const FrameDesc& f, const RaySetup& r, unsigned& nsamp, int vidx, const float* light_to,
                        float cv_rho = 2.f) {
  Accum acc = {0.f, 0.f, 0.f, 0.f};
  float runmax = -INFINITY;  // MIP: largest sample so far
  int cv_phase = 0;          // ClearView: 0 looking for the context surface, 1 for the focus surface
  float cv_a = 1.f, cv_c[3] = {0.f, 0.f, 0.f};
  if (r.hit) {
    const float dt = f.dt;
    const float t0 = r.t0;
    const float V[3] = {-r.dw[0], -r.dw[1], -r.dw[2]};
    Walk wk;
    walk_setup(f, r, wk);
    const int K = wk.K;
    auto exit_k = [&](int ex, int ey, int ez) { return walk_exit(wk, ex, ey, ez); };
    auto pos_of = [&](int kk, float& px, float& py, float& pz) { walk_pos(f, r, kk, px, py, pz); };
    auto run_end = [&](int k0, int lx, int ly, int lz, int hx, int hy, int hz) -> int {
      return walk_run_end(f, r, wk, k0, lx, ly, lz, hx, hy, hz);
    };
    int k = wk.k;
    bool done = false;
    BrickView b;
    int bi = -1, bke = 0;  // current brick and the end of the ray's run in it
    const int sh = f.cell_shift;
    if constexpr (MODE == MODE_MIP) {
      if (f.empty_skip >= 2 && f.smax) {
        // Largest cell first: walk the ray's super-cells (4^3 macro-cells),
        // jumping over bricks the walk skips or that cannot hold a larger
        // maximum, reading only their maxima; then
        // the macro-cells of the ray's stretch through the best one; then
        // sample the best macro-cell.  The walk below starts from its largest
        // sample and leaves every cell and brick that cannot exceed it.  The
        // maximum is over the same samples, so it is the same value.
        constexpr int SS = SUPERCELL_SHIFT;
        const int s2 = sh + SS;
        auto exit_of = [&](int kk, int lx, int ly, int lz, int hx, int hy, int hz) {
          const float kef = ceilf(exit_k(r.dv[0] > 0.f ? hx : lx, r.dv[1] > 0.f ? hy : ly, r.dv[2] > 0.f ? hz : lz));
          return kef >= (float)K ? K : max(kk + 1, (int)kef);
        };
        float best = -INFINITY;
        int b0 = 0, b1 = 0;
        for (int kk = k; kk < K;) {
          float qx, qy, qz;
          pos_of(kk, qx, qy, qz);
          const int gx = clamp_cell(qx, f.dims[0]), gy = clamp_cell(qy, f.dims[1]), gz = clamp_cell(qz, f.dims[2]);
          const int bx = brick_col(f, gx, f.nb[0]), by = brick_col(f, gy, f.nb[1]), bz = brick_col(f, gz, f.nb[2]);
          const int bj = (bz * f.nb[1] + by) * f.nb[0] + bx;
          // a brick the walk skips, or whose largest voxel cannot beat the
          // best super-cell so far, is crossed in one step
          if ((f.empty_skip >= 1 && __ldg(f.skip + bj)) || __ldg(&f.bricks[bj].vmax) <= best) {
            const int I = f.interior;
            kk = exit_of(kk, bx * I, by * I, bz * I, min(bx * I + I, f.dims[0]), min(by * I + I, f.dims[1]),
                         min(bz * I + I, f.dims[2]));
            continue;
          }
          const int sx = max(gx, 0) >> s2, sy = max(gy, 0) >> s2, sz = max(gz, 0) >> s2;
          const float sm = __ldg(f.smax + ((size_t)sz * f.nsc[1] + sy) * f.nsc[0] + sx);
          const int ke = exit_of(kk, sx << s2, sy << s2, sz << s2, min((sx + 1) << s2, f.dims[0]),
                                 min((sy + 1) << s2, f.dims[1]), min((sz + 1) << s2, f.dims[2]));
          if (sm > best) {
            best = sm;
            b0 = kk;
            b1 = ke;
          }
          kk = ke;
        }
        best = -INFINITY;
        int c0 = 0, c1 = 0;
        for (int kk = b0; kk < b1;) {
          float qx, qy, qz;
          pos_of(kk, qx, qy, qz);
          const int cx = max(clamp_cell(qx, f.dims[0]), 0) >> sh, cy = max(clamp_cell(qy, f.dims[1]), 0) >> sh,
                    cz = max(clamp_cell(qz, f.dims[2]), 0) >> sh;
          const float cm = __ldg(&f.cells[((size_t)cz * f.nc[1] + cy) * f.nc[0] + cx].y);
          const int ke = min(exit_of(kk, cx << sh, cy << sh, cz << sh, min((cx + 1) << sh, f.dims[0]),
                                     min((cy + 1) << sh, f.dims[1]), min((cz + 1) << sh, f.dims[2])),
                             b1);
          if (cm > best) {
            best = cm;
            c0 = kk;
            c1 = ke;
          }
          kk = ke;
        }
        for (int kk = c0; kk < c1; ++kk) {
          float qx, qy, qz;
          pos_of(kk, qx, qy, qz);
          const Cell c = make_cell(f, qx, qy, qz);
          const int bj = brick_index(f, c.x, c.y, c.z);
          if (f.empty_skip >= 1 && __ldg(f.skip + bj)) continue;
          BrickView bv;
          load_brick(f, bj, bv);
          ++nsamp;
          runmax = fmaxf(runmax, sample_cell<T, SAMPLER>(f, bv, c.x, c.y, c.z, c.fx, c.fy, c.fz));
        }
        if (runmax >= f.level_max) done = true;
      }
    }
    while (k < K && !done) {
      float px, py, pz;
      pos_of(k, px, py, pz);
      const int gx = clamp_cell(px, f.dims[0]), gy = clamp_cell(py, f.dims[1]), gz = clamp_cell(pz, f.dims[2]);
      if (bi < 0 || k >= bke) {
        bi = brick_index(f, gx, gy, gz);
        load_brick(f, bi, b);
        bke = run_end(k, b.lox, b.loy, b.loz, b.hix, b.hiy, b.hiz);
        bool skip_b = f.empty_skip >= 1 && __ldg(f.skip + bi);
        // MIP: a brick whose largest voxel cannot raise the maximum is skipped
        if constexpr (MODE == MODE_MIP) skip_b = skip_b || (f.empty_skip >= 1 && __ldg(&f.bricks[bi].vmax) <= runmax);
        if (skip_b) {
          k = bke;
          bi = -1;
          continue;
        }
        if (f.touched) f.touched[(long long)vidx * f.touched_stride + bi] = 1;
      }
      int ke = bke;
      if (f.empty_skip >= 2) {
        // Macro-cells: occ holds, per cell, the Chebyshev distance (in
        // cells, capped) to the nearest cell that may contribute; 0 = this
        // cell may contribute.  From an empty cell at distance d the ray may
        // leave the whole cube of 2d-1 cells around it without sampling.
        // Runs are estimated from exit planes only: a sample that rounding
        // places across a face lies within a voxel of it, and every cell's
        // min/max covers one voxel beyond its samples' footprints, so no
        // contributing sample is ever skipped; sampling past a face is
        // harmless.
        const int cx = max(gx, 0) >> sh, cy = max(gy, 0) >> sh, cz = max(gz, 0) >> sh;
        if constexpr (MODE == MODE_MIP) {
          // a super-cell (4^3 macro-cells) whose largest cell maximum cannot
          // raise the maximum is left through its exit face at once
          if (f.smax) {
            constexpr int SS = SUPERCELL_SHIFT;
            const int sx = cx >> SS, sy = cy >> SS, sz = cz >> SS;
            if (__ldg(f.smax + ((size_t)sz * f.nsc[1] + sy) * f.nsc[0] + sx) <= runmax) {
              const int s2 = sh + SS;
              const float kef = ceilf(exit_k(r.dv[0] > 0.f ? min((sx + 1) << s2, f.dims[0]) : sx << s2,
                                             r.dv[1] > 0.f ? min((sy + 1) << s2, f.dims[1]) : sy << s2,
                                             r.dv[2] > 0.f ? min((sz + 1) << s2, f.dims[2]) : sz << s2));
              k = kef >= (float)K ? K : max(k + 1, (int)kef);
              if (k >= bke) bi = -1;
              continue;
            }
          }
        }
        const size_t ci = ((size_t)cz * f.nc[1] + cy) * f.nc[0] + cx;
        int d;
        if constexpr (MODE == MODE_MIP) d = __ldg(&f.cells[ci].y) <= runmax ? 1 : 0;  // one cell at a time
        else d = __ldg(f.occ + ci);
        const int lo_c = d > 0 ? d - 1 : 0;  // cube = cells [c - lo_c, c + lo_c]
        const float kef = ceilf(exit_k(r.dv[0] > 0.f ? min((cx + lo_c + 1) << sh, f.dims[0]) : max(cx - lo_c, 0) << sh,
                                       r.dv[1] > 0.f ? min((cy + lo_c + 1) << sh, f.dims[1]) : max(cy - lo_c, 0) << sh,
                                       r.dv[2] > 0.f ? min((cz + lo_c + 1) << sh, f.dims[2]) : max(cz - lo_c, 0) << sh));
        if (d > 0) {
          k = kef >= (float)K ? K : max(k + 1, (int)kef);
          if (k >= bke) bi = -1;
          continue;
        }
        ke = kef >= (float)ke ? ke : max(k + 1, (int)kef);
        if (f.cell_touched) {
          // algorithmic-bytes accounting: one bit per sampled cell
          unsigned* w = f.cell_touched + (long long)vidx * f.cell_touched_stride + (ci >> 5);
          const unsigned bit = 1u << (ci & 31);
          if (!(*(volatile unsigned*)w & bit)) atomicOr(w, bit);
        }
      }
      if constexpr (MODE == MODE_MIP) {
        for (; k < ke; ++k) {
          float ax, ay, az;
          pos_of(k, ax, ay, az);
          const Cell ca = make_cell(f, ax, ay, az);
          ++nsamp;
          runmax = fmaxf(runmax, sample_cell<T, SAMPLER>(f, b, ca.x, ca.y, ca.z, ca.fx, ca.fy, ca.fz));
        }
        if (runmax >= f.level_max) done = true;
      } else if constexpr (MODE == MODE_1D) {
        if constexpr (SPS == 2) {
          for (; k + 1 < ke; k += 2) {
            float ax, ay, az, bx, by, bz;
            pos_of(k, ax, ay, az);
            pos_of(k + 1, bx, by, bz);
            const Cell ca = make_cell(f, ax, ay, az);
            const Cell cb = make_cell(f, bx, by, bz);
            const float va = sample_cell<T, SAMPLER>(f, b, ca.x, ca.y, ca.z, ca.fx, ca.fy, ca.fz);
            const float vb = sample_cell<T, SAMPLER>(f, b, cb.x, cb.y, cb.z, cb.fx, cb.fy, cb.fz);
            const float4 ta = tf1d(f, va), tb = tf1d(f, vb);
            ++nsamp;
            if (composite<MODE>(f, ta, acc)) {
              done = true;
              break;
            }
            ++nsamp;
            if (composite<MODE>(f, tb, acc)) {
              done = true;
              break;
            }
          }
        }
        for (; k < ke && !done; ++k) {
          float ax, ay, az;
          pos_of(k, ax, ay, az);
          const Cell ca = make_cell(f, ax, ay, az);
          ++nsamp;
          if (composite<MODE>(f, tf1d(f, sample_cell<T, SAMPLER>(f, b, ca.x, ca.y, ca.z, ca.fx, ca.fy, ca.fz)), acc)) {
            done = true;
            break;
          }
        }
      } else {
      for (; k < ke; ++k) {
        pos_of(k, px, py, pz);
        const Cell c = make_cell(f, px, py, pz);
        // 2D TF, software trilinear: the value and later its gradient from shared taps
        constexpr bool kTaps = MODE == MODE_2D && SAMPLER == SAMPLER_SW;
        Taps tp;
        float m[8];
        float v;
        if (kTaps && f.interp) {
          make_taps(f, b, c, tp);
          v = sample_taps<T>(f, tp, c, m);
        } else {
          v = sample_cell<T, SAMPLER>(f, b, c.x, c.y, c.z, c.fx, c.fy, c.fz);
        }
        ++nsamp;
        if (MODE == MODE_ISO) {
          const float thr = (CV && cv_phase) ? f.cv_iso : f.iso;
          if (v >= thr) {
            float tl = k == 0 ? t0 : fmaf((float)k - 0.5f, dt, t0), th = fmaf((float)k + 0.5f, dt, t0);
#pragma unroll 1
            for (int it = 0; it < 4; ++it) {
              float tm = 0.5f * (tl + th);
              const Cell mc = make_cell(f, fmaf(tm, r.dv[0], r.ov[0]), fmaf(tm, r.dv[1], r.ov[1]),
                                        fmaf(tm, r.dv[2], r.ov[2]));
              // within one voxel of this brick's interior its ghosts hold the
              // neighbours' voxels, so the current brick answers (same values;
              // an out-of-core neighbour need not be resident)
              float vm;
              if (mc.x >= b.lox - 1 && mc.x <= b.hix && mc.y >= b.loy - 1 && mc.y <= b.hiy && mc.z >= b.loz - 1 &&
                  mc.z <= b.hiz)
                vm = sample_cell<T, SAMPLER>(f, b, mc.x, mc.y, mc.z, mc.fx, mc.fy, mc.fz);
              else
                vm = sample_anywhere<T, SAMPLER>(f, fmaf(tm, r.dv[0], r.ov[0]), fmaf(tm, r.dv[1], r.ov[1]),
                                                 fmaf(tm, r.dv[2], r.ov[2]));
              if (vm >= thr) th = tm;
              else tl = tm;
            }
            float th2 = 0.5f * (tl + th);
            const Cell hc = make_cell(f, fmaf(th2, r.dv[0], r.ov[0]), fmaf(th2, r.dv[1], r.ov[1]),
                                      fmaf(th2, r.dv[2], r.ov[2]));
            BrickView hb;
            load_brick(f, brick_index(f, hc.x, hc.y, hc.z), hb);
            float g[3], col[3];
            gradient<T, SAMPLER>(f, hb, hc, g);
            g[0] *= f.vox_scale[0];
            g[1] *= f.vox_scale[1];
            g[2] *= f.vox_scale[2];
            const float* rgb = (CV && cv_phase) ? f.cv_rgb : f.iso_rgb;
            if (f.lighting) shade(f, light_to, g, V, rgb, col);
            else { col[0] = rgb[0]; col[1] = rgb[1]; col[2] = rgb[2]; }
            if constexpr (CV) {
              if (cv_phase == 0) {
                const float gl = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
                const float nv = gl > 0.f ? fabsf(g[0] * V[0] + g[1] * V[1] + g[2] * V[2]) / gl : 1.f;
                const float a = cv_rho < 1.f ? __saturatef(fmaf(f.cv_border * cv_rho, cv_rho, f.cv_context * (1.f - nv)))
                                             : 1.f;
                if (a < 1.f) {
                  cv_a = a;
                  cv_c[0] = col[0]; cv_c[1] = col[1]; cv_c[2] = col[2];
                  cv_phase = 1;
                  --k;  // the focus surface may cross at this sample too
                  continue;
                }
              } else {
                // the context over the focus surface
#pragma unroll
                for (int q = 0; q < 3; ++q) col[q] = fmaf(cv_a, cv_c[q], (1.f - cv_a) * col[q]);
              }
            }
            acc.C0 = col[0]; acc.C1 = col[1]; acc.C2 = col[2];
            acc.A = 1.f;
            done = true;
            break;
          }
          continue;
        }
        // 2D transfer function over (value, |gradient|), Phong lit.  A value
        // between two columns without opacity in any gradient row composites
        // nothing (alpha 0 whatever the gradient): its gradient is skipped.
        if (f.tf_col_live) {
          const float ix = fminf(fmaxf((v - f.value_lo) * f.idx_scale, 0.f), (float)(f.tf_w - 1));
          const int x0 = (int)ix;
          if (!(__ldg(f.tf_col_live + x0) | __ldg(f.tf_col_live + min(x0 + 1, f.tf_w - 1)))) continue;
        }
        float g[3];
        if (kTaps && f.interp) gradient_taps<T>(f, tp, c, m, g);
        else gradient<T, SAMPLER>(f, b, c, g);
        const float gm = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        float4 cl = tf2d(f, v, gm);
        if (f.lighting && cl.w > 0.f) {
          float gw[3] = {g[0] * f.vox_scale[0], g[1] * f.vox_scale[1], g[2] * f.vox_scale[2]};
          float col[3] = {cl.x, cl.y, cl.z}, lit[3];
          shade(f, light_to, gw, V, col, lit);
          cl.x = lit[0]; cl.y = lit[1]; cl.z = lit[2];
        }
        if (composite<MODE>(f, cl, acc)) { done = true; break; }
      }
      }
    }
  }
  if constexpr (CV) {
    if (cv_phase == 1 && acc.A < 1.f) {
      // no focus surface behind the context surface
      acc.C0 = cv_a * cv_c[0];
      acc.C1 = cv_a * cv_c[1];
      acc.C2 = cv_a * cv_c[2];
      acc.A = cv_a;
    }
  }
  if constexpr (MODE == MODE_MIP) {
    // the maximum through the 1D TF, composited once (no opacity correction)
    if (runmax > -INFINITY) {
      const float4 c = tf1d(f, runmax);
      acc.C0 = c.x * c.w;
      acc.C1 = c.y * c.w;
      acc.C2 = c.z * c.w;
      acc.A = c.w;
    }
  }
  return make_float4(acc.C0, acc.C1, acc.C2, acc.A);
}

// Background colour of pixel row py (row 0 = top): f.bg, or with a gradient
// (setBGColors with two colours) the colour at the row's centre, linear from
// bg_top at the top edge to bg at the bottom edge.
__device__ __forceinline__ float3 bg_at(const FrameDesc& f, int py) {
  if (!f.bg_grad) return make_float3(f.bg[0], f.bg[1], f.bg[2]);
  const float t = ((float)py + 0.5f) / (float)f.height;
  return make_float3(fmaf(t, f.bg[0] - f.bg_top[0], f.bg_top[0]), fmaf(t, f.bg[1] - f.bg_top[1], f.bg_top[1]),
                     fmaf(t, f.bg[2] - f.bg_top[2], f.bg_top[2]));
}

// 1D TF, software sampler, warp-shared sampling (SPS = CAP = 4 or 8).  Each
// lane walks its own ray -- brick changes, skipped bricks and empty-cell
// jumps, one head step per loop step as march does -- and composites its own
// samples in order; but evaluating the samples (position, cell, 8 voxels,
// trilinear, TF, opacity correction) is shared: every step, the pending
// samples of all lanes' current runs, up to CAP per lane, are laid out one
// after another and the warp evaluates them 32 at a time, each lane fetching
// its task's ray and brick from the owning lane by shuffle.  The owners then
// take their results back by shuffle and composite them in sample order,
// stopping at early termination.  Sample positions, values, compositing order
// and the termination sample are those of march: the same pixels.  All 32
// lanes of the warp must call it together (`live` false for a lane without a
// pixel).
template <typename T, int CAP>
__device__ float4 march_1d_shared(const FrameDesc& f, const RaySetup& r, bool live, unsigned& nsamp, int vidx) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  Accum acc = {0.f, 0.f, 0.f, 0.f};
  Walk wk;
  bool active = live && r.hit;
  if (active) walk_setup(f, r, wk);
  else wk.K = wk.k = 0;
  int k = wk.k, kr = wk.k;  // pending samples of the current run: [k, kr)
  BrickView b;
  b.base = 0;
  b.s0 = b.s1 = b.s2 = 0;
  b.ox = b.oy = b.oz = 0;
  int bi = -1, bke = 0;
  const int sh = f.cell_shift;
  for (;;) {
    // one head step for a lane without pending samples (as an outer step of march)
    if (active && k >= kr) {
      if (k >= wk.K) {
        active = false;
      } else {
        float px, py, pz;
        walk_pos(f, r, k, px, py, pz);
        const int gx = clamp_cell(px, f.dims[0]), gy = clamp_cell(py, f.dims[1]), gz = clamp_cell(pz, f.dims[2]);
        bool run = true;
        if (bi < 0 || k >= bke) {
          bi = brick_index(f, gx, gy, gz);
          load_brick(f, bi, b);
          bke = walk_run_end(f, r, wk, k, b.lox, b.loy, b.loz, b.hix, b.hiy, b.hiz);
          if (f.empty_skip >= 1 && __ldg(f.skip + bi)) {
            k = bke;
            bi = -1;
            run = false;
          } else if (f.touched) {
            f.touched[(long long)vidx * f.touched_stride + bi] = 1;
          }
        }
        if (run) {
          int ke = bke;
          if (f.empty_skip >= 2) {
            const int cx = max(gx, 0) >> sh, cy = max(gy, 0) >> sh, cz = max(gz, 0) >> sh;
            const size_t ci = ((size_t)cz * f.nc[1] + cy) * f.nc[0] + cx;
            const int d = __ldg(f.occ + ci);
            const int lo_c = d > 0 ? d - 1 : 0;  // cube = cells [c - lo_c, c + lo_c]
            const float kef =
                ceilf(walk_exit(wk, r.dv[0] > 0.f ? min((cx + lo_c + 1) << sh, f.dims[0]) : max(cx - lo_c, 0) << sh,
                                r.dv[1] > 0.f ? min((cy + lo_c + 1) << sh, f.dims[1]) : max(cy - lo_c, 0) << sh,
                                r.dv[2] > 0.f ? min((cz + lo_c + 1) << sh, f.dims[2]) : max(cz - lo_c, 0) << sh));
            if (d > 0) {
              k = kef >= (float)wk.K ? wk.K : max(k + 1, (int)kef);
              if (k >= bke) bi = -1;
              run = false;
            } else {
              ke = kef >= (float)ke ? ke : max(k + 1, (int)kef);
              if (f.cell_touched) {
                unsigned* w = f.cell_touched + (long long)vidx * f.cell_touched_stride + (ci >> 5);
                const unsigned bit = 1u << (ci & 31);
                if (!(*(volatile unsigned*)w & bit)) atomicOr(w, bit);
              }
            }
          }
          if (run) kr = ke;
        }
      }
    }
    // this step's tasks: up to CAP pending samples per lane, laid out lane after lane
    const int n = active && k < kr ? min(kr - k, CAP) : 0;
    int off = n;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(FULL, off, d);
      if (lane >= d) off += y;
    }
    off -= n;  // exclusive prefix
    const int total = __shfl_sync(FULL, off + n, 31);
    if (total == 0) {
      if (!__any_sync(FULL, active)) break;
      continue;
    }
    bool stop = false;  // this lane's ray ended within this step
    for (int base = 0; base < total; base += 32) {
      const int t = base + lane;
      // the task's owner: the last lane whose tasks start at or before t
      int own = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int cand = own + step;
        if (__shfl_sync(FULL, off, cand) <= t) own = cand;
      }
      const int o_k = __shfl_sync(FULL, k, own), o_off = __shfl_sync(FULL, off, own);
      const float o_t0 = __shfl_sync(FULL, r.t0, own);
      const float ovx = __shfl_sync(FULL, r.ov[0], own), ovy = __shfl_sync(FULL, r.ov[1], own),
                  ovz = __shfl_sync(FULL, r.ov[2], own);
      const float dvx = __shfl_sync(FULL, r.dv[0], own), dvy = __shfl_sync(FULL, r.dv[1], own),
                  dvz = __shfl_sync(FULL, r.dv[2], own);
      BrickView ob;
      ob.base = __shfl_sync(FULL, b.base, own);
      ob.s0 = __shfl_sync(FULL, b.s0, own);
      ob.s1 = __shfl_sync(FULL, b.s1, own);
      ob.s2 = __shfl_sync(FULL, b.s2, own);
      ob.ox = __shfl_sync(FULL, b.ox, own);
      ob.oy = __shfl_sync(FULL, b.oy, own);
      ob.oz = __shfl_sync(FULL, b.oz, own);
      float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
      if (t < total) {
        const int ks = o_k + (t - o_off);
        const float tt = fmaf((float)ks + 0.5f, f.dt, o_t0);
        const Cell c = make_cell(f, fmaf(tt, dvx, ovx), fmaf(tt, dvy, ovy), fmaf(tt, dvz, ovz));
        const float4 tc = tf1d(f, sample_cell<T, SAMPLER_SW>(f, ob, c.x, c.y, c.z, c.fx, c.fy, c.fz));
        float al = tc.w;
        if (f.opacity_exp != 1.f) al = 1.f - __powf(1.f - al, f.opacity_exp);
        res = make_float4(tc.x, tc.y, tc.z, al);
      }
      // the owners take their tasks of this round back, in sample order
      const int first = max(off - base, 0), last = min(off + n - base, 32);
      const int cnt = last > first ? last - first : 0;
      const int maxcnt = __reduce_max_sync(FULL, (unsigned)cnt);
      for (int j = 0; j < maxcnt; ++j) {
        const int src = (first + j) & 31;
        const float cx = __shfl_sync(FULL, res.x, src), cy = __shfl_sync(FULL, res.y, src),
                    cz = __shfl_sync(FULL, res.z, src), al = __shfl_sync(FULL, res.w, src);
        if (j < cnt && !stop) {
          ++nsamp;
          const float w = (1.f - acc.A) * al;
          acc.C0 = fmaf(w, cx, acc.C0);
          acc.C1 = fmaf(w, cy, acc.C1);
          acc.C2 = fmaf(w, cz, acc.C2);
          acc.A += w;
          if (acc.A >= f.ert) stop = true;
        }
      }
    }
    if (active) {
      if (stop) active = false;
      else k += n;
    }
  }
  return make_float4(acc.C0, acc.C1, acc.C2, acc.A);
}

// What lies behind the volume: the background (adds no opacity), or an
// opaque bounding-box line.
__device__ __forceinline__ float4 behind(const FrameDesc& f, float4 c, unsigned line, int py) {
  const float rem = 1.f - c.w;
  if (line == NO_LINE) {
    const float3 bg = bg_at(f, py);
    return make_float4(fmaf(rem, bg.x, c.x), fmaf(rem, bg.y, c.y), fmaf(rem, bg.z, c.z), c.w);
  }
  const float* lc = f.line_rgb[line & 1u];
  return make_float4(fmaf(rem, lc[0], c.x), fmaf(rem, lc[1], c.y), fmaf(rem, lc[2], c.z), c.w + rem);
}

template <typename T, int MODE, int SAMPLER>
__device__ __forceinline__ void render_tile(const FrameDesc& f, int tile) {
  const int lane = threadIdx.x & 31;
  const int tx = f.tx0 + tile % f.ntx, ty = f.ty0 + tile / f.ntx;
  const int px = tx * f.tile_w + (lane & (f.tile_w - 1));
  const int py = ty * (32 / f.tile_w) + (lane / f.tile_w);
  unsigned nsamp = 0;
  if (px < f.width && py < f.height) {
    RaySetup r;
    setup_ray(f, px, py, r);
    float4 c = behind(f, march<T, MODE, SAMPLER>(f, r, nsamp, 0, f.light_to), NO_LINE, py);
    const size_t o = (size_t)py * f.width + px;
    if (f.out_f32) f.out_f32[o] = c;
    if (f.out_rgba8) {
      f.out_rgba8[o] = make_uchar4((unsigned char)__float2uint_rn(__saturatef(c.x) * 255.f),
                                   (unsigned char)__float2uint_rn(__saturatef(c.y) * 255.f),
                                   (unsigned char)__float2uint_rn(__saturatef(c.z) * 255.f),
                                   (unsigned char)__float2uint_rn(__saturatef(c.w) * 255.f));
    }
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) nsamp += __shfl_xor_sync(0xffffffffu, nsamp, s);
  if (lane == 0 && f.samples && nsamp) atomicAdd(f.samples, (unsigned long long)nsamp);
}

// The same for a batch-uniform descriptor f (kernel parameter) and the view's
// own descriptor fv (camera, image size, outputs, counter).
template <typename T, int MODE, int SAMPLER, int SPS = 1>
__device__ __forceinline__ void render_tile_u(const FrameDesc& f, const FrameDesc& fv, int vidx, int tile) {
  const int lane = threadIdx.x & 31;
  const int tw = f.tile_w;
  const int tx = fv.tx0 + tile % fv.ntx, ty = fv.ty0 + tile / fv.ntx;
  const int px = tx * tw + (lane & (tw - 1));
  const int py = ty * (32 / tw) + (lane / tw);
  unsigned nsamp = 0;
  if constexpr (SPS >= 4) {
    // warp-shared sampling: every lane of the warp takes part
    const bool in = px < f.width && py < f.height;
    RaySetup r{};  // lanes without a pixel still hand their (zero) ray to the shuffles
    r.hit = false;
    if (in) setup_ray(fv, px, py, r);
    const float4 c = behind(f, march_1d_shared<T, SPS>(f, r, in, nsamp, vidx), NO_LINE, py);
    if (in) {
      const size_t o = (size_t)py * f.width + px;
      float4* of = fv.out_f32;
      uchar4* o8 = fv.out_rgba8;
      if (of) of[o] = c;
      if (o8)
        o8[o] = make_uchar4((unsigned char)__float2uint_rn(__saturatef(c.x) * 255.f),
                            (unsigned char)__float2uint_rn(__saturatef(c.y) * 255.f),
                            (unsigned char)__float2uint_rn(__saturatef(c.z) * 255.f),
                            (unsigned char)__float2uint_rn(__saturatef(c.w) * 255.f));
    }
  } else if (px < f.width && py < f.height) {
    RaySetup r;
    setup_ray(fv, px, py, r);
    float4 c = behind(f, march<T, MODE, SAMPLER, false, SPS>(f, r, nsamp, vidx, fv.light_to), NO_LINE, py);
    const size_t o = (size_t)py * f.width + px;
    float4* of = fv.out_f32;
    uchar4* o8 = fv.out_rgba8;
    if (of) of[o] = c;
    if (o8)
      o8[o] = make_uchar4((unsigned char)__float2uint_rn(__saturatef(c.x) * 255.f),
                          (unsigned char)__float2uint_rn(__saturatef(c.y) * 255.f),
                          (unsigned char)__float2uint_rn(__saturatef(c.z) * 255.f),
                          (unsigned char)__float2uint_rn(__saturatef(c.w) * 255.f));
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) nsamp += __shfl_xor_sync(0xffffffffu, nsamp, s);
  if (lane == 0 && nsamp) {
    unsigned long long* cnt = fv.samples;
    if (cnt) atomicAdd(cnt, (unsigned long long)nsamp);
  }
}

constexpr int RENDER_THREADS = 128;
// Resident CTAs per SM each mode's kernels are compiled for (registers =
// 65536 / (128 x this)): the 1D TF and MIP walks 10 (48 registers; measured
// ahead of 6, 8 and 12); the 2D TF path 6 (80 registers: it keeps a sample's
// 8 voxels and 12 tap offsets for its gradient; 7 spills and is 5 % slower);
// the isosurface path 7 (72 registers, no spills; 1.5 % ahead of 8 at 64).
template <int MODE>
constexpr int uniform_ctas_per_sm() { return (MODE == MODE_1D || MODE == MODE_MIP) ? 10 : (MODE == MODE_2D ? 6 : 7); }
// Two samples per step keep two samples' voxels live, and warp-shared
// sampling (4, 8) keeps a task's owner data live: 8 CTAs/SM (64 registers).
template <int MODE, int SPS>
constexpr int uniform_ctas_per_sm_sps() { return SPS >= 2 ? 8 : uniform_ctas_per_sm<MODE>(); }

template <typename T, int MODE, int SAMPLER>
__global__ void __launch_bounds__(RENDER_THREADS, uniform_ctas_per_sm<MODE>())
    k_render_plain(const __grid_constant__ FrameDesc f) {
  int warp = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (warp >= f.ntx * f.nty) return;
  render_tile<T, MODE, SAMPLER>(f, warp);
}

// Work item i belongs to the frame whose tile_prefix range holds it.
__device__ __forceinline__ int find_frame(const int* __restrict__ prefix, int nframes, int item) {
  int lo = 0, hi = nframes - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(prefix + mid) <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <typename T, int MODE, int SAMPLER>
__global__ void __launch_bounds__(RENDER_THREADS, uniform_ctas_per_sm<MODE>())
    k_render_persistent(const FrameDesc* __restrict__ frames, int nframes,
                                                         const int* __restrict__ tile_prefix,
                                                         int* __restrict__ counter) {
  const int lane = threadIdx.x & 31;
  const int total = __ldg(tile_prefix + nframes);
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(counter, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= total) return;
    int fi = find_frame(tile_prefix, nframes, item);
    render_tile<T, MODE, SAMPLER>(frames[fi], item - __ldg(tile_prefix + fi));
  }
}

// Serving batches: the group's frames, frame count and tile prefix come from
// a table in device memory (written before each launch), so one captured
// launch per (voxel type, mode) group serves every batch; a group with no
// frames in a batch returns at once.
template <typename T, int MODE, int SAMPLER>
__global__ void __launch_bounds__(RENDER_THREADS, uniform_ctas_per_sm<MODE>())
    k_render_persistent_g(const FrameDesc* __restrict__ frames, const LaunchGroup* __restrict__ groups, int gi,
                          const int* __restrict__ tile_prefix, int* __restrict__ counters) {
  const LaunchGroup g = groups[gi];
  if (g.count <= 0) return;
  const FrameDesc* fr = frames + g.first;
  const int* prefix = tile_prefix + g.prefix_at;
  int* counter = counters + gi;
  const int lane = threadIdx.x & 31;
  const int total = __ldg(prefix + g.count);
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(counter, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= total) return;
    int fi = find_frame(prefix, g.count, item);
    render_tile<T, MODE, SAMPLER>(fr[fi], item - __ldg(prefix + fi));
  }
}

template <typename T, int MODE>
static cudaError_t persistent_g_t(const FrameDesc* frames, const LaunchGroup* groups, int gi, const int* prefix,
                                  int* counters, int grid, cudaStream_t s) {
  k_render_persistent_g<T, MODE, SAMPLER_SW><<<grid, RENDER_THREADS, 0, s>>>(frames, groups, gi, prefix, counters);
  return cudaGetLastError();
}

cudaError_t launch_render_persistent_group(int dtype, int mode, const FrameDesc* frames, const LaunchGroup* groups,
                                           int gi, const int* prefix, int* counters, int grid, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (grid <= 0) return cudaErrorInvalidValue;
  switch (dtype * 4 + mode) {
    case 0: return persistent_g_t<uint8_t, MODE_1D>(frames, groups, gi, prefix, counters, grid, s);
    case 1: return persistent_g_t<uint8_t, MODE_2D>(frames, groups, gi, prefix, counters, grid, s);
    case 2: return persistent_g_t<uint8_t, MODE_ISO>(frames, groups, gi, prefix, counters, grid, s);
    case 3: return persistent_g_t<uint8_t, MODE_MIP>(frames, groups, gi, prefix, counters, grid, s);
    case 4: return persistent_g_t<uint16_t, MODE_1D>(frames, groups, gi, prefix, counters, grid, s);
    case 5: return persistent_g_t<uint16_t, MODE_2D>(frames, groups, gi, prefix, counters, grid, s);
    case 6: return persistent_g_t<uint16_t, MODE_ISO>(frames, groups, gi, prefix, counters, grid, s);
    case 7: return persistent_g_t<uint16_t, MODE_MIP>(frames, groups, gi, prefix, counters, grid, s);
    case 8: return persistent_g_t<float, MODE_1D>(frames, groups, gi, prefix, counters, grid, s);
    case 9: return persistent_g_t<float, MODE_2D>(frames, groups, gi, prefix, counters, grid, s);
    case 10: return persistent_g_t<float, MODE_ISO>(frames, groups, gi, prefix, counters, grid, s);
    case 11: return persistent_g_t<float, MODE_MIP>(frames, groups, gi, prefix, counters, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

// Resident CTAs per SM of the group kernel of a mode (its launch bounds).
int persistent_group_ctas_per_sm(int mode) {
  int per_sm = 0;
  if (mode == MODE_1D || mode == MODE_MIP)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_persistent_g<uint16_t, MODE_1D, SAMPLER_SW>,
                                                  RENDER_THREADS, 0);
  else if (mode == MODE_2D)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_persistent_g<uint16_t, MODE_2D, SAMPLER_SW>,
                                                  RENDER_THREADS, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_persistent_g<uint16_t, MODE_ISO, SAMPLER_SW>,
                                                  RENDER_THREADS, 0);
  return per_sm < 1 ? 1 : per_sm;
}

// Background outside a frame's tile rectangle.  A block covers FILL_ROWS rows
// of one frame; its threads stride along each row (coalesced 4-byte RGBA8 or
// 16-byte float stores) and skip the rectangle's span on the rows it crosses.
// No division: the row and column come from the loop counters.

__device__ __forceinline__ void fill_outside_rows(const FrameDesc& f, int row_block) {
  const int w = f.width, h = f.height;
  const int y0 = row_block * FILL_ROWS;
  if (y0 >= h) return;
  const int y1 = min(y0 + FILL_ROWS, h);
  const int th = 32 / f.tile_w;
  const int rx0 = f.tx0 * f.tile_w, rx1 = (f.tx0 + f.ntx) * f.tile_w;
  const int ry0 = f.ty0 * th, ry1 = (f.ty0 + f.nty) * th;
  uchar4* o8 = f.out_rgba8;
  float4* o32 = f.out_f32;
  for (int y = y0; y < y1; ++y) {
    const float3 bg = bg_at(f, y);
    const float4 c = make_float4(bg.x, bg.y, bg.z, 0.f);
    const uchar4 c8 = make_uchar4((unsigned char)__float2uint_rn(__saturatef(c.x) * 255.f),
                                  (unsigned char)__float2uint_rn(__saturatef(c.y) * 255.f),
                                  (unsigned char)__float2uint_rn(__saturatef(c.z) * 255.f), 0);
    const size_t base = (size_t)y * w;
    const bool row_in = y >= ry0 && y < ry1;
    // [0, a) and [b, w): the whole row, or the parts left and right of the rectangle
    const int a = row_in ? min(rx0, w) : w, b = row_in ? max(rx1, a) : w;
    for (int x = threadIdx.x; x < a; x += FILL_THREADS) {
      if (o8) o8[base + x] = c8;
      if (o32) o32[base + x] = c;
    }
    for (int x = b + threadIdx.x; x < w; x += FILL_THREADS) {
      if (o8) o8[base + x] = c8;
      if (o32) o32[base + x] = c;
    }
  }
}

__global__ void __launch_bounds__(FILL_THREADS) k_fill_outside(const FrameDesc* __restrict__ frames) {
  fill_outside_rows(frames[blockIdx.x], blockIdx.y);
}

__global__ void __launch_bounds__(FILL_THREADS) k_fill_outside_one(const __grid_constant__ FrameDesc f) {
  fill_outside_rows(f, blockIdx.x);
}

cudaError_t launch_fill_outside_one(const FrameDesc& f, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (f.ntx == f.tiles_x && f.nty == f.tiles_y) return cudaSuccess;  // nothing outside
  if (f.width <= 0 || f.height <= 0) return cudaSuccess;
  k_fill_outside_one<<<(unsigned)((f.height + FILL_ROWS - 1) / FILL_ROWS), FILL_THREADS, 0, s>>>(f);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(FILL_THREADS) k_line_stops(const FrameDesc* __restrict__ frames, int frame0,
                                                              unsigned long long* list, unsigned* count) {
  const FrameDesc& f = frames[blockIdx.x];
  if (f.lines) line_stops_rows(f, frame0 + (int)blockIdx.x, blockIdx.y, list, count);
}

cudaError_t launch_line_stops(const FrameDesc* frames, int frame0, int nframes, int max_height,
                              unsigned long long* list, unsigned* count, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nframes <= 0 || max_height <= 0) return cudaSuccess;
  if ((max_height + FILL_ROWS - 1) / FILL_ROWS > 65535) return cudaErrorInvalidValue;
  k_line_stops<<<dim3((unsigned)nframes, (unsigned)((max_height + FILL_ROWS - 1) / FILL_ROWS)), FILL_THREADS, 0, s>>>(
      frames + frame0, frame0, list, count);
  return cudaGetLastError();
}

// Re-render the pixels a bounding-box line covers (after the frame's render):
// the ray ends at the line's stop, and the line lies behind what the ray
// composited.  One thread per listed pixel; the sample counters keep the
// main render's counts.
template <typename T, int MODE, int SAMPLER>
__global__ void __launch_bounds__(128) k_render_lines(const FrameDesc* __restrict__ frames,
                                                      const unsigned long long* __restrict__ list,
                                                      const unsigned* __restrict__ count) {
  const unsigned n = *count;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned long long e = list[i];
    const FrameDesc& f = frames[e >> 32];
    const size_t p = (size_t)(e & 0xffffffffull);
    const int px = (int)(p % (size_t)f.width), py = (int)(p / (size_t)f.width);
    const unsigned stop = f.lines[p];
    RaySetup r;
    setup_ray(f, px, py, r);
    r.t1 = fminf(r.t1, __uint_as_float(stop));
    r.hit = r.t1 > r.t0 && (r.t1 - r.t0) < 4.0f;
    unsigned nsamp = 0;
    const float4 c = behind(f, march<T, MODE, SAMPLER>(f, r, nsamp, 0, f.light_to), stop, py);
    if (f.out_f32) f.out_f32[p] = c;
    if (f.out_rgba8)
      f.out_rgba8[p] = make_uchar4((unsigned char)__float2uint_rn(__saturatef(c.x) * 255.f),
                                   (unsigned char)__float2uint_rn(__saturatef(c.y) * 255.f),
                                   (unsigned char)__float2uint_rn(__saturatef(c.z) * 255.f),
                                   (unsigned char)__float2uint_rn(__saturatef(c.w) * 255.f));
  }
}

cudaError_t launch_fill_outside(const FrameDesc* frames, int nframes, int max_height, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nframes <= 0 || max_height <= 0) return cudaSuccess;
  if ((max_height + FILL_ROWS - 1) / FILL_ROWS > 65535) return cudaErrorInvalidValue;
  dim3 grid((unsigned)nframes, (unsigned)((max_height + FILL_ROWS - 1) / FILL_ROWS));
  k_fill_outside<<<grid, FILL_THREADS, 0, s>>>(frames);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Bounding-box lines (Tuvok draws them as GL lines, depth-tested against the
// volume: RenderWindow.cpp:2208-2225 setGlobalBBox / setLocalBBox).  One block
// per (segment, view).  The coverage test and the key are FP64 expressions
// with every operation rounded on its own (no contraction), in the order the
// oracle evaluates them, so both pick the same pixels and keys bit for bit;
// the candidate pixels (a band around the projected segment) only need to
// include every covered one.
namespace {
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dd(double a, double b) { return __ddiv_rn(a, b); }

struct SegScreen {
  double sx0, sy0, z0, dx, dy, dz, inv_l2;
  int ok;
  // FP32 copies for rejecting far candidates: used when every coordinate is
  // below 65536 pixels, where the FP32 squared distance errs by under 0.02
  int fast;
  float fx0, fy0, fdx, fdy, finv;
};

__device__ void project_segment(const LineSeg& s, const LineView& v, SegScreen& o) {
  double M[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      M[4 * i + j] = da(da(da(dm(v.proj[4 * i], v.view[j]), dm(v.proj[4 * i + 1], v.view[4 + j])),
                           dm(v.proj[4 * i + 2], v.view[8 + j])),
                        dm(v.proj[4 * i + 3], v.view[12 + j]));
  double c0[4], c1[4];
  for (int i = 0; i < 4; ++i) {
    c0[i] = da(da(da(dm(M[4 * i], s.a[0]), dm(M[4 * i + 1], s.a[1])), dm(M[4 * i + 2], s.a[2])), M[4 * i + 3]);
    c1[i] = da(da(da(dm(M[4 * i], s.b[0]), dm(M[4 * i + 1], s.b[1])), dm(M[4 * i + 2], s.b[2])), M[4 * i + 3]);
  }
  // clip to the near plane z >= -w
  const double n0 = da(c0[2], c0[3]), n1 = da(c1[2], c1[3]);
  o.ok = !(n0 < 0.0 && n1 < 0.0);
  double p0[4], p1[4];
  for (int k = 0; k < 4; ++k) { p0[k] = c0[k]; p1[k] = c1[k]; }
  if (n0 < 0.0) {
    const double u = dd(n0, ds(n0, n1));
    for (int k = 0; k < 4; ++k) p0[k] = da(c0[k], dm(u, ds(c1[k], c0[k])));
  } else if (n1 < 0.0) {
    const double u = dd(n1, ds(n1, n0));
    for (int k = 0; k < 4; ++k) p1[k] = da(c1[k], dm(u, ds(c0[k], c1[k])));
  }
  if (!(p0[3] > 0.0 && p1[3] > 0.0)) o.ok = 0;
  const double hw = 0.5 * (double)v.width, hh = 0.5 * (double)v.height;
  const double sx0 = dm(da(dd(p0[0], p0[3]), 1.0), hw), sy0 = dm(ds(1.0, dd(p0[1], p0[3])), hh);
  const double sx1 = dm(da(dd(p1[0], p1[3]), 1.0), hw), sy1 = dm(ds(1.0, dd(p1[1], p1[3])), hh);
  const double z0 = dd(p0[2], p0[3]), z1 = dd(p1[2], p1[3]);
  o.sx0 = sx0;
  o.sy0 = sy0;
  o.z0 = z0;
  o.dx = ds(sx1, sx0);
  o.dy = ds(sy1, sy0);
  o.dz = ds(z1, z0);
  const double l2 = da(dm(o.dx, o.dx), dm(o.dy, o.dy));
  o.inv_l2 = l2 > 0.0 ? dd(1.0, l2) : 0.0;
  // projections beyond 1e8 pixels (a segment grazing the eye plane) are not drawn
  if (!(fabs(sx0) < 1e8 && fabs(sy0) < 1e8 && fabs(sx1) < 1e8 && fabs(sy1) < 1e8)) o.ok = 0;
  o.fast = fabs(sx0) < 65536.0 && fabs(sy0) < 65536.0 && fabs(sx1) < 65536.0 && fabs(sy1) < 65536.0;
  o.fx0 = (float)sx0;
  o.fy0 = (float)sy0;
  o.fdx = (float)o.dx;
  o.fdy = (float)o.dy;
  o.finv = (float)o.inv_l2;
}

__device__ __forceinline__ void cover_pixel(const SegScreen& g, int color, const LineView& v, int px, int py) {
  if (g.fast) {
    // far from the segment in FP32 (squared distance > 0.3): not covered
    const float cxf = (float)px + 0.5f, cyf = (float)py + 0.5f;
    float sf = ((cxf - g.fx0) * g.fdx + (cyf - g.fy0) * g.fdy) * g.finv;
    sf = fminf(fmaxf(sf, 0.f), 1.f);
    const float exf = cxf - (g.fx0 + sf * g.fdx), eyf = cyf - (g.fy0 + sf * g.fdy);
    if (exf * exf + eyf * eyf > 0.3f) return;
  }
  const double cx = (double)px + 0.5, cy = (double)py + 0.5;
  double s = dm(da(dm(ds(cx, g.sx0), g.dx), dm(ds(cy, g.sy0), g.dy)), g.inv_l2);
  s = s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s);
  const double ex = ds(cx, da(g.sx0, dm(s, g.dx))), ey = ds(cy, da(g.sy0, dm(s, g.dy)));
  const double d2 = da(dm(ex, ex), dm(ey, ey));
  if (!(d2 <= 0.25)) return;
  const double zz = da(da(g.z0, dm(s, g.dz)), 2.0);
  if (!(zz > 0.0)) return;
  atomicMin(v.keys + (size_t)py * v.width + px, line_key(__double2float_rn(zz), color));
}
}  // namespace

__global__ void __launch_bounds__(128) k_raster_lines(const LineSeg* __restrict__ segs,
                                                      const LineView* __restrict__ views) {
  __shared__ SegScreen g;
  const LineView& v = views[blockIdx.y];
  const int color = segs[blockIdx.x].color;
  if (threadIdx.x == 0) project_segment(segs[blockIdx.x], v, g);
  __syncthreads();
  if (!g.ok) return;
  const int W = v.width, H = v.height;
  // march along the major axis; per step the band of 5 pixels around the
  // segment (a covered pixel's centre is within one pixel of the segment's
  // point at its column or row)
  const bool xmaj = fabs(g.dx) >= fabs(g.dy);
  const double a0 = xmaj ? g.sx0 : g.sy0, da_ = xmaj ? g.dx : g.dy;
  const double b0 = xmaj ? g.sy0 : g.sx0, db = xmaj ? g.dy : g.dx;
  const int na = xmaj ? W : H, nb = xmaj ? H : W;
  const double lo = fmax(fmin(a0, a0 + da_) - 1.0, -1.0), hi = fmin(fmax(a0, a0 + da_) + 1.0, (double)na);
  const int i0 = max(0, (int)floor(lo)), i1 = min(na - 1, (int)floor(hi));
  for (int i = i0 + (int)threadIdx.x; i <= i1; i += blockDim.x) {
    double t = da_ != 0.0 ? ((double)i + 0.5 - a0) / da_ : 0.0;
    t = fmin(fmax(t, 0.0), 1.0);
    const int j0 = (int)floor(b0 + t * db) - 2;
    for (int j = max(j0, 0); j <= min(j0 + 4, nb - 1); ++j) {
      if (xmaj) cover_pixel(g, color, v, i, j);
      else cover_pixel(g, color, v, j, i);
    }
  }
}

cudaError_t launch_raster_lines(const LineSeg* segs, int nseg, const LineView* views, int nviews, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nseg <= 0 || nviews <= 0) return cudaSuccess;
  if (nviews > 65535) return cudaErrorInvalidValue;
  k_raster_lines<<<dim3((unsigned)nseg, (unsigned)nviews), 128, 0, s>>>(segs, views);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// 2D slice views (renderRegion2D: a slice at a depth along one axis, or the
// maximum along that axis): one thread per pixel.  The slice fills the
// framebuffer at its aspect ratio, centred, with the background around it;
// screen x follows the lower-numbered in-plane axis, screen y the higher one
// upwards, each optionally mirrored.  The value at the pixel (trilinear on
// the level, the axis coordinate at the slice's voxel centre) goes through
// the 1D TF and over the background.  MIP walks the voxel centres along the
// axis brick by brick, skipping bricks whose largest voxel cannot raise the
// maximum.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_render_slice(const __grid_constant__ FrameDesc f, const __grid_constant__ SliceDesc s) {
  const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y;
  unsigned ns = 0;
  if (px < f.width) {
    float uw = ((float)px + 0.5f - s.half_w) * s.inv_s;
    float vw = (s.half_h - ((float)py + 0.5f)) * s.inv_s;
    if (s.flip_x) uw = -uw;
    if (s.flip_y) vw = -vw;
    const float3 bg = bg_at(f, py);
    float4 out = make_float4(bg.x, bg.y, bg.z, 0.f);
    if (fabsf(uw) <= 0.5f * s.ext_u && fabsf(vw) <= 0.5f * s.ext_v) {
      const float pu = (uw + 0.5f * s.ext_u) * s.scale_u - 0.5f;
      const float pv = (vw + 0.5f * s.ext_v) * s.scale_v - 0.5f;
      auto pos = [&](float pa, float& x, float& y, float& z) {
        x = s.axis == 0 ? pa : pu;
        y = s.axis == 1 ? pa : (s.axis == 0 ? pu : pv);
        z = s.axis == 2 ? pa : pv;
      };
      float v, x, y, z;
      bool empty = false;
      if (!s.mip) {
        pos(s.coord, x, y, z);
        if (s.use_skip) {
          // the in-core pixel of a brick empty under the TF is the background
          const Cell c = make_cell(f, x, y, z);
          empty = __ldg(f.skip + brick_index(f, c.x, c.y, c.z)) != 0;
        }
        v = empty ? 0.f : sample_anywhere<T, SAMPLER_SW>(f, x, y, z);
        ns = empty ? 0 : 1;
      } else {
        v = -INFINITY;
        const int n = f.dims[s.axis];
        int k = 0;
        while (k < n) {
          pos((float)k, x, y, z);
          const Cell c = make_cell(f, x, y, z);
          const int bi = brick_index(f, c.x, c.y, c.z);
          BrickView b;
          load_brick(f, bi, b);
          const int hi = s.axis == 0 ? b.hix : (s.axis == 1 ? b.hiy : b.hiz);
          if (__ldg(&f.bricks[bi].vmax) > v && !(s.use_skip && __ldg(f.skip + bi))) {
            for (; k < hi; ++k) {
              const int cx = s.axis == 0 ? k : c.x, cy = s.axis == 1 ? k : c.y, cz = s.axis == 2 ? k : c.z;
              v = fmaxf(v, sample_cell<T, SAMPLER_SW>(f, b, cx, cy, cz, s.axis == 0 ? 0.f : c.fx,
                                                     s.axis == 1 ? 0.f : c.fy, s.axis == 2 ? 0.f : c.fz));
              ++ns;
            }
          } else {
            k = hi;
          }
          if (v >= f.level_max) break;
        }
      }
      if (!empty) {
        const float4 c = tf1d(f, v);
        out = make_float4(fmaf(c.w, c.x, (1.f - c.w) * bg.x), fmaf(c.w, c.y, (1.f - c.w) * bg.y),
                          fmaf(c.w, c.z, (1.f - c.w) * bg.z), c.w);
      }
    }
    const size_t o = (size_t)py * f.width + px;
    if (f.out_f32) f.out_f32[o] = out;
    if (f.out_rgba8)
      f.out_rgba8[o] = make_uchar4((unsigned char)__float2uint_rn(__saturatef(out.x) * 255.f),
                                   (unsigned char)__float2uint_rn(__saturatef(out.y) * 255.f),
                                   (unsigned char)__float2uint_rn(__saturatef(out.z) * 255.f),
                                   (unsigned char)__float2uint_rn(__saturatef(out.w) * 255.f));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ns += __shfl_xor_sync(0xffffffffu, ns, o);
  if ((threadIdx.x & 31) == 0 && f.samples && ns) atomicAdd(f.samples, (unsigned long long)ns);
}

cudaError_t launch_render_slice(const FrameDesc& f, const SliceDesc& sd, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  dim3 grid((unsigned)((f.width + 127) / 128), (unsigned)f.height);
  if (f.dtype == DT_U8) k_render_slice<uint8_t><<<grid, 128, 0, s>>>(f, sd);
  else if (f.dtype == DT_U16) k_render_slice<uint16_t><<<grid, 128, 0, s>>>(f, sd);
  else k_render_slice<float><<<grid, 128, 0, s>>>(f, sd);
  return cudaGetLastError();
}

// Batch-uniform variant: `shared` (a kernel parameter, so the walk reads it as
// constant-bank operands) holds everything the views have in common; camera,
// image size, outputs and the sample counter come from frames[view].
template <typename T, int MODE, int SAMPLER, int SPS = 1>
__global__ void __launch_bounds__(RENDER_THREADS, uniform_ctas_per_sm_sps<MODE, SPS>())
    k_render_persistent_u(const __grid_constant__ FrameDesc shared, const FrameDesc* __restrict__ frames,
                          int nframes, const int* __restrict__ tile_prefix, int* __restrict__ counter) {
  const int lane = threadIdx.x & 31;
  const int total = __ldg(tile_prefix + nframes);
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(counter, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= total) return;
    int fi = find_frame(tile_prefix, nframes, item);
    render_tile_u<T, MODE, SAMPLER, SPS>(shared, frames[fi], fi, item - __ldg(tile_prefix + fi));
  }
}

// ---------------------------------------------------------------------------
// Empty-space classification.  Values sampled where a brick or macro-cell
// applies lie in [vmin, vmax] of the voxels its samples can touch (trilinear
// weights are convex), so the TF entries such a sample can read are bounded;
// if every one has alpha 0 the region contributes exactly nothing and the
// walk skips it.  Isosurface: skipped when vmax < iso (no sample can reach
// the isovalue).  MIP skips by the running maximum in the walk instead.  One prefix count over the TF columns makes each test O(1).
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned char classify_range(float mn, float mx, const int* __restrict__ prefix, int tf_w,
                                                        int mode, float value_lo, float idx_scale, float iso) {
  if (mode == MODE_ISO) return mx >= iso ? 1 : 0;
  if (mode == MODE_MIP) return 1;  // the maximum goes through the TF: nothing is empty up front
  float ilo = fminf(fmaxf((mn - value_lo) * idx_scale, 0.f), (float)(tf_w - 1));
  float ihi = fminf(fmaxf((mx - value_lo) * idx_scale, 0.f), (float)(tf_w - 1));
  int lo = max((int)floorf(ilo) - 1, 0);
  int hi = min((int)floorf(ihi) + 2, tf_w - 1);
  return (__ldg(prefix + hi + 1) - __ldg(prefix + lo)) > 0 ? 1 : 0;
}

__global__ void k_classify_bricks(const BrickInfo* __restrict__ bricks, int nbricks, const int* __restrict__ prefix,
                                  int tf_w, int mode, float value_lo, float idx_scale, float iso,
                                  unsigned char* __restrict__ skip) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbricks) return;
  skip[i] = classify_range(bricks[i].vmin, bricks[i].vmax, prefix, tf_w, mode, value_lo, idx_scale, iso) ? 0 : 1;
}

__global__ void k_classify_cells(const float2* __restrict__ cells, long long n, const int* __restrict__ prefix, int tf_w,
                                 int mode, float value_lo, float idx_scale, float iso, unsigned char* __restrict__ occ) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float2 c = __ldg(cells + i);
    occ[i] = classify_range(c.x, c.y, prefix, tf_w, mode, value_lo, idx_scale, iso);
  }
}

__global__ void k_count_bits(const unsigned* __restrict__ bits, long long words, unsigned long long* __restrict__ counts) {
  const unsigned* b = bits + (size_t)blockIdx.y * words;
  unsigned long long c = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < words; i += (long long)gridDim.x * blockDim.x)
    c += __popc(__ldg(b + i));
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(counts + blockIdx.y, c);
}

cudaError_t launch_count_bits(const unsigned* bits, long long words, int n, unsigned long long* counts, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (n <= 0 || words <= 0) return cudaSuccess;
  dim3 grid((unsigned)std::min<long long>((words + 255) / 256, 64), (unsigned)n);
  k_count_bits<<<grid, 256, 0, s>>>(bits, words, counts);
  return cudaGetLastError();
}

__global__ void k_occ_to_dist(const unsigned char* __restrict__ occ, unsigned char* __restrict__ d, long long n, int cap) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    d[i] = occ[i] ? 0 : (unsigned char)cap;
}

// Chebyshev distance transform of the macro-cell occupancy, one relaxation
// pass per launch: d'(c) = 0 if c may contribute, else min(cap, 1 + min over
// the 26 neighbours of d(n)); `cap` passes give the exact capped distance.
__global__ void k_cell_distance(const unsigned char* __restrict__ in, unsigned char* __restrict__ out, int nx, int ny,
                                int nz, int cap) {
  const long long n = (long long)nx * ny * nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx);
    const long long t = i / nx;
    const int y = (int)(t % ny), z = (int)(t / ny);
    int d = __ldg(in + i);
    if (d == 0) { out[i] = 0; continue; }
    int m = cap;
    for (int dz = -1; dz <= 1; ++dz) {
      const int zz = z + dz;
      if (zz < 0 || zz >= nz) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        const int yy = y + dy;
        if (yy < 0 || yy >= ny) continue;
        const unsigned char* row = in + ((long long)zz * ny + yy) * nx;
        for (int dx = -1; dx <= 1; ++dx) {
          const int xx = x + dx;
          if (xx < 0 || xx >= nx) continue;
          m = min(m, (int)__ldg(row + xx));
        }
      }
    }
    out[i] = (unsigned char)min(cap, m + 1);
  }
}

cudaError_t launch_cell_distance(unsigned char* occ, unsigned char* tmp, const int nc[3], int cap, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  const long long n = (long long)nc[0] * nc[1] * nc[2];
  if (n <= 0) return cudaSuccess;
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  // occ enters as 1 = may contribute, 0 = empty; convert to distances
  // (0 = may contribute, cap = empty) in tmp, then relax back and forth
  k_occ_to_dist<<<(unsigned)blocks, 256, 0, s>>>(occ, tmp, n, cap);
  unsigned char* a = tmp;
  unsigned char* b = occ;
  for (int p = 0; p < cap; ++p) {
    k_cell_distance<<<(unsigned)blocks, 256, 0, s>>>(a, b, nc[0], nc[1], nc[2], cap);
    unsigned char* t = a;
    a = b;
    b = t;
  }
  // result must end in occ
  if (a != occ) {
    cudaError_t e = cudaMemcpyAsync(occ, a, (size_t)n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

cudaError_t launch_classify_bricks(const BrickInfo* bricks, int nbricks, const int* prefix, int tf_w, int mode,
                                   float value_lo, float idx_scale, float iso, unsigned char* skip, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nbricks <= 0) return cudaSuccess;
  k_classify_bricks<<<(nbricks + 127) / 128, 128, 0, s>>>(bricks, nbricks, prefix, tf_w, mode, value_lo, idx_scale,
                                                         iso, skip);
  return cudaGetLastError();
}

cudaError_t launch_classify_cells(const float2* cells, long long n, const int* prefix, int tf_w, int mode,
                                  float value_lo, float idx_scale, float iso, unsigned char* occ, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (n <= 0) return cudaSuccess;
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  k_classify_cells<<<(unsigned)blocks, 256, 0, s>>>(cells, n, prefix, tf_w, mode, value_lo, idx_scale, iso, occ);
  return cudaGetLastError();
}

template <typename T, int MODE, int SAMPLER>
static cudaError_t plain_t(const FrameDesc& f, cudaStream_t s) {
  (void)cudaGetLastError();
  int tiles = f.ntx * f.nty;  // the frame's tile rectangle (the whole frame unless culled)
  int warps_per_block = RENDER_THREADS / 32;
  int blocks = (tiles + warps_per_block - 1) / warps_per_block;
  if (blocks == 0) return cudaSuccess;
  k_render_plain<T, MODE, SAMPLER><<<blocks, RENDER_THREADS, 0, s>>>(f);
  return cudaGetLastError();
}

template <typename T, int MODE, int SAMPLER>
static cudaError_t persistent_t(const FrameDesc* frames, int nframes, const int* prefix, int* counter, int grid,
                                cudaStream_t s) {
  (void)cudaGetLastError();
  k_render_persistent<T, MODE, SAMPLER><<<grid, RENDER_THREADS, 0, s>>>(frames, nframes, prefix, counter);
  return cudaGetLastError();
}

template <typename T, int MODE, int SAMPLER>
static cudaError_t persistent_u_t(const FrameDesc& shared, const FrameDesc* frames, int nframes, const int* prefix,
                                  int* counter, int grid, cudaStream_t s) {
  (void)cudaGetLastError();
  k_render_persistent_u<T, MODE, SAMPLER><<<grid, RENDER_THREADS, 0, s>>>(shared, frames, nframes, prefix, counter);
  return cudaGetLastError();
}

#define GBVR_DISPATCH(FN, dtype, mode, sampler, ...)                                          \
  do {                                                                                        \
    switch ((dtype) * 8 + (mode) * 2 + (sampler)) {                                           \
      case 0: return FN<uint8_t, MODE_1D, SAMPLER_SW>(__VA_ARGS__);                           \
      case 1: return FN<uint8_t, MODE_1D, SAMPLER_TEX>(__VA_ARGS__);                          \
      case 2: return FN<uint8_t, MODE_2D, SAMPLER_SW>(__VA_ARGS__);                           \
      case 3: return FN<uint8_t, MODE_2D, SAMPLER_TEX>(__VA_ARGS__);                          \
      case 4: return FN<uint8_t, MODE_ISO, SAMPLER_SW>(__VA_ARGS__);                          \
      case 5: return FN<uint8_t, MODE_ISO, SAMPLER_TEX>(__VA_ARGS__);                         \
      case 6: return FN<uint8_t, MODE_MIP, SAMPLER_SW>(__VA_ARGS__);                          \
      case 7: return FN<uint8_t, MODE_MIP, SAMPLER_TEX>(__VA_ARGS__);                         \
      case 8: return FN<uint16_t, MODE_1D, SAMPLER_SW>(__VA_ARGS__);                          \
      case 9: return FN<uint16_t, MODE_1D, SAMPLER_TEX>(__VA_ARGS__);                         \
      case 10: return FN<uint16_t, MODE_2D, SAMPLER_SW>(__VA_ARGS__);                         \
      case 11: return FN<uint16_t, MODE_2D, SAMPLER_TEX>(__VA_ARGS__);                        \
      case 12: return FN<uint16_t, MODE_ISO, SAMPLER_SW>(__VA_ARGS__);                        \
      case 13: return FN<uint16_t, MODE_ISO, SAMPLER_TEX>(__VA_ARGS__);                       \
      case 14: return FN<uint16_t, MODE_MIP, SAMPLER_SW>(__VA_ARGS__);                        \
      case 15: return FN<uint16_t, MODE_MIP, SAMPLER_TEX>(__VA_ARGS__);                       \
      case 16: return FN<float, MODE_1D, SAMPLER_SW>(__VA_ARGS__);                            \
      case 17: return FN<float, MODE_1D, SAMPLER_TEX>(__VA_ARGS__);                           \
      case 18: return FN<float, MODE_2D, SAMPLER_SW>(__VA_ARGS__);                            \
      case 19: return FN<float, MODE_2D, SAMPLER_TEX>(__VA_ARGS__);                           \
      case 20: return FN<float, MODE_ISO, SAMPLER_SW>(__VA_ARGS__);                           \
      case 21: return FN<float, MODE_ISO, SAMPLER_TEX>(__VA_ARGS__);                          \
      case 22: return FN<float, MODE_MIP, SAMPLER_SW>(__VA_ARGS__);                           \
      case 23: return FN<float, MODE_MIP, SAMPLER_TEX>(__VA_ARGS__);                          \
      default: return cudaErrorInvalidValue;                                                  \
    }                                                                                         \
  } while (0)

// ClearView lens pass (isosurface mode), after the frame's render and line
// pass: the pixels inside the lens circle are rendered again with the
// context surface made partly transparent over the focus surface (see march);
// pixels outside keep the main render.  One warp per 8x4 pixel tile of the
// lens's bounding rectangle.
template <typename T, int SAMPLER>
__global__ void __launch_bounds__(128) k_render_cv(const __grid_constant__ FrameDesc f, const CvLens L) {
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  const int tw = (L.x1 - L.x0 + 7) / 8;
  const int px = L.x0 + (warp % tw) * 8 + (lane & 7), py = L.y0 + (warp / tw) * 4 + (lane >> 3);
  if (px >= L.x1 || py >= L.y1) return;
  const float dx = (float)px + 0.5f - L.fx, dy = (float)py + 0.5f - L.fy;
  const float rho = sqrtf(dx * dx + dy * dy) / L.radius;
  if (!(rho < 1.f)) return;
  const size_t p = (size_t)py * f.width + px;
  RaySetup r;
  setup_ray(f, px, py, r);
  unsigned stop = NO_LINE;
  if (f.lines) {
    stop = f.lines[p];
    r.t1 = fminf(r.t1, __uint_as_float(stop));
    r.hit = r.t1 > r.t0 && (r.t1 - r.t0) < 4.0f;
  }
  unsigned nsamp = 0;
  const float4 c = behind(f, march<T, MODE_ISO, SAMPLER, true>(f, r, nsamp, 0, f.light_to, rho), stop, py);
  if (f.out_f32) f.out_f32[p] = c;
  if (f.out_rgba8)
    f.out_rgba8[p] = make_uchar4((unsigned char)__float2uint_rn(__saturatef(c.x) * 255.f),
                                 (unsigned char)__float2uint_rn(__saturatef(c.y) * 255.f),
                                 (unsigned char)__float2uint_rn(__saturatef(c.z) * 255.f),
                                 (unsigned char)__float2uint_rn(__saturatef(c.w) * 255.f));
}

template <typename T, int SAMPLER>
static cudaError_t cv_t(const FrameDesc& f, const CvLens& L, cudaStream_t s) {
  const long long tiles = (long long)((L.x1 - L.x0 + 7) / 8) * ((L.y1 - L.y0 + 3) / 4);
  k_render_cv<T, SAMPLER><<<(unsigned)((tiles + 3) / 4), 128, 0, s>>>(f, L);
  return cudaGetLastError();
}

cudaError_t launch_render_cv(const FrameDesc& f, const CvLens& L, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (L.x1 <= L.x0 || L.y1 <= L.y0 || !(L.radius > 0.f)) return cudaSuccess;
  const bool tex = f.sampler == SAMPLER_TEX;
  switch (f.dtype) {
    case 0: return tex ? cv_t<uint8_t, SAMPLER_TEX>(f, L, s) : cv_t<uint8_t, SAMPLER_SW>(f, L, s);
    case 1: return tex ? cv_t<uint16_t, SAMPLER_TEX>(f, L, s) : cv_t<uint16_t, SAMPLER_SW>(f, L, s);
    case 2: return tex ? cv_t<float, SAMPLER_TEX>(f, L, s) : cv_t<float, SAMPLER_SW>(f, L, s);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T, int MODE, int SAMPLER>
static cudaError_t lines_t(const FrameDesc* frames, const unsigned long long* list, const unsigned* count, int grid,
                           cudaStream_t s) {
  k_render_lines<T, MODE, SAMPLER><<<grid, 128, 0, s>>>(frames, list, count);
  return cudaGetLastError();
}

cudaError_t launch_render_lines(int dtype, int mode, int sampler, const FrameDesc* frames,
                                const unsigned long long* list, const unsigned* count, int grid, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (grid <= 0) return cudaSuccess;
  GBVR_DISPATCH(lines_t, dtype, mode, sampler, frames, list, count, grid, s);
}

cudaError_t launch_render_plain(const FrameDesc& f, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  GBVR_DISPATCH(plain_t, f.dtype, f.mode, f.sampler, f, s);
}

// All frames of one persistent launch share dtype, mode and sampler (the
// host groups a mixed batch by these and issues one launch per group).
cudaError_t launch_render_persistent_typed(int dtype, int mode, int sampler, const FrameDesc* frames, int nframes,
                                           const int* prefix, int* counter, int grid, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  GBVR_DISPATCH(persistent_t, dtype, mode, sampler, frames, nframes, prefix, counter, grid, s);
}

template <typename T, int SPS>
static cudaError_t persistent_u_sps_t(const FrameDesc& shared, const FrameDesc* frames, int nframes, const int* prefix,
                                      int* counter, int grid, cudaStream_t s) {
  k_render_persistent_u<T, MODE_1D, SAMPLER_SW, SPS><<<grid, RENDER_THREADS, 0, s>>>(shared, frames, nframes, prefix,
                                                                                      counter);
  return cudaGetLastError();
}

template <int SPS>
static cudaError_t persistent_u_sps(int dtype, const FrameDesc& shared, const FrameDesc* frames, int nframes,
                                    const int* prefix, int* counter, int grid, cudaStream_t s) {
  if (dtype == DT_U8) return persistent_u_sps_t<uint8_t, SPS>(shared, frames, nframes, prefix, counter, grid, s);
  if (dtype == DT_U16) return persistent_u_sps_t<uint16_t, SPS>(shared, frames, nframes, prefix, counter, grid, s);
  return persistent_u_sps_t<float, SPS>(shared, frames, nframes, prefix, counter, grid, s);
}

cudaError_t launch_render_persistent_uniform(int dtype, int mode, int sampler, const FrameDesc& shared,
                                             const FrameDesc* frames, int nframes, const int* prefix, int* counter,
                                             int grid, cudaStream_t s, int sps) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (mode == MODE_1D && sampler == SAMPLER_SW) {
    if (sps == 2) return persistent_u_sps<2>(dtype, shared, frames, nframes, prefix, counter, grid, s);
    if (sps == 4) return persistent_u_sps<4>(dtype, shared, frames, nframes, prefix, counter, grid, s);
    if (sps == 8) return persistent_u_sps<8>(dtype, shared, frames, nframes, prefix, counter, grid, s);
  }
  GBVR_DISPATCH(persistent_u_t, dtype, mode, sampler, shared, frames, nframes, prefix, counter, grid, s);
}

// Resident CTAs per SM of the batch kernel's variants with 2, 4 or 8 samples
// per step (one launch bound: 8 CTAs of 128 threads, 64 registers).
int persistent_ctas_per_sm_sps2() {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_persistent_u<uint16_t, MODE_1D, SAMPLER_SW, 4>,
                                                RENDER_THREADS, 0);
  return per_sm < 1 ? 1 : per_sm;
}

int persistent_grid_size_uniform(int device, int mode) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  // each mode's own kernel: their launch bounds differ
  if (mode == MODE_1D || mode == MODE_MIP)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_persistent_u<uint16_t, MODE_1D, SAMPLER_SW>,
                                                  RENDER_THREADS, 0);
  else if (mode == MODE_2D)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_persistent_u<uint16_t, MODE_2D, SAMPLER_SW>,
                                                  RENDER_THREADS, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_persistent_u<uint16_t, MODE_ISO, SAMPLER_SW>,
                                                  RENDER_THREADS, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

int persistent_grid_size(int device, int mode) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  // each mode's own kernel: their launch bounds differ
  if (mode == MODE_1D || mode == MODE_MIP)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_persistent<uint16_t, MODE_1D, SAMPLER_SW>,
                                                  RENDER_THREADS, 0);
  else if (mode == MODE_2D)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_persistent<uint16_t, MODE_2D, SAMPLER_SW>,
                                                  RENDER_THREADS, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_persistent<uint16_t, MODE_ISO, SAMPLER_SW>,
                                                  RENDER_THREADS, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace gbvr
