// Raycasting kernels: ray setup, bricked front-to-back walk with empty-brick
// skipping, SW or texture trilinear sampling, 1D / 2D transfer functions with
// opacity correction, FP32 compositing with early ray termination, and the
// isosurface first-hit mode with central-difference Phong shading.
//
// Replaces the fragment-shader raycaster behind Tuvok's AbstrRenderer::Paint
// (reached from LuaScripts/BatchRenderer.lua:35 `renderer.paint()` and
// ImageVis3D/UI/RenderWindow.cpp:2464).  The sampling rule is the project's
// (stated in the design doc): samples at t_k = t_entry + (k + 1/2) dt along the unit
// world-space ray, dt = 1 / (samples_per_voxel * max level dim), trilinear on
// cell-centred voxels with clamp-to-edge, TF index (v - lo) (N - 1) / (hi - lo)
// with linear interpolation between entries, alpha' = 1 - (1 - alpha)^(1/s),
// C += (1 - A) alpha' c, A += (1 - A) alpha', stop at A >= ert, background
// composited last.
//
// One warp renders one 8x4 ray tile.  Two launch forms share render_tile():
//   k_render_plain        one launch per view, one warp per tile (the drop-in
//                         per-view form of AbstrRenderer::Paint)
//   k_render_persistent   grid = SMs x resident CTAs; warps pull (view, tile)
//                         items from one atomic counter spanning every view
//                         of the batch, so views and uneven rays share the GPU.
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

template <typename T>
__device__ __forceinline__ float ldv(const T* p) {
  return (float)__ldg(p);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

struct BrickView {
  unsigned long long off;  // element offset of the brick in the pool
  unsigned long long tex;
  int ox, oy, oz, sx, sy, sz;
  int lox, loy, loz, hix, hiy, hiz;
};

__device__ __forceinline__ void load_brick(const FrameDesc& f, int bi, BrickView& b) {
  const BrickInfo* B = f.bricks + bi;
  const int4 w0 = __ldg(reinterpret_cast<const int4*>(B));      // offset, tex
  const int4 w1 = __ldg(reinterpret_cast<const int4*>(B) + 1);  // ox oy oz sx
  const int4 w2 = __ldg(reinterpret_cast<const int4*>(B) + 2);  // sy sz lox loy
  const int4 w3 = __ldg(reinterpret_cast<const int4*>(B) + 3);  // loz hix hiy hiz
  b.off = ((unsigned long long)(unsigned)w0.y << 32) | (unsigned)w0.x;
  b.tex = ((unsigned long long)(unsigned)w0.w << 32) | (unsigned)w0.z;
  b.ox = w1.x; b.oy = w1.y; b.oz = w1.z; b.sx = w1.w;
  b.sy = w2.x; b.sz = w2.y; b.lox = w2.z; b.loy = w2.w;
  b.loz = w3.x; b.hix = w3.y; b.hiy = w3.z; b.hiz = w3.w;
}

// Value of the level at voxel-centre position p, using brick b (whose stored
// region covers the trilinear footprint of every p whose floor lies in its
// interior, and of p +- 1 voxel, because ghost = 2).  Clamping to the stored
// box equals clamp-to-edge of the whole level: the box ends only at the
// level's boundary.
template <typename T, int SAMPLER>
__device__ __forceinline__ float sample_brick(const FrameDesc& f, const BrickView& b, float px,
                                              float py, float pz) {
  if (SAMPLER == SAMPLER_TEX) {
    cudaTextureObject_t tex = (cudaTextureObject_t)b.tex;
    if (f.interp) {
      return tex3D<float>(tex, px - (float)b.ox + 0.5f, py - (float)b.oy + 0.5f,
                          pz - (float)b.oz + 0.5f) * VoxelTraits<T>::tex_scale;
    }
    int ix = clampi((int)floorf(px + 0.5f) - b.ox, 0, b.sx - 1);
    int iy = clampi((int)floorf(py + 0.5f) - b.oy, 0, b.sy - 1);
    int iz = clampi((int)floorf(pz + 0.5f) - b.oz, 0, b.sz - 1);
    return tex3D<float>(tex, ix + 0.5f, iy + 0.5f, iz + 0.5f) * VoxelTraits<T>::tex_scale;
  }
  const T* base = reinterpret_cast<const T*>(f.pool) + (size_t)b.off;
  if (!f.interp) {
    int ix = clampi((int)floorf(px + 0.5f) - b.ox, 0, b.sx - 1);
    int iy = clampi((int)floorf(py + 0.5f) - b.oy, 0, b.sy - 1);
    int iz = clampi((int)floorf(pz + 0.5f) - b.oz, 0, b.sz - 1);
    return ldv(base + ((size_t)iz * b.sy + iy) * b.sx + ix);
  }
  float fx0 = floorf(px), fy0 = floorf(py), fz0 = floorf(pz);
  float fx = px - fx0, fy = py - fy0, fz = pz - fz0;
  int x0 = (int)fx0 - b.ox, y0 = (int)fy0 - b.oy, z0 = (int)fz0 - b.oz;
  int xa = clampi(x0, 0, b.sx - 1), xb = clampi(x0 + 1, 0, b.sx - 1);
  int ya = clampi(y0, 0, b.sy - 1), yb = clampi(y0 + 1, 0, b.sy - 1);
  int za = clampi(z0, 0, b.sz - 1), zb = clampi(z0 + 1, 0, b.sz - 1);
  const size_t slice = (size_t)b.sx * b.sy;
  const T* pa = base + za * slice;
  const T* pb = base + zb * slice;
  const int ra = ya * b.sx, rb = yb * b.sx;
  float v000 = ldv(pa + ra + xa), v100 = ldv(pa + ra + xb);
  float v010 = ldv(pa + rb + xa), v110 = ldv(pa + rb + xb);
  float v001 = ldv(pb + ra + xa), v101 = ldv(pb + ra + xb);
  float v011 = ldv(pb + rb + xa), v111 = ldv(pb + rb + xb);
  float c00 = fmaf(fx, v100 - v000, v000);
  float c10 = fmaf(fx, v110 - v010, v010);
  float c01 = fmaf(fx, v101 - v001, v001);
  float c11 = fmaf(fx, v111 - v011, v011);
  float c0 = fmaf(fy, c10 - c00, c00);
  float c1 = fmaf(fy, c11 - c01, c01);
  return fmaf(fz, c1 - c0, c0);
}

__device__ __forceinline__ int brick_index(const FrameDesc& f, int gx, int gy, int gz) {
  int bx = gx < 0 ? 0 : min(gx / f.interior, f.nb[0] - 1);
  int by = gy < 0 ? 0 : min(gy / f.interior, f.nb[1] - 1);
  int bz = gz < 0 ? 0 : min(gz / f.interior, f.nb[2] - 1);
  return (bz * f.nb[1] + by) * f.nb[0] + bx;
}

// Voxel cell of a sample, clamped to [-1, n-1]: positions computed in FP32
// can land a rounding error outside the level; clamping keeps brick lookup
// and membership consistent (so the walk always advances), and matches the
// clamp-to-edge sampling rule.  NaN converts to 0.
__device__ __forceinline__ void cell(const FrameDesc& f, float px, float py, float pz, int& gx, int& gy, int& gz) {
  gx = clampi((int)floorf(px), -1, f.dims[0] - 1);
  gy = clampi((int)floorf(py), -1, f.dims[1] - 1);
  gz = clampi((int)floorf(pz), -1, f.dims[2] - 1);
}

__device__ __forceinline__ bool inside(const BrickView& b, int gx, int gy, int gz) {
  return gx >= b.lox && gx < b.hix && gy >= b.loy && gy < b.hiy && gz >= b.loz && gz < b.hiz;
}

// Sample at an arbitrary position (isosurface bisection): find its brick first.
template <typename T, int SAMPLER>
__device__ float sample_anywhere(const FrameDesc& f, float px, float py, float pz) {
  int gx, gy, gz;
  cell(f, px, py, pz, gx, gy, gz);
  int bi = brick_index(f, gx, gy, gz);
  BrickView b;
  load_brick(f, bi, b);
  return sample_brick<T, SAMPLER>(f, b, px, py, pz);
}

// Central differences of the interpolated field at h = 1 voxel (data units
// per voxel).
template <typename T, int SAMPLER>
__device__ __forceinline__ void gradient(const FrameDesc& f, const BrickView& b, float px, float py,
                                         float pz, float g[3]) {
  g[0] = (sample_brick<T, SAMPLER>(f, b, px + 1.f, py, pz) - sample_brick<T, SAMPLER>(f, b, px - 1.f, py, pz)) * 0.5f;
  g[1] = (sample_brick<T, SAMPLER>(f, b, px, py + 1.f, pz) - sample_brick<T, SAMPLER>(f, b, px, py - 1.f, pz)) * 0.5f;
  g[2] = (sample_brick<T, SAMPLER>(f, b, px, py, pz + 1.f) - sample_brick<T, SAMPLER>(f, b, px, py, pz - 1.f)) * 0.5f;
}

// Phong, directional light, two-sided: normal = -grad/|grad| turned towards
// the viewer.  g is a world-space gradient, V the unit vector to the viewer.
__device__ __forceinline__ void shade(const FrameDesc& f, const float g[3], const float V[3],
                                      const float col[3], float out[3]) {
  float gl = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
  if (!(gl > 0.f)) {
    out[0] = col[0] * f.amb[0];
    out[1] = col[1] * f.amb[1];
    out[2] = col[2] * f.amb[2];
    return;
  }
  float n0 = -g[0] / gl, n1 = -g[1] / gl, n2 = -g[2] / gl;
  if (n0 * V[0] + n1 * V[1] + n2 * V[2] < 0.f) { n0 = -n0; n1 = -n1; n2 = -n2; }
  const float* L = f.light_to;
  float nl = fmaxf(0.f, n0 * L[0] + n1 * L[1] + n2 * L[2]);
  float H0 = L[0] + V[0], H1 = L[1] + V[1], H2 = L[2] + V[2];
  float hl = sqrtf(H0 * H0 + H1 * H1 + H2 * H2);
  float nh = hl > 0.f ? fmaxf(0.f, (n0 * H0 + n1 * H1 + n2 * H2) / hl) : 0.f;
  float sp = nh > 0.f ? __powf(nh, f.shininess) : 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = col[k] * (f.amb[k] + f.diff[k] * nl) + f.spec[k] * sp;
}

__device__ __forceinline__ float4 tf1d(const FrameDesc& f, float v) {
  float idx = fminf(fmaxf((v - f.value_lo) * f.idx_scale, 0.f), (float)(f.tf_w - 1));
  float i0f = floorf(idx);
  int i0 = (int)i0f;
  int i1 = min(i0 + 1, f.tf_w - 1);
  float fr = idx - i0f;
  float4 a = __ldg(f.tf + i0), b = __ldg(f.tf + i1);
  return make_float4(fmaf(fr, b.x - a.x, a.x), fmaf(fr, b.y - a.y, a.y), fmaf(fr, b.z - a.z, a.z),
                     fmaf(fr, b.w - a.w, a.w));
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
  float dw[3];         // unit world direction
  float t0, t1;
  bool hit;
};

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
  }
  r.t0 = t0;
  r.t1 = t1;
  // a chord through the unit-normalised box is at most sqrt(3) long; the
  // comparison also rejects NaN rays from degenerate matrices
  r.hit = t1 > t0 && (t1 - t0) < 4.0f;
}

template <typename T, int MODE, int SAMPLER>
__device__ float4 march(const FrameDesc& f, const RaySetup& r, unsigned& nsamp) {
  float C0 = 0.f, C1 = 0.f, C2 = 0.f, A = 0.f;
  if (r.hit) {
    const float dt = f.dt;
    const float t0 = r.t0;
    const int K = max(0, (int)ceilf((r.t1 - t0) / dt - 0.5f));
    const float V[3] = {-r.dw[0], -r.dw[1], -r.dw[2]};
    int k = 0;
    bool done = false;
    while (k < K && !done) {
      float t = fmaf((float)k + 0.5f, dt, t0);
      float px = fmaf(t, r.dv[0], r.ov[0]), py = fmaf(t, r.dv[1], r.ov[1]), pz = fmaf(t, r.dv[2], r.ov[2]);
      int gx, gy, gz;
      cell(f, px, py, pz, gx, gy, gz);
      int bi = brick_index(f, gx, gy, gz);
      BrickView b;
      load_brick(f, bi, b);
      if (__ldg(f.skip + bi)) {
        // Jump past the brick: estimate the exit from its interior planes,
        // then settle the boundary samples by the same floor(pos) rule that
        // assigns samples to bricks, so no sample of a neighbour is skipped.
        float te = INFINITY;
        te = fminf(te, r.dv[0] > 0.f ? ((float)b.hix - r.ov[0]) / r.dv[0]
                                     : (r.dv[0] < 0.f ? ((float)b.lox - r.ov[0]) / r.dv[0] : INFINITY));
        te = fminf(te, r.dv[1] > 0.f ? ((float)b.hiy - r.ov[1]) / r.dv[1]
                                     : (r.dv[1] < 0.f ? ((float)b.loy - r.ov[1]) / r.dv[1] : INFINITY));
        te = fminf(te, r.dv[2] > 0.f ? ((float)b.hiz - r.ov[2]) / r.dv[2]
                                     : (r.dv[2] < 0.f ? ((float)b.loz - r.ov[2]) / r.dv[2] : INFINITY));
        float kef = ceilf((te - t0) / dt - 0.5f);
        int ke = kef >= (float)K ? K : max(k + 1, (int)kef);
        auto in_b = [&](int kk) {
          float tt = fmaf((float)kk + 0.5f, dt, t0);
          int cx, cy, cz;
          cell(f, fmaf(tt, r.dv[0], r.ov[0]), fmaf(tt, r.dv[1], r.ov[1]), fmaf(tt, r.dv[2], r.ov[2]), cx, cy, cz);
          return inside(b, cx, cy, cz);
        };
        while (ke > k + 1 && !in_b(ke - 1)) --ke;
        while (ke < K && in_b(ke)) ++ke;
        k = ke;
        continue;
      }
      if (f.touched) f.touched[bi] = 1;
      for (; k < K; ++k) {
        t = fmaf((float)k + 0.5f, dt, t0);
        px = fmaf(t, r.dv[0], r.ov[0]);
        py = fmaf(t, r.dv[1], r.ov[1]);
        pz = fmaf(t, r.dv[2], r.ov[2]);
        cell(f, px, py, pz, gx, gy, gz);
        if (!inside(b, gx, gy, gz)) break;
        float v = sample_brick<T, SAMPLER>(f, b, px, py, pz);
        ++nsamp;
        if (MODE == MODE_ISO) {
          if (v >= f.iso) {
            float tl = k == 0 ? t0 : fmaf((float)k - 0.5f, dt, t0), th = t;
#pragma unroll 1
            for (int it = 0; it < 4; ++it) {
              float tm = 0.5f * (tl + th);
              float vm = sample_anywhere<T, SAMPLER>(f, fmaf(tm, r.dv[0], r.ov[0]), fmaf(tm, r.dv[1], r.ov[1]),
                                                     fmaf(tm, r.dv[2], r.ov[2]));
              if (vm >= f.iso) th = tm;
              else tl = tm;
            }
            float th2 = 0.5f * (tl + th);
            float hx = fmaf(th2, r.dv[0], r.ov[0]), hy = fmaf(th2, r.dv[1], r.ov[1]), hz = fmaf(th2, r.dv[2], r.ov[2]);
            BrickView hb;
            int hx0, hy0, hz0;
            cell(f, hx, hy, hz, hx0, hy0, hz0);
            load_brick(f, brick_index(f, hx0, hy0, hz0), hb);
            float g[3], col[3];
            gradient<T, SAMPLER>(f, hb, hx, hy, hz, g);
            g[0] *= f.vox_scale[0];
            g[1] *= f.vox_scale[1];
            g[2] *= f.vox_scale[2];
            if (f.lighting) shade(f, g, V, f.iso_rgb, col);
            else { col[0] = f.iso_rgb[0]; col[1] = f.iso_rgb[1]; col[2] = f.iso_rgb[2]; }
            C0 = col[0]; C1 = col[1]; C2 = col[2];
            A = 1.f;
            done = true;
            break;
          }
          continue;
        }
        float4 c;
        if (MODE == MODE_1D) {
          c = tf1d(f, v);
        } else {
          float g[3];
          gradient<T, SAMPLER>(f, b, px, py, pz, g);
          float gm = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
          c = tf2d(f, v, gm);
          if (f.lighting && c.w > 0.f) {
            float gw[3] = {g[0] * f.vox_scale[0], g[1] * f.vox_scale[1], g[2] * f.vox_scale[2]};
            float col[3] = {c.x, c.y, c.z}, lit[3];
            shade(f, gw, V, col, lit);
            c.x = lit[0]; c.y = lit[1]; c.z = lit[2];
          }
        }
        float al = c.w;
        if (f.opacity_exp != 1.f) al = 1.f - __powf(1.f - al, f.opacity_exp);
        float w = (1.f - A) * al;
        C0 = fmaf(w, c.x, C0);
        C1 = fmaf(w, c.y, C1);
        C2 = fmaf(w, c.z, C2);
        A += w;
        if (A >= f.ert) { done = true; break; }
      }
    }
  }
  float rem = 1.f - A;
  return make_float4(fmaf(rem, f.bg[0], C0), fmaf(rem, f.bg[1], C1), fmaf(rem, f.bg[2], C2), A);
}

template <typename T, int MODE, int SAMPLER>
__device__ __forceinline__ void render_tile(const FrameDesc& f, int tile) {
  const int lane = threadIdx.x & 31;
  const int tx = tile % f.tiles_x, ty = tile / f.tiles_x;
  const int px = tx * TILE_W + (lane & (TILE_W - 1));
  const int py = ty * TILE_H + (lane / TILE_W);
  unsigned nsamp = 0;
  if (px < f.width && py < f.height) {
    RaySetup r;
    setup_ray(f, px, py, r);
    float4 c = march<T, MODE, SAMPLER>(f, r, nsamp);
    size_t o = (size_t)py * f.width + px;
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

constexpr int RENDER_THREADS = 128;

template <typename T, int MODE, int SAMPLER>
__global__ void __launch_bounds__(RENDER_THREADS) k_render_plain(const __grid_constant__ FrameDesc f) {
  int warp = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (warp >= f.tiles_x * f.tiles_y) return;
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
__global__ void __launch_bounds__(RENDER_THREADS) k_render_persistent(const FrameDesc* __restrict__ frames, int nframes,
                                                         const int* __restrict__ tile_prefix, int total,
                                                         int* __restrict__ counter) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(counter, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= total) return;
    int fi = find_frame(tile_prefix, nframes, item);
    render_tile<T, MODE, SAMPLER>(frames[fi], item - __ldg(tile_prefix + fi));
  }
}

// ---------------------------------------------------------------------------
// Brick classification: a brick is skipped when no sample inside it can add
// anything.  Values sampled in a brick lie in [vmin, vmax] of its stored
// voxels (trilinear weights are convex), so the TF entries a sample can touch
// are bounded; if every such alpha is 0 the brick contributes exactly nothing.
// Isosurface: skipped when vmax < iso (no sample can reach the isovalue).
// One warp per brick.
// ---------------------------------------------------------------------------
__global__ void k_classify(const BrickInfo* __restrict__ bricks, int nbricks, const float4* __restrict__ tf,
                           int tf_w, int tf_h, int mode, float value_lo, float idx_scale, float iso,
                           unsigned char* __restrict__ skip) {
  int warp = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  int lane = threadIdx.x & 31;
  if (warp >= nbricks) return;
  const BrickInfo& b = bricks[warp];
  if (mode == MODE_ISO) {
    if (lane == 0) skip[warp] = (b.vmax < iso) ? 1 : 0;
    return;
  }
  float ilo = fminf(fmaxf((b.vmin - value_lo) * idx_scale, 0.f), (float)(tf_w - 1));
  float ihi = fminf(fmaxf((b.vmax - value_lo) * idx_scale, 0.f), (float)(tf_w - 1));
  int lo = max((int)floorf(ilo) - 1, 0);
  int hi = min((int)floorf(ihi) + 2, tf_w - 1);
  int rows = mode == MODE_2D ? tf_h : 1;
  int nonzero = 0;
  for (int r = 0; r < rows && !nonzero; ++r) {
    for (int i = lo + lane; i <= hi; i += 32)
      if (tf[r * tf_w + i].w != 0.f) nonzero = 1;
    nonzero = __any_sync(0xffffffffu, nonzero);
  }
  if (lane == 0) skip[warp] = nonzero ? 0 : 1;
}

cudaError_t launch_classify(const BrickInfo* bricks, int nbricks, const float4* tf, int tf_w, int tf_h, int mode,
                            float value_lo, float idx_scale, float iso, unsigned char* skip, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  if (nbricks <= 0) return cudaSuccess;
  int threads = 128;
  int blocks = (nbricks * 32 + threads - 1) / threads;
  k_classify<<<blocks, threads, 0, s>>>(bricks, nbricks, tf, tf_w, tf_h, mode, value_lo, idx_scale, iso, skip);
  return cudaGetLastError();
}

template <typename T, int MODE, int SAMPLER>
static cudaError_t plain_t(const FrameDesc& f, cudaStream_t s) {
  (void)cudaGetLastError();
  int tiles = f.tiles_x * f.tiles_y;
  int warps_per_block = RENDER_THREADS / 32;
  int blocks = (tiles + warps_per_block - 1) / warps_per_block;
  if (blocks == 0) return cudaSuccess;
  k_render_plain<T, MODE, SAMPLER><<<blocks, RENDER_THREADS, 0, s>>>(f);
  return cudaGetLastError();
}

template <typename T, int MODE, int SAMPLER>
static cudaError_t persistent_t(const FrameDesc* frames, int nframes, const int* prefix, int total, int* counter,
                                int grid, cudaStream_t s) {
  (void)cudaGetLastError();
  k_render_persistent<T, MODE, SAMPLER><<<grid, RENDER_THREADS, 0, s>>>(frames, nframes, prefix, total, counter);
  return cudaGetLastError();
}

#define GBVR_DISPATCH(FN, dtype, mode, sampler, ...)                                          \
  do {                                                                                          \
    switch ((dtype) * 6 + (mode) * 2 + (sampler)) {                                             \
      case 0: return FN<uint8_t, MODE_1D, SAMPLER_SW>(__VA_ARGS__);                             \
      case 1: return FN<uint8_t, MODE_1D, SAMPLER_TEX>(__VA_ARGS__);                            \
      case 2: return FN<uint8_t, MODE_2D, SAMPLER_SW>(__VA_ARGS__);                             \
      case 3: return FN<uint8_t, MODE_2D, SAMPLER_TEX>(__VA_ARGS__);                            \
      case 4: return FN<uint8_t, MODE_ISO, SAMPLER_SW>(__VA_ARGS__);                            \
      case 5: return FN<uint8_t, MODE_ISO, SAMPLER_TEX>(__VA_ARGS__);                           \
      case 6: return FN<uint16_t, MODE_1D, SAMPLER_SW>(__VA_ARGS__);                            \
      case 7: return FN<uint16_t, MODE_1D, SAMPLER_TEX>(__VA_ARGS__);                           \
      case 8: return FN<uint16_t, MODE_2D, SAMPLER_SW>(__VA_ARGS__);                            \
      case 9: return FN<uint16_t, MODE_2D, SAMPLER_TEX>(__VA_ARGS__);                           \
      case 10: return FN<uint16_t, MODE_ISO, SAMPLER_SW>(__VA_ARGS__);                          \
      case 11: return FN<uint16_t, MODE_ISO, SAMPLER_TEX>(__VA_ARGS__);                         \
      case 12: return FN<float, MODE_1D, SAMPLER_SW>(__VA_ARGS__);                              \
      case 13: return FN<float, MODE_1D, SAMPLER_TEX>(__VA_ARGS__);                             \
      case 14: return FN<float, MODE_2D, SAMPLER_SW>(__VA_ARGS__);                              \
      case 15: return FN<float, MODE_2D, SAMPLER_TEX>(__VA_ARGS__);                             \
      case 16: return FN<float, MODE_ISO, SAMPLER_SW>(__VA_ARGS__);                             \
      case 17: return FN<float, MODE_ISO, SAMPLER_TEX>(__VA_ARGS__);                            \
      default: return cudaErrorInvalidValue;                                                    \
    }                                                                                           \
  } while (0)

cudaError_t launch_render_plain(const FrameDesc& f, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  GBVR_DISPATCH(plain_t, f.dtype, f.mode, f.sampler, f, s);
}

// All frames of one persistent launch share dtype, mode and sampler (the
// host groups a mixed batch by these and issues one launch per group).
cudaError_t launch_render_persistent_typed(int dtype, int mode, int sampler, const FrameDesc* frames, int nframes,
                                           const int* prefix, int total, int* counter, int grid, cudaStream_t s) {
  (void)cudaGetLastError();  // drop a stale error of an earlier runtime call
  GBVR_DISPATCH(persistent_t, dtype, mode, sampler, frames, nframes, prefix, total, counter, grid, s);
}

int persistent_grid_size(int device) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_persistent<uint16_t, MODE_1D, SAMPLER_SW>,
                                                RENDER_THREADS, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace gbvr
