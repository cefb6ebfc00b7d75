// CPU oracle for the bricked volume raycaster and the UVF build.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
// compared against; nothing in the product links or calls it.  Only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline leg load it.
//
// The reference implementation of this path (Tuvok's GLSL raycaster, its
// ExtendedOctree bricker and its histogram blocks) lives in an un-vendored git
// submodule (https://github.com/SCIInstitute/Tuvok.git, branch master, no
// pinned commit) that is absent from the reference tree, so it cannot be
// compiled.  What this file restates, and where each rule comes from:
//
//  * UVF build call sequence:     UVFReader/DataSource.h:398-683
//      - LOD count rule            DataSource.h:521-529 (halve until it fits)
//      - overlap stored as 2*g     DataSource.h:537-539, CmdLineConverter/main.cpp:145
//      - averaging combiner        DataSource.h:547-572 (CombineAverage<T,1>)
//      - per-brick min/max         DataSource.h:467-469,552 (SimpleMaxMin<T,1>)
//      - 1D histogram + Compress   DataSource.h:601-608
//      - 2D histogram              DataSource.h:609-616
//  * Renderer parameters:          LuaScripts/BatchRenderer.lua:18-41,
//                                  ImageVis3D/UI/RenderWindow.cpp:437-451,2051-2140
//
// Parity is pinned against DemoData/c60.uvf (the reference's own output):
// the 1D histogram, the 2D histogram (bit-exact, including its float32
// max-gradient) and the min/max block.  Rendered images cannot be pinned
// against the reference (no GL stack); the raycaster below is the project's
// documented sampling rule evaluated in FP64.
//
// Build: g++ -O2 -fopenmp -ffp-contract=off -shared -fPIC (see oracle/build.py).
// -ffp-contract=off matters: the integer-exact generators and the f64
// histogram rule must not be contracted into FMAs on any host.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t i64;
typedef uint64_t u64;

enum { DT_U8 = 0, DT_U16 = 1, DT_F32 = 2 };

static inline double load_voxel(const void* p, int dt, i64 i) {
  switch (dt) {
    case DT_U8: return (double)((const uint8_t*)p)[i];
    case DT_U16: return (double)((const uint16_t*)p)[i];
    default: return (double)((const float*)p)[i];
  }
}
static inline size_t dt_size(int dt) { return dt == DT_U8 ? 1 : dt == DT_U16 ? 2 : 4; }

extern "C" {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy
// as 1, 2, 3", SC'11).  Counter-based, so any voxel's draw is independent.
// ---------------------------------------------------------------------------
static inline void mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
  u64 p = (u64)a * (u64)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}
void orc_philox(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(0xD2511F53u, c0, &hi0, &lo0);
    mulhilo(0xCD9E8D57u, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// ---------------------------------------------------------------------------
// LOD pyramid and brick grid (rules stated in the header of this file).
// ---------------------------------------------------------------------------
// Level l+1 has ceil(n/2) voxels per axis.  Levels are added until the
// largest axis fits in one brick interior (brick - 2*ghost), as the
// reference's raster path halves the largest dimension until it fits a brick
// (DataSource.h:521-529).  max_lods > 0 caps the count.
int orc_lod_dims(const i64 dims[3], int brick, int ghost, int max_lods, i64* out /*[L][3]*/) {
  i64 interior = brick - 2 * ghost;
  i64 n[3] = {dims[0], dims[1], dims[2]};
  int count = 0;
  for (;;) {
    out[3 * count + 0] = n[0];
    out[3 * count + 1] = n[1];
    out[3 * count + 2] = n[2];
    ++count;
    i64 mx = std::max(n[0], std::max(n[1], n[2]));
    if (mx <= interior || count == 16) break;
    if (max_lods > 0 && count >= max_lods) break;
    for (int a = 0; a < 3; ++a) n[a] = (n[a] + 1) / 2;
  }
  return count;
}

// A level is a single brick when its largest axis fits the brick interior
// (brick - 2*ghost; c60.uvf: 128^3 in a 256-brick with overlap 4 is one
// brick).  Otherwise it is a grid of interior-sized bricks.  Every stored
// brick carries `ghost` voxels on every face: copies of the neighbouring
// brick's voxels inside the level, and replicated edge voxels (clamp to edge)
// outside it, so a stored brick is (interior + 2 ghost)^3 voxels with its
// origin at interior_start - ghost.
void orc_brick_grid(const i64 dims[3], int brick, int ghost, i64 nb[3], i64* interior) {
  i64 I = brick - 2 * ghost;
  i64 mx = std::max(dims[0], std::max(dims[1], dims[2]));
  if (mx <= I) {
    nb[0] = nb[1] = nb[2] = 1;
    *interior = std::max<i64>(mx, 1);
    return;
  }
  for (int a = 0; a < 3; ++a) nb[a] = (dims[a] + I - 1) / I;
  *interior = I;
}

void orc_brick_extent(const i64 dims[3], int brick, int ghost, const i64 b[3],
                      i64 origin[3], i64 sdims[3]) {
  i64 nb[3], I;
  orc_brick_grid(dims, brick, ghost, nb, &I);
  for (int a = 0; a < 3; ++a) {
    i64 ilo = b[a] * I, ihi = std::min<i64>(ilo + I, dims[a]);
    origin[a] = ilo - ghost;
    sdims[a] = ihi - ilo + 2 * ghost;
  }
}

void orc_extract_brick(const void* vol, int dt, const i64 dims[3], int brick, int ghost,
                       const i64 b[3], void* out) {
  i64 o[3], s[3];
  orc_brick_extent(dims, brick, ghost, b, o, s);
  size_t es = dt_size(dt);
  auto cl = [](i64 v, i64 n) { return v < 0 ? 0 : (v >= n ? n - 1 : v); };
  for (i64 z = 0; z < s[2]; ++z)
    for (i64 y = 0; y < s[1]; ++y)
      for (i64 x = 0; x < s[0]; ++x) {
        i64 src = (cl(o[2] + z, dims[2]) * dims[1] + cl(o[1] + y, dims[1])) * dims[0] + cl(o[0] + x, dims[0]);
        memcpy((char*)out + ((z * s[1] + y) * s[0] + x) * es, (const char*)vol + src * es, es);
      }
}

// 2x2x2 average: each output voxel averages the children that exist (1..8 at
// odd edges).  Integer types take floor(sum / count), i.e. the truncating
// conversion T(double(sum)/count) of an averaging combiner over non-negative
// values; float32 takes float(sum / count) with the sum in double.
void orc_downsample(const void* in, int dt, const i64 dims[3], void* out) {
  i64 od[3] = {(dims[0] + 1) / 2, (dims[1] + 1) / 2, (dims[2] + 1) / 2};
#pragma omp parallel for schedule(static)
  for (i64 z = 0; z < od[2]; ++z)
    for (i64 y = 0; y < od[1]; ++y)
      for (i64 x = 0; x < od[0]; ++x) {
        double sum = 0;
        u64 isum = 0;
        int cnt = 0;
        for (int dz = 0; dz < 2; ++dz)
          for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
              i64 sx = 2 * x + dx, sy = 2 * y + dy, sz = 2 * z + dz;
              if (sx >= dims[0] || sy >= dims[1] || sz >= dims[2]) continue;
              i64 i = (sz * dims[1] + sy) * dims[0] + sx;
              if (dt == DT_F32) sum += ((const float*)in)[i];
              else isum += (u64)load_voxel(in, dt, i);
              ++cnt;
            }
        i64 o = (z * od[1] + y) * od[0] + x;
        if (dt == DT_U8) ((uint8_t*)out)[o] = (uint8_t)(isum / cnt);
        else if (dt == DT_U16) ((uint16_t*)out)[o] = (uint16_t)(isum / cnt);
        else ((float*)out)[o] = (float)(sum / cnt);
      }
}

void orc_minmax(const void* data, int dt, i64 n, double* mn, double* mx) {
  double a = std::numeric_limits<double>::infinity(), b = -a;
  for (i64 i = 0; i < n; ++i) {
    double v = load_voxel(data, dt, i);
    a = std::min(a, v);
    b = std::max(b, v);
  }
  *mn = a;
  *mx = b;
}

// 1D histogram of an integer volume: one bin per value, trailing empty bins
// trimmed (size = max + 1), then merged to at most `max_bins` bins by summing
// runs of f = ceil(size / max_bins) consecutive values.
i64 orc_hist1d(const void* vol, int dt, i64 n, int max_bins, u64* out /* >= 65536 */,
               i64* merge_factor) {
  std::vector<u64> h(dt == DT_U8 ? 256 : 65536, 0);
  for (i64 i = 0; i < n; ++i) h[(size_t)load_voxel(vol, dt, i)]++;
  i64 size = (i64)h.size();
  while (size > 1 && h[size - 1] == 0) --size;
  i64 f = (size + max_bins - 1) / max_bins;
  if (f < 1) f = 1;
  i64 outsize = (size + f - 1) / f;
  for (i64 j = 0; j < outsize; ++j) {
    u64 s = 0;
    for (i64 k = j * f; k < std::min(size, (j + 1) * f); ++k) s += h[k];
    out[j] = s;
  }
  *merge_factor = f;
  return outsize;
}

// 2D histogram, value x gradient magnitude (rule recovered bit-exactly from
// DemoData/c60.uvf; call site DataSource.h:609-616):
//   f(i)  = voxel(i) / maxScalar                     (f64)
//   g_a   = (f(i+1) - f(i-1)) / 2 inside, one-sided first differences on the
//           borders, 0 on an axis of length 1
//   |g|   = sqrt((gx*gx + gy*gy) + gz*gz), x the fastest axis
//   max   = max |g|;  y-bin = floor(|g| / max * 255) (0 when max == 0)
//   x-bin = value / merge_factor (the 1D histogram's merge)
// out is nx * 256 u64, x slowest.  Returns max |g| in f64.
double orc_hist2d(const void* vol, int dt, const i64 dims[3], double max_scalar, i64 nx,
                  i64 merge_factor, u64* out) {
  const i64 X = dims[0], Y = dims[1], Z = dims[2];
  const double c = max_scalar > 0 ? max_scalar : 1.0;
  auto f = [&](i64 x, i64 y, i64 z) { return load_voxel(vol, dt, (z * Y + y) * X + x) / c; };
  auto grad = [&](i64 x, i64 y, i64 z) {
    double gx, gy, gz;
    if (X == 1) gx = 0;
    else if (x == 0) gx = f(1, y, z) - f(0, y, z);
    else if (x == X - 1) gx = f(X - 1, y, z) - f(X - 2, y, z);
    else gx = (f(x + 1, y, z) - f(x - 1, y, z)) / 2.0;
    if (Y == 1) gy = 0;
    else if (y == 0) gy = f(x, 1, z) - f(x, 0, z);
    else if (y == Y - 1) gy = f(x, Y - 1, z) - f(x, Y - 2, z);
    else gy = (f(x, y + 1, z) - f(x, y - 1, z)) / 2.0;
    if (Z == 1) gz = 0;
    else if (z == 0) gz = f(x, y, 1) - f(x, y, 0);
    else if (z == Z - 1) gz = f(x, y, Z - 1) - f(x, y, Z - 2);
    else gz = (f(x, y, z + 1) - f(x, y, z - 1)) / 2.0;
    double s = gx * gx;
    s = s + gy * gy;
    s = s + gz * gz;
    return std::sqrt(s);
  };
  double mg = 0;
#pragma omp parallel for reduction(max : mg) schedule(static)
  for (i64 z = 0; z < Z; ++z)
    for (i64 y = 0; y < Y; ++y)
      for (i64 x = 0; x < X; ++x) mg = std::max(mg, grad(x, y, z));
  memset(out, 0, sizeof(u64) * nx * 256);
  for (i64 z = 0; z < Z; ++z)
    for (i64 y = 0; y < Y; ++y)
      for (i64 x = 0; x < X; ++x) {
        double g = grad(x, y, z);
        i64 by = 0;
        if (mg > 0) {
          double r = g / mg;
          r = r * 255.0;
          by = (i64)std::floor(r);
          if (by > 255) by = 255;
        }
        i64 bx = (i64)load_voxel(vol, dt, (z * Y + y) * X + x) / merge_factor;
        if (bx >= nx) bx = nx - 1;
        out[bx * 256 + by]++;
      }
  return mg;
}

// ---------------------------------------------------------------------------
// Seeded synthetic volumes.  Every voxel is a fixed sequence of float32
// multiplies and adds over per-axis tables, so a CUDA kernel that performs the
// same sequence with round-to-nearest intrinsics reproduces it bit for bit.
// ---------------------------------------------------------------------------
struct orc_blob_tables {
  int nblobs;
  const float* amp;     // [nblobs]
  const float* ex;      // [nblobs][nx]
  const float* ey;      // [nblobs][ny]
  const float* ez;      // [nblobs][nz]
  const float* bgx;     // [nx] or null
  const float* bgy;     // [ny]
  const float* bgz;     // [nz]
  float bg_level;       // background = bg_level + bg_amp * bgx*bgy*bgz
  float bg_amp;
  float scale;          // value = scale * (background + sum of blobs) + noise
  float noise_amp;      // uniform: +-noise_amp; gaussian: sigma
  int noise_kind;       // 0 none, 1 uniform, 2 Irwin-Hall(12) gaussian
  float vmax;           // clamp to [0, vmax]
  uint32_t seed;
};

static inline float blob_noise(const orc_blob_tables* t, u64 idx) {
  uint32_t ctr[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 0x6e6f6973u, 0};
  uint32_t key[2] = {t->seed, 0x766f6c21u};
  uint32_t r[4];
  if (t->noise_kind == 1) {
    orc_philox(ctr, key, r);
    float u = (float)(r[0] >> 8) * (1.0f / 16777216.0f);
    float n = u * (2.0f * t->noise_amp);
    return n - t->noise_amp;
  }
  if (t->noise_kind == 2) {
    uint32_t s = 0;
    for (int k = 0; k < 3; ++k) {
      ctr[3] = (uint32_t)k;
      orc_philox(ctr, key, r);
      for (int j = 0; j < 4; ++j) s += (r[j] >> 16);
    }
    float z = (float)s * (1.0f / 65536.0f);
    z = z - 6.0f;
    return z * t->noise_amp;
  }
  return 0.0f;
}

// Per-axis tables of the blob generator, restated from the recipe:
//  blob k: Philox(ctr {k, 0, 'blob', 0}, key {seed, 'para'}) -> centre
//          u_i * n_i (u_i = top 24 bits / 2^24); Philox(ctr {k, 1, ...})
//          -> sigma = lo + u0 (hi - lo), amplitude = lo + u1 (hi - lo)
//  e_k(i)  = float(exp(-(i - c)^2 / (2 sigma^2)))           (double math)
//  background b(i) = float(cos(2 pi (f (i + 0.5) / n + phase))), phases from
//          Philox(ctr {0xffffffff, 2, 'blob', 0})
// Caller provides storage: amp[nb], ex[nb*nx], ey[nb*ny], ez[nb*nz],
// bg*[n] (when bg_freq > 0).
void orc_blob_tables_make(const i64 dims[3], uint32_t seed, int nb, double sig_lo, double sig_hi,
                          double amp_lo, double amp_hi, double bg_freq, float* amp, float* ex,
                          float* ey, float* ez, float* bgx, float* bgy, float* bgz) {
  const uint32_t key[2] = {seed, 0x70617261u};
  float* tabs[3] = {ex, ey, ez};
  for (int k = 0; k < nb; ++k) {
    uint32_t c0[4] = {(uint32_t)k, 0u, 0x626c6f62u, 0u}, r0[4];
    uint32_t c1[4] = {(uint32_t)k, 1u, 0x626c6f62u, 0u}, r1[4];
    orc_philox(c0, key, r0);
    orc_philox(c1, key, r1);
    double cen[3];
    for (int a = 0; a < 3; ++a) cen[a] = (double)(r0[a] >> 8) / 16777216.0 * (double)dims[a];
    double sig = sig_lo + (double)(r1[0] >> 8) / 16777216.0 * (sig_hi - sig_lo);
    double am = amp_lo + (double)(r1[1] >> 8) / 16777216.0 * (amp_hi - amp_lo);
    amp[k] = (float)am;
    for (int a = 0; a < 3; ++a)
      for (i64 i = 0; i < dims[a]; ++i) {
        double dd = (double)i - cen[a];
        tabs[a][(i64)k * dims[a] + i] = (float)std::exp(-(dd * dd) / (2.0 * sig * sig));
      }
  }
  if (bg_freq > 0) {
    uint32_t c[4] = {0xffffffffu, 2u, 0x626c6f62u, 0u}, r[4];
    orc_philox(c, key, r);
    float* bt[3] = {bgx, bgy, bgz};
    for (int a = 0; a < 3; ++a) {
      double ph = (double)(r[a] >> 8) / 16777216.0;
      for (i64 i = 0; i < dims[a]; ++i)
        bt[a][i] = (float)std::cos(2.0 * M_PI * (bg_freq * ((double)i + 0.5) / (double)dims[a] + ph));
    }
  }
}

void orc_synth_blobs(const orc_blob_tables* t, const i64 dims[3], int dt, void* out) {
  const i64 X = dims[0], Y = dims[1], Z = dims[2];
#pragma omp parallel for schedule(static)
  for (i64 z = 0; z < Z; ++z)
    for (i64 y = 0; y < Y; ++y)
      for (i64 x = 0; x < X; ++x) {
        float acc = 0.0f;
        if (t->bgx) {
          float b = t->bgx[x] * t->bgy[y];
          b = b * t->bgz[z];
          b = b * t->bg_amp;
          acc = t->bg_level + b;
        }
        for (int k = 0; k < t->nblobs; ++k) {
          float w = t->amp[k] * t->ez[(i64)k * Z + z];
          w = w * t->ey[(i64)k * Y + y];
          w = w * t->ex[(i64)k * X + x];
          acc = acc + w;
        }
        float v = acc * t->scale;
        i64 idx = (z * Y + y) * X + x;
        v = v + blob_noise(t, (u64)idx);
        if (dt == DT_F32) {
          ((float*)out)[idx] = v;
          continue;
        }
        float r = std::nearbyint(v);
        if (r < 0.0f) r = 0.0f;
        if (r > t->vmax) r = t->vmax;
        if (dt == DT_U8) ((uint8_t*)out)[idx] = (uint8_t)r;
        else ((uint16_t*)out)[idx] = (uint16_t)r;
      }
}

// ---------------------------------------------------------------------------
// Seeded fractal (fBm) volume: `octaves` octaves of periodic value noise.
// Octave o has a lattice of P = base_period << o cells across every axis,
// lattice values from the integer hash "lowbias32" (C. Wellons, 2018) of the
// wrapped lattice index, smoothstep-weighted trilinear interpolation, and
// weight 2^-o; the sum is normalised, thresholded and scaled:
//   v = clamp((fbm - thr) / (1 - thr), 0, 1) * vmax, rounded to nearest.
// Every step is a single float32 operation in a fixed order.
// ---------------------------------------------------------------------------
static inline uint32_t lowbias32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

static inline float fbm_lattice(uint32_t i, uint32_t j, uint32_t k, uint32_t P, uint32_t salt) {
  uint32_t h = lowbias32(((k * P + j) * P + i) ^ salt);
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}

static inline float fbm_lerp(float a, float b, float t) {
  float d = b - a;
  d = d * t;
  return a + d;
}

float orc_fbm_value(const i64 dims[3], uint32_t seed, int octaves, int base_period, i64 x, i64 y, i64 z) {
  float acc = 0.0f, norm = 0.0f, amp = 1.0f;
  const i64 c[3] = {x, y, z};
  for (int o = 0; o < octaves; ++o) {
    const uint32_t P = (uint32_t)base_period << o;
    const uint32_t salt = seed + 0x9E3779B9u * (uint32_t)(o + 1);
    uint32_t i0[3], i1[3];
    float s[3];
    for (int a = 0; a < 3; ++a) {
      float scale = (float)P / (float)dims[a];
      float u = (float)c[a] + 0.5f;
      u = u * scale;
      float f = std::floor(u);
      float t = u - f;
      float tt = t * t;
      float w = 3.0f - (t + t);
      s[a] = tt * w;
      uint32_t ii = (uint32_t)(i64)f % P;
      i0[a] = ii;
      i1[a] = (ii + 1) % P;
    }
    float c00 = fbm_lerp(fbm_lattice(i0[0], i0[1], i0[2], P, salt), fbm_lattice(i1[0], i0[1], i0[2], P, salt), s[0]);
    float c10 = fbm_lerp(fbm_lattice(i0[0], i1[1], i0[2], P, salt), fbm_lattice(i1[0], i1[1], i0[2], P, salt), s[0]);
    float c01 = fbm_lerp(fbm_lattice(i0[0], i0[1], i1[2], P, salt), fbm_lattice(i1[0], i0[1], i1[2], P, salt), s[0]);
    float c11 = fbm_lerp(fbm_lattice(i0[0], i1[1], i1[2], P, salt), fbm_lattice(i1[0], i1[1], i1[2], P, salt), s[0]);
    float c0 = fbm_lerp(c00, c10, s[1]);
    float c1 = fbm_lerp(c01, c11, s[1]);
    float n = fbm_lerp(c0, c1, s[2]);
    acc = acc + amp * n;
    norm = norm + amp;
    amp = amp * 0.5f;
  }
  return acc / norm;
}

// One voxel of the seeded fractal volume as stored (u8 / u16 rounded to
// nearest, f32 as is): the thresholded, rescaled fBm value.  inv = 1 / (1 - thr).
static inline float fbm_voxel(const i64 dims[3], int dt, uint32_t seed, int octaves, int base_period, float thr,
                              float inv, float vmax, i64 x, i64 y, i64 z) {
  float f = orc_fbm_value(dims, seed, octaves, base_period, x, y, z);
  float v = f - thr;
  v = v * inv;
  v = std::min(std::max(v, 0.0f), 1.0f);
  v = v * vmax;
  return dt == DT_F32 ? v : (float)std::nearbyint(v);
}

void orc_synth_fbm(const i64 dims[3], int dt, uint32_t seed, int octaves, int base_period, float thr, float vmax,
                   void* out) {
  const i64 X = dims[0], Y = dims[1], Z = dims[2];
  const float inv = 1.0f / (1.0f - thr);
#pragma omp parallel for schedule(static)
  for (i64 z = 0; z < Z; ++z)
    for (i64 y = 0; y < Y; ++y)
      for (i64 x = 0; x < X; ++x) {
        const float v = fbm_voxel(dims, dt, seed, octaves, base_period, thr, inv, vmax, x, y, z);
        i64 idx = (z * Y + y) * X + x;
        if (dt == DT_F32) ((float*)out)[idx] = v;
        else if (dt == DT_U8) ((uint8_t*)out)[idx] = (uint8_t)v;
        else ((uint16_t*)out)[idx] = (uint16_t)v;
      }
}

// ---------------------------------------------------------------------------
// FP64 raycaster: the project's sampling rule, evaluated directly on the flat
// volume of the rendered LOD (no bricks: the bricked GPU walk must reproduce
// sampling of the whole level, since ghost voxels are exact copies).
// ---------------------------------------------------------------------------
struct orc_render_params {
  const void* vol;      // flat level, x fastest
  int dtype;
  i64 dims[3];          // dims of the rendered level
  double extent[3];     // world box = [-extent/2, +extent/2] (largest axis 1)
  const float* tf;      // 1D: [n][4]; 2D: [h][w][4] (row = gradient bin)
  int tf_w, tf_h;       // 1D: tf_w entries, tf_h = 1
  int mode;             // 0 1D TF, 1 2D TF + Phong, 2 isosurface, 3 maximum-intensity projection
  int interp;           // 0 nearest, 1 trilinear
  double value_lo, value_hi;   // data value mapped to TF coordinate 0 / 1
  double grad_max;      // 2D TF: |grad| (normalised value per voxel) at the last row
  double samples_per_voxel;
  double ert;           // early ray termination threshold (0.99)
  double iso;           // data value
  double iso_rgb[3];
  int lighting;
  double amb[3], diff[3], spec[3];
  double shininess;
  double light_dir_eye[3];  // direction the light travels, eye space
  double bg[3];
  double inv_viewproj[16];  // row-major inverse of proj*view (column vectors)
  double inv_view[16];      // row-major inverse of view
  int width, height;
  int clip_on;              // clip plane: samples with clip . (x, y, z, 1) > 0 (world) are dropped
  double clip[4];
  // bounding-box lines (the renderer's setGlobalBBox / setLocalBBox)
  int bbox_global, bbox_local;
  double line_rgb[2][3];    // global box, brick boxes
  double view[16], proj[16];  // the float32 view and projection matrices (row-major)
  i64 brick_interior;       // brick edge minus two ghost layers (the level is one brick if it fits)
  const uint32_t* line_keys;  // filled by orc_render: per pixel the nearest line's key or 0xffffffff
  // ClearView (mode 2): the first hit of iso is the context surface; inside the lens (distance to the
  // focus point in pixels over cv_radius < 1) it gets opacity clamp(cv_context (1 - |n.v|) + cv_border
  // rho^2, 0, 1) over the first hit of cv_iso from the context hit's sample on (colour cv_rgb)
  int cv_on;
  double cv_iso, cv_rgb[3], cv_context, cv_border, cv_focus[2], cv_radius;
  // Background gradient (setBGColors with two colours): bg is the bottom
  // edge's colour, bg_top the top edge's; each pixel row takes the colour at
  // its centre, linear in between.
  int bg_grad;
  double bg_top[3];
  // Procedural volume: with proc_fbm set, vol is not read; every voxel is the
  // seeded fractal volume's (orc_synth_fbm with these parameters and dtype),
  // evaluated where a sample needs it.  Lets a pixel subset of a volume too
  // large for host memory be rendered.
  int proc_fbm;
  uint32_t fbm_seed;
  int fbm_octaves, fbm_base_period;
  float fbm_threshold, fbm_vmax;
};

static void bg_row(const orc_render_params* p, int py, double out[3]) {
  if (!p->bg_grad) {
    for (int k = 0; k < 3; ++k) out[k] = p->bg[k];
    return;
  }
  const double t = ((double)py + 0.5) / (double)p->height;
  for (int k = 0; k < 3; ++k) out[k] = p->bg_top[k] + t * (p->bg[k] - p->bg_top[k]);
}

struct Vol {
  const orc_render_params* p;
  double vox(i64 x, i64 y, i64 z) const {
    if (p->proc_fbm)
      return fbm_voxel(p->dims, p->dtype, p->fbm_seed, p->fbm_octaves, p->fbm_base_period, p->fbm_threshold,
                       1.0f / (1.0f - p->fbm_threshold), p->fbm_vmax, x, y, z);
    return load_voxel(p->vol, p->dtype, (z * p->dims[1] + y) * p->dims[0] + x);
  }
  double sample_nearest(double x, double y, double z) const {
    i64 ix = (i64)std::floor(x + 0.5), iy = (i64)std::floor(y + 0.5), iz = (i64)std::floor(z + 0.5);
    ix = std::min(std::max<i64>(ix, 0), p->dims[0] - 1);
    iy = std::min(std::max<i64>(iy, 0), p->dims[1] - 1);
    iz = std::min(std::max<i64>(iz, 0), p->dims[2] - 1);
    return vox(ix, iy, iz);
  }
  double sample(double x, double y, double z) const {
    if (!p->interp) return sample_nearest(x, y, z);
    double fx0 = std::floor(x), fy0 = std::floor(y), fz0 = std::floor(z);
    double fx = x - fx0, fy = y - fy0, fz = z - fz0;
    i64 x0 = (i64)fx0, y0 = (i64)fy0, z0 = (i64)fz0;
    i64 X = p->dims[0], Y = p->dims[1], Z = p->dims[2];
    auto cl = [](i64 v, i64 n) { return v < 0 ? 0 : (v >= n ? n - 1 : v); };
    i64 xa = cl(x0, X), xb = cl(x0 + 1, X), ya = cl(y0, Y), yb = cl(y0 + 1, Y);
    i64 za = cl(z0, Z), zb = cl(z0 + 1, Z);
    auto v = [&](i64 xi, i64 yi, i64 zi) { return vox(xi, yi, zi); };
    auto lerp = [](double a, double b, double t) { return a + t * (b - a); };
    double c00 = lerp(v(xa, ya, za), v(xb, ya, za), fx);
    double c10 = lerp(v(xa, yb, za), v(xb, yb, za), fx);
    double c01 = lerp(v(xa, ya, zb), v(xb, ya, zb), fx);
    double c11 = lerp(v(xa, yb, zb), v(xb, yb, zb), fx);
    double c0 = lerp(c00, c10, fy), c1 = lerp(c01, c11, fy);
    return lerp(c0, c1, fz);
  }
  // central differences of the interpolated field, h = 1 voxel, in data
  // value units per voxel
  void gradient(double x, double y, double z, double g[3]) const {
    g[0] = (sample(x + 1, y, z) - sample(x - 1, y, z)) * 0.5;
    g[1] = (sample(x, y + 1, z) - sample(x, y - 1, z)) * 0.5;
    g[2] = (sample(x, y, z + 1) - sample(x, y, z - 1)) * 0.5;
  }
};

static void mat_vec4(const double* m, const double v[4], double o[4]) {
  for (int r = 0; r < 4; ++r) o[r] = m[4 * r] * v[0] + m[4 * r + 1] * v[1] + m[4 * r + 2] * v[2] + m[4 * r + 3] * v[3];
}

static void tf1d_lookup(const orc_render_params* p, double idx, double c[4]) {
  int n = p->tf_w;
  if (idx < 0) idx = 0;
  if (idx > n - 1) idx = n - 1;
  int i0 = (int)std::floor(idx);
  int i1 = std::min(i0 + 1, n - 1);
  double f = idx - i0;
  for (int k = 0; k < 4; ++k) {
    double a = p->tf[4 * i0 + k], b = p->tf[4 * i1 + k];
    c[k] = a + f * (b - a);
  }
}

static void tf2d_lookup(const orc_render_params* p, double ix, double iy, double c[4]) {
  int w = p->tf_w, h = p->tf_h;
  ix = std::min(std::max(ix, 0.0), (double)(w - 1));
  iy = std::min(std::max(iy, 0.0), (double)(h - 1));
  int x0 = (int)std::floor(ix), y0 = (int)std::floor(iy);
  int x1 = std::min(x0 + 1, w - 1), y1 = std::min(y0 + 1, h - 1);
  double fx = ix - x0, fy = iy - y0;
  for (int k = 0; k < 4; ++k) {
    double a = p->tf[4 * (y0 * w + x0) + k], b = p->tf[4 * (y0 * w + x1) + k];
    double cc = p->tf[4 * (y1 * w + x0) + k], d = p->tf[4 * (y1 * w + x1) + k];
    double t0 = a + fx * (b - a), t1 = cc + fx * (d - cc);
    c[k] = t0 + fy * (t1 - t0);
  }
}

// Phong with a directional light; the normal is the negated normalised
// gradient, flipped to face the viewer (two-sided).
static void shade(const orc_render_params* p, const double g[3], const double vdir[3],
                  const double L[3], const double col[3], double out[3]) {
  double gl = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
  if (gl <= 0) {
    for (int k = 0; k < 3; ++k) out[k] = col[k] * p->amb[k];
    return;
  }
  double n[3] = {-g[0] / gl, -g[1] / gl, -g[2] / gl};
  double V[3] = {-vdir[0], -vdir[1], -vdir[2]};
  double nv = n[0] * V[0] + n[1] * V[1] + n[2] * V[2];
  if (nv < 0) for (int k = 0; k < 3; ++k) n[k] = -n[k];
  double nl = std::max(0.0, n[0] * L[0] + n[1] * L[1] + n[2] * L[2]);
  double H[3] = {L[0] + V[0], L[1] + V[1], L[2] + V[2]};
  double hl = std::sqrt(H[0] * H[0] + H[1] * H[1] + H[2] * H[2]);
  double nh = 0;
  if (hl > 0) nh = std::max(0.0, (n[0] * H[0] + n[1] * H[1] + n[2] * H[2]) / hl);
  double sp = std::pow(nh, p->shininess);
  for (int k = 0; k < 3; ++k) out[k] = col[k] * (p->amb[k] + p->diff[k] * nl) + p->spec[k] * sp;
}

// ---------------------------------------------------------------------------
// Bounding-box lines.  Segments: the 12 edges of the box [-extent/2,
// extent/2] and the lines of the level's brick grid (bounds at multiples of
// the interior size, clamped to the level, at (b / dims) extent - extent/2)
// that are not edges of the drawn box.  A pixel is covered by a segment when
// its centre lies within half a pixel of the segment's projection: the
// segment in clip space (P V x), clipped to the near plane z >= -w, divided
// by w, mapped to pixels (x + 1) W/2, (1 - y) H/2; the covered point's NDC
// depth is interpolated linearly along the projected segment.  Key = the
// float bits of (z + 2) with bit 0 = colour (0 global, 1 brick); the nearest
// line has the smallest key.  Every expression below is evaluated in the
// order written, one rounding per operation (-ffp-contract=off), so the keys
// are reproducible bit for bit.  Projections beyond 1e8 pixels are dropped.
// ---------------------------------------------------------------------------
struct OrcSeg {
  double a[3], b[3];
  int color;
};

static void bbox_segments(const orc_render_params* p, std::vector<OrcSeg>& segs) {
  double h[3];
  for (int a = 0; a < 3; ++a) h[a] = 0.5 * p->extent[a];
  const i64 mx = std::max(p->dims[0], std::max(p->dims[1], p->dims[2]));
  const bool single = mx <= p->brick_interior;
  const i64 I = single ? mx : p->brick_interior;
  i64 nb[3];
  for (int a = 0; a < 3; ++a) nb[a] = single ? 1 : (p->dims[a] + I - 1) / I;
  auto add = [&](int a, double u, double v, int color) {
    const int b = (a + 1) % 3, c = (a + 2) % 3;
    OrcSeg s;
    s.a[a] = -h[a];
    s.b[a] = h[a];
    s.a[b] = s.b[b] = u;
    s.a[c] = s.b[c] = v;
    s.color = color;
    segs.push_back(s);
  };
  for (int a = 0; a < 3; ++a) {
    const int b = (a + 1) % 3, c = (a + 2) % 3;
    if (p->bbox_global)
      for (int k = 0; k < 4; ++k) add(a, (k & 1) ? h[b] : -h[b], (k & 2) ? h[c] : -h[c], 0);
    if (!p->bbox_local) continue;
    auto bound = [&](int ax, i64 j) {
      const i64 bj = std::min(j * I, p->dims[ax]);
      return (double)bj / (double)p->dims[ax] * p->extent[ax] - h[ax];
    };
    for (i64 j = 0; j <= nb[b]; ++j)
      for (i64 k = 0; k <= nb[c]; ++k) {
        const bool edge = (j == 0 || j == nb[b]) && (k == 0 || k == nb[c]);
        if (edge && p->bbox_global) continue;
        add(a, bound(b, j), bound(c, k), 1);
      }
  }
}

static void line_keys(const orc_render_params* p, std::vector<uint32_t>& keys) {
  const int W = p->width, H = p->height;
  keys.assign((size_t)W * H, 0xffffffffu);
  std::vector<OrcSeg> segs;
  bbox_segments(p, segs);
  const double* Pm = p->proj;
  const double* Vm = p->view;
  double M[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      M[4 * i + j] = Pm[4 * i] * Vm[j] + Pm[4 * i + 1] * Vm[4 + j] + Pm[4 * i + 2] * Vm[8 + j] + Pm[4 * i + 3] * Vm[12 + j];
  for (const OrcSeg& s : segs) {
    double c0[4], c1[4];
    for (int i = 0; i < 4; ++i) {
      c0[i] = M[4 * i] * s.a[0] + M[4 * i + 1] * s.a[1] + M[4 * i + 2] * s.a[2] + M[4 * i + 3];
      c1[i] = M[4 * i] * s.b[0] + M[4 * i + 1] * s.b[1] + M[4 * i + 2] * s.b[2] + M[4 * i + 3];
    }
    const double n0 = c0[2] + c0[3], n1 = c1[2] + c1[3];
    if (n0 < 0.0 && n1 < 0.0) continue;
    double p0[4], p1[4];
    for (int k = 0; k < 4; ++k) { p0[k] = c0[k]; p1[k] = c1[k]; }
    if (n0 < 0.0) {
      const double u = n0 / (n0 - n1);
      for (int k = 0; k < 4; ++k) p0[k] = c0[k] + u * (c1[k] - c0[k]);
    } else if (n1 < 0.0) {
      const double u = n1 / (n1 - n0);
      for (int k = 0; k < 4; ++k) p1[k] = c1[k] + u * (c0[k] - c1[k]);
    }
    if (!(p0[3] > 0.0 && p1[3] > 0.0)) continue;
    const double hw = 0.5 * (double)W, hh = 0.5 * (double)H;
    const double sx0 = (p0[0] / p0[3] + 1.0) * hw, sy0 = (1.0 - p0[1] / p0[3]) * hh;
    const double sx1 = (p1[0] / p1[3] + 1.0) * hw, sy1 = (1.0 - p1[1] / p1[3]) * hh;
    if (!(std::fabs(sx0) < 1e8 && std::fabs(sy0) < 1e8 && std::fabs(sx1) < 1e8 && std::fabs(sy1) < 1e8)) continue;
    const double z0 = p0[2] / p0[3], z1 = p1[2] / p1[3];
    const double dx = sx1 - sx0, dy = sy1 - sy0, dz = z1 - z0;
    const double l2 = dx * dx + dy * dy;
    const double inv = l2 > 0.0 ? 1.0 / l2 : 0.0;
    // every pixel of the segment's bounding box, one pixel wider
    const i64 x0 = std::max<i64>(0, (i64)std::floor(std::min(sx0, sx1) - 1.0));
    const i64 x1 = std::min<i64>(W - 1, (i64)std::floor(std::max(sx0, sx1) + 1.0));
    const i64 y0 = std::max<i64>(0, (i64)std::floor(std::min(sy0, sy1) - 1.0));
    const i64 y1 = std::min<i64>(H - 1, (i64)std::floor(std::max(sy0, sy1) + 1.0));
    for (i64 py = y0; py <= y1; ++py)
      for (i64 px = x0; px <= x1; ++px) {
        const double cx = (double)px + 0.5, cy = (double)py + 0.5;
        double t = ((cx - sx0) * dx + (cy - sy0) * dy) * inv;
        t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
        const double ex = cx - (sx0 + t * dx), ey = cy - (sy0 + t * dy);
        const double d2 = ex * ex + ey * ey;
        if (!(d2 <= 0.25)) continue;
        const double zz = (z0 + t * dz) + 2.0;
        if (!(zz > 0.0)) continue;
        const float zf = (float)zz;
        uint32_t u;
        memcpy(&u, &zf, 4);
        u = (u & ~1u) | (uint32_t)s.color;
        uint32_t& k = keys[(size_t)py * W + px];
        if (u < k) k = u;
      }
  }
}

static void render_pixel(const orc_render_params* p, int px, int py, double* out,
                         i64* nsamples) {
  Vol V{p};
  double ndc_x = (px + 0.5) / p->width * 2.0 - 1.0;
  double ndc_y = 1.0 - (py + 0.5) / p->height * 2.0;
  double a[4] = {ndc_x, ndc_y, -1.0, 1.0}, b[4] = {ndc_x, ndc_y, 1.0, 1.0}, na[4], fb[4];
  mat_vec4(p->inv_viewproj, a, na);
  mat_vec4(p->inv_viewproj, b, fb);
  double o[3], d[3];
  for (int k = 0; k < 3; ++k) {
    o[k] = na[k] / na[3];
    d[k] = fb[k] / fb[3] - o[k];
  }
  double dl = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  for (int k = 0; k < 3; ++k) d[k] /= dl;
  double t0 = 0.0, t1 = std::numeric_limits<double>::infinity();
  for (int k = 0; k < 3; ++k) {
    double lo = -0.5 * p->extent[k], hi = 0.5 * p->extent[k];
    if (d[k] == 0.0) {
      if (o[k] < lo || o[k] > hi) { t1 = -1; break; }
      continue;
    }
    double ta = (lo - o[k]) / d[k], tb = (hi - o[k]) / d[k];
    t0 = std::max(t0, std::min(ta, tb));
    t1 = std::min(t1, std::max(ta, tb));
  }
  // a bounding-box line covering the pixel ends the ray at the line's depth
  const uint32_t line = p->line_keys ? p->line_keys[(size_t)py * p->width + px] : 0xffffffffu;
  if (line != 0xffffffffu) {
    const uint32_t u = line & ~1u;
    float zf;
    memcpy(&zf, &u, 4);
    double g[4], gh[4] = {ndc_x, ndc_y, (double)zf - 2.0, 1.0};
    mat_vec4(p->inv_viewproj, gh, g);
    double ts = 0.0;
    for (int k = 0; k < 3; ++k) ts += (g[k] / g[3] - o[k]) * d[k];
    t1 = std::min(t1, ts);
  }
  double C[3] = {0, 0, 0}, A = 0;
  // light: travels along light_dir_eye, transformed to world by the inverse view
  double L[3] = {0, 0, 0};
  {
    double ld[3];
    for (int r = 0; r < 3; ++r)
      ld[r] = p->inv_view[4 * r] * p->light_dir_eye[0] + p->inv_view[4 * r + 1] * p->light_dir_eye[1] +
              p->inv_view[4 * r + 2] * p->light_dir_eye[2];
    double ll = std::sqrt(ld[0] * ld[0] + ld[1] * ld[1] + ld[2] * ld[2]);
    if (ll > 0) for (int k = 0; k < 3; ++k) L[k] = -ld[k] / ll;
  }
  i64 ns = 0;
  if (t1 > t0) {
    i64 maxd = std::max(p->dims[0], std::max(p->dims[1], p->dims[2]));
    double dt = 1.0 / (p->samples_per_voxel * (double)maxd);
    double K = std::ceil((t1 - t0) / dt - 0.5);
    i64 nk = K > 0 ? (i64)K : 0;
    double e = 1.0 / p->samples_per_voxel;
    double scale_v[3], off_v[3];
    for (int k = 0; k < 3; ++k) {
      scale_v[k] = (double)p->dims[k] / p->extent[k];
      off_v[k] = 0.5 * p->extent[k];
    }
    auto to_vox = [&](double t, double x[3]) {
      for (int k = 0; k < 3; ++k) x[k] = (o[k] + t * d[k] + off_v[k]) * scale_v[k] - 0.5;
    };
    double vscale = 1.0 / (p->value_hi - p->value_lo);
    double prev_t = t0;
    double vmax = -std::numeric_limits<double>::infinity();
    bool any = false;
    // ClearView state: phase 0 looks for the context surface, 1 for the focus surface
    int cv_phase = 0;
    double cv_a = 1.0, cv_c[3] = {0, 0, 0};
    double cv_rho = 2.0;
    if (p->cv_on && p->mode == 2) {
      const double dx = px + 0.5 - p->cv_focus[0], dy = py + 0.5 - p->cv_focus[1];
      cv_rho = std::sqrt(dx * dx + dy * dy) / p->cv_radius;
    }
    for (i64 k = 0; k < nk; ++k) {
      double t = t0 + (k + 0.5) * dt;
      if (p->clip_on) {
        // the GPU settles the kept range with the same test per sample
        double s = p->clip[3];
        for (int q = 0; q < 3; ++q) s += p->clip[q] * (o[q] + t * d[q]);
        if (s > 0) {
          prev_t = t;
          continue;
        }
      }
      double x[3];
      to_vox(t, x);
      double v = V.sample(x[0], x[1], x[2]);
      ++ns;
      if (p->mode == 3) {
        vmax = std::max(vmax, v);
        any = true;
        prev_t = t;
        continue;
      }
      if (p->mode == 2) {
        const double thr = cv_phase ? p->cv_iso : p->iso;
        if (v >= thr) {
          double tl = (k == 0) ? t0 : prev_t, th = t;
          for (int it = 0; it < 4; ++it) {
            double tm = 0.5 * (tl + th), xm[3];
            to_vox(tm, xm);
            if (V.sample(xm[0], xm[1], xm[2]) >= thr) th = tm;
            else tl = tm;
          }
          double th_hit = 0.5 * (tl + th), xh[3], g[3], col[3];
          to_vox(th_hit, xh);
          V.gradient(xh[0], xh[1], xh[2], g);
          for (int c = 0; c < 3; ++c) g[c] *= scale_v[c];  // world-space direction
          const double* rgb = cv_phase ? p->cv_rgb : p->iso_rgb;
          if (p->lighting) shade(p, g, d, L, rgb, col);
          else for (int c = 0; c < 3; ++c) col[c] = rgb[c];
          if (p->cv_on && cv_phase == 0) {
            const double gl = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
            const double nv = gl > 0 ? std::fabs(g[0] * d[0] + g[1] * d[1] + g[2] * d[2]) / gl : 1.0;
            double a = 1.0;
            if (cv_rho < 1.0) a = std::min(1.0, std::max(0.0, p->cv_border * cv_rho * cv_rho + p->cv_context * (1.0 - nv)));
            if (a < 1.0) {
              cv_a = a;
              for (int c = 0; c < 3; ++c) cv_c[c] = col[c];
              cv_phase = 1;
              --k;  // the focus surface may cross at this sample too
              continue;
            }
          } else if (p->cv_on) {
            for (int c = 0; c < 3; ++c) col[c] = cv_a * cv_c[c] + (1.0 - cv_a) * col[c];
          }
          for (int c = 0; c < 3; ++c) C[c] = col[c];
          A = 1.0;
          break;
        }
        prev_t = t;
        continue;
      }
      double c[4];
      double vn = (v - p->value_lo) * vscale;
      if (p->mode == 0) {
        tf1d_lookup(p, vn * (p->tf_w - 1), c);
      } else {
        double g[3];
        V.gradient(x[0], x[1], x[2], g);
        double gm = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) * vscale;
        tf2d_lookup(p, vn * (p->tf_w - 1), gm / p->grad_max * (p->tf_h - 1), c);
        if (p->lighting && c[3] > 0) {
          double lit[3], gw[3];
          for (int q = 0; q < 3; ++q) gw[q] = g[q] * scale_v[q];
          shade(p, gw, d, L, c, lit);
          c[0] = lit[0]; c[1] = lit[1]; c[2] = lit[2];
        }
      }
      double al = c[3];
      if (e != 1.0) al = 1.0 - std::pow(1.0 - al, e);
      double w = (1.0 - A) * al;
      C[0] += w * c[0];
      C[1] += w * c[1];
      C[2] += w * c[2];
      A += w;
      if (A >= p->ert) break;
    }
    if (cv_phase == 1 && A < 1.0) {
      // no focus surface behind the context surface
      for (int c = 0; c < 3; ++c) C[c] = cv_a * cv_c[c];
      A = cv_a;
    }
    if (p->mode == 3 && any) {
      // maximum-intensity projection: the maximum through the 1D TF, once
      double c[4];
      tf1d_lookup(p, (vmax - p->value_lo) * vscale * (p->tf_w - 1), c);
      for (int q = 0; q < 3; ++q) C[q] = c[q] * c[3];
      A = c[3];
    }
  }
  if (line != 0xffffffffu) {
    // the opaque line behind the volume's samples
    const double* lc = p->line_rgb[line & 1u];
    for (int k = 0; k < 3; ++k) out[k] = C[k] + (1.0 - A) * lc[k];
    out[3] = A + (1.0 - A);
  } else {
    double bg[3];
    bg_row(p, py, bg);
    for (int k = 0; k < 3; ++k) out[k] = C[k] + (1.0 - A) * bg[k];
    out[3] = A;
  }
  if (nsamples) *nsamples = ns;
}

// 2D slice view: framebuffer pixel -> point on the slice plane (the plane
// fills the image at its aspect ratio, centred; screen x = the lower-numbered
// in-plane axis, screen y = the higher one upwards; flips mirror them); the
// trilinear value at the slice's axis coordinate `coord` (level voxels), or
// with mip the maximum over the voxel centres along the axis, through the 1D
// TF over the background.  out: [height][width][4] doubles.
void orc_render_slice(const orc_render_params* p, int axis, double coord, int flip_x, int flip_y, int mip,
                      double* out) {
  Vol V{p};
  const int ua = axis == 0 ? 1 : 0, va = axis == 2 ? 1 : 2;
  const double eu = p->extent[ua], ev = p->extent[va];
  const double sc = std::min((double)p->width / eu, (double)p->height / ev);
  const double vscale = 1.0 / (p->value_hi - p->value_lo);
#pragma omp parallel for schedule(dynamic, 16)
  for (int py = 0; py < p->height; ++py)
    for (int px = 0; px < p->width; ++px) {
      double uw = (px + 0.5 - 0.5 * p->width) / sc, vw = (0.5 * p->height - (py + 0.5)) / sc;
      if (flip_x) uw = -uw;
      if (flip_y) vw = -vw;
      double* o = out + 4 * ((i64)py * p->width + px);
      double bg[3];
      bg_row(p, py, bg);
      o[0] = bg[0]; o[1] = bg[1]; o[2] = bg[2]; o[3] = 0.0;
      if (std::fabs(uw) > 0.5 * eu || std::fabs(vw) > 0.5 * ev) continue;
      double x[3];
      x[ua] = (uw + 0.5 * eu) * (double)p->dims[ua] / eu - 0.5;
      x[va] = (vw + 0.5 * ev) * (double)p->dims[va] / ev - 0.5;
      double v;
      if (!mip) {
        x[axis] = coord;
        v = V.sample(x[0], x[1], x[2]);
      } else {
        v = -std::numeric_limits<double>::infinity();
        for (i64 k = 0; k < p->dims[axis]; ++k) {
          x[axis] = (double)k;
          v = std::max(v, V.sample(x[0], x[1], x[2]));
        }
      }
      double c[4];
      tf1d_lookup(p, (v - p->value_lo) * vscale * (p->tf_w - 1), c);
      for (int q = 0; q < 3; ++q) o[q] = c[3] * c[q] + (1.0 - c[3]) * bg[q];
      o[3] = c[3];
    }
}

// Render `npix` pixels (indices into the width*height image, row 0 = top) or
// the whole image when pixels == null.  out: [npix][4] doubles.  Returns the
// number of samples taken.
i64 orc_render(const orc_render_params* pin, const int64_t* pixels, i64 npix, double* out, int threads) {
  orc_render_params pc = *pin;
  const orc_render_params* p = &pc;
  std::vector<uint32_t> keys;
  if (pc.bbox_global || pc.bbox_local) {
    line_keys(p, keys);
    pc.line_keys = keys.data();
  } else {
    pc.line_keys = nullptr;
  }
  i64 total = pixels ? npix : (i64)p->width * p->height;
  i64 ns_total = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : ns_total)
  for (i64 i = 0; i < total; ++i) {
    i64 pix = pixels ? pixels[i] : i;
    i64 ns = 0;
    render_pixel(p, (int)(pix % p->width), (int)(pix / p->width), out + 4 * i, &ns);
    ns_total += ns;
  }
  return ns_total;
}

// The per-pixel line keys alone (for the tests of the GPU rasteriser).
void orc_line_keys(const orc_render_params* p, uint32_t* out) {
  std::vector<uint32_t> keys;
  line_keys(p, keys);
  memcpy(out, keys.data(), sizeof(uint32_t) * keys.size());
}

// LZ4 block decoding, restated from the published block format (test
// oracle for the library's codec): sequences of a token (literal count in
// the high nibble, match length - 4 in the low one, 15 = continued by bytes
// added until one below 255), the literals, a 2-byte little-endian offset
// and the match; the last sequence carries literals only.  Returns the
// decoded size, or -1 when the block is malformed or exceeds out_n.
i64 orc_lz4_decompress(const uint8_t* in, i64 n, uint8_t* out, i64 out_n) {
  i64 ip = 0, op = 0;
  while (ip < n) {
    const int token = in[ip++];
    i64 lit = token >> 4;
    if (lit == 15) {
      int b;
      do {
        if (ip >= n) return -1;
        b = in[ip++];
        lit += b;
      } while (b == 255);
    }
    if (ip + lit > n || op + lit > out_n) return -1;
    for (i64 i = 0; i < lit; ++i) out[op++] = in[ip++];
    if (ip == n) return op;
    if (ip + 2 > n) return -1;
    const i64 off = in[ip] + 256 * (i64)in[ip + 1];
    ip += 2;
    i64 len = (token & 15);
    if (len == 15) {
      int b;
      do {
        if (ip >= n) return -1;
        b = in[ip++];
        len += b;
      } while (b == 255);
    }
    len += 4;
    if (off < 1 || off > op || op + len > out_n) return -1;
    for (i64 i = 0; i < len; ++i, ++op) out[op] = out[op - off];
  }
  return -1;  // a block ends with a literal-only sequence
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// ---------------------------------------------------------------------------
// 2D transfer-function rasterisation from .2dt swatches, restated from the
// editor's drawing (ImageVis3D/UI/Q2DTransferFunction.cpp:436-473 swatch
// fill with QLinearGradient / QRadialGradient, 1138-1153 the 1D TF image
// stretched underneath, 1182-1217 drawing order, 156-160 gradient 0 at the
// bottom).  Tuvok's own table renderer is not in the tree: parity of this
// rule with the reference is unpinned; the GPU rasteriser must equal it bit
// for bit (float arithmetic, the same operation order, no contraction).
// Swatch layout: radial, npoints, nstops, reserved (int32), points[128],
// grad[4], stops[80] (float), as gbvr_tf2d_swatch.
// ---------------------------------------------------------------------------
struct orc_swatch {
  int32_t radial, npoints, nstops, reserved;
  float points[128];
  float grad[4];
  float stops[80];
};

static bool sw_covers(const orc_swatch& s, float cx, float cy, float fw, float fh) {
  bool in = false;
  for (int i = 0, j = s.npoints - 1; i < s.npoints; j = i++) {
    const float xi = s.points[2 * i] * fw, yi = s.points[2 * i + 1] * fh;
    const float xj = s.points[2 * j] * fw, yj = s.points[2 * j + 1] * fh;
    if ((yi > cy) != (yj > cy)) {
      const float xc = xi + ((cy - yi) * (xj - xi)) / (yj - yi);
      if (cx < xc) in = !in;
    }
  }
  return in;
}

static float sw_pos(const orc_swatch& s, float cx, float cy, float fw, float fh) {
  const float g0x = s.grad[0] * fw, g0y = s.grad[1] * fh, g1x = s.grad[2] * fw, g1y = s.grad[3] * fh;
  const float qx = cx - g0x, qy = cy - g0y, dx = g1x - g0x, dy = g1y - g0y;
  const float dd = dx * dx + dy * dy;
  float t;
  if (s.radial) {
    const float r = std::sqrt(dd);
    const float d = std::sqrt(qx * qx + qy * qy);
    t = r > 0.f ? d / r : 1.f;
  } else {
    t = dd > 0.f ? (qx * dx + qy * dy) / dd : 0.f;
  }
  return std::min(std::max(t, 0.f), 1.f);
}

static void sw_colour(const orc_swatch& s, float t, float c[4]) {
  const int n = s.nstops;
  const float* st = s.stops;
  if (!(t > st[0]) || n == 1) {
    for (int k = 0; k < 4; ++k) c[k] = st[1 + k];
    return;
  }
  if (t >= st[5 * (n - 1)]) {
    for (int k = 0; k < 4; ++k) c[k] = st[5 * (n - 1) + 1 + k];
    return;
  }
  int i = 0;
  while (i + 2 < n && st[5 * (i + 1)] <= t) ++i;
  const float w = (t - st[5 * i]) / (st[5 * (i + 1)] - st[5 * i]);
  for (int k = 0; k < 4; ++k) {
    const float a = st[5 * i + 1 + k], b = st[5 * (i + 1) + 1 + k];
    c[k] = a + w * (b - a);
  }
}

void orc_raster_tf2d(const orc_swatch* sw, int ns, const float* tf1d, int n1d, int W, int H, float* out) {
  const float fw = (float)W, fh = (float)H;
  for (int r = 0; r < H; ++r)
    for (int x = 0; x < W; ++x) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      if (n1d > 0) {
        const i64 j = (i64)x * n1d / W;
        for (int k = 0; k < 4; ++k) d[k] = tf1d[4 * j + k];
      }
      const float cx = (float)x + 0.5f, cy = (float)(H - 1 - r) + 0.5f;
      for (int k = 0; k < ns; ++k) {
        if (!sw_covers(sw[k], cx, cy, fw, fh)) continue;
        float c[4];
        sw_colour(sw[k], sw_pos(sw[k], cx, cy, fw, fh), c);
        const float as = c[3];
        const float kd = d[3] * (1.f - as);
        const float a = as + kd;
        for (int j = 0; j < 3; ++j) d[j] = a > 0.f ? (c[j] * as + d[j] * kd) / a : 0.f;
        d[3] = a;
      }
      for (int k = 0; k < 4; ++k) out[4 * ((i64)r * W + x) + k] = d[k];
    }
}

// ---------------------------------------------------------------------------
// Cameras, restated in FP64 for the CPU reference arm and as an independent
// check of the library's camera code: the look-at view matrix and the OpenGL
// perspective projection (gluLookAt / gluPerspective, row-major, column
// vectors), and the orbit of the 360-degree capture
// (ImageVis3D/UI/ImageVis3D_Capturing.cpp:170: angle i / N * 360 about +y;
// RenderWindow.cpp:207-214) at an elevation above the xz plane, looking at
// the volume centre, clip planes one unit either side of the centre's depth.
// Results are rounded to float32 once, at the end.
// ---------------------------------------------------------------------------
static void cam_look_at(const double eye[3], const double at[3], const double up[3], double V[16]) {
  double fwd[3], side[3], upv[3];
  for (int i = 0; i < 3; ++i) fwd[i] = at[i] - eye[i];
  const double fn = std::sqrt(fwd[0] * fwd[0] + fwd[1] * fwd[1] + fwd[2] * fwd[2]);
  for (double& v : fwd) v /= fn;
  side[0] = fwd[1] * up[2] - fwd[2] * up[1];
  side[1] = fwd[2] * up[0] - fwd[0] * up[2];
  side[2] = fwd[0] * up[1] - fwd[1] * up[0];
  const double sn = std::sqrt(side[0] * side[0] + side[1] * side[1] + side[2] * side[2]);
  for (double& v : side) v /= sn;
  upv[0] = side[1] * fwd[2] - side[2] * fwd[1];
  upv[1] = side[2] * fwd[0] - side[0] * fwd[2];
  upv[2] = side[0] * fwd[1] - side[1] * fwd[0];
  const double* axes[3] = {side, upv, fwd};
  for (int r = 0; r < 3; ++r) {
    const double sg = r == 2 ? -1.0 : 1.0;  // the camera looks down -z
    double dot = 0.0;
    for (int k = 0; k < 3; ++k) {
      V[4 * r + k] = sg * axes[r][k];
      dot += V[4 * r + k] * eye[k];
    }
    V[4 * r + 3] = -dot;
  }
  V[12] = V[13] = V[14] = 0.0;
  V[15] = 1.0;
}

static void cam_perspective(double fovy_deg, double aspect, double zn, double zf, double P[16]) {
  const double f = 1.0 / std::tan(fovy_deg * M_PI / 360.0);
  for (int i = 0; i < 16; ++i) P[i] = 0.0;
  P[0] = f / aspect;
  P[5] = f;
  P[10] = (zf + zn) / (zn - zf);
  P[11] = 2.0 * zf * zn / (zn - zf);
  P[14] = -1.0;
}

void orc_orbit_camera(double az_deg, double el_deg, double radius, double fov_deg, int w, int h, float view[16],
                      float proj[16]) {
  const double az = az_deg * M_PI / 180.0, el = el_deg * M_PI / 180.0;
  const double eye[3] = {radius * std::cos(el) * std::sin(az), radius * std::sin(el),
                         radius * std::cos(el) * std::cos(az)};
  const double at[3] = {0.0, 0.0, 0.0}, up[3] = {0.0, 1.0, 0.0};
  double V[16], P[16];
  cam_look_at(eye, at, up, V);
  cam_perspective(fov_deg, (double)w / (double)h, std::max(0.01, radius - 2.0), radius + 2.0, P);
  for (int i = 0; i < 16; ++i) {
    view[i] = (float)V[i];
    proj[i] = (float)P[i];
  }
}

void orc_look_at_camera(const double eye[3], const double at[3], const double up[3], double fov_deg, double zn,
                        double zf, int w, int h, float view[16], float proj[16]) {
  double V[16], P[16];
  cam_look_at(eye, at, up, V);
  cam_perspective(fov_deg, (double)w / (double)h, zn, zf, P);
  for (int i = 0; i < 16; ++i) {
    view[i] = (float)V[i];
    proj[i] = (float)P[i];
  }
}

// ---------------------------------------------------------------------------
// The CPU UVF build of a flat level-0 volume, timed phase by phase for the
// CPU baseline: the LOD pyramid (orc_downsample), every level's bricks with
// ghosts (orc_extract_brick) and their min/max, the 1D histogram and the 2D
// histogram -- the converter's sequence (UVFReader/DataSource.h:475-616) on
// `threads` OpenMP threads (bricks in parallel; the histograms as written
// above).  phase_s[4]: pyramid, bricks + min/max, hist1d, hist2d seconds.
// Returns the total seconds.
// ---------------------------------------------------------------------------
double orc_uvf_build_timed(const void* vol, int dt, const i64 dims[3], int brick, int ghost, int threads,
                           double* phase_s) {
#ifdef _OPENMP
  const int saved = omp_get_max_threads();
  omp_set_num_threads(threads > 0 ? threads : saved);
#endif
  auto now = [] {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
  };
  const size_t es = dt_size(dt);
  i64 ld[16 * 3];
  const int nl = orc_lod_dims(dims, brick, ghost, 0, ld);
  std::vector<std::vector<char>> lv(nl);
  double t0 = now();
  for (int l = 1; l < nl; ++l) {
    lv[l].resize((size_t)ld[3 * l] * ld[3 * l + 1] * ld[3 * l + 2] * es);
    orc_downsample(l == 1 ? vol : lv[l - 1].data(), dt, ld + 3 * (l - 1), lv[l].data());
  }
  double t1 = now();
  double sink = 0.0;
  for (int l = 0; l < nl; ++l) {
    const void* src = l == 0 ? vol : lv[l].data();
    i64 nb[3], I;
    orc_brick_grid(ld + 3 * l, brick, ghost, nb, &I);
    const i64 n = nb[0] * nb[1] * nb[2];
#pragma omp parallel reduction(+ : sink)
    {
      std::vector<char> buf;
#pragma omp for schedule(dynamic, 1)
      for (i64 i = 0; i < n; ++i) {
        const i64 b[3] = {i % nb[0], (i / nb[0]) % nb[1], i / (nb[0] * nb[1])};
        i64 o[3], sd[3];
        orc_brick_extent(ld + 3 * l, brick, ghost, b, o, sd);
        buf.resize((size_t)sd[0] * sd[1] * sd[2] * es);
        orc_extract_brick(src, dt, ld + 3 * l, brick, ghost, b, buf.data());
        double mn, mx;
        orc_minmax(buf.data(), dt, sd[0] * sd[1] * sd[2], &mn, &mx);
        sink += mn + mx;
      }
    }
  }
  double t2 = now();
  std::vector<u64> h1(65536);
  i64 merge = 1, nx = 1;
  if (dt != DT_F32) nx = orc_hist1d(vol, dt, dims[0] * dims[1] * dims[2], 4096, h1.data(), &merge);
  double t3 = now();
  if (dt != DT_F32) {
    double mn, mx;
    orc_minmax(vol, dt, dims[0] * dims[1] * dims[2], &mn, &mx);
    std::vector<u64> h2((size_t)nx * 256);
    orc_hist2d(vol, dt, dims, mx, nx, merge, h2.data());
  }
  double t4 = now();
#ifdef _OPENMP
  omp_set_num_threads(saved);
#endif
  phase_s[0] = t1 - t0;
  phase_s[1] = t2 - t1;
  phase_s[2] = t3 - t2;
  phase_s[3] = t4 - t3;
  return (t4 - t0) + 0.0 * sink;
}

}  // extern "C"
