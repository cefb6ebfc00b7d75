// Internal structures shared by the host runtime and the CUDA kernels.
//
// Data layout in HBM (one dataset):
//   pool      one device allocation holding every brick of every LOD level,
//             each brick a dense x-fastest block of its stored voxels
//             (interior + up to `ghost` voxels copied from each neighbour),
//             starting on a 256-byte boundary.
//   bricks    BrickInfo[total bricks], level-major, then z, y, x brick order.
//   skip      one byte per brick, recomputed by the classify kernel whenever
//             the transfer function, render mode or isovalue changes.
//   frames    FrameDesc[n] for the views rendered by one launch.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace gbvr {

enum DType { DT_U8 = 0, DT_U16 = 1, DT_F32 = 2 };
enum Mode { MODE_1D = 0, MODE_2D = 1, MODE_ISO = 2, MODE_MIP = 3 };
enum Sampler { SAMPLER_SW = 0, SAMPLER_TEX = 1 };

inline size_t dtype_size(int dt) { return dt == DT_U8 ? 1 : dt == DT_U16 ? 2 : 4; }

// One stored brick.  All coordinates are voxel indices of its LOD level.
struct __align__(16) BrickInfo {
  unsigned long long offset;  // element offset of voxel (0,0,0) in the pool
  unsigned long long tex;     // cudaTextureObject_t when the texture sampler is built
  int ox, oy, oz;             // level coordinate of stored voxel (0,0,0)
  int sx, sy, sz;             // stored dims
  int lox, loy, loz;          // interior [lo, hi): a sample whose floor(pos) lies
  int hix, hiy, hiz;          //   here is taken from this brick (lo = -1 on the low face)
  float vmin, vmax;           // over the stored voxels, ghosts included
  // Layout copies: the pool may hold the same bricks up to three times, with
  // x, y or z as the fastest axis; a view samples the copy whose fastest
  // axis is closest to its screen x axis so a warp's rays coalesce.
  int level;
  int pad;
};

struct LevelInfo {
  int dims[3];
  int nb[3];
  int interior;
  int brick_base;  // index of the level's first brick
};

// Everything one view needs; read by every warp working on one of its tiles.
struct __align__(16) FrameDesc {
  // dataset
  const void* pool;
  const BrickInfo* bricks;   // the rendered level's bricks
  const unsigned char* skip; // skip flags of the rendered level's bricks
  int dtype;
  int sampler;
  int dims[3];               // rendered level
  int nb[3];
  int interior;
  float inv_interior;        // 1 / interior (estimate of the brick column, settled exactly)
  float vox_scale[3];        // world -> voxel-centre coordinates: (p + extent/2) * scale - 0.5
  float half_extent[3];
  // classification
  const float4* tf;          // 1D: [tf_w]; 2D: [tf_h][tf_w]
  int tf_w, tf_h;
  int mode;
  int interp;
  float value_lo;
  float idx_scale;           // (tf_w - 1) / (value_hi - value_lo)
  float grad_scale;          // 2D: (tf_h - 1) / (grad_max * (value_hi - value_lo))
  const unsigned char* tf_col_live;  // 2D: per value column, 1 if any gradient row has opacity (or null)
  float dt;                  // step, world units
  float opacity_exp;         // dt / dt0 = 1 / samples_per_voxel
  float ert;
  float iso;
  float iso_rgb[3];
  int lighting;
  float amb[3], diff[3], spec[3];
  float shininess;
  float light_to[3];         // unit vector towards the light, world space
  float bg[3];               // background; with bg_grad the bottom edge's colour
  float bg_top[3];           // bg_grad: the top edge's colour (setBGColors' top)
  int bg_grad;               // 1: vertical gradient from bg_top (top edge) to bg (bottom edge)
  // camera
  float inv_vp[16];          // row-major inverse of proj*view
  int width, height;
  int tiles_x, tiles_y;
  // the view's ray tiles that can meet the volume: tx0 .. tx0 + ntx - 1 by
  // ty0 .. ty0 + nty - 1 (the whole frame unless a batch culls it); pixels
  // outside hold the background
  int tx0, ty0, ntx, nty;
  // empty-space skipping: 0 none, 1 whole bricks, 2 bricks and macro-cells
  int empty_skip;
  const unsigned char* occ; // per macro-cell: capped distance (cells) to one that may contribute
  int nc[3];                 // macro-cell grid of the level
  int cell_shift;            // macro-cell edge = 1 << cell_shift voxels
  const float2* cells;       // MIP: per macro-cell min/max of the level (footprint + 1 voxel)
  const float* smax;         // MIP: per super-cell (4^3 macro-cells) the largest cell maximum, or null
  int nsc[3];                // super-cell grid
  float level_max;           // MIP: largest voxel of the level; no sample exceeds it
  int clip_on;               // clip plane: samples with clip . (x, y, z, 1) > 0 are dropped
  float clip[4];
  // bounding-box lines: per pixel the key of the nearest covering line (see
  // line_key), then the ray parameter where that line ends the ray (float
  // bits, bit 0 = colour), or 0xffffffff; null when no lines are drawn.  Per
  // view.
  const unsigned* lines;
  float line_rgb[2][3];      // colour of the global box (key bit 0 = 0) and of the brick boxes (1)
  // ClearView (isosurface mode, the lens pass only): the focus surface's
  // iso value and colour, the context and border scales of the context
  // surface's opacity
  float cv_iso, cv_rgb[3], cv_context, cv_border;
  int tile_w;                // ray tile of one warp: tile_w x (32 / tile_w) pixels
  int perm;                  // brick layout copy: 0 x-fastest, 1 y-fastest, 2 z-fastest, 3 4^3 blocks
  unsigned long long copy_off;  // element offset of that copy in the pool
  // outputs
  uchar4* out_rgba8;         // may be null
  float4* out_f32;           // may be null
  unsigned long long* samples;  // per-frame sample counter
  unsigned char* touched;    // per-frame flag per brick of the rendered level
  unsigned* cell_touched;    // per-frame bitmap of sampled non-empty macro-cells (or null)
  // batch-uniform descriptors only: view v's flags start at touched +
  // v * touched_stride (cell_touched likewise); 0 in per-view descriptors
  long long touched_stride, cell_touched_stride;
};

// Bounding-box lines (setGlobalBBox / setLocalBBox).  Segments in world
// coordinates; a pixel is covered by a segment when its centre lies within
// half a pixel of the segment's projection (clipped to the near plane).  The
// covered point's NDC depth z varies linearly along the projected segment.
// Key = bits of the float (z + 2) with bit 0 replaced by the colour index, so
// the smallest key is the nearest line, and of two lines at one depth the
// global box wins.
struct LineSeg {
  double a[3], b[3];
  int color;  // 0 global box, 1 brick box
  int pad;
};
struct LineView {
  float view[16], proj[16];  // row-major, column vectors (as gbvr_view)
  int width, height;
  unsigned* keys;            // width * height, 0xffffffff where no line
};

__host__ __device__ inline unsigned line_key(float z_plus_2, int color) {
  unsigned u;
  memcpy(&u, &z_plus_2, 4);
  return (u & ~1u) | (unsigned)color;
}
__host__ __device__ inline float line_ndc_z(unsigned key) {
  const unsigned u = key & ~1u;
  float z;
  memcpy(&z, &u, 4);
  return z - 2.f;
}

// A 2D slice view: screen pixels map to the plane through the slice (or to
// rays along its axis for MIP).
struct SliceDesc {
  int axis;            // 0 x (sagittal), 1 y (axial), 2 z (coronal)
  float coord;         // level voxel coordinate of the slice along `axis`
  float inv_s;         // world units per pixel
  float half_w, half_h;  // framebuffer half size, pixels
  float ext_u, ext_v;  // world extents of the in-plane axes (u = lower-numbered, v = higher)
  float scale_u, scale_v;  // level voxels per world unit along u, v
  int flip_x, flip_y, mip;
  int use_skip;        // out of core: a brick flagged in f.skip (empty under the TF, or not resident) is background
};

// Default ray tile handled by one warp: 8 x 4 pixels.
constexpr int TILE_W = 8;

// ---- launch wrappers (kernels_render.cu) ----
// Classification of value ranges against the transfer function.  tf_prefix
// holds tf_w + 1 counts: tf_prefix[i] = number of TF columns j < i with a
// non-zero alpha (in any row of a 2D TF).  Writes 1 = may contribute.
cudaError_t launch_classify_bricks(const BrickInfo* bricks, int nbricks, const int* tf_prefix, int tf_w,
                                   int mode, float value_lo, float idx_scale, float iso,
                                   unsigned char* skip, cudaStream_t s);
// Turn occ (1 = may contribute) into the capped Chebyshev distance to the
// nearest such cell, in place (tmp: scratch of the same size).
cudaError_t launch_cell_distance(unsigned char* occ, unsigned char* tmp, const int nc[3], int cap, cudaStream_t s);
cudaError_t launch_classify_cells(const float2* cells, long long ncells, const int* tf_prefix, int tf_w,
                                  int mode, float value_lo, float idx_scale, float iso,
                                  unsigned char* occ, cudaStream_t s);
cudaError_t launch_render_plain(const FrameDesc& f, cudaStream_t s);
// popcount of n_frames bitmaps of `words` words each into counts[n_frames]
cudaError_t launch_count_bits(const unsigned* bits, long long words, int n_frames, unsigned long long* counts,
                              cudaStream_t s);
// tile_prefix[0..nframes]: the first tile of each frame and, last, the total;
// the kernels read the total from device memory, so a graph replay takes the
// count of the descriptors uploaded before it
cudaError_t launch_render_persistent_typed(int dtype, int mode, int sampler, const FrameDesc* frames,
                                           int nframes, const int* tile_prefix, int* counter, int grid,
                                           cudaStream_t s);
int persistent_grid_size(int device, int mode);
// One (voxel type, mode) group of a serving batch: frames [first, first +
// count) of the batch's descriptor array, tile prefix at prefix_at.
struct LaunchGroup {
  int first, count, prefix_at, pad;
};
cudaError_t launch_render_persistent_group(int dtype, int mode, const FrameDesc* frames, const LaunchGroup* groups,
                                           int gi, const int* prefix, int* counters, int grid, cudaStream_t s);
int persistent_group_ctas_per_sm(int mode);
// Background (RGBA = bg, 0) into every pixel of each frame outside its tile
// rectangle, as a ray that misses the volume leaves it.
// (frames of different sizes: max_height is the tallest; each block checks its frame's size)
cudaError_t launch_fill_outside(const FrameDesc* frames, int nframes, int max_height, cudaStream_t s);
cudaError_t launch_fill_outside_one(const FrameDesc& f, cudaStream_t s);
// Batches whose views share everything but camera, light direction, outputs
// and counters: the shared part travels as a kernel parameter (constant
// bank), each view's part is read from `frames` (camera, light direction,
// outputs, sample counter).
// sps: samples per step of the inner loop (2 only for the 1D TF with the
// software sampler; otherwise 1)
cudaError_t launch_render_persistent_uniform(int dtype, int mode, int sampler, const FrameDesc& shared,
                                             const FrameDesc* frames, int nframes, const int* prefix, int* counter,
                                             int grid, cudaStream_t s, int sps = 1);
int persistent_ctas_per_sm_sps2();
int persistent_grid_size_uniform(int device, int mode);
cudaError_t launch_render_slice(const FrameDesc& f, const SliceDesc& sd, cudaStream_t s);
// then, for frames [frame0, frame0 + n) of `frames` (device), each covered
// pixel's key <- the ray parameter where its ray ends (float bits; bit 0
// keeps the colour), and the pixel (frame << 32 | pixel) is appended to list
// (*count entries, zeroed beforehand)
cudaError_t launch_line_stops(const FrameDesc* frames, int frame0, int nframes, int max_height,
                              unsigned long long* list, unsigned* count, cudaStream_t s);
// after the frames' render: re-render the listed pixels with the ray ending
// at the line and the line behind (grid-stride over *count)
cudaError_t launch_render_lines(int dtype, int mode, int sampler, const FrameDesc* frames,
                                const unsigned long long* list, const unsigned* count, int grid, cudaStream_t s);
// ClearView lens: the pixel rectangle [x0, x1) x [y0, y1) around the focus
// point (fx, fy) (pixels, row 0 = top) and the lens radius in pixels
struct CvLens {
  int x0, y0, x1, y1;
  float fx, fy, radius;
};
cudaError_t launch_render_cv(const FrameDesc& f, const CvLens& L, cudaStream_t s);
// keys of every view (set to 0xffffffff beforehand) <- the nearest covering line
cudaError_t launch_raster_lines(const LineSeg* segs, int nseg, const LineView* views, int nviews, cudaStream_t s);

// ---- launch wrappers (kernels_build.cu) ----
struct BlobTablesDev {
  int nblobs;
  const float* amp;
  const float* ex;
  const float* ey;
  const float* ez;
  const float* bgx;
  const float* bgy;
  const float* bgz;
  float bg_level, bg_amp, scale, noise_amp;
  int noise_kind;
  float vmax;
  uint32_t seed;
};
cudaError_t launch_synth_blobs(const BlobTablesDev& t, const long long dims[3], int dtype, void* out,
                               cudaStream_t s);
// planes [z0, z0 + nz) of the volume into out (nz planes)
cudaError_t launch_synth_blobs_planes(const BlobTablesDev& t, const long long dims[3], int dtype, long long z0,
                                      long long nz, void* out, cudaStream_t s);
cudaError_t launch_synth_fbm(const long long dims[3], int dtype, uint32_t seed, int octaves, int base_period,
                             float thr, float vmax, void* out, cudaStream_t s);
cudaError_t launch_downsample(const void* in, int dtype, const long long dims[3], void* out,
                              cudaStream_t s);
// perm: 0 stores x fastest, 1 y fastest (then z, x), 2 z fastest (then x, y),
// 3 in 4x4x4 blocks of 64 contiguous voxels (x fastest within and between blocks)
cudaError_t launch_gather_bricks(const void* level, int dtype, const long long dims[3],
                                 const BrickInfo* bricks_dev, int nbricks, void* pool,
                                 int perm, cudaStream_t s);
// bricks from a window of the level holding planes vz0.. (their stored boxes,
// clamped to the level, must lie in the window)
// The flat level back from the interiors of its bricks (x-fastest copy).
cudaError_t launch_scatter_interiors(const void* pool, int dtype, const BrickInfo* bricks, int nbricks,
                                     const long long dims[3], void* level, cudaStream_t s);
cudaError_t launch_gather_bricks_window(const void* level, int dtype, const long long dims[3], long long vz0,
                                        const BrickInfo* bricks_dev, int nbricks, void* pool, int perm,
                                        cudaStream_t s);
cudaError_t launch_brick_minmax(const void* pool, int dtype, BrickInfo* bricks_dev, int nbricks,
                                cudaStream_t s);
// In one pass over a whole level: its bricks into the x-fastest copy (pool0),
// into the 4x4x4-blocked copy when pool1 is not null (the same offsets), and
// each brick's vmin / vmax (which must be +inf / -inf on entry).  max_sz: the
// largest stored z extent of the bricks.
cudaError_t launch_gather_fused(const void* level, int dtype, const long long dims[3], BrickInfo* bricks_dev,
                                int nbricks, int max_sz, void* pool0, void* pool1, cudaStream_t s);
// Macro-cell min/max of a flat level: cell c covers sample cells [c M, c M + M)
// per axis, whose trilinear footprints span voxels [c M, c M + M]; the range
// is taken over [c M - 1, c M + M + 1] (clamped) so that a sample rounded
// across a cell face is still covered.
cudaError_t launch_cell_minmax(const void* level, int dtype, const long long dims[3], int cell_shift,
                               const int nc[3], float2* out, cudaStream_t s);
// cell layers [cz0, cz1) from a window of the level holding planes vz0.. (the
// layers' footprints must lie in the window)
cudaError_t launch_cell_minmax_layers(const void* level, int dtype, const long long dims[3], long long vz0,
                                      int cell_shift, const int nc[3], int cz0, int cz1, float2* out, cudaStream_t s);
// Super-cells of 4^3 macro-cells (clamped at the grid's end): the largest
// cell maximum of each, out[(sz nsc1 + sy) nsc0 + sx].
constexpr int SUPERCELL_SHIFT = 2;
cudaError_t launch_supercell_max(const float2* cells, const int nc[3], float* out, const int nsc[3], cudaStream_t s);
cudaError_t launch_hist1d(const void* vol, int dtype, long long n, unsigned long long* hist,
                          int nbins, cudaStream_t s);
// 2D histogram passes; scratch holds the pass-1 reduction state.
struct Hist2DScratch {
  unsigned long long smax;      // max integer squared central-difference sum
  unsigned long long gmax_bits; // max f64 |grad| among voxels attaining smax
};
// narrow: 16-bit data known to lie below 16384 (gradient sums in 32 bits)
cudaError_t launch_hist2d(const void* vol, int dtype, const long long dims[3], double max_scalar,
                          long long nx, long long merge, unsigned long long* hist,
                          Hist2DScratch* scratch, cudaStream_t s, bool narrow = false);
// LZ4-compressed brick chunks to decode on the device: the compressed bytes
// at stage + src (comp bytes; bit 31 set: stored uncompressed) become raw
// bytes at pool + dst.
struct Lz4Chunk {
  unsigned long long src, dst;
  unsigned comp, raw;
};
// one warp per chunk; a malformed chunk sets *err (nonzero) and is left partly written
cudaError_t launch_lz4_decode(const void* stage, void* pool, const Lz4Chunk* chunks, int nchunks, int* err,
                              cudaStream_t s);

// zlib-compressed chunks (the same table; comp bit 31: stored raw): one warp
// per chunk; a malformed chunk or a wrong Adler-32 sets *err (nonzero)
cudaError_t launch_inflate(const void* stage, void* pool, const Lz4Chunk* chunks, int nchunks, int* err,
                           cudaStream_t s);

// One of the three passes (1: Smax, 2: f64 max |grad| at Smax, 3: binning)
// over the planes [zb, ze) of a volume streamed in z: `slab` holds planes
// zlo .. (zlo <= zb - 1 unless zb = 0, and plane ze unless ze = Z).  The
// scratch is zeroed once before the first slab of pass 1; every slab of a
// pass before the next pass.
cudaError_t launch_hist2d_slab(const void* slab, int dtype, const long long dims[3], long long zb, long long ze,
                               long long zlo, double max_scalar, long long nx, long long merge, int pass,
                               unsigned long long* hist, Hist2DScratch* scratch, cudaStream_t s);

}  // namespace gbvr
