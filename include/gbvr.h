/*
 * gbvr.h - C ABI of the GB300-native bricked volume raycaster and UVF builder.
 *
 * This is the drop-in boundary for ImageVis3D's raycast path.  The reference
 * reaches its renderer through Tuvok's AbstrRenderer, created by
 * `tuvok.renderer.new` and driven by Lua method calls (the sequence in
 * LuaScripts/BatchRenderer.lua:22-41); each entry point below names the call
 * it replaces.  Conventions:
 *   - every function returns GBVR_OK (0) or a negative GBVR_E* status; the
 *     message of the last failure on the calling thread is returned by
 *     gbvr_last_error().  No C++ exception crosses this boundary.
 *   - handles are opaque; host buffers are owned by the caller; device memory
 *     is owned by the library.
 *   - one renderer per host thread; calls on one renderer are not reentrant
 *     (as paint is not, ImageVis3D/UI/RenderWindow.cpp:2455-2458).
 *   - matrices are row-major float[16] acting on column vectors (p' = M p),
 *     OpenGL clip conventions (near plane at z_ndc = -1).
 *   - volumes are x-fastest; dims[0] = x.  dtype: GBVR_U8, GBVR_U16, GBVR_F32.
 */
#ifndef GBVR_H
#define GBVR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBVR_OK 0
#define GBVR_EINVAL (-1)      /* invalid argument */
#define GBVR_ECUDA (-2)       /* CUDA runtime error */
#define GBVR_ENOMEM (-3)      /* device or pinned allocation failed */
#define GBVR_EIO (-4)         /* file could not be read or written */
#define GBVR_EFORMAT (-5)     /* malformed or unsupported UVF content */
#define GBVR_ECHECKSUM (-6)   /* UVF checksum mismatch */
#define GBVR_ESTATE (-7)      /* call out of order (e.g. paint before load) */
#define GBVR_EOVERSIZED (-8)  /* brick larger than the device limit */
#define GBVR_ETIMEOUT (-9)    /* a wait ran out of time */

#define GBVR_U8 0
#define GBVR_U16 1
#define GBVR_F32 2

/* Renderer types.  Tuvok's MasterController::EVolumeRendererType ordinals are
 * persisted as integers (ImageVis3D/UI/ImageVis3D_Settings.cpp:480; names at
 * ImageVis3D/UI/RenderWindowGL.cpp:176-188 and SettingsDlg.cpp:486-515), so
 * the new type is appended after them and none is renumbered. */
#define GBVR_OPENGL_SBVR 0
#define GBVR_OPENGL_RAYCASTER 1
#define GBVR_DIRECTX_SBVR 2
#define GBVR_DIRECTX_RAYCASTER 3
#define GBVR_OPENGL_2DSBVR 4
#define GBVR_DIRECTX_2DSBVR 5
#define GBVR_OPENGL_GRIDLEAPER 6
#define GBVR_DIRECTX_GRIDLEAPER 7
#define GBVR_OPENGL_CHOOSE 8
#define GBVR_CUDA_RAYCASTER 9 /* this library; the only type it creates */

/* Render modes (AbstrRenderer::ERenderMode, RenderWindow.cpp:2051-2059). */
#define GBVR_RM_1DTRANS 0
#define GBVR_RM_2DTRANS 1
#define GBVR_RM_ISOSURFACE 2
/* Maximum-intensity projection: the largest sample along the ray through the
 * 1D TF, composited once over the background.  Tuvok has no such render
 * mode: MIP is a property of its 2D render regions (setUseMIP,
 * RenderWindow.cpp:286-289; CaptureMIPFrame, :1690-1713); here it takes any
 * camera, e.g. an orthographic one along a slice axis. */
#define GBVR_RM_MIP 3

/* Interpolants (RenderWindow.cpp:437-446, ImageVis3D.cpp:881-888). */
#define GBVR_NEAREST 0
#define GBVR_LINEAR 1

/* Trilinear sampler: FP32 software interpolation or texture hardware. */
#define GBVR_SAMPLER_SW 0
#define GBVR_SAMPLER_TEX 1

/* gbvr_create flags */
#define GBVR_FLAG_FLOAT_FB 1u /* also keep float RGBA framebuffers (for error measurement) */

typedef struct gbvr_renderer gbvr_renderer;

typedef struct gbvr_brick_params {
  int32_t brick_size;   /* largest stored brick edge incl. ghosts (uvfconvert
                           -bricksize, CmdLineConverter/main.cpp:172-174) */
  int32_t overlap;      /* ghost voxels per face (DEFAULT_BRICKOVERLAP = 2,
                           CmdLineConverter/main.cpp:145) */
  int32_t max_lods;     /* 0 = halve until one brick holds the level */
  int32_t build_texture;/* also build 3D textures for GBVR_SAMPLER_TEX */
  int32_t layouts;      /* 1: bricks stored x-fastest only; 3: also y- and z-fastest
                           copies (3x device memory), each view samples the copy
                           whose fastest axis is closest to its screen x axis;
                           4: also a copy in 4x4x4 voxel blocks (2x memory),
                           sampled by every view; 5: the blocks of that copy
                           also hold their +1 neighbours (5x5x5 voxels in 128
                           elements, 3x memory), so a trilinear footprint is
                           read at fixed offsets from one address; 6: both
                           blocked copies (4x memory), isosurfaces sampled from
                           the overlapped one, the other modes from the other */
  int32_t compression;  /* out-of-core host store: 0 raw, 1 zlib, 3 LZ4 (the UVF codec ids
                           CT_ZLIB and CT_LZ4, UVFReader/BlockInfo.h:60-93; zlib is the
                           converter's default, CmdLineConverter/main.cpp:146): 16 KiB chunks
                           compressed by host threads at build, decoded on the GPU when paged */
  int32_t brick_order;  /* out-of-core host store: order of the bricks of each level (the
                           converter's -bricklayout, CmdLineConverter/main.cpp:175-178): 0
                           scanline (brick index), 1 Morton, 2 Hilbert, 3 random (seeded);
                           a paint copies each stretch of adjacent missing bricks at once */
  int32_t reserved;     /* 0 */
  double aspect[3];     /* voxel spacing; 0 = (1,1,1) */
} gbvr_brick_params;

typedef struct gbvr_dataset_info {
  int64_t dims[3];
  int32_t dtype;
  int32_t bit_width;      /* getBitWidth (ImageVis3D_WindowHandling.cpp:862-946) */
  double range[2];        /* getRange: global min / max of LOD 0 */
  int32_t lod_count;      /* getLODLevelCount */
  int32_t brick_size, overlap;
  int64_t lod_dims[16][3];/* getDomainSize(lod) */
  int32_t lod_bricks[16][3];
  int64_t total_bricks;
  uint64_t device_bytes;  /* bytes of the brick pool (sum of stored bricks) */
  int32_t hist1d_size;    /* bins of the 1D histogram (<= 4096) */
  float hist2d_max_grad;  /* max gradient magnitude of the 2D histogram */
  uint64_t host_bytes;    /* out of core: bytes of the page-locked host brick store */
  int32_t device_slots;   /* out of core: bricks the device pool holds at once */
  int32_t compression;    /* out of core: the store's codec (0 raw, 1 zlib, 3 LZ4) */
  uint64_t host_raw_bytes;/* out of core: the store's bytes uncompressed */
} gbvr_dataset_info;

/* One view of a batch: camera, output size and (optionally) its own TF. */
typedef struct gbvr_view {
  float view[16];
  float proj[16];
} gbvr_view;

typedef struct gbvr_stats {
  uint64_t frames;             /* views rendered by the last paint call */
  uint64_t samples;            /* volume samples evaluated (all views) */
  uint64_t bricks_touched;     /* sum over views of distinct non-skipped bricks sampled */
  uint64_t bricks_skipped;     /* bricks of the rendered level classified empty */
  uint64_t brick_bytes;        /* sum over views of stored bytes of touched bricks */
  uint64_t brick_misses;       /* bricks not resident when requested */
  uint64_t bytes_paged;        /* host->device brick bytes of the last paint */
  uint64_t h2d_bytes;          /* host->device bytes copied by the last paint (view descriptors) */
  int32_t lod;                 /* level rendered (getMinLODIndex) */
  int32_t subframes;           /* getCurrentSubFrameCount: always 1 */
  double gpu_ms;               /* device time of the last paint (CUDA events) */
  double kernel_ms;            /* device time of its raycast kernel launch(es) alone */
  uint64_t cells_touched;      /* stats level 2: sum over views of distinct non-empty macro-cells sampled */
  uint64_t cell_bytes;         /* ... times the cell's voxel bytes (4^3 voxels) */
  double page_ms;              /* out of core: device time of the last paint's brick uploads */
  uint64_t bytes_paged_compressed; /* out of core, compressed store: host->device bytes of those bricks */
  uint64_t host_copies;        /* out of core: host->device copies that brought those bricks */
} gbvr_stats;

/* ---- brick orders (the converter's -bricklayout, CmdLineConverter/main.cpp:175-178) ----
 * gbvr_brick_order: the bricks of an nb[0] x nb[1] x nb[2] grid (index
 * (z ny + y) nx + x) in storage order for order 0 scanline, 1 Morton, 2 Hilbert
 * (positions along the curve of the enclosing power-of-two cube), 3 random
 * (seeded): perm[k] = the brick stored k-th.  gbvr_hilbert3: the position of
 * (x, y, z) along the 3D Hilbert curve of a 2^bits cube. */
int gbvr_brick_order(const int32_t nb[3], int32_t order, uint64_t seed, int32_t* perm, size_t n);
uint64_t gbvr_hilbert3(uint32_t x, uint32_t y, uint32_t z, int32_t bits);

/* ---- errors / device ---- */
int gbvr_last_error(char* buf, size_t size);
int gbvr_device_info(int* sm_count, size_t* free_bytes, size_t* total_bytes);

/* ---- renderer lifetime ----
 * gbvr_create replaces tuvok.renderer.new(type, pow2, 8bit, noBorder, biasTF)
 *   (LuaScripts/BatchRenderer.lua:22, ImageVis3D/UI/RenderWindowGL.cpp:97-100);
 *   only GBVR_CUDA_RAYCASTER is accepted.  flags are reserved (0).
 * gbvr_destroy replaces renderer.cleanup() + deleteClass (BatchRenderer.lua:40-41,
 *   RenderWindow.cpp:1591-1603). */
int gbvr_create(int renderer_type, uint32_t flags, gbvr_renderer** out);
int gbvr_destroy(gbvr_renderer* r);

/* ---- datasets ----
 * gbvr_load_uvf replaces renderer.loadDataset(path) (BatchRenderer.lua:25,
 *   RenderWindowGL.cpp:111): reads a UVF v2/v3 file (raster data block,
 *   histograms, min/max), verifies its MD5 unless verify == 0
 *   (ImageVis3D_FileHandling.cpp:567-585), and bricks it on the device.
 * gbvr_load_volume takes a flat host volume and runs the GPU UVF build
 *   (bricks + LOD pyramid + min/max + histograms) into the device pool,
 *   replacing tuvok.io.convertDataset (ImageVis3D_FileHandling.cpp:609-611)
 *   followed by loadDataset.
 * gbvr_load_synthetic generates a seeded volume directly on the device (see
 *   gbvr_synth_params) and builds it the same way. */
int gbvr_load_uvf(gbvr_renderer* r, const char* path, int verify, const gbvr_brick_params* bp);
int gbvr_load_volume(gbvr_renderer* r, const void* host, const int64_t dims[3], int dtype,
                     const gbvr_brick_params* bp);
int gbvr_get_dataset_info(gbvr_renderer* r, gbvr_dataset_info* info);
/* getHistogram / get2DHistogram (ImageVis3D_WindowHandling.cpp:880-946) */
int gbvr_get_hist1d(gbvr_renderer* r, uint64_t* out, size_t n);
int gbvr_get_hist2d(gbvr_renderer* r, uint64_t* out, size_t nx, size_t ny, float* max_grad);
/* per-brick min/max of one level in brick order (MaxMinDataBlock) */
int gbvr_get_brick_minmax(gbvr_renderer* r, int lod, double* out_minmax, size_t nbricks);
/* the macro-cell min/max grid of a level (the empty-space skipping structure
 * inside bricks): cell (cx, cy, cz) of edge M voxels (4 in core, 8 out of
 * core) holds the min and max of the voxels [c M - 1, c M + M + 1] per axis
 * (clamped to the level), at out_minmax[2 ((cz ny + cy) nx + cx)]; nc
 * receives (nx, ny, nz) and cell_edge M.  ncells: capacity in cells. */
int gbvr_get_cell_minmax(gbvr_renderer* r, int lod, float* out_minmax, size_t ncells, int32_t nc[3],
                         int32_t* cell_edge);
/* copy one stored brick (interior + ghosts) back to the host */
int gbvr_get_brick(gbvr_renderer* r, int lod, const int32_t brick[3], void* out, size_t bytes,
                   int64_t origin[3], int64_t stored_dims[3]);
/* write the loaded dataset as a UVF v2 file (raster + 1D/2D histogram + min/max
 * + key/value blocks, MD5 checksum), the sequence of UVFReader/DataSource.h:453-667 */
int gbvr_write_uvf(gbvr_renderer* r, const char* path);

/* ---- render state (setters of RenderWindow.h:77-314) ---- */
int gbvr_resize(gbvr_renderer* r, int width, int height);                 /* resize(UINTVECTOR2) */
int gbvr_set_render_mode(gbvr_renderer* r, int mode);                     /* setRenderMode */
int gbvr_set_tf1d(gbvr_renderer* r, const float* rgba, int n);            /* changed1DTrans */
int gbvr_set_tf2d(gbvr_renderer* r, const float* rgba, int w, int h, float max_grad); /* changed2DTrans */
/* A camera path (the fly-through animator's frames, LuaScripts/FlyThroughAnimator.lua, painted one by one
 * in the reference) in one call: frame i into framebuffer i (read them with gbvr_read_framebuffers).  Out of
 * core every frame renders at the finest level whose bricks fit the device pool, as gbvr_paint does, and
 * the bricks of frame i + 1 are paged in on a copy stream while frame i renders.  Per frame (optional arrays
 * of n entries): the level rendered, the bricks missed at the target level, the bytes paged in.  In-core
 * datasets render the frames one after the other.  gbvr_get_stats then reports the whole path. */
int gbvr_paint_path(gbvr_renderer* r, const gbvr_view* views, int n, int32_t* lod, uint64_t* misses,
                    uint64_t* bytes_paged);
/* The same path with every frame captured (the capture sequence of ImageVis3D_Capturing.cpp:63-96 and
 * RenderWindow.cpp:1718-1725, one image per frame): frame i's RGBA8 pixels (rows top first, as
 * gbvr_read_framebuffers gives them) go to rgba8 + i * width * height * 4 as soon as frame i is done, on a
 * copy stream of their own, while the following frames page and render; returns when every frame is in
 * host memory.  rgba8 must hold n frames (bytes >= n * width * height * 4); page-locked memory lets the
 * copies overlap the path. */
int gbvr_paint_path_capture(gbvr_renderer* r, const gbvr_view* views, int n, int32_t* lod, uint64_t* misses,
                            uint64_t* bytes_paged, uint8_t* rgba8, size_t bytes);

/* 2D render region (tuvok.renderRegion2D.new(mode, sliceIndex, renderer), setSliceDepth, set2DFlipMode,
 * setUseMIP: RenderWindow.cpp:1548-1571, 235-239, 270-289) into framebuffer 0.  axis = the window mode:
 * 0 sagittal (x), 1 axial (y), 2 coronal (z), as the reference indexes getDomainSize() by it; index = the
 * slice in voxels of the finest level, rendered at the LOD limit's level.  The slice fills the framebuffer
 * at its aspect ratio, centred, background around it; screen x follows the lower-numbered in-plane axis,
 * screen y the higher one upwards; flip_x / flip_y mirror them.  Each pixel: the trilinear value at the
 * slice through the 1D TF over the background.  use_mip: the maximum along the axis instead (maximum-
 * intensity projection of the whole volume).  Out of core, the bricks the slice needs are paged in first
 * (every brick for use_mip), on a coarser level when they do not fit the device slots. */
int gbvr_paint_slice(gbvr_renderer* r, int axis, int64_t index, int flip_x, int flip_y, int use_mip);
/* setClipPlane / setClipPlaneEnabled (RenderWindow.cpp:1920-1927, RenderWindow.h:131,168): samples at world
 * points p (the normalised volume box) with plane[0..2] . p + plane[3] > 0 are dropped; enabled = 0 turns the
 * plane off (plane may then be NULL). */
int gbvr_set_clip_plane(gbvr_renderer* r, int enabled, const float plane[4]);
/* setGlobalBBox / setLocalBBox (RenderWindow.cpp:2208-2225, RenderWindow.h:165-166): global draws the 12
 * edges of the dataset box, local the lines of the rendered level's brick grid (brick interior bounds).
 * Lines are opaque, one pixel wide (a pixel whose centre lies within half a pixel of a line's projection,
 * after clipping to the near plane), at their depth: the volume in front of a line composites over it, and
 * the line replaces the background behind the ray (alpha 1).  Of two lines at one depth the global box
 * wins.  rgb may be NULL (keep; defaults: global (1, 1, 1), local (0.6, 0.6, 0.6)).  3D views only. */
int gbvr_set_bboxes(gbvr_renderer* r, int global, int local, const float global_rgb[3], const float local_rgb[3]);
/* ClearView (setCV, setCVIsoValue, setCVColor, setCVSize, setCVContextScale, setCVBorderScale, setCVFocusPos:
 * RenderWindow.cpp:2155-2206,2337-2367; the focus-and-context technique of Krueger, Schneider and Westermann,
 * IEEE Vis 2006), isosurface mode only.  The first hit of the iso value (gbvr_set_iso) is the context
 * surface, the first hit of `iso` behind it the focus surface (colour rgb, shaded alike).  Inside the lens,
 * a circle of radius size * min(width, height) / 2 pixels around the focus point (focus_x, focus_y in pixels,
 * row 0 = top), the context surface gets opacity a = clamp(context_scale (1 - |n.v|) + border_scale rho^2,
 * 0, 1) (n its normal, v the view direction, rho the distance to the focus point over the radius) and is
 * composited over the focus surface (or the background); elsewhere it is opaque.  Rays that meet no
 * context surface show the background, as in isosurface mode.  rgb may be NULL (keep). */
int gbvr_set_clearview(gbvr_renderer* r, int enabled, float iso, const float rgb[3], float size, float context_scale,
                       float border_scale, float focus_x, float focus_y);
int gbvr_set_value_range(gbvr_renderer* r, double lo, double hi);         /* TF domain (biasScaleTF) */
int gbvr_set_iso(gbvr_renderer* r, float value, const float rgb[3]);      /* setIsoValue, setIsosurfaceColor */
/* setIsoValueRelative (RenderWindow.cpp:2144-2153): iso = clamp(fraction, 0, 1) x the integer top of the
 * value range (the TF domain's upper end), as the script command maps it (ImageVis3D.cpp:478-484).  Needs a
 * loaded dataset. */
int gbvr_set_iso_relative(gbvr_renderer* r, float fraction, const float rgb[3]);
/* setBlendPrecision (RenderWindow.cpp:1618-1623): 8, 16 or 32 bits; this renderer composites in FP32 for
 * every setting (the value is recorded and returned by nothing else). */
int gbvr_set_blend_precision(gbvr_renderer* r, int bits);
int gbvr_set_lighting(gbvr_renderer* r, int enabled, const float amb[4], const float diff[4],
                      const float spec[4], const float dir[3]);          /* setLightingEnabled, setLightColors */
int gbvr_set_sample_rate(gbvr_renderer* r, float samples_per_voxel);      /* setSampleRateModifier */
int gbvr_set_interpolant(gbvr_renderer* r, int interp);                   /* setInterpolant */
int gbvr_set_sampler(gbvr_renderer* r, int sampler);                      /* SW or texture trilinear */
int gbvr_set_lod_limits(gbvr_renderer* r, int min_lod, int max_lod);      /* setLODLimits */
int gbvr_set_view(gbvr_renderer* r, const float view[16], const float proj[16]); /* setRotation4x4/... */
int gbvr_set_background(gbvr_renderer* r, const float top[3], const float bottom[3]); /* setBGColors */
int gbvr_set_early_termination(gbvr_renderer* r, float alpha);           /* 0.99 by default */
/* Launch shape of the raycast kernels: a warp renders tile_w x (32 / tile_w)
 * pixels (tile_w in 4, 8, 16, 32); ctas_per_sm sizes the persistent grid as
 * SMs x ctas_per_sm (0 = as many as fit).  No counterpart in the reference
 * (GL rasterisation chose its own fragment order). */
int gbvr_set_launch_shape(gbvr_renderer* r, int tile_w, int ctas_per_sm);

/* Empty-space skipping: 0 none (every sample is evaluated), 1 whole bricks
 * classified empty by their min/max against the TF, 2 (default) also
 * 4^3-voxel macro-cells inside bricks (jumping whole empty cubes by a
 * distance field over them), the finer acceleration grid of the
 * reference's GridLeaper renderer type (RenderWindowGL.cpp:176-188).  All
 * three give identical pixels: a skipped region contributes exactly zero. */
int gbvr_set_empty_skipping(gbvr_renderer* r, int mode);

typedef struct gbvr_tune_result {
  int32_t tile_w;
  int32_t ctas_per_sm;
  int32_t candidates;
  float best_ms;        /* kernel time of the chosen shape on the tuning batch */
  float default_ms;     /* kernel time of the default shape (8, 0) */
} gbvr_tune_result;

/* Autotuner: times every candidate launch shape on `views` with the batched
 * kernel (after one warm-up each), keeps the fastest and returns the result.
 * The frame content does not depend on the shape (rays are independent). */
int gbvr_autotune(gbvr_renderer* r, const gbvr_view* views, int n, gbvr_tune_result* out);

/* Samples per step of the batched kernel's inner loop (1D TF, software
 * sampler): 1 (default), 2, 4 or 8.  With 2 each lane evaluates two
 * consecutive samples of its ray per step -- both samples' voxel and TF loads
 * in flight together.  With 4 or 8 the warp shares the work: each lane still
 * walks its own ray and composites its own samples, but the pending samples of
 * all the warp's rays (up to 4 or 8 per ray per step) are evaluated by the
 * whole warp, 32 at a time.  Every setting composites the same samples in the
 * same order and stops at the same one: the same pixels.  No counterpart in
 * the reference. */
int gbvr_set_samples_per_step(gbvr_renderer* r, int sps);

/* Extended autotuner: the launch-shape sweep of gbvr_autotune (tile width x
 * CTAs per SM) for every brick size in brick_sizes (the dataset is rebuilt at
 * each from its finest level: same pixels, other bricks; the uvfconvert
 * -bricksize setting, CmdLineConverter/main.cpp:172-174, and the max brick
 * size of ImageVis3D/UI/ImageVis3D_Settings.cpp:516-520) and every value in
 * samples_per_step (gbvr_set_samples_per_step).  The fastest combination on
 * `views` stays set (the dataset left at its brick size).  Zero entries end
 * each list; an empty list keeps the current setting.  In-core datasets only. */
typedef struct gbvr_tune_params {
  int32_t brick_sizes[4];
  int32_t samples_per_step[4];
} gbvr_tune_params;

typedef struct gbvr_tune_result_ex {
  int32_t tile_w, ctas_per_sm, brick_size, samples_per_step;
  int32_t candidates;
  float best_ms;     /* kernel time of the chosen combination on the tuning batch */
  float default_ms;  /* ... of the settings at the call (tile 8, CTAs as fit, 1 sample per step, its brick size) */
  float worst_ms;    /* ... of the slowest candidate */
} gbvr_tune_result_ex;

int gbvr_autotune_ex(gbvr_renderer* r, const gbvr_view* views, int n, const gbvr_tune_params* p,
                     gbvr_tune_result_ex* out);

/* ---- paint ----
 * gbvr_paint replaces renderer.paint() (BatchRenderer.lua:35,
 *   RenderWindow.cpp:2464): one plain launch for the current view.
 * gbvr_paint_batch renders n views of the loaded dataset in one persistent
 *   launch over a shared ray-tile queue (CUDA-graph replayed when the batch
 *   shape repeats); framebuffer i holds view i.  This is the batched form of
 *   the 360-degree capture loop (ImageVis3D_Capturing.cpp:159-202).
 * gbvr_paint_views renders the same n views with n plain launches, the
 *   per-view form timed beside the batch. */
int gbvr_paint(gbvr_renderer* r);
int gbvr_paint_batch(gbvr_renderer* r, const gbvr_view* views, int n);
int gbvr_paint_views(gbvr_renderer* r, const gbvr_view* views, int n);

/* ---- asynchronous batches (a pipeline of steps; no counterpart in the reference, whose paint is
 * synchronous) ----
 * gbvr_paint_batch_async renders n views into framebuffer set `slot` (0 or 1, in-core datasets) and returns
 * once the work is queued.  gbvr_read_framebuffers_async copies views of a set into host memory
 * (page-locked for a true overlap) after that set's render, on its own stream, so the read-back of one step
 * overlaps the render of the next; a set is rendered again only after its read-back.  gbvr_wait_read
 * returns once every read-back queued for `slot` has landed in host memory (the render queued since keeps
 * running); gbvr_wait_async waits for everything queued.  The synchronous calls first let queued work
 * finish, then render into and read the set selected last (set 0 until an asynchronous batch picks 1). */
int gbvr_paint_batch_async(gbvr_renderer* r, const gbvr_view* views, int n, int slot);
int gbvr_read_framebuffers_async(gbvr_renderer* r, int slot, int first, int n, void* host, size_t bytes);
int gbvr_wait_read(gbvr_renderer* r, int slot);
int gbvr_wait_async(gbvr_renderer* r);

/* ---- readback (captureSingleFrame, RenderWindow.cpp:1642-1671; RGBA8 model
 * StandaloneTuvok/CmdRenderer.cpp:34-56).  Row 0 is the top image row. ---- */
int gbvr_read_framebuffer(gbvr_renderer* r, int view, uint8_t* rgba8, size_t bytes);
int gbvr_read_framebuffer_f32(gbvr_renderer* r, int view, float* rgba, size_t bytes);
/* views [first, first + n) of the last paint in one copy: n x height x width
 * RGBA8, view-major.  Faster into page-locked host memory. */
int gbvr_read_framebuffers(gbvr_renderer* r, int first, int n, uint8_t* rgba8, size_t bytes);
int gbvr_capture_single_frame(gbvr_renderer* r, const char* path, int preserve_transparency);
/* capture view i of the last paint (the capture-sequence frames of
 * ImageVis3D_Capturing.cpp:188 / RenderWindow.cpp:1718-1725) */
int gbvr_capture_view(gbvr_renderer* r, int view, const char* path, int preserve_transparency);
int gbvr_get_stats(gbvr_renderer* r, gbvr_stats* out);
/* What paint records for gbvr_get_stats: 0 sample counts only, 1 (default)
 * also the bricks each view touched, 2 also the macro-cells each view
 * sampled (a bitmap per view; costs an atomic per new cell). */
int gbvr_set_stats_level(gbvr_renderer* r, int level);

/* ---- seeded synthetic volumes ----
 * Sum of isotropic Gaussian blobs (+ optional low-frequency background and
 * uniform or Irwin-Hall Gaussian noise), drawn with Philox4x32-10 from seed;
 * the volume kinds of the UVFReader generator (UVFReader/DataSource.h:335-396)
 * re-specified so CPU and GPU agree bit for bit. */
typedef struct gbvr_synth_params {
  int64_t dims[3];
  int32_t dtype;
  uint32_t seed;
  int32_t nblobs;
  float sigma_lo, sigma_hi;    /* voxels */
  float amp_lo, amp_hi;
  float bg_freq;               /* 0 = no background */
  float bg_level, bg_amp;
  float scale;                 /* value = scale * (background + blobs) + noise */
  int32_t noise_kind;          /* 0 none, 1 uniform +-noise_amp, 2 Gaussian sigma noise_amp */
  float noise_amp;
  float vmax;                  /* integer types clamp to [0, vmax] */
} gbvr_synth_params;

int gbvr_synth_volume(const gbvr_synth_params* p, void* host_out, size_t bytes);
/* Out of core (the reference's GPU-memory-capped brick cache, GPUMemMan with
 * MaxGPUMem, ImageVis3D_Settings.cpp:509-514): the seeded volume is generated
 * and bricked on the device in z-slabs straight into a page-locked host
 * brick store (all LOD levels, same bricks as the in-core build), and the
 * device keeps at most device_pool_bytes of bricks.  Each paint pages in the
 * bricks its views need (non-empty under the TF, inside a view frustum) on a
 * side stream, evicting least-recently-used ones; when they do not fit, the
 * paint falls back to the finest coarser level that fits.  gbvr_get_stats
 * reports the level used, brick misses, bytes paged and their device time.
 * The 2D histogram is not built out of core (max gradient 0). */
int gbvr_load_synthetic_ooc(gbvr_renderer* r, const gbvr_synth_params* p, const gbvr_brick_params* bp,
                            uint64_t device_pool_bytes);
int gbvr_load_synthetic(gbvr_renderer* r, const gbvr_synth_params* p, const gbvr_brick_params* bp);

/* Seeded fractal volume: `octaves` octaves of periodic value noise (lattice
 * of base_period << o cells per axis at octave o, hashed lattice values,
 * smoothstep trilinear, weight 2^-o), normalised to [0, 1], then
 * v = clamp((f - threshold) / (1 - threshold), 0, 1) * vmax: sparse
 * structures in empty space. */
typedef struct gbvr_fbm_params {
  int64_t dims[3];
  int32_t dtype;
  uint32_t seed;
  int32_t octaves;
  int32_t base_period;
  float threshold;
  float vmax;
} gbvr_fbm_params;

int gbvr_synth_fbm_volume(const gbvr_fbm_params* p, void* host_out, size_t bytes);
int gbvr_load_synthetic_fbm(gbvr_renderer* r, const gbvr_fbm_params* p, const gbvr_brick_params* bp);

/* Device time and bytes of the last in-core UVF build of a renderer's dataset
 * (gbvr_load_volume, gbvr_load_synthetic, gbvr_load_uvf), phase by phase:
 * the work of TOCBlock::FlatDataToBrickedLOD and the histogram blocks
 * (UVFReader/DataSource.h:475-500, 601-616), timed with CUDA events around
 * each phase's launches.  Synthesis, host uploads and texture building are
 * not part of it.  bytes = what each phase must read and write at least:
 * pyramid: every level read once and the next written; cells: every level
 * read; bricks: every level read once for the x-fastest and 4x4x4-blocked
 * copies (written together, with each brick's min/max reduced on the way,
 * so minmax is 0 ms and 0 bytes) and once more per other copy, plus every
 * stored brick written per copy (twice its size for the overlapped blocks);
 * hist1d: level 0 read;
 * hist2d: level 0 read twice (the largest squared gradient, then the bins;
 * the f64 maximum-gradient pass between them revisits only the voxels that
 * attain it). */
typedef struct gbvr_build_stats {
  double total_ms;
  double pyramid_ms, cells_ms, bricks_ms, minmax_ms, hist1d_ms, hist2d_ms;
  uint64_t total_bytes;
  uint64_t pyramid_bytes, cells_bytes, bricks_bytes, minmax_bytes, hist1d_bytes, hist2d_bytes;
  uint64_t level0_bytes;   /* bytes of the finest level */
  int32_t lod_count;
  int32_t layout_copies;
} gbvr_build_stats;
int gbvr_get_build_stats(gbvr_renderer* r, gbvr_build_stats* out);

/* ---- GPU UVF build without a renderer (uvfconvert, CmdLineConverter/main.cpp:406-408):
 * host volume in, UVF v2 file out. ---- */
int gbvr_build_uvf(const void* host, const int64_t dims[3], int dtype, const gbvr_brick_params* bp,
                   const char* out_path);

/* ---- device-resident build kernels, for callers that keep volumes in HBM.
 * Pointers are device pointers; sizes are elements. ---- */
int gbvr_dev_hist1d(const void* dev_vol, int dtype, int64_t n, uint64_t* dev_hist, int nbins,
                    void* stream);
int gbvr_dev_hist2d(const void* dev_vol, int dtype, const int64_t dims[3], double max_scalar,
                    int64_t nx, int64_t merge, uint64_t* dev_hist, float* max_grad, void* stream);
int gbvr_dev_downsample(const void* dev_in, int dtype, const int64_t dims[3], void* dev_out,
                        void* stream);

/* ---- seeded synthesis into caller-owned device memory, allocating nothing.
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they call: a host application that owns the GPU memory budget
 * and hands out only pre-allocated buffers, or code issuing work beside other
 * streams, where cudaFree (and often cudaMalloc) would synchronise the whole
 * device.  Same volume as gbvr_synth_volume, written to dev_out (a device
 * pointer of at least X*Y*Z*element bytes) on `stream` (a cudaStream_t, or
 * null for the default stream); the call returns once the work is queued.
 * The generator's tables go through a fixed device array of
 * GBVR_NOALLOC_SYNTH_MAX_FLOATS floats (1 MiB, held on every GPU that loads
 * the library until the process exits): parameters needing more than
 * nblobs * (1 + X + Y + Z) + X + Y + Z <= that many floats are rejected with
 * GBVR_EINVAL.  The first call on a device sets the array up there (it loads
 * the library's device code and resolves the array's address), so make one
 * call on each device before any stream capture.  All calls share the array:
 * calls that overlap on the GPU (different streams, no ordering) race. */
#define GBVR_NOALLOC_SYNTH_MAX_FLOATS 262144
int gbvr_dev_synth_volume_noalloc(const gbvr_synth_params* p, void* dev_out, size_t bytes, void* stream);

/* ---- serving (continuous batching) ----
 * A server keeps many datasets and transfer-function presets and renders
 * requests submitted from any thread.  A worker thread keeps up to `slots`
 * batches in flight, each on its own CUDA stream: whenever a slot is free and
 * requests are pending it launches a batch of them at once, so batches
 * overlap on the device (a new batch's ray tiles fill the SMs that earlier
 * batches' tails leave idle).  A batch takes pending requests in arrival
 * order until it holds max_batch of them or its framebuffer share
 * (fb_budget_bytes / slots) is full.  Its requests are grouped by (voxel
 * type, render mode); each group is one persistent launch over the group's
 * ray tiles, replayed from a CUDA graph, with the group's launch shape from
 * gbvr_server_autotune.  Admission by memory: with device_pool_bytes > 0 the
 * datasets' brick pools share that budget; a request whose dataset is not
 * resident waits until its pool fits (idle datasets are evicted, least
 * recently used first, and the pool is uploaded from page-locked host memory
 * ahead of the batch), while requests for resident datasets go ahead.  A
 * request's image does not depend on the batch it lands in.  No counterpart
 * in the reference (its GUI renders one window per paint,
 * ImageVis3D/UI/RenderWindow.cpp:2453-2502). */
typedef struct gbvr_server gbvr_server;

typedef struct gbvr_server_params {
  int32_t max_batch;          /* requests per batch (0 = 64) */
  int32_t tile_w;             /* default warp tile width (0 = 8) */
  uint64_t fb_budget_bytes;   /* device + pinned framebuffer memory, shared by the slots (0 = 2 GiB) */
  int32_t slots;              /* batches in flight, one stream each (0 = 3; at most 8) */
  int32_t reserved;
  uint64_t device_pool_bytes; /* brick-pool memory the datasets share (0 = no limit: all stay resident) */
} gbvr_server_params;

typedef struct gbvr_request {
  int32_t dataset;            /* id from gbvr_server_add_* */
  int32_t tf;                 /* id from gbvr_server_add_tf (of that dataset) */
  int32_t width, height;
  float view[16], proj[16];
  float samples_per_voxel;    /* 0 = 1 */
  int32_t reserved;
  uint8_t* out_rgba8;         /* caller's host buffer, width*height*4 bytes, valid until waited for */
} gbvr_request;

typedef struct gbvr_request_result {
  int32_t status;
  int32_t batch_size;         /* requests in the batch that rendered it */
  uint64_t batch;
  double latency_ms;          /* submit to completion (host clock) */
  double queue_ms;            /* submit to launch */
  double gpu_ms;              /* device time of its batch */
} gbvr_request_result;

typedef struct gbvr_server_stats {
  uint64_t submitted, completed, batches;
  double mean_batch;
  double p50_ms, p99_ms, max_ms;  /* request latency percentiles */
  double frames_per_s;            /* completed requests / (last completion - first submit) */
  uint64_t overlap_checked;       /* pairs of consecutive batches whose kernel spans were compared */
  uint64_t overlapped;            /* ... of which the later batch's kernels started before the earlier's ended */
  uint64_t uploads, evictions;    /* brick pools made resident / evicted under device_pool_bytes */
  uint64_t upload_bytes;
  uint64_t resident_bytes;        /* brick-pool bytes resident now */
} gbvr_server_stats;

int gbvr_server_create(const gbvr_server_params* params, gbvr_server** out);
int gbvr_server_destroy(gbvr_server* s);
int gbvr_server_add_volume(gbvr_server* s, const void* host, const int64_t dims[3], int dtype,
                           const gbvr_brick_params* bp, int* dataset_id);
int gbvr_server_add_synthetic(gbvr_server* s, const gbvr_synth_params* p, const gbvr_brick_params* bp,
                              int* dataset_id);
/* A transfer-function preset of one dataset, classified once for empty-space
 * skipping: mode GBVR_RM_1DTRANS (w entries, h ignored), GBVR_RM_2DTRANS
 * (w x h, grad_max as gbvr_set_tf2d) or GBVR_RM_ISOSURFACE (rgba may be null;
 * iso, iso_rgb).  [lo, hi] is the value range mapped onto the TF (hi <= lo:
 * the dataset's default). */
int gbvr_server_add_tf(gbvr_server* s, int dataset, int mode, const float* rgba, int w, int h, float grad_max,
                       float iso, const float iso_rgb[3], double lo, double hi, int* tf_id);
/* Fails with GBVR_EINVAL for a request that can never be admitted (unknown
 * ids, a framebuffer above the slot's share, a brick pool above
 * device_pool_bytes). */
int gbvr_server_submit(gbvr_server* s, const gbvr_request* req, uint64_t* ticket);
/* Blocks until the request is done (timeout_s <= 0: no limit; GBVR_ETIMEOUT
 * when it runs out, the ticket then stays valid); its pixels are then in
 * req.out_rgba8.  A ticket can be waited for once. */
int gbvr_server_wait(gbvr_server* s, uint64_t ticket, double timeout_s, gbvr_request_result* out);
int gbvr_server_get_stats(gbvr_server* s, gbvr_server_stats* out);
int gbvr_server_reset_stats(gbvr_server* s);

/* Launch shape of one (voxel type, render mode) group of the server. */
typedef struct gbvr_server_tune {
  int32_t dtype, mode;
  int32_t tile_w, ctas_per_sm;  /* chosen */
  int32_t candidates;
  float best_ms, default_ms;    /* kernel time of the tuning batch: chosen shape, default shape */
} gbvr_server_tune;

/* Autotuner of the serving launches: for every (voxel type, mode) group that
 * has a transfer-function preset, renders a batch of `n` requests of
 * width x height (orbit cameras around one dataset of the group, its presets
 * in turn) with every candidate tile width and CTAs-per-SM, keeps the
 * fastest, and writes one entry per group to out (up to cap; count to
 * *n_out).  Waits for the batches in flight first; requests submitted
 * meanwhile wait.  The pixels do not depend on the shape. */
int gbvr_server_autotune(gbvr_server* s, int width, int height, int n, gbvr_server_tune* out, int cap, int* n_out);

/* Orbit camera around the volume centre: the rotation the 360-degree capture
 * applies per frame (ImageVis3D_Capturing.cpp:170 fAngle = i/N * 360,
 * RenderWindow.cpp:207-214 RotationY).  Eye at radius (world units, the
 * largest volume axis spans 1), azimuth about +y, elevation above the xz
 * plane, looking at the origin with +y up; perspective fov_deg vertical. */
int gbvr_orbit_camera(float azimuth_deg, float elevation_deg, float radius, float fov_deg, int width,
                      int height, float view[16], float proj[16]);

/* ---- transfer-function files (host only) ----
 * .1dt: first token N, then N lines "r g b a" (DemoData/c60.1dt), the format
 * TransferFunction1D::Load reads (Q1DTransferFunction.cpp:573-588).  With
 * target_size > 0 the table is resampled linearly to that many entries (as
 * loadFromFileWithSize does for the dataset's histogram size); 0 keeps N.
 * Writes at most `capacity` entries and the count to *n_out. */
int gbvr_load_tf1d_file(const char* path, int target_size, float* rgba_out, int capacity, int* n_out);

/* .2dt (DemoData/c60.2dt; TransferFunction2D::Load / Save, reached through
 * Q2DTransferFunction::LoadFromFile, Q2DTransferFunction.cpp:1234-1261):
 * "W H", the embedded 1D TF (N, then N lines "r g b a"), the swatch count,
 * then per swatch: the radial flag, the vertex count, one "x y" line per
 * vertex, the gradient end points "x0 y0 x1 y1", the stop count and one
 * "pos r g b a" line per stop.  Coordinates are normalised to the editor
 * canvas: x = value, y from the top (maximum gradient magnitude) down to 1
 * (gradient magnitude 0). */
#define GBVR_TF2D_MAX_POINTS 64
#define GBVR_TF2D_MAX_STOPS 16
typedef struct gbvr_tf2d_swatch {
  int32_t radial;  /* 0: linear gradient from grad[0..1] to grad[2..3]; 1: radial around grad[0..1] */
  int32_t npoints; /* polygon vertices, 3 .. GBVR_TF2D_MAX_POINTS */
  int32_t nstops;  /* gradient stops, 1 .. GBVR_TF2D_MAX_STOPS, increasing positions */
  int32_t reserved;
  float points[2 * GBVR_TF2D_MAX_POINTS]; /* x0 y0 x1 y1 ... */
  float grad[4];
  float stops[5 * GBVR_TF2D_MAX_STOPS]; /* pos r g b a ... */
} gbvr_tf2d_swatch;

/* Parse a .2dt file (host only).  Writes the canvas size, up to tf1d_cap
 * entries of the embedded 1D TF (count to *tf1d_n) and up to swatch_cap
 * swatches (count to *nswatches).  Output pointers may be NULL (with cap 0)
 * to query the counts. */
int gbvr_load_tf2d_file(const char* path, int* width, int* height, float* tf1d, int tf1d_cap, int* tf1d_n,
                        gbvr_tf2d_swatch* swatches, int swatch_cap, int* nswatches);

/* Rasterise swatches into a width x height RGBA float table on the GPU (the
 * step Tuvok's TransferFunction2D performs before changed2DTrans; the editor
 * draws it the same way, Q2DTransferFunction.cpp:436-473,1138-1153,
 * 1182-1217): every entry starts as the 1D TF entry of its column
 * (floor(x * tf1d_n / width)), then each swatch in order is composited over
 * it ("source over", non-premultiplied RGBA) where the entry's centre lies
 * inside the polygon (even-odd rule), with the colour of the gradient at the
 * centre (position clamped to [0, 1], linear between stops).  Row r of the
 * table is gradient bin r, i.e. canvas y = 1 - (r + 0.5) / height.  With no
 * 1D TF (tf1d_n = 0) the table starts transparent black.  out_rgba: host,
 * width * height * 4 floats. */
int gbvr_tf2d_rasterize(const gbvr_tf2d_swatch* swatches, int nswatches, const float* tf1d, int tf1d_n, int width,
                        int height, float* out_rgba);

/* changed2DTrans from a file: parse, rasterise on the GPU at the file's canvas
 * size and set the result as the renderer's 2D TF (gbvr_set_tf2d). */
int gbvr_set_tf2d_file(gbvr_renderer* r, const char* path, float max_grad);

/* Camera at `eye` looking at `ref` with up vector `up` (world units, the
 * largest volume axis spans 1), perspective fov_deg vertical, clip planes
 * znear / zfar: the keyframe camera of the fly-through animator
 * (LuaScripts/FlyThroughAnimator.lua: eye, ref, vup). */
int gbvr_look_at_camera(const float eye[3], const float ref[3], const float up[3], float fov_deg, float znear,
                        float zfar, int width, int height, float view[16], float proj[16]);

/* ---- host-only UVF inspection (the UVFReader tool, UVFReader/main.cpp:23-205,
 * UVFReader/BlockInfo.h:27-401).  No GPU is used. ---- */
typedef struct gbvr_uvf_summary {
  uint64_t version;
  uint64_t checksum_semantic;  /* 0 none, 1 crc32, 2 MD5 */
  uint8_t checksum[16];
  int32_t checksum_verified;   /* 1 when verify was requested and matched */
  int32_t nblocks;
  uint64_t block_semantics[32];
  int64_t dims[3];
  int32_t dtype;
  int32_t lod_count;
  int64_t brick_size[3];
  int64_t overlap[3];          /* as stored: 2 x ghost voxels */
  uint64_t data_offset;        /* file offset of the voxels */
  int64_t hist1d_size;
  int64_t hist2d_nx, hist2d_ny;
  float hist2d_max_grad;
  int64_t minmax_count;
  double minmax_first[4];      /* min, max, min gradient, max gradient of brick 0 */
} gbvr_uvf_summary;

int gbvr_uvf_inspect(const char* path, int verify, gbvr_uvf_summary* out);
int gbvr_uvf_read_volume(const char* path, void* out, size_t bytes);
int gbvr_uvf_read_hist1d(const char* path, uint64_t* out, size_t n);
int gbvr_uvf_read_hist2d(const char* path, uint64_t* out, size_t n, float* max_grad);
/* Write a single-brick, single-LOD UVF v2 file from host arrays: raster block
 * `raster_id`, then the given 1D / 2D histograms and min/max entries (each
 * may be empty), MD5 over bytes 49..end.  This is the layout of c60.uvf. */
int gbvr_uvf_write_raster(const char* path, const char* raster_id, const void* voxels,
                          const int64_t dims[3], int dtype, int32_t brick_size, int32_t overlap,
                          const uint64_t* hist1d, size_t n1, const uint64_t* hist2d, size_t nx,
                          size_t ny, float max_grad, const double* minmax, size_t nminmax);

/* ---- LZ4 block codec (UVF brick compression id 3, CT_LZ4: UVFReader/BlockInfo.h:60-93), host side.  The
 * out-of-core brick store compresses with it (gbvr_brick_params.compression) and the GPU decodes paged
 * bricks.  gbvr_lz4_compress returns the compressed size (0: does not fit in cap); gbvr_lz4_decompress
 * decodes into exactly out_n bytes (GBVR_EFORMAT when malformed). ---- */
size_t gbvr_lz4_bound(size_t n);
size_t gbvr_lz4_compress(const void* src, size_t n, void* dst, size_t cap);
int gbvr_lz4_decompress(const void* src, size_t n, void* dst, size_t out_n);

/* ---- zlib streams (RFC 1950) of DEFLATE data (RFC 1951): UVF brick compression id 1, CT_ZLIB
 * (UVFReader/BlockInfo.h:60-93), the converter's default (CmdLineConverter/main.cpp:146).  The
 * out-of-core brick store compresses with it when gbvr_brick_params.compression = 1 and the GPU
 * decodes paged bricks.  gbvr_zlib_compress writes one zlib stream (dynamic Huffman blocks, or stored
 * blocks where smaller) and returns its size (0: does not fit cap); gbvr_zlib_decompress decodes any
 * zlib stream (stored, fixed and dynamic blocks) into exactly out_n bytes, checking its Adler-32
 * (GBVR_EFORMAT when malformed).  Host only. ---- */
size_t gbvr_zlib_bound(size_t n);
size_t gbvr_zlib_compress(const void* src, size_t n, void* dst, size_t cap);
int gbvr_zlib_decompress(const void* src, size_t n, void* dst, size_t out_n);

/* One chunk of a batch of zlib streams for the GPU decoder: the stream at byte
 * src of the source buffer, decoded to `raw` bytes at byte dst of the output
 * buffer; bit 31 of comp marks a chunk stored raw (comp & 0x7fffffff == raw). */
typedef struct gbvr_zchunk {
  uint64_t src, dst;
  uint32_t comp, raw;
} gbvr_zchunk;

/* GPU decoding of many zlib streams at once, the decoder of paged bricks: one
 * warp per chunk (device pointers: dev_src, dev_dst, the chunk table
 * dev_chunks and the flag dev_err, which a malformed stream or a wrong
 * Adler-32 sets nonzero; the call neither clears nor reads it).  The call
 * returns once the work is queued on `stream` (a cudaStream_t, or null). */
int gbvr_dev_zlib_decode(const void* dev_src, void* dev_dst, const gbvr_zchunk* dev_chunks, int n, int* dev_err,
                         void* stream);
/* The same for LZ4 blocks (codec id 3; gbvr_lz4_compress writes them), the
 * decoder of paged bricks when gbvr_brick_params.compression = 3: one warp
 * per chunk, each block decoded to exactly `raw` bytes; a malformed block
 * sets *dev_err nonzero and is left partly written. */
int gbvr_dev_lz4_decode(const void* dev_src, void* dev_dst, const gbvr_zchunk* dev_chunks, int n, int* dev_err,
                        void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBVR_H */
