// Host-only UVF entry points of the C ABI (the UVFReader inspection tool and
// a raster writer); they touch no GPU.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gbvr.h"
#include "abi_guard.h"
#include "uvf.h"

namespace gbvr {
int set_error(int code, const std::string& msg);
}

using namespace gbvr;

extern "C" {

int gbvr_uvf_inspect(const char* path, int verify, gbvr_uvf_summary* out) {
  GBVR_ABI_TRY
  if (!path || !out) return set_error(GBVR_EINVAL, "null argument");
  UvfFile f;
  std::string msg;
  int rc = uvf_read(path, verify != 0, f, msg);
  if (rc) return set_error(rc, msg);
  memset(out, 0, sizeof(*out));
  out->version = f.version;
  out->checksum_semantic = f.checksum_semantic;
  if (!f.checksum.empty()) memcpy(out->checksum, f.checksum.data(), f.checksum.size() < 16 ? f.checksum.size() : 16);
  out->checksum_verified = verify && f.checksum_ok;
  out->nblocks = (int)f.blocks.size();
  for (size_t i = 0; i < f.blocks.size() && i < 32; ++i) out->block_semantics[i] = f.blocks[i].semantic;
  const UvfRaster& r = f.raster;
  for (int a = 0; a < 3; ++a) {
    out->dims[a] = (int64_t)r.dims[a];
    out->brick_size[a] = (int64_t)r.brick_size[a];
    out->overlap[a] = (int64_t)r.overlap[a];
  }
  out->dtype = r.is_float ? GBVR_F32 : (r.bit_size == 8 ? GBVR_U8 : GBVR_U16);
  out->lod_count = r.lod_counts.empty() ? 1 : (int)r.lod_counts[0];
  out->data_offset = r.data_pos;
  out->hist1d_size = (int64_t)f.hist1d.size();
  out->hist2d_nx = (int64_t)f.hist2d_nx;
  out->hist2d_ny = (int64_t)f.hist2d_ny;
  out->hist2d_max_grad = f.hist2d_max_grad;
  out->minmax_count = (int64_t)f.minmax.size();
  if (!f.minmax.empty()) {
    out->minmax_first[0] = f.minmax[0].min_scalar;
    out->minmax_first[1] = f.minmax[0].max_scalar;
    out->minmax_first[2] = f.minmax[0].min_grad;
    out->minmax_first[3] = f.minmax[0].max_grad;
  }
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_uvf_read_volume(const char* path, void* out, size_t bytes) {
  GBVR_ABI_TRY
  if (!path || !out) return set_error(GBVR_EINVAL, "null argument");
  UvfFile f;
  std::string msg;
  int rc = uvf_read(path, false, f, msg);
  if (rc) return set_error(rc, msg);
  const UvfRaster& r = f.raster;
  const size_t need = (size_t)r.dims[0] * r.dims[1] * r.dims[2] * (r.bit_size / 8);
  if (bytes < need) return set_error(GBVR_EINVAL, "buffer too small for the raster data");
  rc = uvf_read_voxels(path, f, out, need, msg);
  if (rc) return set_error(rc, msg);
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_uvf_read_hist1d(const char* path, uint64_t* out, size_t n) {
  GBVR_ABI_TRY
  UvfFile f;
  std::string msg;
  int rc = uvf_read(path ? path : "", false, f, msg);
  if (rc) return set_error(rc, msg);
  if (!out || n < f.hist1d.size()) return set_error(GBVR_EINVAL, "buffer too small");
  if (!f.hist1d.empty()) memcpy(out, f.hist1d.data(), 8 * f.hist1d.size());
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_uvf_read_hist2d(const char* path, uint64_t* out, size_t n, float* max_grad) {
  GBVR_ABI_TRY
  UvfFile f;
  std::string msg;
  int rc = uvf_read(path ? path : "", false, f, msg);
  if (rc) return set_error(rc, msg);
  if (!out || n < f.hist2d.size()) return set_error(GBVR_EINVAL, "buffer too small");
  if (!f.hist2d.empty()) memcpy(out, f.hist2d.data(), 8 * f.hist2d.size());
  if (max_grad) *max_grad = f.hist2d_max_grad;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_uvf_write_raster(const char* path, const char* raster_id, const void* voxels, const int64_t dims[3], int dtype,
                          int32_t brick_size, int32_t overlap, const uint64_t* hist1d, size_t n1, const uint64_t* hist2d,
                          size_t nx, size_t ny, float max_grad, const double* minmax, size_t nminmax) {
  GBVR_ABI_TRY
  if (!path || !voxels || !dims || dtype < 0 || dtype > 2) return set_error(GBVR_EINVAL, "bad argument");
  UvfWriteSpec s;
  s.raster.id = raster_id ? raster_id : "";
  const size_t es = dtype == GBVR_U8 ? 1 : dtype == GBVR_U16 ? 2 : 4;
  for (int a = 0; a < 3; ++a) {
    s.raster.dims[a] = (uint64_t)dims[a];
    s.raster.brick_size[a] = (uint64_t)brick_size;
    s.raster.overlap[a] = (uint64_t)(2 * overlap);
  }
  s.raster.bit_size = 8 * es;
  s.raster.mantissa = dtype == GBVR_F32 ? 23 : 8 * es;
  s.raster.is_signed = dtype == GBVR_F32;
  s.voxels = voxels;
  s.voxel_bytes = (uint64_t)dims[0] * dims[1] * dims[2] * es;
  if (hist1d && n1) s.hist1d.assign(hist1d, hist1d + n1);
  if (hist2d && nx * ny) {
    s.hist2d.assign(hist2d, hist2d + nx * ny);
    s.hist2d_nx = nx;
    s.hist2d_ny = ny;
    s.hist2d_max_grad = max_grad;
  }
  for (size_t i = 0; minmax && i < nminmax; ++i)
    s.minmax.push_back({minmax[4 * i], minmax[4 * i + 1], minmax[4 * i + 2], minmax[4 * i + 3]});
  std::string msg;
  int rc = uvf_write(path, s, msg);
  if (rc) return set_error(rc, msg);
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_load_tf1d_file(const char* path, int target_size, float* rgba_out, int capacity, int* n_out) {
  GBVR_ABI_TRY
  if (!path || !rgba_out || capacity <= 0) return set_error(GBVR_EINVAL, "bad argument");
  FILE* f = fopen(path, "r");
  if (!f) return set_error(GBVR_EIO, std::string("cannot open ") + path);
  long n = 0;
  std::vector<float> t;
  bool ok = fscanf(f, "%ld", &n) == 1 && n > 0 && n <= (1 << 20);
  if (ok) {
    t.resize(4 * (size_t)n);
    for (long i = 0; ok && i < 4 * n; ++i) ok = fscanf(f, "%f", &t[i]) == 1;
  }
  fclose(f);
  if (!ok) return set_error(GBVR_EFORMAT, std::string("not a 1D transfer function file: ") + path);
  const long m = target_size > 0 ? target_size : n;
  if (m > capacity) return set_error(GBVR_EINVAL, "capacity below the table size");
  for (long j = 0; j < m; ++j) {
    // linear resampling: entry j sits at position j (n - 1) / (m - 1)
    double pos = m > 1 ? (double)j * (double)(n - 1) / (double)(m - 1) : 0.0;
    long i0 = (long)pos;
    if (i0 > n - 1) i0 = n - 1;
    long i1 = i0 + 1 < n ? i0 + 1 : n - 1;
    double w = pos - (double)i0;
    for (int c = 0; c < 4; ++c) rgba_out[4 * j + c] = (float)((1.0 - w) * t[4 * i0 + c] + w * t[4 * i1 + c]);
  }
  if (n_out) *n_out = (int)m;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_load_tf2d_file(const char* path, int* width, int* height, float* tf1d, int tf1d_cap, int* tf1d_n,
                        gbvr_tf2d_swatch* swatches, int swatch_cap, int* nswatches) {
  GBVR_ABI_TRY
  if (!path) return set_error(GBVR_EINVAL, "bad argument");
  FILE* f = fopen(path, "r");
  if (!f) return set_error(GBVR_EIO, std::string("cannot open ") + path);
  auto bad = [&](const char* what) {
    fclose(f);
    return set_error(GBVR_EFORMAT, std::string("not a 2D transfer function file (") + what + "): " + path);
  };
  int w = 0, h = 0;
  long n = 0;
  if (fscanf(f, "%d %d", &w, &h) != 2 || w <= 0 || h <= 0 || w > 16384 || h > 16384) return bad("size");
  if (fscanf(f, "%ld", &n) != 1 || n < 0 || n > (1 << 20)) return bad("1D size");
  for (long i = 0; i < 4 * n; ++i) {
    float v;
    if (fscanf(f, "%f", &v) != 1) return bad("1D entries");
    if (tf1d && i < 4L * tf1d_cap) tf1d[i] = v;
  }
  int ns = 0;
  if (fscanf(f, "%d", &ns) != 1 || ns < 0 || ns > (1 << 16)) return bad("swatch count");
  for (int k = 0; k < ns; ++k) {
    gbvr_tf2d_swatch sw;
    memset(&sw, 0, sizeof(sw));
    if (fscanf(f, "%d %d", &sw.radial, &sw.npoints) != 2 || sw.radial < 0 || sw.radial > 1 || sw.npoints < 3 ||
        sw.npoints > GBVR_TF2D_MAX_POINTS)
      return bad("swatch header");
    for (int j = 0; j < 2 * sw.npoints; ++j)
      if (fscanf(f, "%f", &sw.points[j]) != 1) return bad("vertex");
    for (int j = 0; j < 4; ++j)
      if (fscanf(f, "%f", &sw.grad[j]) != 1) return bad("gradient");
    if (fscanf(f, "%d", &sw.nstops) != 1 || sw.nstops < 1 || sw.nstops > GBVR_TF2D_MAX_STOPS) return bad("stop count");
    for (int j = 0; j < 5 * sw.nstops; ++j)
      if (fscanf(f, "%f", &sw.stops[j]) != 1) return bad("stop");
    for (int j = 1; j < sw.nstops; ++j)
      if (!(sw.stops[5 * j] >= sw.stops[5 * (j - 1)])) return bad("stop order");
    if (swatches && k < swatch_cap) swatches[k] = sw;
  }
  fclose(f);
  if (width) *width = w;
  if (height) *height = h;
  if (tf1d_n) *tf1d_n = (int)n;
  if (nswatches) *nswatches = ns;
  return GBVR_OK;
  GBVR_ABI_CATCH
}

}  // extern "C"
