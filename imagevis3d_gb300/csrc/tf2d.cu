// 2D transfer functions from swatches: the rasteriser that turns the
// polygons-with-gradients of a .2dt file into the value x gradient-magnitude
// RGBA table the raycaster samples.
//
// The reference's editor draws the same table with Qt
// (Q2DTransferFunction.cpp:436-473 swatches with QLinearGradient /
// QRadialGradient brushes, 1138-1153 the 1D TF image stretched underneath,
// 1182-1217 the drawing order); Tuvok's TransferFunction2D, which produces the
// table for the GPU, is not in the tree.  The rule here:
//   * entry (x, r) has its centre at canvas pixel (x + 0.5, H - 1 - r + 0.5):
//     row r is gradient bin r, and the canvas has gradient 0 at the bottom as
//     the editor's histogram image (Q2DTransferFunction.cpp:156-160);
//   * it starts as 1D TF entry floor(x * N / W) (an unsmoothed stretch);
//   * each swatch in file order, where the centre lies inside its polygon
//     (even-odd rule, Qt's default fill rule), composites the gradient colour
//     at the centre over it ("source over" on non-premultiplied RGBA);
//   * linear gradient: t = projection of the centre onto g0 -> g1; radial:
//     t = |centre - g0| / |g1 - g0|; both clamped to [0, 1] (pad spread);
//     colour linear between the stops around t, the end stops outside them.
// Geometry is evaluated in canvas pixels (normalised coordinates x W, x H),
// as the editor does, so radial swatches stay round on non-square tables.
// Every float operation is an explicitly rounded intrinsic in a fixed order,
// which the oracle's restatement repeats, so both give identical bits.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/gbvr.h"
#include "abi_guard.h"
#include "gbvr_internal.h"

namespace gbvr {
int set_error(int code, const std::string& msg);
}

using namespace gbvr;

namespace {

__device__ bool swatch_covers(const gbvr_tf2d_swatch& s, float cx, float cy, float fw, float fh) {
  bool in = false;
  const int n = s.npoints;
  for (int i = 0, j = n - 1; i < n; j = i++) {
    const float xi = __fmul_rn(s.points[2 * i], fw), yi = __fmul_rn(s.points[2 * i + 1], fh);
    const float xj = __fmul_rn(s.points[2 * j], fw), yj = __fmul_rn(s.points[2 * j + 1], fh);
    if ((yi > cy) != (yj > cy)) {
      const float xc = __fadd_rn(xi, __fdiv_rn(__fmul_rn(__fsub_rn(cy, yi), __fsub_rn(xj, xi)), __fsub_rn(yj, yi)));
      if (cx < xc) in = !in;
    }
  }
  return in;
}

__device__ float gradient_pos(const gbvr_tf2d_swatch& s, float cx, float cy, float fw, float fh) {
  const float g0x = __fmul_rn(s.grad[0], fw), g0y = __fmul_rn(s.grad[1], fh);
  const float g1x = __fmul_rn(s.grad[2], fw), g1y = __fmul_rn(s.grad[3], fh);
  const float qx = __fsub_rn(cx, g0x), qy = __fsub_rn(cy, g0y);
  const float dx = __fsub_rn(g1x, g0x), dy = __fsub_rn(g1y, g0y);
  const float dd = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
  float t;
  if (s.radial) {
    const float r = __fsqrt_rn(dd);
    const float d = __fsqrt_rn(__fadd_rn(__fmul_rn(qx, qx), __fmul_rn(qy, qy)));
    t = r > 0.f ? __fdiv_rn(d, r) : 1.f;
  } else {
    t = dd > 0.f ? __fdiv_rn(__fadd_rn(__fmul_rn(qx, dx), __fmul_rn(qy, dy)), dd) : 0.f;
  }
  return fminf(fmaxf(t, 0.f), 1.f);
}

__device__ void stop_colour(const gbvr_tf2d_swatch& s, float t, float c[4]) {
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
  while (i + 2 < n && st[5 * (i + 1)] <= t) ++i;  // st[5 i] <= t < st[5 (i + 1)]
  const float p0 = st[5 * i], p1 = st[5 * (i + 1)];
  const float w = __fdiv_rn(__fsub_rn(t, p0), __fsub_rn(p1, p0));
  for (int k = 0; k < 4; ++k) {
    const float a = st[5 * i + 1 + k], b = st[5 * (i + 1) + 1 + k];
    c[k] = __fadd_rn(a, __fmul_rn(w, __fsub_rn(b, a)));
  }
}

__global__ void k_raster_tf2d(const gbvr_tf2d_swatch* __restrict__ sw, int ns, const float* __restrict__ tf1d,
                              int n1d, int W, int H, float4* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
  if (x >= W) return;
  float d[4] = {0.f, 0.f, 0.f, 0.f};
  if (n1d > 0) {
    const long long j = (long long)x * n1d / W;
    for (int k = 0; k < 4; ++k) d[k] = tf1d[4 * j + k];
  }
  const float fw = (float)W, fh = (float)H;
  const float cx = __fadd_rn((float)x, 0.5f), cy = __fadd_rn((float)(H - 1 - r), 0.5f);
  for (int k = 0; k < ns; ++k) {
    const gbvr_tf2d_swatch& s = sw[k];
    if (!swatch_covers(s, cx, cy, fw, fh)) continue;
    float c[4];
    stop_colour(s, gradient_pos(s, cx, cy, fw, fh), c);
    const float as = c[3];
    const float kd = __fmul_rn(d[3], __fsub_rn(1.f, as));
    const float a = __fadd_rn(as, kd);
    for (int j = 0; j < 3; ++j)
      d[j] = a > 0.f ? __fdiv_rn(__fadd_rn(__fmul_rn(c[j], as), __fmul_rn(d[j], kd)), a) : 0.f;
    d[3] = a;
  }
  out[(long long)r * W + x] = make_float4(d[0], d[1], d[2], d[3]);
}

struct DevMem {
  void* p = nullptr;
  ~DevMem() {
    if (p) cudaFree(p);
  }
};

int cuda_fail(cudaError_t e, const char* what) {
  return set_error(GBVR_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" {

int gbvr_tf2d_rasterize(const gbvr_tf2d_swatch* swatches, int nswatches, const float* tf1d, int tf1d_n, int width,
                        int height, float* out_rgba) {
  GBVR_ABI_TRY
  if (!out_rgba || width <= 0 || height <= 0 || width > 16384 || height > 16384 || nswatches < 0 || tf1d_n < 0 ||
      (nswatches > 0 && !swatches) || (tf1d_n > 0 && !tf1d))
    return set_error(GBVR_EINVAL, "bad argument");
  for (int k = 0; k < nswatches; ++k) {
    const gbvr_tf2d_swatch& s = swatches[k];
    if (s.radial < 0 || s.radial > 1 || s.npoints < 3 || s.npoints > GBVR_TF2D_MAX_POINTS || s.nstops < 1 ||
        s.nstops > GBVR_TF2D_MAX_STOPS)
      return set_error(GBVR_EINVAL, "swatch " + std::to_string(k) + " out of range");
    for (int j = 1; j < s.nstops; ++j)
      if (!(s.stops[5 * j] >= s.stops[5 * (j - 1)]))
        return set_error(GBVR_EINVAL, "swatch " + std::to_string(k) + ": stops not in increasing order");
  }
  (void)cudaGetLastError();
  DevMem dsw, dtf, dout;
  const size_t nout = (size_t)width * height * 4 * sizeof(float);
  cudaError_t e;
  if (nswatches > 0) {
    if ((e = cudaMalloc(&dsw.p, sizeof(gbvr_tf2d_swatch) * nswatches)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    if ((e = cudaMemcpy(dsw.p, swatches, sizeof(gbvr_tf2d_swatch) * nswatches, cudaMemcpyHostToDevice)) != cudaSuccess)
      return cuda_fail(e, "upload swatches");
  }
  if (tf1d_n > 0) {
    if ((e = cudaMalloc(&dtf.p, sizeof(float) * 4 * tf1d_n)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    if ((e = cudaMemcpy(dtf.p, tf1d, sizeof(float) * 4 * tf1d_n, cudaMemcpyHostToDevice)) != cudaSuccess)
      return cuda_fail(e, "upload 1D TF");
  }
  if ((e = cudaMalloc(&dout.p, nout)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  dim3 grid((unsigned)((width + 127) / 128), (unsigned)height);
  k_raster_tf2d<<<grid, 128>>>((const gbvr_tf2d_swatch*)dsw.p, nswatches, (const float*)dtf.p, tf1d_n, width, height,
                               (float4*)dout.p);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "k_raster_tf2d");
  if ((e = cudaMemcpy(out_rgba, dout.p, nout, cudaMemcpyDeviceToHost)) != cudaSuccess) return cuda_fail(e, "readback");
  return GBVR_OK;
  GBVR_ABI_CATCH
}

int gbvr_set_tf2d_file(gbvr_renderer* r, const char* path, float max_grad) {
  GBVR_ABI_TRY
  if (!r) return set_error(GBVR_EINVAL, "null renderer");
  int w = 0, h = 0, n1 = 0, ns = 0;
  int st = gbvr_load_tf2d_file(path, &w, &h, nullptr, 0, &n1, nullptr, 0, &ns);
  if (st != GBVR_OK) return st;
  std::vector<float> tf1d(4 * (size_t)n1);
  std::vector<gbvr_tf2d_swatch> sw(ns);
  st = gbvr_load_tf2d_file(path, &w, &h, tf1d.data(), n1, &n1, sw.data(), ns, &ns);
  if (st != GBVR_OK) return st;
  std::vector<float> table((size_t)w * h * 4);
  st = gbvr_tf2d_rasterize(sw.data(), ns, tf1d.data(), n1, w, h, table.data());
  if (st != GBVR_OK) return st;
  return gbvr_set_tf2d(r, table.data(), w, h, max_grad);
  GBVR_ABI_CATCH
}

}  // extern "C"
