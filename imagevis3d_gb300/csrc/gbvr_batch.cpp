// gbvr_batch: headless batch renderer over the C ABI.
//
// Replays the call sequence of the reference's batch renderer script
// (LuaScripts/BatchRenderer.lua:22-41, run by BatchRenderer/main.cpp:67-112):
//   renderer = tuvok.renderer.new(...)          -> gbvr_create
//   renderer.loadDataset(uvf)                   -> gbvr_load_uvf
//   renderer.resize({w, h})                     -> gbvr_resize
//   renderer.paint()                            -> gbvr_paint (or one batch for an orbit)
//   renderer.captureSingleFrame(png, true)      -> gbvr_capture_single_frame / gbvr_capture_view
//   renderer.cleanup(); deleteClass(renderer)   -> gbvr_destroy
// The GL context creation of BatchContext.cpp has no counterpart: the
// framebuffer lives in device memory.
//
// usage: gbvr_batch -f data.uvf -o out.png [-tf tf.1dt] [-size W H] [-spv S]
//                   [-views N] [-elevation DEG] [-radius R] [-noverify]
// With -views N > 1 the N frames of a 360-degree orbit (ImageVis3D_Capturing.cpp)
// are rendered by one batched paint and written as out_0000.png ...
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gbvr.h"

static int die(const char* what) {
  char msg[1024];
  gbvr_last_error(msg, sizeof(msg));
  fprintf(stderr, "gbvr_batch: %s failed: %s\n", what, msg);
  return 1;
}

int main(int argc, char** argv) {
  std::string data, out = "render.png", tf;
  int w = 640, h = 480, views = 1, verify = 1;
  float spv = 1.f, elev = 20.f, radius = 2.5f * std::sqrt(3.f);
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&](int k) { return i + k < argc; };
    if (a == "-f" && next(1)) data = argv[++i];
    else if (a == "-o" && next(1)) out = argv[++i];
    else if (a == "-tf" && next(1)) tf = argv[++i];
    else if (a == "-size" && next(2)) { w = atoi(argv[++i]); h = atoi(argv[++i]); }
    else if (a == "-spv" && next(1)) spv = (float)atof(argv[++i]);
    else if (a == "-views" && next(1)) views = atoi(argv[++i]);
    else if (a == "-elevation" && next(1)) elev = (float)atof(argv[++i]);
    else if (a == "-radius" && next(1)) radius = (float)atof(argv[++i]);
    else if (a == "-noverify") verify = 0;
    else {
      fprintf(stderr, "usage: %s -f data.uvf -o out.png [-tf tf.1dt] [-size W H] [-spv S] [-views N] "
                      "[-elevation DEG] [-radius R] [-noverify]\n", argv[0]);
      return 2;
    }
  }
  if (data.empty() || views < 1) return die("arguments");
  gbvr_renderer* r = nullptr;
  if (gbvr_create(GBVR_CUDA_RAYCASTER, 0, &r) != GBVR_OK) return die("renderer.new");
  int rc = 0;
  do {
    if (gbvr_load_uvf(r, data.c_str(), verify, nullptr) != GBVR_OK) { rc = die("loadDataset"); break; }
    if (!tf.empty()) {
      gbvr_dataset_info info;
      gbvr_get_dataset_info(r, &info);
      std::vector<float> t(4 * 65536);
      int n = 0;
      if (gbvr_load_tf1d_file(tf.c_str(), info.hist1d_size, t.data(), 65536, &n) != GBVR_OK ||
          gbvr_set_tf1d(r, t.data(), n) != GBVR_OK) { rc = die("transfer function"); break; }
    }
    if (gbvr_resize(r, w, h) != GBVR_OK) { rc = die("resize"); break; }
    if (gbvr_set_sample_rate(r, spv) != GBVR_OK) { rc = die("setSampleRateModifier"); break; }
    std::vector<gbvr_view> vs(views);
    for (int i = 0; i < views; ++i)
      gbvr_orbit_camera(360.f * i / views, elev, radius, 45.f, w, h, vs[i].view, vs[i].proj);
    if (views == 1) {
      if (gbvr_set_view(r, vs[0].view, vs[0].proj) != GBVR_OK || gbvr_paint(r) != GBVR_OK) { rc = die("paint"); break; }
      if (gbvr_capture_single_frame(r, out.c_str(), 1) != GBVR_OK) { rc = die("captureSingleFrame"); break; }
    } else {
      if (gbvr_paint_batch(r, vs.data(), views) != GBVR_OK) { rc = die("paint"); break; }
      std::string stem = out, ext = ".png";
      size_t dot = out.rfind('.');
      if (dot != std::string::npos) { stem = out.substr(0, dot); ext = out.substr(dot); }
      for (int i = 0; i < views && rc == 0; ++i) {
        char name[4096];
        snprintf(name, sizeof(name), "%s_%04d%s", stem.c_str(), i, ext.c_str());
        if (gbvr_capture_view(r, i, name, 1) != GBVR_OK) rc = die("capture");
      }
    }
    gbvr_stats st;
    gbvr_get_stats(r, &st);
    printf("gbvr_batch: %d view(s) %dx%d, %.3f ms on the GPU, %llu samples\n", views, w, h, st.gpu_ms,
           (unsigned long long)st.samples);
  } while (0);
  gbvr_destroy(r);
  return rc;
}
