// The library's host-side parsers, codec and image writer under
// AddressSanitizer and UndefinedBehaviorSanitizer: the UVF reader and writer,
// the .1dt / .2dt parsers and the LZ4 block codec on valid inputs and on
// truncated, bit-flipped and overwritten ones, and the PNG / BMP / PPM frame
// writer at odd sizes.  A malformed input must come back as a
// status: no crash, no out-of-bounds access, no undefined behaviour.  Built
// and run by test_host_sanitizers.py (no GPU); usage: sanitize_host DIR SEED.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "gbvr.h"

namespace gbvr {
// the renderer's error store lives in the CUDA part of the library
int set_error(int code, const std::string&) { return code; }
bool write_image(const std::string& path, const unsigned char* rgba, int w, int h, bool alpha);
}  // namespace gbvr

namespace {

uint64_t g_rng = 88172645463325252ull;
uint32_t rnd() {
  g_rng ^= g_rng << 13;
  g_rng ^= g_rng >> 7;
  g_rng ^= g_rng << 17;
  return (uint32_t)(g_rng >> 11);
}

int g_failures = 0;
#define CHECK(c)                                                     \
  do {                                                               \
    if (!(c)) {                                                      \
      std::fprintf(stderr, "check failed at line %d: %s\n", __LINE__, #c); \
      ++g_failures;                                                  \
    }                                                                \
  } while (0)

// an exact-size heap buffer, so that the sanitizer sees any access past it
struct Heap {
  std::unique_ptr<uint8_t[]> p;
  size_t n;
  explicit Heap(size_t size) : p(new uint8_t[size ? size : 1]), n(size) {}
  uint8_t* data() { return p.get(); }
};

std::vector<uint8_t> slurp(const std::string& path) {
  std::vector<uint8_t> d;
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return d;
  uint8_t buf[65536];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) d.insert(d.end(), buf, buf + got);
  std::fclose(f);
  return d;
}

void spit(const std::string& path, const std::vector<uint8_t>& d) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return;
  if (!d.empty()) std::fwrite(d.data(), 1, d.size(), f);
  std::fclose(f);
}

// one random damage: a flipped byte, a truncation, or 8 bytes overwritten
// with a large or random value (where the size fields are)
std::vector<uint8_t> damage(const std::vector<uint8_t>& d, size_t hot) {
  std::vector<uint8_t> m = d;
  if (m.empty()) return m;
  const size_t at = (rnd() % 2 && hot) ? rnd() % std::min(hot, m.size()) : rnd() % m.size();
  switch (rnd() % 3) {
    case 0:
      m[at] ^= (uint8_t)(1 + rnd() % 255);
      break;
    case 1:
      m.resize(at);
      break;
    default: {
      uint64_t v = rnd() % 2 ? ~0ull >> (rnd() % 64) : ((uint64_t)rnd() << 32 | rnd());
      for (int i = 0; i < 8 && at + i < m.size(); ++i) m[at + i] = (uint8_t)(v >> (8 * i));
    }
  }
  return m;
}

void lz4_cases() {
  const size_t sizes[] = {0, 1, 4, 5, 12, 13, 17, 255, 256, 4096, 16384, 16385, 65535, 65536, 65537, 100000};
  for (size_t n : sizes)
    for (int pat = 0; pat < 4; ++pat) {
      Heap src(n);
      for (size_t i = 0; i < n; ++i)
        src.data()[i] = pat == 0   ? (uint8_t)rnd()
                        : pat == 1 ? 0
                        : pat == 2 ? (uint8_t)(i % 3)
                                   : (uint8_t)(rnd() % 16 == 0 ? rnd() : i / 64);
      const size_t cap = gbvr_lz4_bound(n);
      Heap comp(cap);
      const size_t c = gbvr_lz4_compress(src.data(), n, comp.data(), cap);
      CHECK(c > 0 && c <= cap);
      Heap out(n);
      CHECK(gbvr_lz4_decompress(comp.data(), c, out.data(), n) == GBVR_OK);
      CHECK(std::memcmp(out.data(), src.data(), n) == 0);
      if (n > 0) {
        Heap shorter(n - 1);
        CHECK(gbvr_lz4_decompress(comp.data(), c, shorter.data(), n - 1) != GBVR_OK);
      }
      if (c > 1) {
        Heap small(c - 1);
        CHECK(gbvr_lz4_compress(src.data(), n, small.data(), c - 1) == 0);
      }
      std::vector<uint8_t> good(comp.data(), comp.data() + c);
      for (int m = 0; m < 48; ++m) {
        std::vector<uint8_t> bad = damage(good, 16);
        Heap in(bad.size());
        if (!bad.empty()) std::memcpy(in.data(), bad.data(), bad.size());
        Heap o(n);
        (void)gbvr_lz4_decompress(in.data(), bad.size(), o.data(), n);
      }
    }
}

void uvf_cases(const std::string& dir) {
  const int64_t dims[3] = {24, 20, 16};
  const size_t nvox = 24 * 20 * 16;
  for (int dtype = GBVR_U8; dtype <= GBVR_F32; ++dtype) {
    const size_t es = dtype == GBVR_U8 ? 1 : dtype == GBVR_U16 ? 2 : 4;
    Heap vox(nvox * es);
    for (size_t i = 0; i < nvox * es; ++i) vox.data()[i] = (uint8_t)rnd();
    if (dtype == GBVR_F32)
      for (size_t i = 0; i < nvox; ++i) {
        const float v = (float)(rnd() % 1000) * 0.5f;
        std::memcpy(vox.data() + 4 * i, &v, 4);
      }
    std::vector<uint64_t> h1(dtype == GBVR_U8 ? 256 : 1024), h2(64 * 32);
    for (auto& v : h1) v = rnd() % 100;
    for (auto& v : h2) v = rnd() % 100;
    const double mm[4] = {0.0, 255.0, 0.0, 17.5};
    const std::string path = dir + "/valid.uvf";
    CHECK(gbvr_uvf_write_raster(path.c_str(), "sanitizer volume", vox.data(), dims, dtype, 64, 2, h1.data(), h1.size(),
                                h2.data(), 64, 32, 3.5f, mm, 1) == GBVR_OK);
    gbvr_uvf_summary s;
    CHECK(gbvr_uvf_inspect(path.c_str(), 1, &s) == GBVR_OK);
    CHECK(s.checksum_verified == 1 && s.dims[0] == 24 && s.dims[1] == 20 && s.dims[2] == 16 && s.dtype == dtype);
    Heap back(nvox * es);
    CHECK(gbvr_uvf_read_volume(path.c_str(), back.data(), nvox * es) == GBVR_OK);
    CHECK(std::memcmp(back.data(), vox.data(), nvox * es) == 0);
    std::vector<uint64_t> r1(h1.size()), r2(h2.size());
    CHECK(gbvr_uvf_read_hist1d(path.c_str(), r1.data(), r1.size()) == GBVR_OK && r1 == h1);
    float mg = 0.f;
    CHECK(gbvr_uvf_read_hist2d(path.c_str(), r2.data(), r2.size(), &mg) == GBVR_OK && r2 == h2 && mg == 3.5f);

    const std::vector<uint8_t> file = slurp(path);
    const std::string bad_path = dir + "/damaged.uvf";
    for (int m = 0; m < 400; ++m) {
      const std::vector<uint8_t> bad = damage(file, 600);
      spit(bad_path, bad);
      const bool changed = bad != file;
      gbvr_uvf_summary t;
      // the MD5 covers bytes 49 .. end: damage there must not verify
      const int rv = gbvr_uvf_inspect(bad_path.c_str(), 1, &t);
      if (changed && bad.size() > 49 && file.size() == bad.size() &&
          std::memcmp(bad.data(), file.data(), 49) == 0)
        CHECK(rv != GBVR_OK);
      if (gbvr_uvf_inspect(bad_path.c_str(), 0, &t) != GBVR_OK) continue;
      const uint64_t need = (uint64_t)t.dims[0] * (uint64_t)t.dims[1] * (uint64_t)t.dims[2] *
                            (t.dtype == GBVR_U8 ? 1u : t.dtype == GBVR_U16 ? 2u : 4u);
      if (need <= (64u << 20)) {
        Heap v(need);
        (void)gbvr_uvf_read_volume(bad_path.c_str(), v.data(), need);
      }
      if (t.hist1d_size >= 0 && t.hist1d_size <= (1 << 20)) {
        std::vector<uint64_t> a((size_t)t.hist1d_size + 1);
        (void)gbvr_uvf_read_hist1d(bad_path.c_str(), a.data(), (size_t)t.hist1d_size);
      }
      const uint64_t n2 = (uint64_t)t.hist2d_nx * (uint64_t)t.hist2d_ny;
      if (t.hist2d_nx >= 0 && t.hist2d_ny >= 0 && n2 <= (1u << 20)) {
        std::vector<uint64_t> a((size_t)n2 + 1);
        (void)gbvr_uvf_read_hist2d(bad_path.c_str(), a.data(), (size_t)n2, nullptr);
      }
    }
  }
}

void tf_cases(const std::string& dir) {
  // .1dt
  std::string t1 = "16\n";
  for (int i = 0; i < 16; ++i) {
    char line[96];
    std::snprintf(line, sizeof(line), "%g %g %g %g\n", i / 15.0, 0.5, 1.0 - i / 15.0, i / 30.0);
    t1 += line;
  }
  const std::string p1 = dir + "/valid.1dt";
  spit(p1, std::vector<uint8_t>(t1.begin(), t1.end()));
  std::vector<float> rgba(4 * 64);
  int n = 0;
  CHECK(gbvr_load_tf1d_file(p1.c_str(), 0, rgba.data(), 16, &n) == GBVR_OK && n == 16);
  CHECK(gbvr_load_tf1d_file(p1.c_str(), 64, rgba.data(), 64, &n) == GBVR_OK && n == 64);
  CHECK(gbvr_load_tf1d_file(p1.c_str(), 0, rgba.data(), 15, &n) == GBVR_EINVAL);
  const std::vector<uint8_t> f1(t1.begin(), t1.end());
  const std::string b1 = dir + "/damaged.1dt";
  for (int m = 0; m < 300; ++m) {
    spit(b1, damage(f1, 8));
    Heap out(4 * 64 * sizeof(float));
    (void)gbvr_load_tf1d_file(b1.c_str(), rnd() % 2 ? 0 : 64, (float*)out.data(), 64, &n);
  }
  const char* bad1[] = {"2000000\n0 0 0 0\n", "-5\n", "3\n1 2 3 4\n5 6 7\n", "x\n", ""};
  for (const char* b : bad1) {
    spit(b1, std::vector<uint8_t>(b, b + std::strlen(b)));
    CHECK(gbvr_load_tf1d_file(b1.c_str(), 0, rgba.data(), 64, &n) == GBVR_EFORMAT);
  }
  // .2dt: canvas, embedded 1D TF, two swatches
  std::string t2 = "256 128\n4\n0 0 0 0\n0.2 0.2 0.2 0.1\n0.6 0.6 0.6 0.5\n1 1 1 1\n2\n";
  t2 += "0 4\n0.1 0.1\n0.5 0.1\n0.5 0.6\n0.1 0.6\n0.1 0.1 0.5 0.6\n2\n0 1 0 0 0.5\n1 0 1 0 0.8\n";
  t2 += "1 3\n0.6 0.2\n0.9 0.3\n0.7 0.8\n0.75 0.4 0.9 0.9\n3\n0 0 0 1 0\n0.5 0 1 1 0.5\n1 1 1 1 1\n";
  const std::string p2 = dir + "/valid.2dt";
  spit(p2, std::vector<uint8_t>(t2.begin(), t2.end()));
  int w = 0, h = 0, n1 = 0, ns = 0;
  CHECK(gbvr_load_tf2d_file(p2.c_str(), &w, &h, nullptr, 0, &n1, nullptr, 0, &ns) == GBVR_OK);
  CHECK(w == 256 && h == 128 && n1 == 4 && ns == 2);
  std::vector<float> tf1(16);
  std::vector<gbvr_tf2d_swatch> sw(2);
  CHECK(gbvr_load_tf2d_file(p2.c_str(), &w, &h, tf1.data(), 4, &n1, sw.data(), 2, &ns) == GBVR_OK);
  CHECK(sw[0].npoints == 4 && sw[1].radial == 1 && sw[1].nstops == 3);
  const std::vector<uint8_t> f2(t2.begin(), t2.end());
  const std::string b2 = dir + "/damaged.2dt";
  for (int m = 0; m < 300; ++m) {
    spit(b2, damage(f2, 16));
    std::vector<float> a(16);
    std::vector<gbvr_tf2d_swatch> s2(2);
    (void)gbvr_load_tf2d_file(b2.c_str(), &w, &h, a.data(), 4, &n1, s2.data(), 2, &ns);
  }
  const char* bad2[] = {"0 5\n", "256 128\n2000000\n", "8 8\n0\n1\n0 100\n", "8 8\n0\n1\n0 3\n0 0\n1 0\n1 1\n0 0 1 1\n0\n",
                        "8 8\n0\n1\n0 3\n0 0\n1 0\n1 1\n0 0 1 1\n2\n0.5 1 1 1 1\n0.2 1 1 1 1\n"};
  for (const char* b : bad2) {
    spit(b2, std::vector<uint8_t>(b, b + std::strlen(b)));
    CHECK(gbvr_load_tf2d_file(b2.c_str(), &w, &h, nullptr, 0, &n1, nullptr, 0, &ns) == GBVR_EFORMAT);
  }
}

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

// PNG (stored deflate blocks), BMP and PPM frames of odd sizes: the PNG is
// decoded back (chunks, stored blocks, filter bytes) and must give the pixels
void image_cases(const std::string& dir) {
  const int sizes[][2] = {{1, 1}, {3, 5}, {100, 7}, {7, 300}, {200, 200}};
  for (const auto& sz : sizes)
    for (int alpha = 0; alpha < 2; ++alpha) {
      const int w = sz[0], h = sz[1], ch = alpha ? 4 : 3;
      Heap rgba((size_t)w * h * 4);
      for (size_t i = 0; i < (size_t)w * h * 4; ++i) rgba.data()[i] = (uint8_t)rnd();
      const std::string png = dir + "/frame.png";
      CHECK(gbvr::write_image(png, rgba.data(), w, h, alpha != 0));
      const std::vector<uint8_t> f = slurp(png);
      CHECK(f.size() > 33 && std::memcmp(f.data() + 12, "IHDR", 4) == 0);
      if (f.size() <= 33) continue;
      CHECK(be32(f.data() + 16) == (uint32_t)w && be32(f.data() + 20) == (uint32_t)h && f[25] == (alpha ? 6 : 2));
      std::vector<uint8_t> z;  // the IDAT payloads
      for (size_t at = 8; at + 12 <= f.size();) {
        const uint32_t n = be32(f.data() + at);
        if (at + 12 + n > f.size()) break;
        if (std::memcmp(f.data() + at + 4, "IDAT", 4) == 0) z.insert(z.end(), f.begin() + at + 8, f.begin() + at + 8 + n);
        at += 12 + n;
      }
      std::vector<uint8_t> raw;  // stored blocks after the 2-byte zlib header
      size_t q = 2;
      bool last = false;
      while (!last && q + 5 <= z.size()) {
        last = z[q] & 1;
        const size_t n = z[q + 1] | (size_t)z[q + 2] << 8;
        CHECK((z[q + 3] | (size_t)z[q + 4] << 8) == (~n & 0xffff));
        if (q + 5 + n > z.size()) break;
        raw.insert(raw.end(), z.begin() + q + 5, z.begin() + q + 5 + n);
        q += 5 + n;
      }
      CHECK(last && raw.size() == (size_t)h * (1 + (size_t)w * ch));
      bool same = raw.size() == (size_t)h * (1 + (size_t)w * ch);
      for (int y = 0; same && y < h; ++y) {
        same = raw[(size_t)y * (1 + w * ch)] == 0;
        for (int x = 0; same && x < w; ++x)
          same = std::memcmp(&raw[(size_t)y * (1 + w * ch) + 1 + (size_t)x * ch], rgba.data() + 4 * ((size_t)y * w + x),
                             ch) == 0;
      }
      CHECK(same);
      const std::string bmp = dir + "/frame.BMP", ppm = dir + "/frame.ppm";
      CHECK(gbvr::write_image(bmp, rgba.data(), w, h, false));
      CHECK(slurp(bmp).size() == 54 + (size_t)((w * 3 + 3) & ~3) * h);
      CHECK(gbvr::write_image(ppm, rgba.data(), w, h, false));
      char hdr[64];
      std::snprintf(hdr, sizeof(hdr), "P6\n%d %d\n255\n", w, h);
      CHECK(slurp(ppm).size() == std::strlen(hdr) + (size_t)w * h * 3);
    }
  CHECK(!gbvr::write_image(dir + "/no/such/dir/frame.png", nullptr, 0, 0, false));
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s DIR SEED\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  g_rng ^= std::strtoull(argv[2], nullptr, 10) * 0x9E3779B97F4A7C15ull;
  lz4_cases();
  uvf_cases(dir);
  tf_cases(dir);
  image_cases(dir);
  std::printf("%s: %d failed checks\n", g_failures ? "FAILED" : "ok", g_failures);
  return g_failures ? 1 : 0;
}
