// Framebuffer capture to image files, the headless stand-in for
// captureSingleFrame (ImageVis3D/UI/RenderWindow.cpp:1642-1671) and for the
// RGBA8 readback model of StandaloneTuvok/CmdRenderer.cpp:34-56.
// PNG is written with stored (uncompressed) deflate blocks, so no zlib is
// needed; .bmp and .ppm are also accepted.
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace gbvr {

// CRC-32 (the PNG chunk checksum), table built once on first use (a
// function-local static: safe when several threads capture at once)
struct CrcTable {
  uint32_t t[256];
  CrcTable() {
    for (uint32_t n = 0; n < 256; ++n) {
      uint32_t c = n;
      for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      t[n] = c;
    }
  }
};
static uint32_t crc32(const unsigned char* p, size_t n, uint32_t c = 0xFFFFFFFFu) {
  static const CrcTable table;
  for (size_t i = 0; i < n; ++i) c = table.t[(c ^ p[i]) & 0xFF] ^ (c >> 8);
  return c;
}

static void be32(std::vector<unsigned char>& v, uint32_t x) {
  v.push_back((unsigned char)(x >> 24));
  v.push_back((unsigned char)(x >> 16));
  v.push_back((unsigned char)(x >> 8));
  v.push_back((unsigned char)x);
}

static void chunk(std::vector<unsigned char>& out, const char* type, const std::vector<unsigned char>& data) {
  be32(out, (uint32_t)data.size());
  size_t start = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  uint32_t c = crc32(out.data() + start, out.size() - start) ^ 0xFFFFFFFFu;
  be32(out, c);
}

// rgba: width*height*4 bytes, row 0 = top.  alpha == false drops alpha.
bool write_image(const std::string& path, const unsigned char* rgba, int w, int h, bool alpha) {
  std::string ext = path.size() >= 4 ? path.substr(path.size() - 4) : "";
  for (auto& ch : ext) ch = (char)tolower((unsigned char)ch);
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return false;
  bool ok = true;
  const int ch = alpha ? 4 : 3;
  if (ext == ".ppm") {
    fprintf(f, "P6\n%d %d\n255\n", w, h);
    for (int i = 0; ok && i < w * h; ++i) ok = fwrite(rgba + 4 * i, 1, 3, f) == 3;
  } else if (ext == ".bmp") {
    const int row = (w * 3 + 3) & ~3;
    const uint32_t size = 54 + (uint32_t)row * h;
    unsigned char hd[54] = {'B', 'M'};
    auto le = [&](int off, uint32_t v, int n) { for (int i = 0; i < n; ++i) hd[off + i] = (unsigned char)(v >> (8 * i)); };
    le(2, size, 4); le(10, 54, 4); le(14, 40, 4); le(18, (uint32_t)w, 4); le(22, (uint32_t)h, 4);
    le(26, 1, 2); le(28, 24, 2); le(34, (uint32_t)row * h, 4);
    ok = fwrite(hd, 1, 54, f) == 54;
    std::vector<unsigned char> line(row, 0);
    for (int y = h - 1; ok && y >= 0; --y) {  // BMP rows run bottom-up
      for (int x = 0; x < w; ++x) {
        const unsigned char* p = rgba + 4 * ((size_t)y * w + x);
        line[3 * x] = p[2]; line[3 * x + 1] = p[1]; line[3 * x + 2] = p[0];
      }
      ok = fwrite(line.data(), 1, row, f) == (size_t)row;
    }
  } else {
    std::vector<unsigned char> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<unsigned char> ihdr;
    be32(ihdr, (uint32_t)w);
    be32(ihdr, (uint32_t)h);
    ihdr.push_back(8);
    ihdr.push_back(alpha ? 6 : 2);
    ihdr.push_back(0); ihdr.push_back(0); ihdr.push_back(0);
    chunk(png, "IHDR", ihdr);
    std::vector<unsigned char> raw;
    raw.reserve((size_t)h * (w * ch + 1));
    for (int y = 0; y < h; ++y) {
      raw.push_back(0);  // filter: none
      for (int x = 0; x < w; ++x) raw.insert(raw.end(), rgba + 4 * ((size_t)y * w + x), rgba + 4 * ((size_t)y * w + x) + ch);
    }
    std::vector<unsigned char> z = {0x78, 0x01};
    size_t pos = 0;
    uint32_t a = 1, b = 0;
    for (unsigned char c : raw) { a = (a + c) % 65521u; b = (b + a) % 65521u; }
    do {
      size_t n = raw.size() - pos;
      if (n > 65535) n = 65535;
      bool last = pos + n == raw.size();
      z.push_back(last ? 1 : 0);
      z.push_back((unsigned char)(n & 0xFF)); z.push_back((unsigned char)(n >> 8));
      z.push_back((unsigned char)(~n & 0xFF)); z.push_back((unsigned char)((~n >> 8) & 0xFF));
      z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
      pos += n;
    } while (pos < raw.size());
    be32(z, (b << 16) | a);
    chunk(png, "IDAT", z);
    chunk(png, "IEND", {});
    ok = fwrite(png.data(), 1, png.size(), f) == png.size();
  }
  fclose(f);
  return ok;
}

}  // namespace gbvr
