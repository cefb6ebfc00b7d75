// UVF container I/O and MD5 (RFC 1321).  See uvf.h for the layout notes.
#include "uvf.h"

#include <algorithm>
#include <cmath>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>

#include "../../include/gbvr.h"

namespace gbvr {

// ---------------------------------------------------------------------------
// MD5, written from RFC 1321: 64 steps per 512-bit block in four rounds,
// per-step constants floor(|sin(i + 1)| * 2^32).
// ---------------------------------------------------------------------------
static uint32_t md5_k[64];
static const int md5_r[64] = {7, 12, 17, 22, 7, 12, 17, 22, 7, 12, 17, 22, 7, 12, 17, 22,
                              5, 9,  14, 20, 5, 9,  14, 20, 5, 9,  14, 20, 5, 9,  14, 20,
                              4, 11, 16, 23, 4, 11, 16, 23, 4, 11, 16, 23, 4, 11, 16, 23,
                              6, 10, 15, 21, 6, 10, 15, 21, 6, 10, 15, 21, 6, 10, 15, 21};
static std::once_flag md5_once;
// Filled once, by whichever thread opens or writes a UVF file first.
static void md5_init_table() {
  std::call_once(md5_once, [] {
    for (int i = 0; i < 64; ++i)
      md5_k[i] = (uint32_t)(uint64_t)std::floor(std::fabs(std::sin((double)(i + 1))) * 4294967296.0);
  });
}

static inline uint32_t rotl(uint32_t x, int c) { return (x << c) | (x >> (32 - c)); }

static void md5_block(Md5& m, const unsigned char* p) {
  uint32_t w[16];
  for (int i = 0; i < 16; ++i)
    w[i] = (uint32_t)p[4 * i] | ((uint32_t)p[4 * i + 1] << 8) | ((uint32_t)p[4 * i + 2] << 16) | ((uint32_t)p[4 * i + 3] << 24);
  uint32_t a = m.a, b = m.b, c = m.c, d = m.d;
  for (int i = 0; i < 64; ++i) {
    uint32_t f;
    int g;
    if (i < 16) { f = (b & c) | (~b & d); g = i; }
    else if (i < 32) { f = (d & b) | (~d & c); g = (5 * i + 1) & 15; }
    else if (i < 48) { f = b ^ c ^ d; g = (3 * i + 5) & 15; }
    else { f = c ^ (b | ~d); g = (7 * i) & 15; }
    uint32_t t = d;
    d = c;
    c = b;
    b = b + rotl(a + f + md5_k[i] + w[g], md5_r[i]);
    a = t;
  }
  m.a += a; m.b += b; m.c += c; m.d += d;
}

Md5::Md5() : a(0x67452301u), b(0xefcdab89u), c(0x98badcfeu), d(0x10325476u), len(0), fill(0) { md5_init_table(); }

void Md5::update(const void* data, size_t n) {
  const unsigned char* p = (const unsigned char*)data;
  len += n;
  while (n > 0) {
    size_t take = 64 - fill;
    if (take > n) take = n;
    memcpy(buf + fill, p, take);
    fill += take;
    p += take;
    n -= take;
    if (fill == 64) {
      md5_block(*this, buf);
      fill = 0;
    }
  }
}

void Md5::final(unsigned char out[16]) {
  uint64_t bits = len * 8;
  unsigned char pad = 0x80;
  update(&pad, 1);
  unsigned char z = 0;
  while (fill != 56) update(&z, 1);
  unsigned char lb[8];
  for (int i = 0; i < 8; ++i) lb[i] = (unsigned char)(bits >> (8 * i));
  update(lb, 8);
  uint32_t v[4] = {a, b, c, d};
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) out[4 * i + j] = (unsigned char)(v[i] >> (8 * j));
}

// ---------------------------------------------------------------------------
// Reader
// ---------------------------------------------------------------------------
namespace {
struct File {
  FILE* f = nullptr;
  explicit File(const std::string& p, const char* mode) { f = fopen(p.c_str(), mode); }
  ~File() { if (f) fclose(f); }
};

bool rd(FILE* f, uint64_t off, void* dst, size_t n) {
  if (fseeko(f, (off_t)off, SEEK_SET) != 0) return false;
  return fread(dst, 1, n, f) == n;
}
bool rd64(FILE* f, uint64_t off, uint64_t& v) {
  unsigned char b[8];
  if (!rd(f, off, b, 8)) return false;
  v = 0;
  for (int i = 7; i >= 0; --i) v = (v << 8) | b[i];
  return true;
}
}  // namespace

namespace {
// a * b, false when it does not fit 64 bits
bool mul_ok(uint64_t a, uint64_t b, uint64_t& r) { return !__builtin_mul_overflow(a, b, &r); }
// count items of `each` bytes fit in [from, end)
bool fits(uint64_t from, uint64_t end, uint64_t count, uint64_t each) {
  if (from > end) return false;
  uint64_t bytes;
  return mul_ok(count, each, bytes) && bytes <= end - from;
}

// The parse proper.  Every read of a block's fields stays inside the block,
// every count read from the file is checked against the bytes that remain
// before anything is allocated, so a truncated or corrupted file ends in a
// status.
int uvf_parse(const std::string& path, bool verify, UvfFile& out, std::string& msg) {
  File fh(path, "rb");
  if (!fh.f) { msg = "cannot open " + path; return GBVR_EIO; }
  FILE* f = fh.f;
  fseeko(f, 0, SEEK_END);
  const uint64_t size = (uint64_t)ftello(f);
  char magic[8];
  if (size < 57 || !rd(f, 0, magic, 8) || memcmp(magic, "UVF-DATA", 8) != 0) {
    msg = "not a UVF file: " + path;
    return GBVR_EFORMAT;
  }
  unsigned char endian = 1;
  rd(f, 8, &endian, 1);
  if (endian != 0) { msg = "big-endian UVF is not supported"; return GBVR_EFORMAT; }
  uint64_t p = 9, cs_len = 0;
  if (!rd64(f, p, out.version) || !rd64(f, p + 8, out.checksum_semantic) || !rd64(f, p + 16, cs_len) || cs_len > 64) {
    msg = "truncated UVF global header";
    return GBVR_EFORMAT;
  }
  if (out.version < 2 || out.version > 3) { msg = "unsupported UVF version"; return GBVR_EFORMAT; }
  p += 24;
  out.checksum.resize(cs_len);
  if (cs_len && !rd(f, p, out.checksum.data(), cs_len)) { msg = "truncated checksum"; return GBVR_EFORMAT; }
  const uint64_t md5_from = p + cs_len;
  p += cs_len;
  uint64_t addl = 0;
  if (!rd64(f, p, addl) || addl > size - (p + 8)) { msg = "truncated UVF global header"; return GBVR_EFORMAT; }
  p += 8 + addl;
  if (verify && out.checksum_semantic == 2) {
    if (cs_len != 16) { msg = "MD5 checksum must be 16 bytes"; return GBVR_EFORMAT; }
    Md5 m;
    std::unique_ptr<unsigned char[]> buf(new unsigned char[1 << 20]);
    fseeko(f, (off_t)md5_from, SEEK_SET);
    size_t got;
    while ((got = fread(buf.get(), 1, 1 << 20, f)) > 0) m.update(buf.get(), got);
    unsigned char dg[16];
    m.final(dg);
    out.checksum_ok = memcmp(dg, out.checksum.data(), 16) == 0;
    if (!out.checksum_ok) { msg = "UVF MD5 checksum mismatch: " + path; return GBVR_ECHECKSUM; }
  }
  // blocks
  for (int guard = 0; guard < 4096; ++guard) {
    UvfBlock b;
    b.start = p;
    uint64_t slen = 0;
    if (p > size || !rd64(f, p, slen) || slen > (1 << 20) || slen + 32 > size - p) {
      msg = "truncated block header";
      return GBVR_EFORMAT;
    }
    b.id.resize(slen);
    if (slen) rd(f, p + 8, &b.id[0], slen);
    uint64_t q = p + 8 + slen;
    b.semantic = b.compression = b.next = 0;
    rd64(f, q, b.semantic);
    rd64(f, q + 8, b.compression);
    rd64(f, q + 16, b.next);
    b.payload = q + 24;
    out.blocks.push_back(b);
    if (b.next > size - b.start) { msg = "block extends past end of file"; return GBVR_EFORMAT; }
    const uint64_t end = b.next ? b.start + b.next : size;
    if (end < b.payload) { msg = "block extends past end of file"; return GBVR_EFORMAT; }
    // reads of the block's fields: inside [payload, end) or the parse fails
    bool ok = true;
    auto get = [&](uint64_t off, uint64_t& v) {
      v = 0;
      if (!(off >= b.payload && off <= end && end - off >= 8 && rd64(f, off, v))) ok = false;
    };
    if (b.compression != 0 && (b.semantic == 1 || b.semantic == 5 || b.semantic == 6 || b.semantic == 7)) {
      msg = "compressed UVF blocks are not supported";
      return GBVR_EFORMAT;
    }
    if (b.semantic == 1 && !out.has_raster) {
      UvfRaster& r = out.raster;
      r.id = b.id;
      uint64_t w = b.payload, nd = 0;
      get(w, nd);
      if (!ok || nd != 3) { msg = "raster block is not 3-dimensional"; return GBVR_EFORMAT; }
      w += 8 + 3 * 8;  // domain semantics
      for (int i = 0; i < 16; ++i) {
        uint64_t bits;
        get(w + 8 * i, bits);
        memcpy(&r.transform[i], &bits, 8);
      }
      w += 16 * 8;
      for (int i = 0; i < 3; ++i) get(w + 8 * i, r.dims[i]);
      w += 24;
      for (int i = 0; i < 3; ++i) get(w + 8 * i, r.brick_size[i]);
      w += 24;
      for (int i = 0; i < 3; ++i) get(w + 8 * i, r.overlap[i]);
      w += 24;
      for (int i = 0; i < 3; ++i) get(w + 8 * i, r.lod_factor[i]);
      w += 24;
      uint64_t ngroups = 0;
      for (int i = 0; i < 3; ++i) {
        get(w + 8 * i, r.lod_groups[i]);
        if (r.lod_groups[i] >= 64) { msg = "bad LOD groups in the raster block"; return GBVR_EFORMAT; }
        if (r.lod_groups[i] + 1 > ngroups) ngroups = r.lod_groups[i] + 1;
      }
      w += 24;
      if (!ok) { msg = "truncated raster block"; return GBVR_EFORMAT; }
      r.lod_counts.assign(ngroups, 1);
      for (uint64_t g = 0; g < ngroups; ++g) get(w + 8 * g, r.lod_counts[g]);
      w += 8 * ngroups;
      uint64_t nel = 0, eldim = 0;
      get(w, nel);
      get(w + 8, eldim);
      if (!ok) { msg = "truncated raster block"; return GBVR_EFORMAT; }
      if (nel != 1 || eldim != 1) { msg = "only scalar raster data is supported"; return GBVR_EFORMAT; }
      w += 16;
      get(w, r.elem_semantic);
      get(w + 8, r.bit_size);
      get(w + 16, r.mantissa);
      w += 24;
      unsigned char sg = 0;
      if (!(w < end && rd(f, w, &sg, 1))) ok = false;
      r.is_signed = sg != 0;
      w += 1;
      get(w, r.data_offset_field);
      w += 8;
      if (!ok) { msg = "truncated raster block"; return GBVR_EFORMAT; }
      if (r.bit_size != 8 && r.bit_size != 16 && r.bit_size != 32) {
        msg = "unsupported raster element size";
        return GBVR_EFORMAT;
      }
      // the voxels (finest level) must lie inside the file
      uint64_t nvox = 1, nbytes = 0;
      for (int i = 0; i < 3; ++i)
        if (r.dims[i] == 0 || !mul_ok(nvox, r.dims[i], nvox)) { msg = "bad raster dimensions"; return GBVR_EFORMAT; }
      if (!mul_ok(nvox, r.bit_size / 8, nbytes) || r.data_offset_field > size - w) {
        msg = "bad raster dimensions";
        return GBVR_EFORMAT;
      }
      r.data_pos = w + r.data_offset_field;
      if (nbytes > size - r.data_pos) { msg = "truncated raster data"; return GBVR_EFORMAT; }
      r.is_float = r.bit_size == 32 && r.mantissa == 23;
      out.has_raster = true;
    } else if (b.semantic == 5) {
      uint64_t n = 0;
      get(b.payload, n);
      if (!ok || !fits(b.payload + 8, end, n, 8)) { msg = "truncated 1D histogram"; return GBVR_EFORMAT; }
      out.hist1d.resize(n);
      for (uint64_t i = 0; i < n; ++i) get(b.payload + 8 + 8 * i, out.hist1d[i]);
      if (!ok) { msg = "truncated 1D histogram"; return GBVR_EFORMAT; }
    } else if (b.semantic == 6) {
      uint64_t nx = 0, ny = 0, n = 0;
      if (!(end - b.payload >= 4 && rd(f, b.payload, &out.hist2d_max_grad, 4))) ok = false;
      get(b.payload + 4, nx);
      get(b.payload + 12, ny);
      if (!ok || !mul_ok(nx, ny, n) || !fits(b.payload + 20, end, n, 8)) {
        msg = "truncated 2D histogram";
        return GBVR_EFORMAT;
      }
      out.hist2d_nx = nx;
      out.hist2d_ny = ny;
      out.hist2d.resize(n);
      std::vector<unsigned char> raw(8 * n);
      if (n && !rd(f, b.payload + 20, raw.data(), raw.size())) { msg = "truncated 2D histogram"; return GBVR_EFORMAT; }
      for (uint64_t i = 0; i < n; ++i) {
        uint64_t v = 0;
        for (int k = 7; k >= 0; --k) v = (v << 8) | raw[8 * i + k];
        out.hist2d[i] = v;
      }
      out.hist2d_id = b.id;
    } else if (b.semantic == 7) {
      uint64_t nb = 0, nc = 0, n = 0;
      get(b.payload, nb);
      get(b.payload + 8, nc);
      if (!ok || !mul_ok(nb, nc, n) || !fits(b.payload + 16, end, n, 32)) {
        msg = "truncated min/max block";
        return GBVR_EFORMAT;
      }
      out.minmax_components = nc;
      out.minmax.resize(n);
      for (uint64_t i = 0; i < n; ++i)
        if (!rd(f, b.payload + 16 + 32 * i, &out.minmax[i], 32)) { msg = "truncated min/max block"; return GBVR_EFORMAT; }
    } else if (b.semantic == 4) {
      uint64_t n = 0, w = b.payload;
      get(w, n);
      w += 8;
      for (uint64_t i = 0; ok && i < n && i < 4096; ++i) {
        uint64_t kl = 0, vl = 0;
        get(w, kl);
        if (!ok || kl > end - (w + 8)) break;
        std::string k(kl, '\0');
        if (kl) rd(f, w + 8, &k[0], kl);
        w += 8 + kl;
        get(w, vl);
        if (!ok || vl > end - (w + 8)) break;
        std::string v(vl, '\0');
        if (vl) rd(f, w + 8, &v[0], vl);
        w += 8 + vl;
        out.kv.emplace_back(k, v);
      }
      if (!ok || out.kv.size() < std::min<uint64_t>(n, 4096)) { msg = "truncated key/value block"; return GBVR_EFORMAT; }
    }
    if (b.next == 0) break;
    p = b.start + b.next;
  }
  if (!out.has_raster) { msg = "UVF file holds no raster data block"; return GBVR_EFORMAT; }
  return GBVR_OK;
}
}  // namespace

int uvf_read(const std::string& path, bool verify, UvfFile& out, std::string& msg) {
  try {
    return uvf_parse(path, verify, out, msg);
  } catch (const std::bad_alloc&) {
    msg = "out of host memory reading " + path;
    return GBVR_ENOMEM;
  } catch (const std::exception& e) {
    msg = std::string("UVF read failed: ") + e.what();
    return GBVR_EFORMAT;
  }
}

int uvf_read_voxels(const std::string& path, const UvfFile& uf, void* out, size_t bytes, std::string& msg) {
  File fh(path, "rb");
  if (!fh.f) { msg = "cannot open " + path; return GBVR_EIO; }
  if (!rd(fh.f, uf.raster.data_pos, out, bytes)) { msg = "truncated raster data"; return GBVR_EFORMAT; }
  return GBVR_OK;
}

// ---------------------------------------------------------------------------
// Writer
// ---------------------------------------------------------------------------
namespace {
struct Buf {
  std::vector<unsigned char> v;
  void u64(uint64_t x) { for (int i = 0; i < 8; ++i) v.push_back((unsigned char)(x >> (8 * i))); }
  void f64(double d) { uint64_t b; memcpy(&b, &d, 8); u64(b); }
  void f32(float f) { unsigned char b[4]; memcpy(b, &f, 4); v.insert(v.end(), b, b + 4); }
  void bytes(const void* p, size_t n) { v.insert(v.end(), (const unsigned char*)p, (const unsigned char*)p + n); }
  void str(const std::string& s) { u64(s.size()); bytes(s.data(), s.size()); }
};

void block_header(Buf& b, const std::string& id, uint64_t sem, uint64_t next) {
  b.str(id);
  b.u64(sem);
  b.u64(0);  // no compression
  b.u64(next);
}
}  // namespace

int uvf_write(const std::string& path, const UvfWriteSpec& s, std::string& msg) {
  // Each block is assembled in memory except the raster voxels, which are
  // streamed; block sizes are known up front so every "next" offset is exact.
  std::vector<Buf> blocks;
  std::vector<uint64_t> voxel_tail;  // voxel bytes appended after block i's header/payload
  // raster
  {
    Buf h;
    const UvfRaster& r = s.raster;
    Buf p;
    p.u64(3);
    p.u64(1); p.u64(2); p.u64(3);
    for (int i = 0; i < 16; ++i) p.f64(r.transform[i]);
    for (int i = 0; i < 3; ++i) p.u64(r.dims[i]);
    for (int i = 0; i < 3; ++i) p.u64(r.brick_size[i]);
    for (int i = 0; i < 3; ++i) p.u64(r.overlap[i]);
    for (int i = 0; i < 3; ++i) p.u64(r.lod_factor[i]);
    for (int i = 0; i < 3; ++i) p.u64(r.lod_groups[i]);
    for (uint64_t c : r.lod_counts) p.u64(c);
    p.u64(1);
    p.u64(1);
    p.u64(r.elem_semantic);
    p.u64(r.bit_size);
    p.u64(r.mantissa);
    unsigned char sg = r.is_signed ? 1 : 0;
    p.bytes(&sg, 1);
    p.u64(0);
    const uint64_t hdr = 8 + r.id.size() + 24;
    const bool last = s.hist1d.empty() && s.hist2d.empty() && s.minmax.empty() && s.kv.empty();
    block_header(h, r.id, 1, last ? 0 : hdr + p.v.size() + s.voxel_bytes);
    h.bytes(p.v.data(), p.v.size());
    blocks.push_back(h);
    voxel_tail.push_back(s.voxel_bytes);
  }
  std::vector<Buf> rest;
  if (!s.hist1d.empty()) {
    Buf p;
    p.u64(s.hist1d.size());
    for (uint64_t x : s.hist1d) p.u64(x);
    rest.push_back(p);
  }
  std::vector<std::string> ids;
  std::vector<uint64_t> sems;
  if (!s.hist1d.empty()) { ids.push_back(s.hist1d_id); sems.push_back(5); }
  if (!s.hist2d.empty()) {
    Buf p;
    p.f32(s.hist2d_max_grad);
    p.u64(s.hist2d_nx);
    p.u64(s.hist2d_ny);
    for (uint64_t x : s.hist2d) p.u64(x);
    rest.push_back(p);
    ids.push_back("2D Histogram for datablock " + s.raster.id);
    sems.push_back(6);
  }
  if (!s.minmax.empty()) {
    Buf p;
    p.u64(s.minmax.size());
    p.u64(1);
    for (const UvfMinMax& m : s.minmax) {
      p.f64(m.min_scalar); p.f64(m.max_scalar); p.f64(m.min_grad); p.f64(m.max_grad);
    }
    rest.push_back(p);
    ids.push_back(s.minmax_id);
    sems.push_back(7);
  }
  if (!s.kv.empty()) {
    Buf p;
    p.u64(s.kv.size());
    for (auto& kv : s.kv) { p.str(kv.first); p.str(kv.second); }
    rest.push_back(p);
    ids.push_back("Key/Value Pairs");
    sems.push_back(4);
  }
  for (size_t i = 0; i < rest.size(); ++i) {
    Buf h;
    const uint64_t hdr = 8 + ids[i].size() + 24;
    block_header(h, ids[i], sems[i], i + 1 == rest.size() ? 0 : hdr + rest[i].v.size());
    h.bytes(rest[i].v.data(), rest[i].v.size());
    blocks.push_back(h);
    voxel_tail.push_back(0);
  }
  // global header with a zero checksum, patched after hashing
  Buf g;
  g.bytes("UVF-DATA", 8);
  unsigned char endian = 0;
  g.bytes(&endian, 1);
  g.u64(2);
  g.u64(2);
  g.u64(16);
  const size_t cs_pos = g.v.size();
  unsigned char zero[16] = {0};
  g.bytes(zero, 16);
  g.u64(0);  // additional header bytes
  Md5 m;
  m.update(g.v.data() + 49, g.v.size() - 49);
  for (size_t i = 0; i < blocks.size(); ++i) {
    m.update(blocks[i].v.data(), blocks[i].v.size());
    if (voxel_tail[i]) m.update(s.voxels, s.voxel_bytes);
  }
  unsigned char dg[16];
  m.final(dg);
  memcpy(g.v.data() + cs_pos, dg, 16);
  File fh(path, "wb");
  if (!fh.f) { msg = "cannot create " + path; return GBVR_EIO; }
  bool ok = fwrite(g.v.data(), 1, g.v.size(), fh.f) == g.v.size();
  for (size_t i = 0; ok && i < blocks.size(); ++i) {
    ok = fwrite(blocks[i].v.data(), 1, blocks[i].v.size(), fh.f) == blocks[i].v.size();
    if (ok && voxel_tail[i]) ok = fwrite(s.voxels, 1, s.voxel_bytes, fh.f) == s.voxel_bytes;
  }
  if (!ok) { msg = "write failed: " + path; return GBVR_EIO; }
  return GBVR_OK;
}

}  // namespace gbvr
