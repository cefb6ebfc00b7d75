// LZ4 block format (the codec CT_LZ4 = 3 of the UVF brick compression ids,
// UVFReader/BlockInfo.h:60-93 and CmdLineConverter/main.cpp:175-178),
// restated from the published block format description:
//   a block is a sequence of sequences; each starts with a token byte whose
//   high nibble is the literal count and low nibble the match length minus 4
//   (15 = more length bytes follow, each added, until one below 255), then
//   the literals, then a 2-byte little-endian match offset (1 .. 65535 bytes
//   back into the output) and the match length bytes.  The last sequence has
//   literals only; the last 5 bytes of a block are literals and the last
//   match starts at least 12 bytes before the block's end.
// The compressor is a greedy hash-chain matcher: every position is linked
// into the chain of its 4-byte hash, and at each position up to `chain`
// earlier positions of that chain within 65535 bytes are compared, the
// longest match winning (the nearest on ties), and taken when it is at least
// `min_match` bytes long (4, the format's minimum, by default; a larger one
// trades ratio for fewer sequences).  Fewer, longer sequences make a faster
// decode, whose cost on the GPU is per sequence.  The host decoder checks every bound and fails on malformed
// input; the GPU decoder is in kernels_build.cu.
#include "lz4.h"

#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/gbvr.h"
#include "abi_guard.h"

namespace gbvr {

namespace {
constexpr int kHashBits = 14;
constexpr size_t kMinMatch = 4, kLastLiterals = 5, kMatchLimit = 12, kMaxOffset = 65535;

inline uint32_t rd32(const uint8_t* p) {
  uint32_t v;
  memcpy(&v, p, 4);
  return v;
}

inline uint32_t hash4(uint32_t v) { return (v * 2654435761u) >> (32 - kHashBits); }

// a length above 14 (literals) or 18 (matches): the nibble is 15 and the
// remainder goes in bytes of 255 and a last one below 255
inline bool put_len(uint8_t*& op, const uint8_t* oend, size_t rem) {
  while (rem >= 255) {
    if (op >= oend) return false;
    *op++ = 255;
    rem -= 255;
  }
  if (op >= oend) return false;
  *op++ = (uint8_t)rem;
  return true;
}

bool emit(uint8_t*& op, const uint8_t* oend, const uint8_t* lit, size_t nlit, size_t off, size_t mlen) {
  if (op >= oend) return false;
  uint8_t* token = op++;
  const size_t ln = nlit < 15 ? nlit : 15;
  *token = (uint8_t)(ln << 4);
  if (nlit >= 15 && !put_len(op, oend, nlit - 15)) return false;
  if ((size_t)(oend - op) < nlit) return false;
  memcpy(op, lit, nlit);
  op += nlit;
  if (mlen == 0) return true;  // the last sequence
  if (oend - op < 2) return false;
  *op++ = (uint8_t)(off & 0xff);
  *op++ = (uint8_t)(off >> 8);
  const size_t m = mlen - kMinMatch;
  *token |= (uint8_t)(m < 15 ? m : 15);
  if (m >= 15 && !put_len(op, oend, m - 15)) return false;
  return true;
}
}  // namespace

size_t lz4_bound(size_t n) { return n + n / 255 + 16; }

// Compress src[0, n) into dst (capacity cap); returns the compressed size or
// 0 when it does not fit.
size_t lz4_compress(const uint8_t* src, size_t n, uint8_t* dst, size_t cap, int chain, int min_match) {
  uint8_t* op = dst;
  const uint8_t* oend = dst + cap;
  size_t anchor = 0;
  if (chain < 1) chain = 1;
  if (n >= kMatchLimit + 1) {
    // head: latest position of each hash; prev: the previous position of the
    // same hash, per position modulo the 64 KiB window
    std::vector<int32_t> head((size_t)1 << kHashBits, -1);
    std::vector<int32_t> prev((size_t)1 << 16, -1);
    const size_t last_start = n - kMatchLimit;   // a match starts before this
    const size_t match_end = n - kLastLiterals;  // and ends at or before this
    size_t ins = 0;                              // positions below this are linked
    auto link_to = [&](size_t end) {
      for (; ins < end; ++ins) {
        const uint32_t h = hash4(rd32(src + ins));
        prev[ins & 0xffff] = head[h];
        head[h] = (int32_t)ins;
      }
    };
    size_t ip = 0;
    while (ip < last_start) {
      link_to(ip);
      const uint32_t seq = rd32(src + ip);
      size_t best_len = 0, best_off = 0;
      int32_t ref = head[hash4(seq)];
      for (int k = 0; k < chain && ref >= 0 && ip - (size_t)ref <= kMaxOffset; ++k) {
        if (rd32(src + ref) == seq) {
          size_t len = kMinMatch;
          while (ip + len < match_end && src[ref + len] == src[ip + len]) ++len;
          if (len > best_len) {
            best_len = len;
            best_off = ip - (size_t)ref;
            if (ip + len >= match_end) break;
          }
        }
        const int32_t nx = prev[(size_t)ref & 0xffff];
        if (nx >= ref) break;  // the window wrapped past this chain
        ref = nx;
      }
      if (best_len && best_len >= (size_t)min_match) {
        if (!emit(op, oend, src + anchor, ip - anchor, best_off, best_len)) return 0;
        ip += best_len;
        anchor = ip;
      } else {
        ++ip;
      }
    }
  }
  if (!emit(op, oend, src + anchor, n - anchor, 0, 0)) return 0;
  return (size_t)(op - dst);
}

// Decode a block of `in_n` bytes into exactly `out_n` bytes; false when the
// block is malformed or does not produce exactly out_n bytes.
bool lz4_decompress(const uint8_t* in, size_t in_n, uint8_t* out, size_t out_n) {
  size_t ip = 0, op = 0;
  for (;;) {
    if (ip >= in_n) return false;
    const uint8_t token = in[ip++];
    size_t nlit = token >> 4;
    if (nlit == 15) {
      uint8_t b;
      do {
        if (ip >= in_n) return false;
        b = in[ip++];
        nlit += b;
      } while (b == 255);
    }
    if (nlit > in_n - ip || nlit > out_n - op) return false;
    memcpy(out + op, in + ip, nlit);
    ip += nlit;
    op += nlit;
    if (ip == in_n) return op == out_n;  // the last sequence
    if (in_n - ip < 2) return false;
    const size_t off = (size_t)in[ip] | ((size_t)in[ip + 1] << 8);
    ip += 2;
    size_t mlen = (token & 15);
    if (mlen == 15) {
      uint8_t b;
      do {
        if (ip >= in_n) return false;
        b = in[ip++];
        mlen += b;
      } while (b == 255);
    }
    mlen += kMinMatch;
    if (off == 0 || off > op || mlen > out_n - op) return false;
    for (size_t i = 0; i < mlen; ++i) out[op + i] = out[op - off + i];  // may overlap: byte order
    op += mlen;
  }
}

}  // namespace gbvr

extern "C" {

size_t gbvr_lz4_bound(size_t n) { return gbvr::lz4_bound(n); }

size_t gbvr_lz4_compress(const void* src, size_t n, void* dst, size_t cap) {
  GBVR_ABI_TRY
  if (!src || !dst) return 0;
  return gbvr::lz4_compress((const uint8_t*)src, n, (uint8_t*)dst, cap, 16);
  GBVR_ABI_CATCH_SIZE
}

int gbvr_lz4_decompress(const void* src, size_t n, void* dst, size_t out_n) {
  GBVR_ABI_TRY
  if (!src || !dst) return GBVR_EINVAL;
  return gbvr::lz4_decompress((const uint8_t*)src, n, (uint8_t*)dst, out_n) ? GBVR_OK : GBVR_EFORMAT;
  GBVR_ABI_CATCH
}

}  // extern "C"
