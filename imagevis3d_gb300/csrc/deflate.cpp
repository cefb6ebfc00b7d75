// zlib / DEFLATE codec, host side, written from RFC 1950 (zlib stream format)
// and RFC 1951 (DEFLATE).  The encoder is this library's own: greedy LZ77 over
// hash chains, dynamic Huffman codes limited to the format's code lengths by
// lengthening and refilling to a complete code, stored blocks where that is
// smaller.  The decoder reads every block type and checks the stream.
#include "deflate.h"

#include <algorithm>
#include <cstring>
#include <queue>
#include <vector>

#include "../../include/gbvr.h"
#include "abi_guard.h"

namespace gbvr {

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

uint32_t adler32(const uint8_t* p, size_t n) {
  constexpr uint32_t M = 65521;  // the largest prime below 2^16
  uint32_t a = 1, b = 0;
  while (n) {
    // the modulo can wait while b stays below 2^32: after k bytes b grows by at
    // most 255 k (k + 1) / 2 + (k + 1) (M - 1), which fits for k = 5000
    size_t k = std::min<size_t>(n, 5000);
    n -= k;
    for (; k; --k) {
      a += *p++;
      b += a;
    }
    a %= M;
    b %= M;
  }
  return (b << 16) | a;
}

namespace {

constexpr size_t kWindow = 32768;
// input bytes per DEFLATE block: a block that ends in a match (at most 258
// bytes past this) still fits one stored block of at most 65535 bytes
constexpr size_t kBlockInput = 65535 - 258;
constexpr int kMinMatch = 3, kMaxMatch = 258;

struct BitOut {
  uint8_t* p;
  size_t cap, n = 0;
  uint64_t acc = 0;
  int bits = 0;
  bool over = false;
  void byte(uint8_t b) {
    if (n < cap) p[n] = b;
    else over = true;
    ++n;
  }
  void put(uint32_t v, int nb) {  // nb <= 32, least significant bit first
    acc |= (uint64_t)v << bits;
    bits += nb;
    while (bits >= 8) {
      byte((uint8_t)acc);
      acc >>= 8;
      bits -= 8;
    }
  }
  void align() {
    if (bits) byte((uint8_t)acc);
    acc = 0;
    bits = 0;
  }
};

uint32_t reverse_bits(uint32_t c, int len) {
  uint32_t r = 0;
  for (int i = 0; i < len; ++i) {
    r = (r << 1) | (c & 1u);
    c >>= 1;
  }
  return r;
}

// Canonical codes from code lengths (RFC 1951 3.2.2), bit-reversed because
// DEFLATE sends Huffman codes most significant bit first into an LSB-first
// stream.
void canonical_codes(const uint8_t* len, int n, uint16_t* code) {
  int count[16] = {0};
  for (int i = 0; i < n; ++i) ++count[len[i]];
  count[0] = 0;
  int next[16] = {0};
  int c = 0;
  for (int b = 1; b < 16; ++b) {
    c = (c + count[b - 1]) << 1;
    next[b] = c;
  }
  for (int i = 0; i < n; ++i) code[i] = len[i] ? (uint16_t)reverse_bits((uint32_t)next[len[i]]++, len[i]) : 0;
}

// Huffman code lengths of at most maxbits for the frequencies, forming a
// complete code (every DEFLATE decoder accepts it): a single used symbol gets
// a partner of length 1; lengths above maxbits are cut to maxbits, then the
// longest codes below the limit are lengthened until the code is not
// over-subscribed, then the longest codes are shortened until it is complete.
void huff_lengths(const uint32_t* freq, int n, int maxbits, uint8_t* len) {
  std::fill(len, len + n, 0);
  std::vector<int> used;
  for (int i = 0; i < n; ++i)
    if (freq[i]) used.push_back(i);
  if (used.size() < 2) {
    const int a = used.empty() ? 0 : used[0];
    len[a] = 1;
    len[a == 0 ? 1 : 0] = 1;
    return;
  }
  struct Node {
    uint64_t w;
    int left, right, sym;
  };
  std::vector<Node> nodes;
  typedef std::pair<uint64_t, int> Item;
  std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
  for (int s : used) {
    nodes.push_back({freq[s], -1, -1, s});
    heap.push({freq[s], (int)nodes.size() - 1});
  }
  while (heap.size() > 1) {
    const Item a = heap.top();
    heap.pop();
    const Item b = heap.top();
    heap.pop();
    nodes.push_back({a.first + b.first, a.second, b.second, -1});
    heap.push({a.first + b.first, (int)nodes.size() - 1});
  }
  std::vector<int> depth(nodes.size(), 0);
  for (int i = (int)nodes.size() - 1; i >= 0; --i) {  // parents come after their children
    if (nodes[i].left >= 0) {
      depth[nodes[i].left] = depth[i] + 1;
      depth[nodes[i].right] = depth[i] + 1;
    }
  }
  for (size_t i = 0; i < nodes.size(); ++i)
    if (nodes[i].sym >= 0) len[nodes[i].sym] = (uint8_t)std::min(depth[i], maxbits);
  const uint64_t full = 1ull << maxbits;
  uint64_t kraft = 0;
  for (int s : used) kraft += 1ull << (maxbits - len[s]);
  while (kraft > full) {  // lengthen the longest code below the limit (the least frequent on a tie)
    int pick = -1;
    for (int s : used)
      if (len[s] < maxbits && (pick < 0 || len[s] > len[pick] || (len[s] == len[pick] && freq[s] < freq[pick])))
        pick = s;
    kraft -= 1ull << (maxbits - len[pick] - 1);
    ++len[pick];
  }
  while (kraft < full) {  // shorten the longest code whose shortening still fits (the most frequent on a tie)
    int pick = -1;
    for (int s : used)
      if (len[s] > 1 && kraft + (1ull << (maxbits - len[s])) <= full &&
          (pick < 0 || len[s] > len[pick] || (len[s] == len[pick] && freq[s] > freq[pick])))
        pick = s;
    if (pick < 0) break;
    kraft += 1ull << (maxbits - len[pick]);
    --len[pick];
  }
}

int len_code(int L) {  // 3..258 -> 0..28 (symbol 257 + index)
  int i = 28;
  while (kLenBase[i] > L) --i;
  return i;
}
int dist_code(int d) {  // 1..32768 -> 0..29
  int i = 29;
  while (kDistBase[i] > d) --i;
  return i;
}

struct Token {
  uint16_t v;     // literal byte, or match length
  uint16_t dist;  // 0 for a literal
};

// Code-length sequence of HLIT + HDIST lengths, run-length coded with the
// symbols 16 (repeat previous 3-6), 17 (3-10 zeros), 18 (11-138 zeros).
void rle_lengths(const uint8_t* l, int n, std::vector<std::pair<int, int>>& out) {
  for (int i = 0; i < n;) {
    int run = 1;
    while (i + run < n && l[i + run] == l[i]) ++run;
    if (l[i] == 0) {
      int r = run;
      while (r >= 11) {
        const int k = std::min(r, 138);
        out.push_back({18, k - 11});
        r -= k;
      }
      if (r >= 3) {
        out.push_back({17, r - 3});
        r = 0;
      }
      while (r-- > 0) out.push_back({0, 0});
    } else {
      out.push_back({l[i], 0});
      int r = run - 1;
      while (r >= 3) {
        const int k = std::min(r, 6);
        out.push_back({16, k - 3});
        r -= k;
      }
      while (r-- > 0) out.push_back({l[i], 0});
    }
    i += run;
  }
}

// One block of tokens covering input [s0, s1): dynamic Huffman, or stored
// blocks (at most 65535 bytes each) when that is smaller.
void emit_block(BitOut& bo, const std::vector<Token>& tok, size_t t0, size_t t1, const uint8_t* in, size_t s0,
                size_t s1, bool last) {
  uint32_t lf[286] = {0}, df[30] = {0};
  for (size_t t = t0; t < t1; ++t) {
    if (tok[t].dist == 0) ++lf[tok[t].v];
    else {
      ++lf[257 + len_code(tok[t].v)];
      ++df[dist_code(tok[t].dist)];
    }
  }
  lf[256] = 1;
  uint8_t ll[286], dl[30];
  huff_lengths(lf, 286, 15, ll);
  huff_lengths(df, 30, 15, dl);
  int hlit = 286, hdist = 30;
  while (hlit > 257 && ll[hlit - 1] == 0) --hlit;
  while (hdist > 1 && dl[hdist - 1] == 0) --hdist;
  uint8_t all[316];
  memcpy(all, ll, hlit);
  memcpy(all + hlit, dl, hdist);
  std::vector<std::pair<int, int>> rle;
  rle_lengths(all, hlit + hdist, rle);
  uint32_t cf[19] = {0};
  for (auto& e : rle) ++cf[e.first];
  uint8_t cl[19];
  huff_lengths(cf, 19, 7, cl);
  int hclen = 19;
  while (hclen > 4 && cl[kClOrder[hclen - 1]] == 0) --hclen;
  // sizes in bits
  uint64_t dyn = 3 + 5 + 5 + 4 + 3 * (uint64_t)hclen;
  for (auto& e : rle) dyn += cl[e.first] + (e.first == 16 ? 2 : e.first == 17 ? 3 : e.first == 18 ? 7 : 0);
  for (int s = 0; s < 286; ++s) dyn += (uint64_t)lf[s] * ll[s];
  for (int s = 257; s < 286; ++s) dyn += (uint64_t)lf[s] * kLenExtra[s - 257];
  for (int s = 0; s < 30; ++s) dyn += (uint64_t)df[s] * (dl[s] + kDistExtra[s]);
  const uint64_t stored = (3 + 7 + 32) * ((s1 - s0) / 65535 + 1) + 8 * (uint64_t)(s1 - s0);
  if (stored <= dyn) {
    for (size_t a = s0;;) {
      const size_t b = std::min(s1, a + 65535);
      bo.put(last && b == s1 ? 1 : 0, 1);
      bo.put(0, 2);
      bo.align();
      const uint32_t L = (uint32_t)(b - a);
      bo.put(L & 0xffffu, 16);
      bo.put(~L & 0xffffu, 16);
      for (size_t i = a; i < b; ++i) bo.byte(in[i]);
      if (b == s1) break;
      a = b;
    }
    return;
  }
  uint16_t lc[286], dc[30], cc[19];
  canonical_codes(ll, 286, lc);
  canonical_codes(dl, 30, dc);
  canonical_codes(cl, 19, cc);
  bo.put(last ? 1 : 0, 1);
  bo.put(2, 2);
  bo.put((uint32_t)(hlit - 257), 5);
  bo.put((uint32_t)(hdist - 1), 5);
  bo.put((uint32_t)(hclen - 4), 4);
  for (int i = 0; i < hclen; ++i) bo.put(cl[kClOrder[i]], 3);
  for (auto& e : rle) {
    bo.put(cc[e.first], cl[e.first]);
    if (e.first == 16) bo.put((uint32_t)e.second, 2);
    else if (e.first == 17) bo.put((uint32_t)e.second, 3);
    else if (e.first == 18) bo.put((uint32_t)e.second, 7);
  }
  for (size_t t = t0; t < t1; ++t) {
    if (tok[t].dist == 0) {
      bo.put(lc[tok[t].v], ll[tok[t].v]);
    } else {
      const int li = len_code(tok[t].v), di = dist_code(tok[t].dist);
      bo.put(lc[257 + li], ll[257 + li]);
      if (kLenExtra[li]) bo.put((uint32_t)(tok[t].v - kLenBase[li]), kLenExtra[li]);
      bo.put(dc[di], dl[di]);
      if (kDistExtra[di]) bo.put((uint32_t)(tok[t].dist - kDistBase[di]), kDistExtra[di]);
    }
  }
  bo.put(lc[256], ll[256]);
}

// ---- decoding ----
struct BitIn {
  const uint8_t* p;
  size_t n, pos = 0;
  uint64_t acc = 0;
  int bits = 0;
  size_t past = 0;  // bytes taken beyond the input (zeros)
  void need(int k) {
    while (bits < k) {
      uint64_t b = 0;
      if (pos < n) b = p[pos];
      else ++past;
      ++pos;
      acc |= b << bits;
      bits += 8;
    }
  }
  uint32_t get(int k) {  // k <= 32
    if (k == 0) return 0;
    need(k);
    const uint32_t v = (uint32_t)(acc & ((1ull << k) - 1));
    acc >>= k;
    bits -= k;
    return v;
  }
  // bits beyond the input were consumed
  bool exhausted() const { return past > 0 && (uint64_t)bits < 8 * past; }
};

// Canonical decoding: per length the number of codes and the symbols in code
// order; a code of length l is decoded by comparing against the first code of
// that length.
struct Huff {
  int count[16];
  int sym[320];
  bool build(const uint8_t* len, int n) {
    for (int& c : count) c = 0;
    for (int i = 0; i < n; ++i) ++count[len[i]];
    count[0] = 0;
    int left = 1;
    for (int b = 1; b < 16; ++b) {
      left = 2 * left - count[b];
      if (left < 0) return false;  // over-subscribed
    }
    int offs[16];
    offs[1] = 0;
    for (int b = 1; b < 15; ++b) offs[b + 1] = offs[b] + count[b];
    for (int i = 0; i < n; ++i)
      if (len[i]) sym[offs[len[i]]++] = i;
    return true;
  }
  int decode(BitIn& in) const {
    int code = 0, first = 0, index = 0;
    for (int b = 1; b < 16; ++b) {
      code |= (int)in.get(1);
      const int c = count[b];
      if (code - first < c) return sym[index + code - first];
      index += c;
      first = (first + c) << 1;
      code <<= 1;
    }
    return -1;
  }
};

// The fixed codes' lengths (RFC 1951 3.2.6).
struct FixedLengths {
  uint8_t ll[288], dl[30];
  FixedLengths() {
    for (int i = 0; i < 288; ++i) ll[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
    for (int i = 0; i < 30; ++i) dl[i] = 5;
  }
};

}  // namespace

size_t zlib_bound(size_t n) { return n + 5 * (n / (kBlockInput - 1) + 1) + 6; }

size_t zlib_compress(const void* src, size_t n, void* dst, size_t cap, int chain) {
  const uint8_t* in = (const uint8_t*)src;
  BitOut bo{(uint8_t*)dst, cap};
  bo.byte(0x78);  // CM 8 (deflate), CINFO 7 (32 KiB window)
  bo.byte(0x9C);  // FLEVEL 2, no dictionary; (0x78 * 256 + 0x9C) % 31 == 0
  std::vector<int> head(1 << 15, -1), prev(std::max<size_t>(n, 1), -1);
  auto hash = [&](size_t i) { return ((in[i] << 10) ^ (in[i + 1] << 5) ^ in[i + 2]) & 0x7fff; };
  auto insert = [&](size_t i) {
    if (i + kMinMatch > n) return;
    const int h = hash(i);
    prev[i] = head[h];
    head[h] = (int)i;
  };
  std::vector<Token> tok;
  size_t i = 0, block_start = 0, block_tok = 0;
  if (n == 0) emit_block(bo, tok, 0, 0, in, 0, 0, true);
  while (i < n) {
    int best = 0, best_d = 0;
    if (i + kMinMatch <= n) {
      int cand = head[hash(i)];
      const int maxl = (int)std::min<size_t>(kMaxMatch, n - i);
      for (int depth = chain; cand >= 0 && i - (size_t)cand <= kWindow && depth > 0; --depth) {
        if (in[cand + best] == in[i + best]) {
          int l = 0;
          while (l < maxl && in[cand + l] == in[i + l]) ++l;
          if (l > best) {
            best = l;
            best_d = (int)(i - cand);
            if (l == maxl) break;
          }
        }
        cand = prev[cand];
      }
    }
    if (best >= kMinMatch) {
      tok.push_back({(uint16_t)best, (uint16_t)best_d});
      for (int k = 0; k < best; ++k) insert(i + k);
      i += best;
    } else {
      tok.push_back({in[i], 0});
      insert(i);
      ++i;
    }
    if (i - block_start >= kBlockInput || i == n) {
      emit_block(bo, tok, block_tok, tok.size(), in, block_start, i, i == n);
      block_start = i;
      block_tok = tok.size();
    }
  }
  bo.align();
  const uint32_t ad = adler32(in, n);
  for (int s = 24; s >= 0; s -= 8) bo.byte((uint8_t)(ad >> s));
  return bo.over ? 0 : bo.n;
}

bool zlib_decompress(const void* src, size_t n, void* dst, size_t out_n) {
  const uint8_t* p = (const uint8_t*)src;
  uint8_t* out = (uint8_t*)dst;
  if (n < 6) return false;
  const unsigned cmf = p[0], flg = p[1];
  if ((cmf & 15) != 8 || (cmf >> 4) > 7 || (cmf * 256 + flg) % 31 != 0 || (flg & 0x20)) return false;
  BitIn in{p + 2, n - 6};  // the Adler-32 is not DEFLATE input
  size_t o = 0;
  static const FixedLengths fixed;  // initialised once, thread-safely
  for (bool last = false; !last;) {
    last = in.get(1) != 0;
    const unsigned type = in.get(2);
    if (in.exhausted()) return false;
    if (type == 0) {
      in.get(in.bits & 7);  // to the byte boundary
      const uint32_t L = in.get(16), NL = in.get(16);
      if (in.exhausted() || (L ^ 0xffffu) != NL || o + L > out_n) return false;
      for (uint32_t k = 0; k < L; ++k) {
        out[o++] = (uint8_t)in.get(8);
        if (in.exhausted()) return false;
      }
      continue;
    }
    if (type == 3) return false;
    Huff lit, dist;
    if (type == 1) {
      lit.build(fixed.ll, 288);
      dist.build(fixed.dl, 30);
    } else {
      const int hlit = (int)in.get(5) + 257, hdist = (int)in.get(5) + 1, hclen = (int)in.get(4) + 4;
      if (hlit > 286 || hdist > 30) return false;
      uint8_t cl[19] = {0};
      for (int k = 0; k < hclen; ++k) cl[kClOrder[k]] = (uint8_t)in.get(3);
      Huff clh;
      if (!clh.build(cl, 19)) return false;
      uint8_t lens[316] = {0};
      for (int k = 0; k < hlit + hdist;) {
        const int s = clh.decode(in);
        if (s < 0 || in.exhausted()) return false;
        if (s < 16) {
          lens[k++] = (uint8_t)s;
        } else {
          int rep, val = 0;
          if (s == 16) {
            if (k == 0) return false;
            val = lens[k - 1];
            rep = 3 + (int)in.get(2);
          } else if (s == 17) {
            rep = 3 + (int)in.get(3);
          } else {
            rep = 11 + (int)in.get(7);
          }
          if (k + rep > hlit + hdist) return false;
          while (rep--) lens[k++] = (uint8_t)val;
        }
      }
      if (lens[256] == 0) return false;
      if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist)) return false;
    }
    for (;;) {
      const int s = lit.decode(in);
      if (s < 0 || in.exhausted()) return false;
      if (s < 256) {
        if (o >= out_n) return false;
        out[o++] = (uint8_t)s;
      } else if (s == 256) {
        break;
      } else {
        const int li = s - 257;
        if (li >= 29) return false;
        const size_t L = kLenBase[li] + in.get(kLenExtra[li]);
        const int ds = dist.decode(in);
        if (ds < 0 || ds >= 30) return false;
        const size_t D = kDistBase[ds] + in.get(kDistExtra[ds]);
        if (in.exhausted() || D > o || o + L > out_n) return false;
        for (size_t k = 0; k < L; ++k, ++o) out[o] = out[o - D];
      }
    }
  }
  if (o != out_n) return false;
  // the Adler-32 follows the last block at the next byte boundary
  const size_t used = in.pos - (size_t)(in.bits / 8);
  if (used + 4 > n - 2) return false;
  const uint8_t* a = p + 2 + used;
  const uint32_t want = ((uint32_t)a[0] << 24) | ((uint32_t)a[1] << 16) | ((uint32_t)a[2] << 8) | a[3];
  return want == adler32(out, out_n);
}

}  // namespace gbvr

// ---- C ABI (host only) ----
extern "C" {

size_t gbvr_zlib_bound(size_t n) { return gbvr::zlib_bound(n); }

size_t gbvr_zlib_compress(const void* src, size_t n, void* dst, size_t cap) {
  GBVR_ABI_TRY
  if ((!src && n) || !dst) return 0;
  return gbvr::zlib_compress(src, n, dst, cap);
  GBVR_ABI_CATCH_SIZE
}

int gbvr_zlib_decompress(const void* src, size_t n, void* dst, size_t out_n) {
  GBVR_ABI_TRY
  if (!src || (!dst && out_n)) return gbvr::set_error(GBVR_EINVAL, "null argument");
  if (!gbvr::zlib_decompress(src, n, dst, out_n)) return gbvr::set_error(GBVR_EFORMAT, "malformed zlib stream");
  return GBVR_OK;
  GBVR_ABI_CATCH
}

}  // extern "C"
