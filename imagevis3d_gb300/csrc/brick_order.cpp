// Brick orders of a store, as the converter offers them for the bricks of a
// UVF file (CmdLineConverter/main.cpp:175-178: scanline, Morton, Hilbert or
// random order).  Here they order the out-of-core host store: the bricks
// one view needs lie closer together along a space-filling curve, so a paint
// copies them in fewer, longer stretches.
//
// The Hilbert index follows J. Skilling, "Programming the Hilbert curve",
// AIP Conf. Proc. 707, 381 (2004): the coordinates are turned into the
// "transposed" index by undoing, from the top bit down, the reflections and
// axis exchanges of each level, then Gray-coded; the index is the bits of the
// transposed form read level by level, axis by axis.
#include "brick_order.h"

#include <algorithm>
#include <numeric>

#include "../../include/gbvr.h"
#include "abi_guard.h"

namespace gbvr {

uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  uint64_t key = 0;
  for (int k = 0; k < 21; ++k) {
    key |= (uint64_t)((x >> k) & 1u) << (3 * k);
    key |= (uint64_t)((y >> k) & 1u) << (3 * k + 1);
    key |= (uint64_t)((z >> k) & 1u) << (3 * k + 2);
  }
  return key;
}

uint64_t hilbert3(uint32_t x, uint32_t y, uint32_t z, int bits) {
  if (bits <= 0) return 0;
  uint32_t c[3] = {x, y, z};
  const uint32_t top = 1u << (bits - 1);
  // undo each level's reflection (bit set on an axis: flip the lower bits of
  // axis 0) or exchange (bit clear: swap the lower bits of axes 0 and a)
  for (uint32_t q = top; q > 1; q >>= 1) {
    const uint32_t low = q - 1;
    for (int a = 0; a < 3; ++a) {
      if (c[a] & q) {
        c[0] ^= low;
      } else {
        const uint32_t t = (c[0] ^ c[a]) & low;
        c[0] ^= t;
        c[a] ^= t;
      }
    }
  }
  // Gray code of the transposed index
  c[1] ^= c[0];
  c[2] ^= c[1];
  uint32_t flip = 0;
  for (uint32_t q = top; q > 1; q >>= 1)
    if (c[2] & q) flip ^= q - 1;
  for (int a = 0; a < 3; ++a) c[a] ^= flip;
  // read the transposed index: level by level from the top, axis 0 first
  uint64_t h = 0;
  for (int b = bits - 1; b >= 0; --b)
    for (int a = 0; a < 3; ++a) h = (h << 1) | ((c[a] >> b) & 1u);
  return h;
}

bool brick_order(const int nb[3], int order, uint64_t seed, std::vector<int>& perm) {
  const int n = nb[0] * nb[1] * nb[2];
  perm.resize((size_t)std::max(n, 0));
  std::iota(perm.begin(), perm.end(), 0);
  if (order == 0) return true;
  if (order == 3) {
    // Fisher-Yates with a splitmix64 stream
    uint64_t s = seed;
    auto next = [&]() {
      uint64_t z = (s += 0x9e3779b97f4a7c15ull);
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      return z ^ (z >> 31);
    };
    for (int i = n - 1; i > 0; --i) std::swap(perm[(size_t)i], perm[(size_t)(next() % (uint64_t)(i + 1))]);
    return true;
  }
  if (order != 1 && order != 2) return false;
  int bits = 0;
  while ((1 << bits) < std::max(nb[0], std::max(nb[1], nb[2]))) ++bits;
  std::vector<uint64_t> key((size_t)std::max(n, 0));
  for (int i = 0; i < n; ++i) {
    const uint32_t x = (uint32_t)(i % nb[0]), y = (uint32_t)((i / nb[0]) % nb[1]), z = (uint32_t)(i / (nb[0] * nb[1]));
    key[(size_t)i] = order == 1 ? morton3(x, y, z) : hilbert3(x, y, z, bits);
  }
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return key[(size_t)a] < key[(size_t)b]; });
  return true;
}

}  // namespace gbvr

extern "C" {

int gbvr_brick_order(const int32_t nb[3], int32_t order, uint64_t seed, int32_t* perm, size_t n) {
  GBVR_ABI_TRY
  if (!nb || nb[0] < 1 || nb[1] < 1 || nb[2] < 1) return gbvr::set_error(GBVR_EINVAL, "bad brick grid");
  const size_t total = (size_t)nb[0] * nb[1] * nb[2];
  if (!perm || n < total) return gbvr::set_error(GBVR_EINVAL, "buffer too small");
  const int g[3] = {nb[0], nb[1], nb[2]};
  std::vector<int> p;
  if (!gbvr::brick_order(g, order, seed, p)) return gbvr::set_error(GBVR_EINVAL, "brick order must be 0..3");
  std::copy(p.begin(), p.end(), perm);
  return GBVR_OK;
  GBVR_ABI_CATCH
}

uint64_t gbvr_hilbert3(uint32_t x, uint32_t y, uint32_t z, int32_t bits) { return gbvr::hilbert3(x, y, z, bits); }

}  // extern "C"
