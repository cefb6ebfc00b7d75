// LZ4 block codec (host side): see lz4.cpp.
#pragma once
#include <cstddef>
#include <cstdint>

namespace gbvr {
// largest compressed size of n bytes
size_t lz4_bound(size_t n);
// compress src[0, n) into dst (capacity cap), comparing up to `chain`
// candidates per position and taking matches of at least min_match bytes:
// the compressed size, or 0 when it does not fit
size_t lz4_compress(const uint8_t* src, size_t n, uint8_t* dst, size_t cap, int chain = 16, int min_match = 4);
// decode a block into exactly out_n bytes: false when malformed or of another size
bool lz4_decompress(const uint8_t* in, size_t in_n, uint8_t* out, size_t out_n);
}  // namespace gbvr
