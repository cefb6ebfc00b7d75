// zlib streams (RFC 1950) of DEFLATE data (RFC 1951): the UVF brick codec
// CT_ZLIB (UVFReader/BlockInfo.h:60-93), the converter's default
// (CmdLineConverter/main.cpp:146).  Host encoder and decoder; the GPU decoder
// of paged bricks is k_inflate (kernels_build.cu).
#pragma once
#include <cstddef>
#include <cstdint>

namespace gbvr {

// Largest zlib stream zlib_compress writes for n input bytes (stored blocks
// plus header and checksum).
size_t zlib_bound(size_t n);
// One zlib stream: 2-byte header, DEFLATE blocks of at most 64 KiB of input
// (LZ77 over a 32 KiB window, hash chains of at most `chain` candidates,
// dynamic Huffman codes, or stored blocks where that is smaller), Adler-32.
// Returns the stream's size, 0 when it does not fit cap.
size_t zlib_compress(const void* src, size_t n, void* dst, size_t cap, int chain = 32);
// Decodes a zlib stream into exactly out_n bytes (all block types; header,
// lengths, distances and the Adler-32 checked).  False when malformed.
bool zlib_decompress(const void* src, size_t n, void* dst, size_t out_n);
uint32_t adler32(const uint8_t* p, size_t n);

// DEFLATE's length and distance code tables (RFC 1951 section 3.2.5).
extern const uint16_t kLenBase[29];
extern const uint8_t kLenExtra[29];
extern const uint16_t kDistBase[30];
extern const uint8_t kDistExtra[30];
// order of the code-length code lengths in a dynamic block header (3.2.7)
extern const uint8_t kClOrder[19];

}  // namespace gbvr
