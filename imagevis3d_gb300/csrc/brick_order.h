// Brick orders of a store (the converter's on-disk brick layouts,
// CmdLineConverter/main.cpp:175-178: 0 scanline, 1 Morton, 2 Hilbert, 3
// random): see brick_order.cpp.
#pragma once
#include <cstdint>
#include <vector>

namespace gbvr {
// Morton key of (x, y, z): bit k of x, y, z at bits 3k, 3k + 1, 3k + 2.
uint64_t morton3(uint32_t x, uint32_t y, uint32_t z);
// Position of (x, y, z) along the 3D Hilbert curve of a 2^bits cube.
uint64_t hilbert3(uint32_t x, uint32_t y, uint32_t z, int bits);
// The bricks of an nx x ny x nz grid (index (z ny + y) nx + x) in storage
// order: perm[k] = the brick stored k-th.  False for an unknown order.
bool brick_order(const int nb[3], int order, uint64_t seed, std::vector<int>& perm);
}  // namespace gbvr
