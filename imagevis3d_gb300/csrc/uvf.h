// UVF container I/O (host side): global header, block headers, raster data,
// 1D / 2D histogram, min/max and key/value blocks, MD5 checksum.
//
// Byte layout follows doc/import.adoc:904-1147 and, where that text stops
// ("see the source"), the fields of DemoData/c60.uvf: the raster header
// carries element semantic / bit size / mantissa words, then one signed byte,
// then a u64 data offset, then the voxels.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gbvr {

struct Md5 {
  uint32_t a, b, c, d;
  uint64_t len;
  unsigned char buf[64];
  size_t fill;
  Md5();
  void update(const void* p, size_t n);
  void final(unsigned char out[16]);
};

struct UvfBlock {
  uint64_t start;      // file offset of the block header
  std::string id;
  uint64_t semantic;
  uint64_t compression;
  uint64_t next;       // relative to start, 0 = last
  uint64_t payload;    // file offset of the payload
};

struct UvfRaster {
  std::string id;
  uint64_t dims[3] = {0, 0, 0};          // x, y, z
  uint64_t brick_size[3] = {256, 256, 256};
  uint64_t overlap[3] = {4, 4, 4};        // stored as 2 * ghost voxels
  uint64_t lod_factor[3] = {2, 2, 2};
  uint64_t lod_groups[3] = {0, 0, 0};
  std::vector<uint64_t> lod_counts = {1};
  double transform[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  uint64_t elem_semantic = 0;
  uint64_t bit_size = 8;
  uint64_t mantissa = 8;
  bool is_signed = false;
  bool is_float = false;
  uint64_t data_offset_field = 0;
  uint64_t data_pos = 0;                 // file offset of the voxel data (reader)
};

struct UvfMinMax {
  double min_scalar, max_scalar, min_grad, max_grad;
};

struct UvfFile {
  uint64_t version = 2;
  uint64_t checksum_semantic = 2;
  std::vector<unsigned char> checksum;
  std::vector<UvfBlock> blocks;
  bool has_raster = false;
  UvfRaster raster;
  std::vector<uint64_t> hist1d;
  float hist2d_max_grad = 0.f;
  uint64_t hist2d_nx = 0, hist2d_ny = 0;
  std::vector<uint64_t> hist2d;
  std::string hist2d_id;
  std::vector<UvfMinMax> minmax;
  uint64_t minmax_components = 1;
  std::vector<std::pair<std::string, std::string>> kv;
  bool checksum_ok = false;
};

// Reads headers and small blocks; voxel data stays in the file (data_pos).
// Returns 0 or a GBVR_E* status with msg filled.
int uvf_read(const std::string& path, bool verify, UvfFile& out, std::string& msg);
int uvf_read_voxels(const std::string& path, const UvfFile& f, void* out, size_t bytes, std::string& msg);

// Writes a v2 file: raster block (voxels given as one contiguous buffer), then
// the 1D histogram, 2D histogram, min/max and (if any) key/value blocks, then
// the MD5 of everything from byte 49 on into the global header.
struct UvfWriteSpec {
  UvfRaster raster;
  const void* voxels = nullptr;
  uint64_t voxel_bytes = 0;
  std::vector<uint64_t> hist1d;
  std::string hist1d_id = "1D Histrogram";  // block id string as ImageVis3D writes it
  std::vector<uint64_t> hist2d;
  uint64_t hist2d_nx = 0, hist2d_ny = 0;
  float hist2d_max_grad = 0.f;
  std::vector<UvfMinMax> minmax;
  std::string minmax_id = "Brick Max/Min Values";
  std::vector<std::pair<std::string, std::string>> kv;
};
int uvf_write(const std::string& path, const UvfWriteSpec& spec, std::string& msg);

}  // namespace gbvr
