// Host side of the seeded blob generator (gbvr_synth_params): parameter
// checks and the per-axis tables, shared by every synthesis entry point (the
// allocating ones in gbvr_api.cu and the no-allocation one in noalloc.cu).
#pragma once
#include <cstddef>

#include "../../include/gbvr.h"

namespace gbvr {

// k_synth_blobs keeps one float per blob of the current row in dynamic shared
// memory, within the 48 KiB a block gets without opting in.
constexpr int kMaxSynthBlobs = 12288;

// Checks p for the device generator: dims > 0, a known dtype, 0 <= nblobs <=
// kMaxSynthBlobs, the voxel count times the element size and the table size
// without 64-bit overflow, rows within the launch grid (Y < 2^31) and, when
// whole_volume (one launch over every plane), Z <= 65535.  On success writes
// the table size in floats and the volume's bytes; otherwise returns
// GBVR_EINVAL with the message set.
int check_synth_params(const gbvr_synth_params* p, bool whole_volume, long long* table_floats, size_t* volume_bytes);

// The generator's tables as one array of check_synth_params' table_floats:
// amp[nb] | ex[nb X] | ey[nb Y] | ez[nb Z] | bgx[X] | bgy[Y] | bgz[Z], the
// background tables only when bg_freq > 0.  Blob centres, widths and
// amplitudes are Philox4x32-10 draws keyed by the seed; the tables are
// evaluated in double and rounded to float once.
void fill_blob_tables(const gbvr_synth_params& p, float* t);

}  // namespace gbvr
