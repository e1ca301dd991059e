// mc_tma_host.h -- host helpers of the TMA kernels (tma_host.cu).
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>

namespace mc {

// cuTensorMapEncodeTiled from the driver (nullptr if unavailable).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();

// 2-D uint8 tensor of `rows` rows of `row_bytes` bytes (pitch = row_bytes),
// boxes of box_bytes x 1 (the tile::gather4 shape), 128-byte swizzle.
bool encode_row_gather_u8(CUtensorMap* map, const void* base, long long rows, long long row_bytes, int box_bytes);

// 2-D uint8 tensor of `rows` rows of `row_bytes` bytes (pitch = row_bytes),
// boxes of box_bytes (64 or 128) x box_rows, swizzled at the box width (the
// resident SpMM's slices).
bool encode_slice_u8(CUtensorMap* map, const void* base, long long rows, long long row_bytes, int box_bytes,
                     int box_rows);

// 2-D uint8 tensor of `rows` rows of `row_bytes` bytes (pitch = row_bytes),
// unswizzled boxes of box_bytes x box_rows (the dense-tile SpMM's B chunks);
// rows past the end read as zero.
bool encode_box_u8(CUtensorMap* map, const void* base, long long rows, long long row_bytes, int box_bytes,
                   int box_rows);

// Device address of the counter of bounded waits that ran out, and its value.
unsigned int* async_timeout_counter();
unsigned int async_timeouts();

}  // namespace mc
