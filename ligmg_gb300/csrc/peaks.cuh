// peaks.cuh — the measured gather ceiling of the running GPU (peaks.cu).
#pragma once
#include "common.cuh"

namespace lg {

// Random rows of `width` bytes (4, 8 or 128) per second gathered from a table
// of `rows` rows (L2-resident when it fits), `count` rows per timed launch,
// blocks_per_sm blocks of 256 threads per SM (0: 8, every warp slot).
double gather_peak(i64 rows, int width, i64 count, int blocks_per_sm);

}  // namespace lg
