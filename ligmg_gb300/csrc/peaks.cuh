// peaks.cuh — the measured gather ceiling of the running GPU (peaks.cu).
#pragma once
#include "common.cuh"

namespace lg {

// Random rows of `width` bytes (4, 8 or 128) per second gathered from a table
// of `rows` rows (L2-resident when it fits), `count` rows per timed launch.
double gather_peak(i64 rows, int width, i64 count);

}  // namespace lg
