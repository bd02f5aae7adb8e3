// prims.cuh — device-wide primitives: exclusive scan, stable LSD radix sort,
// stream compaction.  Used by the setup phase, whose integer results must be
// bit-identical run to run (no atomics decide an order anywhere).
#pragma once
#include "common.cuh"

namespace lg {

// out[i] = sum(in[0..i-1]); returns nothing; if total != nullptr the sum of
// all n inputs is written to *total (device pointer).
template <typename T>
void exclusive_scan(const T *in, T *out, i64 n, cudaStream_t s, T *total = nullptr);

// Stable LSD radix sort of (key, payload) pairs on bits [0, key_bits).
// keys/vals are sorted in place (alternate buffers are allocated inside).
void radix_sort_pairs(u64 *keys, u32 *vals, i64 n, int key_bits, cudaStream_t s);

// Stable compaction of indices: out[k] = i for the k-th i with flag[i] != 0.
// Returns the count (synchronises).
i64 compact_indices(const uint8_t *flags, i64 n, i32 *out, cudaStream_t s);

int bits_for(i64 maxval);  // number of bits to represent values in [0, maxval]

}  // namespace lg
