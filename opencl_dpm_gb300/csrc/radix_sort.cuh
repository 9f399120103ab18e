// Stable device radix sort of (uint32 key, uint32 value) pairs.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace dpm {

// Scratch (device) bytes needed to sort n pairs.
size_t radix_sort_scratch_bytes(int n);
int radix_sort_passes(int key_bits);

// Sorts the low key_bits bits of keys[0..n), carrying vals, stably.  The
// sorted pairs end in (keys, vals) or, when *result_in_alt is set, in
// (keys_alt, vals_alt).  All launches go to `stream`; nothing is allocated.
cudaError_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt,
                             uint32_t *vals_alt, int n, int key_bits,
                             uint32_t *scratch, cudaStream_t stream,
                             bool *result_in_alt);

} // namespace dpm
