// prt_sort.cuh - host entry points of the onesweep radix sort (prt_sort.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

namespace prt {

// Device scratch of one sort: 8 x 256 digit histograms, 8 tile counters and a status
// array of sort_status_words(n) words.
struct SortScratch {
	uint32_t *hist = nullptr;
	uint32_t *tile_counters = nullptr;
	uint32_t *status = nullptr;
};

size_t sort_status_words(uint32_t n);

// Stable LSD sort of n (key, value) pairs by the low 8 * n_digits bits of the key.
// Ping-pongs between (keys, vals) and (keys_alt, vals_alt); returns 0 when the sorted
// result is in (keys, vals), 1 when it is in the alternate pair.  Queued on `st`.
int sort_pairs_u32(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt, uint32_t *vals_alt,
                   uint32_t n, int n_digits, SortScratch &s, cudaStream_t st, uint32_t *d_err);
int sort_pairs_u64(uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt,
                   uint32_t n, int n_digits, SortScratch &s, cudaStream_t st, uint32_t *d_err);

} // namespace prt
