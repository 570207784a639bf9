// prt_sort.cu - onesweep-style LSD radix sort of (key, uint32 value) pairs.
//
// One pass over the keys builds the histograms of every 8-bit digit; then each digit
// pass is a single kernel over tiles of 4,096 pairs (Adinets & Merrill, "Onesweep",
// 2022): a tile ranks its keys stably inside the block (warp match + per-warp digit
// counters), publishes its per-digit counts, finds the counts of all earlier tiles by
// decoupled look-back over a status array, and scatters.  Tiles are numbered by an
// atomic counter in the order blocks start, so a tile only waits on tiles whose blocks
// are already running; every wait is additionally bounded and, if the bound is hit,
// flags kErrLookback and moves on (destinations then stay in range, results are
// reported as an error by the host).
//
// Bytes per pair and digit pass: key + value read and written once (8 B each for
// 32-bit keys), plus 4 B per pair for the one histogram pass over all digits.
#include <algorithm>

#include "prt_internal.cuh"
#include "prt_sort.cuh"

namespace prt {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kSortWarps = kSortThreads / 32;
constexpr uint32_t kStAgg = 1u << 30;
constexpr uint32_t kStInc = 2u << 30;
constexpr uint32_t kStMask = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit = 1u << 22;

template <typename K, int DIGITS>
__global__ void __launch_bounds__(256) k_histogram(const K *__restrict__ keys, uint32_t n,
                                                   int first_digit, uint32_t *__restrict__ ghist) {
	__shared__ uint32_t h[DIGITS][256];
	for (int i = threadIdx.x; i < DIGITS * 256; i += blockDim.x)
		(&h[0][0])[i] = 0;
	__syncthreads();
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		K k = keys[i];
#pragma unroll
		for (int d = 0; d < DIGITS; ++d)
			atomicAdd(&h[d][(uint32_t)(k >> (8 * (first_digit + d))) & 255u], 1u);
	}
	__syncthreads();
	for (int i = threadIdx.x; i < DIGITS * 256; i += blockDim.x) {
		uint32_t v = (&h[0][0])[i];
		if (v)
			atomicAdd(&ghist[i], v);
	}
}

// Exclusive scan of each 256-bin histogram (one block per digit).
__global__ void __launch_bounds__(256) k_scan_digits(uint32_t *ghist) {
	__shared__ uint32_t s[256];
	uint32_t *h = ghist + 256 * blockIdx.x;
	uint32_t v = h[threadIdx.x];
	s[threadIdx.x] = v;
	__syncthreads();
	for (int off = 1; off < 256; off <<= 1) {
		uint32_t add = threadIdx.x >= off ? s[threadIdx.x - off] : 0u;
		__syncthreads();
		s[threadIdx.x] += add;
		__syncthreads();
	}
	h[threadIdx.x] = s[threadIdx.x] - v;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
	uint32_t m;
	asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
	return *(const volatile uint32_t *)p;
}

template <typename K>
__global__ void __launch_bounds__(kSortThreads)
    k_onesweep(const K *__restrict__ kin, const uint32_t *__restrict__ vin, K *__restrict__ kout,
               uint32_t *__restrict__ vout, uint32_t n, int shift,
               const uint32_t *__restrict__ digit_base, uint32_t *status, uint32_t *tile_counter,
               uint32_t *err) {
	__shared__ uint32_t s_cnt[kSortWarps][256];
	__shared__ uint32_t s_base[256];
	__shared__ uint32_t s_tile;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

	if (tid == 0)
		s_tile = atomicAdd(tile_counter, 1u);
	for (int i = tid; i < kSortWarps * 256; i += kSortThreads)
		(&s_cnt[0][0])[i] = 0;
	__syncthreads();
	const uint32_t tile = s_tile;

	// Warp-striped load: item j of lane l is element seg + 32 j + l, so walking j then
	// l visits the warp's segment in index order, which makes the ranking stable.
	const uint32_t seg = tile * kSortTile + warp * 32 * kSortItems;
	K key[kSortItems];
	uint32_t val[kSortItems];
	uint32_t dig[kSortItems];
	uint32_t rank[kSortItems];
#pragma unroll
	for (int j = 0; j < kSortItems; ++j) {
		uint32_t idx = seg + 32 * j + lane;
		if (idx < n) {
			key[j] = kin[idx];
			val[j] = vin[idx];
			dig[j] = (uint32_t)(key[j] >> shift) & 255u;
		} else {
			key[j] = 0;
			val[j] = 0;
			dig[j] = 256u;
		}
	}
	const uint32_t lt = lanemask_lt();
#pragma unroll
	for (int j = 0; j < kSortItems; ++j) {
		uint32_t d = dig[j];
		uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
		uint32_t before = __popc(peers & lt);
		uint32_t base = (d < 256u) ? s_cnt[warp][d] : 0u;
		__syncwarp();
		if (d < 256u && before == 0)
			s_cnt[warp][d] = base + __popc(peers);
		__syncwarp();
		rank[j] = base + before;
	}
	__syncthreads();

	// Per digit (thread tid owns digit tid): offsets of each warp inside the tile and
	// the tile's total, then the look-back for the count of all earlier tiles.
	{
		const uint32_t d = tid;
		uint32_t total = 0;
#pragma unroll
		for (int w = 0; w < kSortWarps; ++w) {
			uint32_t c = s_cnt[w][d];
			s_cnt[w][d] = total;
			total += c;
		}
		uint32_t *my = status + (size_t)tile * 256 + d;
		uint32_t prefix = 0;
		if (tile == 0) {
			atomicExch(my, kStInc | total);
		} else {
			atomicExch(my, kStAgg | total);
			int j = (int)tile - 1;
			uint32_t spins = 0;
			while (j >= 0) {
				uint32_t s = ld_volatile(status + (size_t)j * 256 + d);
				uint32_t flag = s & ~kStMask;
				if (flag == 0u) {
					if (++spins > kSpinLimit) {
						atomicOr(err, kErrLookback);
						break;
					}
					__nanosleep(32);
					continue;
				}
				prefix += s & kStMask;
				if (flag == kStInc)
					break;
				--j;
			}
			atomicExch(my, kStInc | (prefix + total));
		}
		s_base[d] = digit_base[d] + prefix;
	}
	__syncthreads();

#pragma unroll
	for (int j = 0; j < kSortItems; ++j) {
		uint32_t d = dig[j];
		if (d < 256u) {
			uint32_t dst = s_base[d] + s_cnt[warp][d] + rank[j];
			if (dst < n) {
				kout[dst] = key[j];
				vout[dst] = val[j];
			}
		}
	}
}

template <typename K>
int sort_pairs_impl(K *keys, uint32_t *vals, K *keys_alt, uint32_t *vals_alt, uint32_t n,
                    int n_digits, SortScratch &s, cudaStream_t st, uint32_t *d_err) {
	if (n <= 1 || n_digits == 0)
		return 0;
	const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
	cudaMemsetAsync(s.hist, 0, sizeof(uint32_t) * 256 * n_digits, st);
	cudaMemsetAsync(s.tile_counters, 0, sizeof(uint32_t) * n_digits, st);
	int hist_blocks = (int)std::min<uint32_t>(1024u, (n + 4095u) / 4096u);
	if (sizeof(K) == 4) {
		k_histogram<K, 4><<<hist_blocks, 256, 0, st>>>(keys, n, 0, s.hist);
	} else {
		k_histogram<K, 4><<<hist_blocks, 256, 0, st>>>(keys, n, 0, s.hist);
		if (n_digits > 4)
			k_histogram<K, 4><<<hist_blocks, 256, 0, st>>>(keys, n, 4, s.hist + 4 * 256);
	}
	k_scan_digits<<<n_digits, 256, 0, st>>>(s.hist);
	K *ki = keys, *ko = keys_alt;
	uint32_t *vi = vals, *vo = vals_alt;
	for (int p = 0; p < n_digits; ++p) {
		cudaMemsetAsync(s.status, 0, sizeof(uint32_t) * 256 * (size_t)tiles, st);
		k_onesweep<K><<<tiles, kSortThreads, 0, st>>>(ki, vi, ko, vo, n, 8 * p, s.hist + 256 * p,
		                                              s.status, s.tile_counters + p, d_err);
		K *tk = ki; ki = ko; ko = tk;
		uint32_t *tv = vi; vi = vo; vo = tv;
	}
	return n_digits & 1; // odd pass count: result is in the alternate buffers
}

} // namespace

size_t sort_status_words(uint32_t n) {
	return 256 * (size_t)((n + kSortTile - 1) / kSortTile + 1);
}

int sort_pairs_u32(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt, uint32_t *vals_alt,
                   uint32_t n, int n_digits, SortScratch &s, cudaStream_t st, uint32_t *d_err) {
	return sort_pairs_impl<uint32_t>(keys, vals, keys_alt, vals_alt, n, n_digits, s, st, d_err);
}

int sort_pairs_u64(uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt,
                   uint32_t n, int n_digits, SortScratch &s, cudaStream_t st, uint32_t *d_err) {
	return sort_pairs_impl<uint64_t>(keys, vals, keys_alt, vals_alt, n, n_digits, s, st, d_err);
}

} // namespace prt
