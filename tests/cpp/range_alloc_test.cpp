// Unit test of prt::RangeAllocator (the request server's budget allocator): fixed cases,
// then random alloc/release sequences checked against a byte-occupancy model.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "prt_range_alloc.h"

#define REQUIRE(c)                                                                             \
	do {                                                                                       \
		if (!(c)) {                                                                            \
			std::printf("FAILED %s at line %d\n", #c, __LINE__);                               \
			return 1;                                                                          \
		}                                                                                      \
	} while (0)

int main() {
	using prt::RangeAllocator;
	RangeAllocator a(4096, 256);
	REQUIRE(a.capacity() == 4096 && a.used() == 0);
	const uint64_t x = a.alloc(1), y = a.alloc(300), z = a.alloc(256);
	REQUIRE(x == 0 && y == 256 && z == 768);
	REQUIRE(a.used() == 1024 && a.peak() == 1024);
	a.release(y, 300);
	REQUIRE(a.alloc(512) == 256); // first fit reuses the hole
	a.release(256, 512);
	a.release(x, 1);
	a.release(z, 256);
	REQUIRE(a.used() == 0 && a.fragments() == 1 && a.largest_free() == 4096);
	REQUIRE(a.alloc(4097) == RangeAllocator::kFail && a.fits_ever(4096) && !a.fits_ever(4097));
	REQUIRE(a.alloc(4096) == 0 && a.alloc(1) == RangeAllocator::kFail);

	std::mt19937_64 rng(7);
	for (int trial = 0; trial < 50; ++trial) {
		const uint64_t cap = 256 * (1 + rng() % 200);
		RangeAllocator r(cap, 256);
		std::vector<int> owner(cap / 256, -1);
		struct Live {
			uint64_t off, bytes;
		};
		std::vector<Live> live;
		for (int step = 0; step < 2000; ++step) {
			if (!live.empty() && (rng() % 3 == 0)) {
				const size_t i = rng() % live.size();
				const Live l = live[i];
				for (uint64_t b = l.off / 256; b < (l.off + r.round(l.bytes)) / 256; ++b)
					owner[b] = -1;
				r.release(l.off, l.bytes);
				live[i] = live.back();
				live.pop_back();
			} else {
				const uint64_t bytes = 1 + rng() % (cap / 4 + 1);
				const uint64_t off = r.alloc(bytes);
				// A failure means no run of free blocks is long enough (first fit finds
				// any hole that fits).
				const uint64_t need = r.round(bytes) / 256;
				uint64_t run = 0, best = 0;
				for (int o : owner) {
					run = (o < 0) ? run + 1 : 0;
					best = std::max(best, run);
				}
				if (off == RangeAllocator::kFail) {
					REQUIRE(best < need);
					continue;
				}
				REQUIRE(off % 256 == 0 && off + r.round(bytes) <= cap);
				for (uint64_t b = off / 256; b < off / 256 + need; ++b) {
					REQUIRE(owner[b] < 0);
					owner[b] = step;
				}
				live.push_back({off, bytes});
			}
			uint64_t used = 0;
			for (int o : owner)
				used += (o >= 0) ? 256 : 0;
			REQUIRE(used == r.used() && r.peak() >= r.used());
		}
		for (const Live &l : live)
			r.release(l.off, l.bytes);
		REQUIRE(r.used() == 0 && r.fragments() == 1 && r.largest_free() == r.capacity());
	}
	std::printf("range allocator: ok\n");
	return 0;
}
