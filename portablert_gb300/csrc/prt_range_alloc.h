// prt_range_alloc.h - first-fit allocator of byte ranges inside one fixed region.
//
// The request server (prt_serve.cu) reserves one device region of its memory budget
// at start-up and carves each admitted request's rays and records out of it; a request
// that does not fit waits until earlier ones release their ranges.  Plain C++ (no CUDA),
// so it is tested on the CPU.  Not thread-safe: the server calls it under its lock.
#pragma once

#include <stdint.h>

#include <algorithm>
#include <iterator>
#include <map>

namespace prt {

class RangeAllocator {
  public:
	static constexpr uint64_t kFail = ~0ull;

	explicit RangeAllocator(uint64_t capacity = 0, uint64_t align = 256) { reset(capacity, align); }

	void reset(uint64_t capacity, uint64_t align) {
		align_ = align ? align : 1;
		cap_ = capacity / align_ * align_;
		free_.clear();
		if (cap_)
			free_[0] = cap_;
		used_ = peak_ = 0;
	}

	uint64_t round(uint64_t bytes) const { return (bytes + align_ - 1) / align_ * align_; }

	// Offset of a free range of round(bytes) bytes (the lowest that fits), or kFail.
	uint64_t alloc(uint64_t bytes) {
		const uint64_t need = round(std::max<uint64_t>(bytes, 1));
		for (auto it = free_.begin(); it != free_.end(); ++it) {
			if (it->second < need)
				continue;
			const uint64_t off = it->first, left = it->second - need;
			free_.erase(it);
			if (left)
				free_[off + need] = left;
			used_ += need;
			peak_ = std::max(peak_, used_);
			return off;
		}
		return kFail;
	}

	// Returns a range given by alloc (same byte count), merging it with free neighbours.
	void release(uint64_t off, uint64_t bytes) {
		uint64_t size = round(std::max<uint64_t>(bytes, 1));
		used_ -= size;
		auto next = free_.lower_bound(off);
		if (next != free_.end() && off + size == next->first) {
			size += next->second;
			next = free_.erase(next);
		}
		if (next != free_.begin()) {
			auto prev = std::prev(next);
			if (prev->first + prev->second == off) {
				prev->second += size;
				return;
			}
		}
		free_[off] = size;
	}

	bool fits_ever(uint64_t bytes) const { return round(std::max<uint64_t>(bytes, 1)) <= cap_; }
	uint64_t capacity() const { return cap_; }
	uint64_t used() const { return used_; }
	uint64_t peak() const { return peak_; }
	size_t fragments() const { return free_.size(); }
	uint64_t largest_free() const {
		uint64_t m = 0;
		for (const auto &f : free_)
			m = std::max(m, f.second);
		return m;
	}

  private:
	std::map<uint64_t, uint64_t> free_; // offset -> size of each free range
	uint64_t cap_ = 0, align_ = 256, used_ = 0, peak_ = 0;
};

} // namespace prt
