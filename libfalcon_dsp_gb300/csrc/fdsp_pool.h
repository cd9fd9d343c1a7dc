// First-fit allocator over one contiguous range [0, size): 256-byte-aligned
// pieces, neighbours coalesced on release.  Host-only bookkeeping (no CUDA),
// so it is tested on the CPU (tests/cpp/pool_check.cc); DevPool
// (fdsp_internal.h) puts it over one cudaMalloc'd region.
#pragma once

#include <cstddef>
#include <cstdint>
#include <iterator>
#include <map>

namespace fdsp {

class RangePool {
 public:
  static constexpr size_t kNone = ~(size_t)0;
  static constexpr size_t kAlign = 256;

  void init(size_t size) {
    size_ = size & ~(kAlign - 1);
    free_.clear();
    used_.clear();
    if (size_) free_[0] = size_;
  }
  // offset of a free piece of at least `bytes` (rounded up to kAlign), or kNone
  size_t alloc(size_t bytes) {
    const size_t n = ((bytes ? bytes : 1) + kAlign - 1) & ~(kAlign - 1);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < n) continue;
      const size_t off = it->first, len = it->second;
      free_.erase(it);
      if (len > n) free_[off + n] = len - n;
      used_[off] = n;
      return off;
    }
    return kNone;
  }
  // returns a piece alloc() gave out (anything else is ignored)
  void release(size_t off) {
    auto u = used_.find(off);
    if (u == used_.end()) return;
    size_t start = off, len = u->second;
    used_.erase(u);
    auto nx = free_.lower_bound(start);
    if (nx != free_.end() && nx->first == start + len) {  // merge with the next free piece
      len += nx->second;
      nx = free_.erase(nx);
    }
    if (nx != free_.begin()) {  // and with the previous one
      auto pv = std::prev(nx);
      if (pv->first + pv->second == start) {
        start = pv->first;
        len += pv->second;
        free_.erase(pv);
      }
    }
    free_[start] = len;
  }
  size_t size() const { return size_; }
  size_t free_bytes() const {
    size_t f = 0;
    for (const auto& kv : free_) f += kv.second;
    return f;
  }
  size_t free_pieces() const { return free_.size(); }
  size_t used_pieces() const { return used_.size(); }

 private:
  size_t size_ = 0;
  std::map<size_t, size_t> free_;  // offset -> bytes
  std::map<size_t, size_t> used_;  // offset -> bytes
};

}  // namespace fdsp
