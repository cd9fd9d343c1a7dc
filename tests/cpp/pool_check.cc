// RangePool (libfalcon_dsp_gb300/csrc/fdsp_pool.h), the bookkeeping of the
// stream server's device pool, against a byte map on random alloc/release
// sequences: pieces 256-byte aligned, inside the range, never overlapping;
// failing allocations only when no free run fits; after everything is
// released one free piece spans the whole range again.
//
// Usage: pool_check <rounds>; prints "ok <rounds> <allocs> <failed>".
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "fdsp_pool.h"

using fdsp::RangePool;

int main(int argc, char** argv) {
  const int rounds = argc > 1 ? std::atoi(argv[1]) : 200;
  std::mt19937_64 rng(7);
  long long allocs = 0, failed = 0;
  for (int rd = 0; rd < rounds; ++rd) {
    const size_t size = 256 * (size_t)(1 + rng() % 4096);
    RangePool p;
    p.init(size);
    std::vector<unsigned char> owner(size / 256, 0);  // 256-byte units in use
    std::vector<std::pair<size_t, size_t>> live;      // (offset, units)
    for (int op = 0; op < 2000; ++op) {
      if (live.empty() || rng() % 3 != 0) {
        const size_t bytes = 1 + rng() % (size / 8 + 1);
        const size_t units = (bytes + 255) / 256;
        const size_t off = p.alloc(bytes);
        ++allocs;
        if (off == RangePool::kNone) {
          ++failed;
          // no run of `units` free units may exist
          size_t run = 0, best = 0;
          for (unsigned char o : owner) {
            run = o ? 0 : run + 1;
            if (run > best) best = run;
          }
          if (best >= units) {
            std::printf("FAIL: refused %zu units with a free run of %zu\n", units, best);
            return 1;
          }
          continue;
        }
        if (off % 256 != 0 || off + units * 256 > size) {
          std::printf("FAIL: piece [%zu, +%zu) outside or unaligned (size %zu)\n", off, units * 256, size);
          return 1;
        }
        for (size_t u = off / 256; u < off / 256 + units; ++u) {
          if (owner[u]) {
            std::printf("FAIL: overlap at unit %zu\n", u);
            return 1;
          }
          owner[u] = 1;
        }
        live.push_back({off, units});
      } else {
        const size_t i = rng() % live.size();
        for (size_t u = live[i].first / 256; u < live[i].first / 256 + live[i].second; ++u) owner[u] = 0;
        p.release(live[i].first);
        live[i] = live.back();
        live.pop_back();
      }
      size_t used_units = 0;
      for (unsigned char o : owner) used_units += o;
      if (p.free_bytes() != size - 256 * used_units) {
        std::printf("FAIL: free bytes %zu, expected %zu\n", p.free_bytes(), size - 256 * used_units);
        return 1;
      }
    }
    for (auto& l : live) p.release(l.first);
    p.release(12345);  // not a piece: ignored
    if (p.free_pieces() != 1 || p.free_bytes() != size || p.used_pieces() != 0) {
      std::printf("FAIL: after releasing everything %zu free pieces, %zu bytes\n", p.free_pieces(), p.free_bytes());
      return 1;
    }
  }
  std::printf("ok %d %lld %lld\n", rounds, allocs, failed);
  return 0;
}
