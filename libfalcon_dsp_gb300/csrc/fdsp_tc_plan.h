// Launch planning of the tensor-core polyphase kernel (host only): merge
// sets, staging geometry, shared-memory budget and the row split.  Kept
// apart from the kernel so that its bounds can be checked on the CPU
// (tests/cpp/tc_plan_check.cc restates the kernel's shared-memory indexing
// over these plans).
#pragma once

#include <stdint.h>

#include <algorithm>
#include <vector>

#include "fdsp_internal.h"

namespace fdsp {

constexpr uint32_t kTcDCols = 128;    // accumulator columns per slot (N <= 128)
constexpr int kTcMaxKw = 128;         // taps of a merged window (before pair rounding)
constexpr size_t kTcSmemMax = 222 * 1024;  // + ~4.3 KB static (barriers, epilogue phasors) <= 227 KB
constexpr int kTcMaxBuf = 4;          // input buffers
constexpr size_t kTcRawMax = 48 * 1024; // raw span buffer (bulk-copy staging) at most

struct TcChunk;

// One work set of the group for this apply, before merging.
struct TcWsPlan {
  const TcChunk* ch;
  int T = 0;      // taps per phase of its chunk (even)
  int n = 0;      // channels of its chunk
  uint32_t phi;   // tap phase
  int64_t delta;  // window end of row 0
  int64_t J;
  uint32_t U, r;
};

struct TcMsetPlan {
  std::vector<int> ws;   // indices into the work-set list
  int64_t E = 0;         // latest window end
  int64_t S0 = 0;        // earliest window start of its work sets
  int64_t S = 0;         // merged window start (row 0): E - Kw + 1, Kw rounded up to even
  int Kw = 0;
  int cols = 0;          // 8-column groups x 8
};

struct TcLaunchPlan {
  std::vector<int> ms;   // merge-set indices
  int nws = 0, nslots = 0;
  int64_t B0 = 0;
  int V = 0, Qp = 0, wrap = 0, nbuf = 1;
  int pair = 0;          // 1: pair records (even D: 16-byte records of two samples)
  int raw_span = 0;      // > 0: tiles staged through one bulk copy of their input span
  int nraw = 0;          // raw span buffers (1 or 2)
  size_t b_bytes = 0, meta_bytes = 0, tab_bytes = 0, in_bytes = 0, raw_bytes = 0, raw_stride = 0;
};

// [B of each merge set | slot constants | A-offset tables | raw span | input buffers]
inline size_t tc_smem_need(const TcLaunchPlan& p, int nbuf) {
  return ((p.b_bytes + p.meta_bytes + p.tab_bytes + 127) & ~(size_t)127) + p.raw_bytes + (size_t)nbuf * p.in_bytes;
}

// Staging geometry of a launch covering merge sets p.ms.
inline void tc_geometry(const std::vector<TcMsetPlan>& msets, TcLaunchPlan& p, uint32_t D, int raw_bufs = 2) {
  const int tpm = p.pair ? 4 : 2;  // taps per MMA
  p.B0 = INT64_MAX;
  p.b_bytes = p.meta_bytes = p.tab_bytes = 0;
  p.nws = p.nslots = 0;
  for (int m : p.ms) {
    p.B0 = std::min(p.B0, msets[m].S);
    const int N = ((msets[m].cols + 15) / 16) * 16;
    p.nws += (int)msets[m].ws.size();
    p.nslots += N / 2;
    p.b_bytes += (size_t)N * msets[m].Kw * 16;
    p.meta_bytes += (size_t)(N / 2) * (8 * sizeof(float2) + 9 * sizeof(uint32_t));
    p.tab_bytes += (size_t)((msets[m].Kw / tpm + 3) & ~3) * 4;
  }
  int64_t W = 0;
  for (int m : p.ms) W = std::max<int64_t>(W, msets[m].S - p.B0 + msets[m].Kw);
  p.wrap = W > (int64_t)D ? 1 : 0;
  if (p.pair)
    p.V = p.wrap ? (int)D / 2 + 1 : (int)W / 2;
  else
    p.V = p.wrap ? (int)D + 1 : (int)W;
  p.Qp = p.wrap ? 128 + (int)((W - 1) / D) : 128;
  // wrapped windows read (nearly) every sample of the tile's span: stage
  // them with one bulk copy when the span is small enough (Qp odd keeps the
  // record writes free of bank conflicts)
  p.raw_span = 0;
  p.nraw = 0;
  p.raw_bytes = p.raw_stride = 0;
  if (p.wrap && raw_bufs > 0) {
    const int qp = p.Qp | 1;
    const size_t span = (size_t)qp * D + (p.pair ? 2 : 1);
    const size_t bytes = (((span + 2) * 8) + 127) & ~(size_t)127;
    if (bytes <= kTcRawMax) {
      p.Qp = qp;
      p.raw_span = (int)span;
      p.nraw = raw_bufs;
      p.raw_stride = bytes;
      p.raw_bytes = bytes * (size_t)raw_bufs;
    }
  }
  p.in_bytes = (((size_t)p.V * p.Qp * 16) + 127) & ~(size_t)127;
}

// Merge sets: consecutive (by window end) work sets while N <= cap columns
// and the merged window stays within kTcMaxKw taps.
inline std::vector<TcMsetPlan> tc_merge(const std::vector<TcWsPlan>& wl, const std::vector<int>& order, int cap) {
  std::vector<TcMsetPlan> msets;
  for (int wi : order) {
    const TcWsPlan& w = wl[wi];
    const int64_t s = w.delta - w.T + 1;
    const int cols = 2 * w.n;
    bool joined = false;
    if (!msets.empty()) {
      TcMsetPlan& m = msets.back();
      const int64_t E = std::max(m.E, w.delta);
      const int64_t S0 = std::min(m.S0, s);
      const int Kw = (int)(((E - S0 + 1) + 1) & ~1LL);
      if (m.cols + cols <= cap && Kw <= kTcMaxKw) {
        m.ws.push_back(wi);
        m.E = E;
        m.S0 = S0;
        m.S = E - Kw + 1;
        m.Kw = Kw;
        m.cols += cols;
        joined = true;
      }
    }
    if (!joined) {
      TcMsetPlan m;
      m.ws.push_back(wi);
      m.E = w.delta;
      m.Kw = w.T;
      m.S0 = s;
      m.S = m.E - m.Kw + 1;
      m.cols = cols;
      msets.push_back(m);
    }
  }
  return msets;
}

// Pair records (even D) read taps four at a time from records of two
// samples: every merged window starts on an even sample and spans a multiple
// of four taps (the extra taps are zero).
inline void tc_pair_windows(std::vector<TcMsetPlan>& msets) {
  for (auto& m : msets) {
    const int64_t S = m.S0 & ~1LL;  // even, at or before every work set's window start
    m.Kw = (int)(((m.E - S + 1) + 3) & ~3LL);
    m.S = S;
  }
}

// Launches: consecutive merge sets while shared memory allows; false when a
// single merge set does not fit.
inline bool tc_pack(const std::vector<TcMsetPlan>& msets, uint32_t D, int pair, std::vector<TcLaunchPlan>& plans) {
  plans.clear();
  for (int mi = 0; mi < (int)msets.size(); ++mi) {
    bool joined = false;
    if (!plans.empty() && (int)plans.back().ms.size() < kMaxTcMsets) {
      TcLaunchPlan p = plans.back();
      p.ms.push_back(mi);
      tc_geometry(msets, p, D);
      if (tc_smem_need(p, 1) > kTcSmemMax) tc_geometry(msets, p, D, 1);
      if (tc_smem_need(p, 1) > kTcSmemMax) tc_geometry(msets, p, D, 0);
      if (tc_smem_need(p, 1) <= kTcSmemMax && p.nws <= kMaxTcWorkSets && p.nslots <= kMaxTcSlots) {
        plans.back() = p;
        joined = true;
      }
    }
    if (!joined) {
      TcLaunchPlan p;
      p.pair = pair;
      p.ms.push_back(mi);
      tc_geometry(msets, p, D);
      if (tc_smem_need(p, 1) > kTcSmemMax) tc_geometry(msets, p, D, 1);
      if (tc_smem_need(p, 1) > kTcSmemMax) tc_geometry(msets, p, D, 0);
      if (tc_smem_need(p, 1) > kTcSmemMax || p.nws > kMaxTcWorkSets || p.nslots > kMaxTcSlots) return false;
      plans.push_back(p);
    }
  }
  for (auto& p : plans) {
    p.nbuf = 1;
    while (p.nbuf < kTcMaxBuf && tc_smem_need(p, p.nbuf + 1) <= kTcSmemMax) p.nbuf++;
  }
  return true;
}

// Row split of a group whose channel columns (2 x channels x up rate, over
// its chunks) are few: the largest S <= limit (at most 8) with S x cols
// columns in one product and a merged window of T + (S - 1) D taps (plus
// pair rounding) within kTcMaxKw.
inline uint32_t tc_row_split(int cols, int tmax, uint32_t D, int limit) {
  uint32_t split = 1;
  while ((int)split < std::min(limit, 8) && cols > 0 && cols * (int)(split + 1) <= (int)kTcDCols &&
         (int64_t)tmax + (int64_t)split * D + 4 <= kTcMaxKw)
    ++split;
  return split;
}

}  // namespace fdsp
