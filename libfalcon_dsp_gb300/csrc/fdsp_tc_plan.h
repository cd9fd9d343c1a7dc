// Launch planning of the tensor-core filter-bank kernel (host only).
//
// One launch covers every decimation group computed on the tensor cores.
// Per group the output rows (windows ending D apart) become 128-row tiles of
// a matrix product Y = A B:
//
//   A[j][k]  input sample  j D' + a + k  of [history | block], split into
//            16-bit {hi, lo} parts: 4 K elements per sample
//            (re_hi, im_hi, re_lo, im_lo), a Hankel matrix that TMA loads
//            16 samples (128 bytes) at a time through a tensor map whose
//            row stride is D' samples;
//   B[k][n]  the NCO-modulated taps of each output stream ("slot") at its
//            offset inside the merged window, hi taps in columns [0, 2 NS),
//            lo taps in [2 NS, 4 NS) (Re, Im per slot): the epilogue adds
//            the two halves, so each output is (x_hi + x_lo)(g_hi + g_lo)
//            with FP32 accumulation.
//
// A slot is one output class of one channel: output m = r + U j of channel
// c uses tap phase phi and the window ending at delta + j D (block relative).
// A row split S (rows j = S i + b become S slots whose rows are S D apart)
// widens groups with few slots, and makes an odd D even (TMA strides are
// multiples of 16 bytes = 2 samples).  Slots sorted by window start are
// kept together per channel (a bundle, in output order) and partitioned into
// merge sets ("msets") of <= 64 slots (N <= 256) by the fewest K chunks; an
// mset's window starts on an even sample (TMA x coordinates are multiples of
// 16 bytes) and is chunked in 16 taps.
//
// Kept apart from the kernel so that its bounds can be checked on the CPU
// (tests/cpp/tc_plan_check.cc).
#pragma once

#include <stdint.h>

#include <algorithm>
#include <climits>
#include <cstddef>
#include <vector>

#if defined(__CUDACC__)
#define FDSP_HD __host__ __device__
#else
#define FDSP_HD
#endif

namespace fdsp {

constexpr int kTcMaxGroups = 16;
constexpr int kTcSideStreams = 3;  // streams of launch packs 1.. (pack 0 runs on the caller's)
constexpr int kTcMaxMsets = 64;
constexpr int kTcMaxSlots = 512;
constexpr int kTcRows = 128;           // rows per tile (MMA M)
constexpr int kTcChunkTaps = 16;       // taps per K chunk: 128 bytes of A per row
constexpr int kTcTileBytes = kTcRows * 128;
constexpr int kTcMsetSlots = 64;       // slots per merge set (N = 4 NS <= 256)
constexpr int kTcStageMaxBytes = 49152;
constexpr int kTcSmemDyn = 223 * 1024; // dynamic shared memory ceiling (227 KB minus static and alignment)
constexpr int kTcMaxStages = 6;
constexpr int kTcEpiSlotBytes = 48;    // per-slot epilogue constants staged in shared memory

// ---- launch records (kernel parameters; shared with the device code) -----
struct TcGroup {
  int32_t D;        // row stride D' = S D (samples, even)
  int32_t S;        // row split
  int32_t pad_[2];
};

struct TcMset {
  uint64_t b;       // device address of its B image: [nchunks][N][128 B]
  int32_t a;        // window start of row 0 in [history | block] samples (even)
  int32_t items;    // work items (R tiles each)
  int16_t group, slot0, NS, nchunks, R, pad_;
  int32_t ntiles;   // 128-row tiles with an output
};

struct TcSlot {
  uint64_t out;     // float2*: output of row 0 (channel output + r)
  int32_t w0;       // window start of row 0, block relative (delta - T + 1)
  int32_t J;        // rows with an output (0: padding slot)
  uint16_t ch;      // channel
  uint16_t T;       // taps per phase
  uint16_t U;       // output stride (up rate x row split)
  uint16_t o;       // window start inside the merge set's window (taps)
  uint16_t phi;     // tap phase
  uint16_t flags;   // bit 0: the next slot holds the same channel's next output (pair store)
  uint16_t pad_[2];
};
static_assert(sizeof(TcSlot) == 32, "slot record");
static_assert(sizeof(TcMset) == 32, "merge-set record");

// ---- planner input ----------------------------------------------------------
struct TcSlotIn {
  int ch, T, U, r, phi;
  int64_t delta;    // window end of row 0 (block relative)
  int64_t J;        // rows with an output this apply
};
struct TcGroupIn {
  int D;
  int max_split;    // largest row split allowed (power of two, 1..32)
  std::vector<TcSlotIn> slots;
};

struct TcPlanGroup {
  int D, S;
  int64_t Wx;       // samples a row of its tensor map spans (max over its msets of (a mod D') + Kw)
};

struct TcPlan {
  std::vector<TcPlanGroup> groups;
  std::vector<TcMset> ms;         // b = byte offset into the B buffer (the engine adds the base)
  std::vector<TcSlot> slots;      // out = 0 (the engine fills it)
  std::vector<int> slot_r;        // output offset r of each slot (for the out pointer)
  size_t b_bytes = 0;
  int64_t xhl_samples = 0;        // [history | block | zero pad] samples the split writes
  int stages = 0, stage_bytes = 0, smem = 0;  // smem: stages, then the epilogue slot table
  int G = 0;                      // grid (CTAs)
  int64_t Lc = 0;                 // samples of the time range each CTA owns
  int64_t items = 0;
};

inline int64_t tc_round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

// A slot of a split group: output m = r + U j, window ending at delta + j D'.
struct TcSlotX {
  TcSlotIn s;
  int64_t start;  // window start of row 0 (block relative)
};

// A bundle: every slot of one channel under row split S, in output order
// (offset r + b U = 0 .. U S - 1), so that row j of the bundle holds the
// channel's consecutive outputs U S j .. U S j + U S - 1 and the epilogue
// writes them as contiguous pairs (a slot at an even position of its merge
// set and the next one of the same bundle).  Its width is its slot count:
// bundles sit back to back, a one-slot bundle takes one column pair.
struct TcBundle {
  std::vector<TcSlotX> slots;
  int64_t start;  // earliest window start of its slots
  int64_t end;    // latest window end
  int width;
};

inline std::vector<TcBundle> tc_bundles(const TcGroupIn& g, int S) {
  std::vector<TcSlotX> xs;
  for (const TcSlotIn& s : g.slots) {
    for (int b = 0; b < S; ++b) {
      if (s.J <= b) continue;
      TcSlotX x;
      x.s = s;
      x.s.delta = s.delta + (int64_t)b * g.D;
      x.s.J = (s.J - b + S - 1) / S;
      x.s.U = s.U * S;
      x.s.r = s.r + b * s.U;
      x.start = x.s.delta - s.T + 1;
      xs.push_back(x);
    }
  }
  std::stable_sort(xs.begin(), xs.end(), [](const TcSlotX& a, const TcSlotX& b) {
    return a.s.ch != b.s.ch ? a.s.ch < b.s.ch : a.s.r < b.s.r;
  });
  std::vector<TcBundle> bs;
  for (size_t i = 0; i < xs.size();) {
    size_t j = i;
    TcBundle b;
    b.start = xs[i].start;
    b.end = xs[i].s.delta;
    while (j < xs.size() && xs[j].s.ch == xs[i].s.ch) {
      b.start = std::min(b.start, xs[j].start);
      b.end = std::max(b.end, xs[j].s.delta);
      b.slots.push_back(xs[j]);
      ++j;
    }
    b.width = (int)b.slots.size();
    bs.push_back(b);
    i = j;
  }
  std::stable_sort(bs.begin(), bs.end(), [](const TcBundle& a, const TcBundle& b) {
    return a.start != b.start ? a.start < b.start : a.end < b.end;
  });
  return bs;
}

// Merge-set window of bundles [i, j) (sorted by start): its start in
// [history | block] samples rounded down to even, and its K chunks.
inline void tc_window(const std::vector<TcBundle>& bs, size_t i, size_t j, int H, int64_t* a, int64_t* chunks) {
  int64_t st = bs[i].start + H;
  if (st & 1) st -= 1;
  int64_t end = bs[i].end;
  for (size_t q = i + 1; q < j; ++q) end = std::max(end, bs[q].end);
  *a = st;
  *chunks = (end + H - st + 1 + kTcChunkTaps - 1) / kTcChunkTaps;
}

// Partition of the sorted bundles into merge sets of at most kTcMsetSlots
// slots minimising the total K chunks: one MMA of M = 128, K = 16 costs the
// same for any N up to 256, so the work of a tile is its merge sets' chunks
// (dynamic programming over the split points).  Returns the cut points and
// the chunks per tile row; -1 when a bundle alone exceeds a merge set.
inline int64_t tc_partition(const std::vector<TcBundle>& bs, int H, std::vector<size_t>& cuts) {
  const size_t n = bs.size();
  std::vector<int64_t> best(n + 1, INT64_MAX);
  std::vector<size_t> from(n + 1, 0);
  best[0] = 0;
  for (size_t i = 0; i < n; ++i) {
    if (best[i] == INT64_MAX) continue;
    int64_t st = bs[i].start + H;
    if (st & 1) st -= 1;
    int64_t end = bs[i].end;
    int width = 0;
    for (size_t j = i + 1; j <= n; ++j) {
      width += bs[j - 1].width;
      if (width > kTcMsetSlots) break;
      end = std::max(end, bs[j - 1].end);
      const int64_t c = best[i] + (end + H - st + 1 + kTcChunkTaps - 1) / kTcChunkTaps;
      if (c < best[j]) {
        best[j] = c;
        from[j] = i;
      }
    }
  }
  cuts.clear();
  if (best[n] == INT64_MAX) return -1;
  for (size_t j = n; j > 0; j = from[j]) cuts.push_back(j);
  cuts.push_back(0);
  std::reverse(cuts.begin(), cuts.end());
  return best[n];
}

// Row split of a group: the power of two up to max_split (S even for odd D,
// so that rows start 16 bytes apart) with the fewest K chunks over all its
// tiles (chunks per tile row x rows / S); ties keep the smaller split.  A
// channel's bundle (U S slots) fits one merge set, and the group's slots
// stay within four full merge sets.
inline int tc_choose_split(const TcGroupIn& g, int H) {
  int64_t J = 0;
  int Umax = 1;
  for (const TcSlotIn& s : g.slots) {
    J = std::max(J, s.J);
    Umax = std::max(Umax, s.U);
  }
  int bestS = 0;
  double bestc = 0;
  for (int S = 1; S <= std::max((g.D & 1) ? 2 : 1, g.max_split); S *= 2) {
    if ((g.D & 1) && (S & 1)) continue;
    if ((int64_t)Umax * S > kTcMsetSlots) break;
    if (S > 2 && (int64_t)g.slots.size() * S > 4 * kTcMsetSlots) break;
    const std::vector<TcBundle> bs = tc_bundles(g, S);
    if (bs.empty()) continue;
    std::vector<size_t> cuts;
    const int64_t ch = tc_partition(bs, H, cuts);
    if (ch < 0) continue;
    const double c = (double)ch * (double)((J + (int64_t)S * kTcRows - 1) / ((int64_t)S * kTcRows));
    if (bestS == 0 || c < bestc) {
      bestS = S;
      bestc = c;
    }
  }
  return bestS;
}

// Returns 0 on success, -1 when the apply exceeds a launch's record limits
// (the caller keeps those groups on the FP32 kernel).
inline int tc_plan(const std::vector<TcGroupIn>& gin, int64_t N, int H, int num_sms, TcPlan& p) {
  p = TcPlan();
  int64_t wx_max = 0;
  for (const TcGroupIn& g : gin) {
    if (g.slots.empty()) continue;
    const int S = tc_choose_split(g, H);
    if (S == 0) return -1;
    const int64_t Dp = (int64_t)S * g.D;
    const std::vector<TcBundle> bs = tc_bundles(g, S);
    if (bs.empty()) continue;
    if ((int)p.groups.size() >= kTcMaxGroups) return -1;
    const int gi = (int)p.groups.size();
    TcPlanGroup pg;
    pg.D = (int)Dp;
    pg.S = S;
    pg.Wx = 0;
    std::vector<size_t> cuts;
    if (tc_partition(bs, H, cuts) < 0) return -1;
    for (size_t ci = 0; ci + 1 < cuts.size(); ++ci) {
      const size_t i = cuts[ci], j = cuts[ci + 1];
      int64_t a, nchunks;
      tc_window(bs, i, j, H, &a, &nchunks);
      int width = 0;
      for (size_t q = i; q < j; ++q) width += bs[q].width;
      // record field ranges (16-bit taps, strides and offsets)
      if (nchunks * kTcChunkTaps > 65535) return -1;
      for (size_t q = i; q < j; ++q)
        for (const TcSlotX& x : bs[q].slots)
          if (x.s.T > 65535 || x.s.U > 65535 || x.s.phi > 65535 || x.s.J > INT32_MAX) return -1;
      const int NS = (int)tc_round_up(width, 8);
      if ((int)p.ms.size() >= kTcMaxMsets || (int)p.slots.size() + NS > kTcMaxSlots) return -1;
      TcMset m{};
      m.a = (int32_t)a;
      m.group = (int16_t)gi;
      m.slot0 = (int16_t)p.slots.size();
      m.NS = (int16_t)NS;
      m.nchunks = (int16_t)nchunks;
      m.R = (int16_t)(4 * NS <= 128 ? 2 : 1);
      int64_t Jmax = 0;
      for (size_t q = i; q < j; ++q) {
        const TcBundle& b = bs[q];
        const size_t pos0 = p.slots.size() - (size_t)m.slot0;  // the bundle's first position in the merge set
        for (size_t k = 0; k < b.slots.size(); ++k) {
          const TcSlotX& x = b.slots[k];
          TcSlot s{};
          s.w0 = (int32_t)x.start;
          s.J = (int32_t)x.s.J;
          s.ch = (uint16_t)x.s.ch;
          s.T = (uint16_t)x.s.T;
          s.U = (uint16_t)x.s.U;
          s.o = (uint16_t)(x.start + H - a);
          s.phi = (uint16_t)x.s.phi;
          // a slot at an even position followed by the channel's next output:
          // one 16-byte store
          s.flags = ((pos0 + k) % 2 == 0 && k + 1 < b.slots.size() && b.slots[k + 1].s.r == x.s.r + 1) ? 1 : 0;
          p.slots.push_back(s);
          p.slot_r.push_back(x.s.r);
          Jmax = std::max(Jmax, x.s.J);
        }
      }
      for (int q = width; q < NS; ++q) {
        p.slots.push_back(TcSlot{});
        p.slot_r.push_back(0);
      }
      m.ntiles = (int32_t)((Jmax + kTcRows - 1) / kTcRows);
      m.items = (m.ntiles + m.R - 1) / m.R;
      m.b = p.b_bytes;
      p.b_bytes += (size_t)tc_round_up((int64_t)m.nchunks * 4 * NS * 128, 1024);
      pg.Wx = std::max<int64_t>(pg.Wx, a % Dp + (int64_t)m.nchunks * kTcChunkTaps);
      p.ms.push_back(m);
    }
    wx_max = std::max(wx_max, pg.Wx);
    p.groups.push_back(pg);
  }
  if (p.ms.empty()) return 0;
  // the split writes [history | block] and a zero tail: every row a tensor
  // map can address ((rows - 1) D' + Wx samples) stays inside it
  p.xhl_samples = tc_round_up(N + H + wx_max + 16, 16);
  // pipeline stages: R A tiles + one B chunk each
  int sb = 0;
  for (const TcMset& m : p.ms)
    sb = std::max<int>(sb, m.R * kTcTileBytes + (int)tc_round_up((int64_t)4 * m.NS * 128, 1024));
  if (sb > kTcStageMaxBytes) return -1;
  p.stage_bytes = sb;
  const int table = (int)tc_round_up((int64_t)p.slots.size() * kTcEpiSlotBytes, 1024);
  p.stages = std::min(kTcMaxStages, (kTcSmemDyn - 1024 - table) / sb);
  if (p.stages < 2) return -1;
  p.smem = p.stages * sb + table + 1024;
  // schedule: each CTA owns a contiguous range of input samples and runs the
  // items of every merge set that start in it, in input order
  int64_t umax = 0;
  for (const TcMset& m : p.ms) {
    const int64_t P = (int64_t)m.R * kTcRows * p.groups[m.group].D;
    umax = std::max<int64_t>(umax, m.a + (int64_t)m.items * P);
    p.items += m.items;
  }
  p.G = (int)std::max<int64_t>(1, std::min<int64_t>(num_sms, p.items));
  p.Lc = (umax + p.G - 1) / p.G;
  return 0;
}

// Item range [first, last) of merge set m owned by CTA b (shared with the
// device code: every role walks the same sequence).
FDSP_HD inline void tc_item_range(int64_t a, int64_t P, int64_t items, int64_t Lc, int b, int G, int64_t* first,
                          int64_t* last) {
  const int64_t v0 = (int64_t)b * Lc - a, v1 = (int64_t)(b + 1) * Lc - a;
  int64_t f = v0 <= 0 ? 0 : (v0 + P - 1) / P;
  int64_t l = v1 <= 0 ? 0 : (v1 + P - 1) / P;
  *first = f < items ? f : items;
  *last = (b == G - 1) ? items : (l < items ? l : items);
}

}  // namespace fdsp
