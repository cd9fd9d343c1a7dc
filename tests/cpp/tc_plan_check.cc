// Bounds and coverage of the tensor-core planner (libfalcon_dsp_gb300/csrc/
// fdsp_tc_plan.h) on random channel sets, checked on the CPU before any plan
// reaches a GPU.  For every plan it restates what the kernels derive from it:
//
//   * the TMA tile loads of A: x coordinates 16-byte aligned and inside the
//     tensor map's row span, every row an output needs inside the map's rows,
//     and the map's last addressable sample inside the split buffer;
//   * each slot's window inside its merge set's chunked window, and the merge
//     set's row-j window equal to the slot's own input window;
//   * the samples each valid output reads lie in [history | block];
//   * B images inside the B buffer, stages inside shared memory, N and R
//     inside one accumulator slot of tensor memory;
//   * the per-CTA item ranges partition every merge set's items;
//   * every output of every channel is written by exactly one (slot, row).
//
// Usage: tc_plan_check <cases>; prints "ok <cases> <msets> <items>".
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "fdsp_tc_plan.h"

using namespace fdsp;

static int g_fail = 0;
#define CHECK(c, ...)                                     \
  do {                                                    \
    if (!(c)) {                                           \
      if (g_fail < 20) {                                  \
        std::printf("FAIL %s:%d: %s | ", __FILE__, __LINE__, #c); \
        std::printf(__VA_ARGS__);                         \
        std::printf("\n");                                \
      }                                                   \
      g_fail++;                                           \
    }                                                     \
  } while (0)

// Outputs the reference loop emits for n inputs from (phase, xoffset).
static uint64_t out_count(uint32_t up, uint32_t down, uint32_t phase, uint64_t xoffset, uint64_t n) {
  if (xoffset >= n) return 0;
  const unsigned __int128 lim = (unsigned __int128)up * (n - xoffset);
  return (uint64_t)((lim - phase + down - 1) / down);
}

int main(int argc, char** argv) {
  const int cases = argc > 1 ? std::atoi(argv[1]) : 2000;
  std::mt19937_64 rng(12345);
  auto U = [&](int64_t lo, int64_t hi) { return (int64_t)(lo + (int64_t)(rng() % (uint64_t)(hi - lo + 1))); };
  int64_t total_ms = 0, total_items = 0;
  for (int cs = 0; cs < cases; ++cs) {
    // channels of a few classes; classes of the same down rate form a group
    const int ngroups = (int)U(1, 6);
    std::vector<TcGroupIn> gin;
    struct Cls {
      int up, down, phase;
      int64_t xoff;
      std::vector<int> T;  // per channel
      std::vector<int> ch;
    };
    std::vector<Cls> classes;
    int nch = 0, Tmax = 1;
    const bool long_fir = (cs % 17) == 0;
    for (int g = 0; g < ngroups; ++g) {
      const int D = long_fir ? (int)U(1, 12) : (int)U(1, 400);
      const int ncls = (int)U(1, 3);
      for (int k = 0; k < ncls; ++k) {
        Cls c;
        c.down = D;
        c.up = long_fir ? 1 : (int)U(1, 4);
        c.phase = (int)U(0, c.up - 1);
        c.xoff = U(0, D);
        const int n = long_fir ? 1 : (int)U(1, 24);
        for (int i = 0; i < n; ++i) {
          const int T = long_fir ? (int)U(200, 5000) : (int)U(1, 70);
          c.T.push_back(T);
          c.ch.push_back(nch++);
          Tmax = std::max(Tmax, T);
        }
        classes.push_back(c);
      }
      if (long_fir) break;
    }
    if (nch > 512) continue;
    const int H = Tmax - 1;
    const int64_t N = U(1, 3) == 1 ? U(1, 5000) : U(20000, 3000000);
    const int max_split = 1 << U(0, 5);
    // planner input (as PolyEngine::launch_tc builds it)
    std::vector<int> gd;
    for (const Cls& c : classes)
      if (std::find(gd.begin(), gd.end(), c.down) == gd.end()) gd.push_back(c.down);
    std::vector<int64_t> M(nch, 0);
    std::vector<int> ch_up(nch), ch_T(nch);
    for (int D : gd) {
      TcGroupIn in;
      in.D = D;
      in.max_split = max_split;
      for (const Cls& c : classes) {
        if (c.down != D) continue;
        const uint64_t m = out_count(c.up, c.down, c.phase, c.xoff, N);
        for (size_t i = 0; i < c.ch.size(); ++i) {
          M[c.ch[i]] = (int64_t)m;
          ch_up[c.ch[i]] = c.up;
          ch_T[c.ch[i]] = c.T[i];
        }
        for (int r = 0; r < c.up; ++r) {
          if ((int64_t)m <= r) continue;
          const uint64_t tt = (uint64_t)c.phase + (uint64_t)r * D;
          for (size_t i = 0; i < c.ch.size(); ++i) {
            TcSlotIn s;
            s.ch = c.ch[i];
            s.T = c.T[i];
            s.U = c.up;
            s.r = r;
            s.phi = (int)(tt % c.up);
            s.delta = (int64_t)(c.xoff + tt / c.up);
            s.J = (int64_t)((m - r + c.up - 1) / c.up);
            in.slots.push_back(s);
          }
        }
      }
      gin.push_back(in);
    }
    TcPlan p;
    const int num_sms = (int)U(1, 152);
    if (tc_plan(gin, N, H, num_sms, p) != 0) continue;  // beyond the record limits: FP32 form
    total_ms += (int64_t)p.ms.size();
    total_items += p.items;
    CHECK(p.ms.size() <= (size_t)kTcMaxMsets && p.slots.size() <= (size_t)kTcMaxSlots &&
              p.groups.size() <= (size_t)kTcMaxGroups,
          "record limits");
    if (p.ms.empty()) continue;
    CHECK(p.smem <= kTcSmemDyn && p.stages >= 2 && p.stages <= kTcMaxStages, "smem %d stages %d", p.smem, p.stages);
    CHECK((int64_t)p.stages * p.stage_bytes + (int64_t)p.slots.size() * kTcEpiSlotBytes + 1024 <= p.smem,
          "stages + epilogue table inside the dynamic shared memory");
    CHECK(p.xhl_samples >= N + H, "split buffer");
    // coverage: one writer per output
    std::vector<std::vector<uint8_t>> hit(nch);
    for (int c = 0; c < nch; ++c) hit[c].assign((size_t)M[c], 0);
    size_t bsum = 0;
    for (size_t mi = 0; mi < p.ms.size(); ++mi) {
      const TcMset& m = p.ms[mi];
      const TcPlanGroup& g = p.groups[m.group];
      const int64_t D = g.D;
      const int N4 = 4 * m.NS;
      CHECK(D % 2 == 0 && D > 0, "row stride %lld", (long long)D);
      CHECK(m.a % 2 == 0 && m.a >= 0, "window start %d", m.a);
      CHECK(m.NS % 8 == 0 && N4 >= 32 && N4 <= 256 && N4 % 16 == 0, "N %d", N4);
      CHECK(m.R * N4 <= 256 && (m.R == 1 || m.R == 2), "tmem R %d N %d", m.R, N4);
      CHECK(m.R * kTcTileBytes + tc_round_up((int64_t)N4 * 128, 1024) <= p.stage_bytes, "stage");
      CHECK(m.b % 1024 == 0 && m.b + (uint64_t)m.nchunks * N4 * 128 <= p.b_bytes, "B image");
      bsum += (size_t)m.nchunks * N4 * 128;
      const int64_t Kw = (int64_t)m.nchunks * kTcChunkTaps;
      // TMA: x coordinates and the map's rows
      const int64_t x0 = 4 * (m.a % D);
      CHECK(x0 % 8 == 0, "x alignment");
      CHECK(x0 / 4 + Kw <= g.Wx, "x range: a mod D %lld Kw %lld Wx %lld", (long long)(m.a % D), (long long)Kw,
            (long long)g.Wx);
      const int64_t rows = (p.xhl_samples - g.Wx) / D + 1;
      CHECK((rows - 1) * D + g.Wx <= p.xhl_samples, "map end");
      int64_t Jmax = 0;
      for (int s = 0; s < m.NS; ++s) {
        const TcSlot& sl = p.slots[m.slot0 + s];
        if (sl.J == 0) continue;
        Jmax = std::max<int64_t>(Jmax, sl.J);
        CHECK(sl.o + sl.T <= Kw, "slot window in merged window: o %d T %d Kw %lld", sl.o, sl.T, (long long)Kw);
        CHECK(m.a + sl.o == (int64_t)sl.w0 + H, "slot offset");
        if (sl.flags & 1) {  // pair store: the next slot is the same channel's next output
          const TcSlot& nx = p.slots[m.slot0 + s + 1];
          CHECK(s % 2 == 0 && s + 1 < m.NS && nx.J > 0 && nx.ch == sl.ch && nx.U == sl.U &&
                    p.slot_r[m.slot0 + s + 1] == p.slot_r[m.slot0 + s] + 1 && nx.J <= sl.J && nx.J + 1 >= sl.J,
                "pair flag");
        }
        // the last valid row reads only [history | block] and lies inside the map
        const int64_t jl = sl.J - 1;
        const int64_t first = jl * D + sl.w0 + H, last = first + sl.T - 1;
        CHECK(sl.w0 + H >= 0 && last < N + H, "window samples [%lld, %lld] of %lld", (long long)(sl.w0 + H),
              (long long)last, (long long)(N + H));
        CHECK(jl + m.a / D < rows, "row inside the map");
        const int c = sl.ch;
        const int r = p.slot_r[m.slot0 + s];
        CHECK(sl.T == ch_T[c], "taps");
        for (int64_t j = 0; j < sl.J; ++j) {
          const int64_t o = r + (int64_t)sl.U * j;
          if (o < 0 || o >= M[c]) {
            CHECK(false, "output %lld of channel %d beyond %lld", (long long)o, c, (long long)M[c]);
            break;
          }
          hit[c][(size_t)o]++;
        }
      }
      CHECK(m.ntiles == (Jmax + kTcRows - 1) / kTcRows && m.items == (m.ntiles + m.R - 1) / m.R, "tiles");
      // item ranges partition [0, items)
      const int64_t P = (int64_t)m.R * kTcRows * D;
      int64_t next = 0;
      for (int b = 0; b < p.G; ++b) {
        int64_t f, l;
        tc_item_range(m.a, P, m.items, p.Lc, b, p.G, &f, &l);
        CHECK(f == next && l >= f, "item ranges: cta %d [%lld, %lld) after %lld", b, (long long)f, (long long)l,
              (long long)next);
        next = l;
      }
      CHECK(next == m.items, "items covered %lld of %d", (long long)next, m.items);
    }
    for (int c = 0; c < nch; ++c)
      for (int64_t o = 0; o < M[c]; ++o)
        if (hit[c][(size_t)o] != 1) {
          CHECK(false, "channel %d output %lld written %d times", c, (long long)o, (int)hit[c][(size_t)o]);
          break;
        }
    if (g_fail) break;
  }
  if (g_fail) {
    std::printf("FAILED %d\n", g_fail);
    return 1;
  }
  std::printf("ok %d %lld %lld\n", cases, (long long)total_ms, (long long)total_items);
  return 0;
}
