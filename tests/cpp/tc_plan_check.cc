// CPU check of the tensor-core kernel's launch plans (fdsp_tc_plan.h):
// random decimation groups are planned exactly as PolyEngine::launch_tc_group
// plans them (row split, merge sets, pair windows, launches), and every
// shared-memory access the kernel derives from a plan is checked against the
// plan's own sizes:
//   * A operand: MMA kp of merge set m reads records (v, q .. q + 127) and
//     (v + 1, q .. q + 127) of the staged tile, with s = a + tpm kp,
//     q = wrap ? s / D : 0, v = (s - q D) / (tpm / 2) (the kernel's A-offset
//     table); both must lie inside the V x Qp records, and record (v, q) must
//     hold the tile sample q D + v (tpm / 2) that tap s of row 0 needs;
//   * B operand: every work set's taps [o, o + T) inside the merged window;
//   * pair records: even window starts, windows a multiple of four taps;
//   * bulk-copy staging: every staged sample inside the copied span, the span
//     buffer within its limit;
//   * shared memory of the chosen buffer count within the kernel's budget,
//     work sets, slots and merge sets within the launch limits;
//   * row split: S x columns within one product, the merged window in range.
// Prints "ok <cases> <launches> <mmas>" and exits 0, else the first failure
// and exits 1.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "fdsp_tc_plan.h"

using namespace fdsp;

static int fail(const char* what, long long a, long long b) {
  std::printf("FAIL %s (%lld, %lld)\n", what, a, b);
  return 1;
}

int main(int argc, char** argv) {
  const int cases = argc > 1 ? std::atoi(argv[1]) : 3000;
  std::mt19937_64 rng(20261203);
  auto uni = [&](long long lo, long long hi) { return lo + (long long)(rng() % (unsigned long long)(hi - lo + 1)); };
  long long launches = 0, mmas = 0;
  for (int c = 0; c < cases; ++c) {
    // a decimation group: classes (up U, taps T per phase, n channels)
    const uint32_t Dg = (uint32_t)(c % 5 == 0 ? uni(2, 8) : uni(2, 400));
    const int nclass = (int)uni(1, 4);
    struct Cls {
      uint32_t U;
      int T, n;
      int64_t delta0;
      int64_t J;
    };
    std::vector<Cls> cls;
    int cols = 0, tmax = 0;
    for (int k = 0; k < nclass; ++k) {
      Cls q;
      q.U = (uint32_t)uni(1, 4);
      q.T = (int)(uni(1, 32) * 2);  // padded to even, <= 64
      q.n = (int)uni(1, 32);
      q.delta0 = uni(-64, 3 * (long long)Dg);
      q.J = uni(1, 5000);
      cols += 2 * q.n * (int)q.U;
      tmax = std::max(tmax, q.T);
      cls.push_back(q);
    }
    const int limit = (int)uni(1, 8);
    const uint32_t split = tc_row_split(cols, tmax, Dg, limit);
    if (split < 1 || (int)split > std::max(1, limit)) return fail("split range", split, limit);
    if (split > 1 && (cols * (int)split > (int)kTcDCols || tmax + (int)(split - 1) * (int)Dg + 4 > kTcMaxKw))
      return fail("split does not fit one product", split, cols);
    const uint32_t D = Dg * split;
    // work sets as launch_tc_group builds them (window ends of the output
    // phases r spread over about D, then row classes b, b D later)
    std::vector<TcWsPlan> wl;
    for (const Cls& q : cls) {
      for (uint32_t r = 0; r < q.U; ++r) {
        const int64_t J = (q.J - r + q.U - 1) / q.U;
        if (J <= 0) continue;
        const int64_t delta = q.delta0 + (int64_t)((uint64_t)r * Dg / q.U);
        for (uint32_t b = 0; b < split; ++b) {
          if (J <= (int64_t)b) continue;
          TcWsPlan w;
          w.ch = nullptr;
          w.T = q.T;
          w.n = q.n;
          w.phi = 0;
          w.delta = delta + (int64_t)b * Dg;
          w.J = (J - (int64_t)b + split - 1) / split;
          w.U = q.U * split;
          w.r = r + b * q.U;
          wl.push_back(w);
        }
      }
    }
    if (wl.empty()) continue;
    std::vector<int> order(wl.size());
    for (size_t i = 0; i < wl.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return wl[a].delta < wl[b].delta; });
    const int pair = (D % 2 == 0) ? 1 : 0;
    std::vector<TcMsetPlan> msets;
    std::vector<TcLaunchPlan> plans;
    bool fits = false;
    for (int cap = (int)kTcDCols; cap >= 16 && !fits; cap /= 2) {
      msets = tc_merge(wl, order, cap);
      if (pair) tc_pair_windows(msets);
      fits = tc_pack(msets, D, pair, plans);
    }
    if (!fits) continue;  // the group takes the FP32 kernel
    std::vector<int> seen(wl.size(), 0);
    for (const TcLaunchPlan& p : plans) {
      ++launches;
      if (p.pair != pair) return fail("pair flag", p.pair, pair);
      if (p.nbuf < 1 || p.nbuf > kTcMaxBuf) return fail("buffers", p.nbuf, kTcMaxBuf);
      if (tc_smem_need(p, p.nbuf) > kTcSmemMax) return fail("shared memory", (long long)tc_smem_need(p, p.nbuf), kTcSmemMax);
      if (p.nws > kMaxTcWorkSets || p.nslots > kMaxTcSlots || (int)p.ms.size() > kMaxTcMsets)
        return fail("launch limits", p.nws, p.nslots);
      const int tpm = p.pair ? 4 : 2;
      const int rstep = tpm / 2;  // samples of a record
      if (p.pair && (p.B0 & 1)) return fail("pair B0 odd", p.B0, 0);
      int64_t Wmax = 0;
      for (int mi : p.ms) {
        const TcMsetPlan& m = msets[mi];
        const int N = ((m.cols + 15) / 16) * 16;
        if (N > (int)kTcDCols) return fail("N", N, kTcDCols);
        if (m.Kw % tpm) return fail("Kw multiple", m.Kw, tpm);
        const int64_t a = m.S - p.B0;
        if (a < 0) return fail("window before B0", a, 0);
        if (p.pair && (a & 1)) return fail("pair window start odd", a, 0);
        Wmax = std::max<int64_t>(Wmax, a + m.Kw);
        for (int wi : m.ws) {
          const TcWsPlan& w = wl[wi];
          seen[wi]++;
          const int64_t o = (w.delta - w.T + 1) - m.S;
          if (o < 0 || o + w.T > m.Kw) return fail("taps outside the merged window", o, m.Kw);
        }
        const int nkp = m.Kw / tpm;
        for (int kp = 0; kp < nkp; ++kp) {
          ++mmas;
          const int64_t s = a + (int64_t)tpm * kp;
          const int64_t q = p.wrap ? s / D : 0;
          const int64_t off = s - q * D;
          if (off % rstep) return fail("tap offset not on a record", off, rstep);
          const int64_t v = off / rstep;
          if (v < 0 || v + 1 >= p.V) return fail("A phase out of range", v, p.V);
          if (q + 127 >= p.Qp) return fail("A rows out of range", q, p.Qp);
          if (!p.wrap && s + tpm > (int64_t)D) return fail("unwrapped window past D", s, D);
          // record (v', q') holds tile sample q' D + v' rstep (+ 0 .. rstep-1):
          // row 0's taps s .. s + tpm - 1 are records (v, q) and (v + 1, q)
          // (phase D / rstep of row q is phase 0 of row q + 1)
          const int64_t smp0 = q * D + v * rstep, smp1 = q * D + (v + 1) * rstep;
          if (smp0 != s || smp1 != s + rstep) return fail("record holds the wrong sample", smp0, s);
        }
      }
      if (Wmax > (p.wrap ? INT64_MAX : (int64_t)D)) return fail("wrap flag", Wmax, D);
      const int64_t need_v = p.wrap ? (int64_t)D / rstep + 1 : Wmax / rstep;
      if (p.V != need_v) return fail("staged phases", p.V, need_v);
      if ((size_t)p.V * p.Qp * 16 > p.in_bytes) return fail("input buffer", (long long)p.V * p.Qp * 16, (long long)p.in_bytes);
      if (p.raw_span > 0) {
        // the producers read samples q D + v rstep (+ rstep - 1) for q < Qp,
        // v < V from the span copied at the tile's first sample
        const int64_t last = (int64_t)(p.Qp - 1) * D + (int64_t)(p.V - 1) * rstep + (rstep - 1);
        if (last >= p.raw_span) return fail("raw span", last, p.raw_span);
        if (p.raw_stride > kTcRawMax || (size_t)(p.raw_span + 2) * 8 > p.raw_stride)
          return fail("raw buffer", (long long)p.raw_stride, (long long)kTcRawMax);
        if (!(p.Qp & 1)) return fail("raw Qp even", p.Qp, 0);
      }
    }
    for (size_t i = 0; i < seen.size(); ++i)
      if (seen[i] != 1) return fail("work set planned != once", (long long)i, seen[i]);
  }
  std::printf("ok %d %lld %lld\n", cases, launches, mmas);
  return 0;
}
