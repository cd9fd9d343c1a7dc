// Tensor-core form of the polyphase engine (tcgen05 + TMA, sm_103a).
//
// The fused shift + polyphase contraction of the decimation groups of an
// apply runs as persistent launches of matrix products over 128-row tiles,
// one per launch pack (as many groups as the launch records hold; the
// planner, fdsp_tc_plan.h, describes the operands):
//
//     Y[j][n] = sum_k A[j][k] B[k][n]
//
//   A  input samples j D' + a + k of [history | block] as 16-bit {hi, lo}
//      parts (4 K elements a sample), loaded 16 samples at a time by TMA
//      into the 128-byte-swizzled K-major layout: a tensor map whose rows
//      are D' samples apart (rows overlap when D' < 16) turns the Hankel
//      matrix of each tile into one TMA copy per K chunk, no staging code;
//   B  the NCO-modulated taps of the merge set's output streams ("slots"),
//      hi taps in the first half of the columns and lo taps in the second,
//      prebuilt per apply in the same swizzled image and copied per chunk;
//   Y  FP32 in tensor memory; the epilogue adds the hi and lo halves,
//      rotates by the NCO phase of each window start (exact integer phase)
//      and stores.  Windows across the NCO rollover are stored unrotated and
//      rotated exactly (split sum) by tc_fix_kernel, launched after the
//      filter bank: keeping that rare path out of the filter-bank kernel
//      roughly halved its MMA issue time.
//
// Per CTA (one per SM, 608 threads):
//   warp 0      producer: takes the CTA's items from the scheduler's queue
//               and announces each in a ring with its first stage; per
//               item (R tiles of one merge set) and K chunk,
//               waits for a free stage, then R TMA tile loads of A and one
//               bulk copy of the B chunk, completing on the stage barrier;
//   warp 1      MMA issuer: per chunk 4 MMAs (K = 16) per tile into the
//               item's accumulator slot, commit frees the stage; the last
//               chunk's commit hands the slot to the epilogue;
//   warps 2-17  epilogue: four warps per TMEM lane quarter; each reads its
//               (at most two) 8-slot column chunks out of tensor memory,
//               releases the slot, then rotates and stores;
//   warp 18     scheduler: finds the CTA's next items (a warp-parallel
//               cursor over the merge sets) and queues them for warp 0.
// Warps 0 and 1 run their loops in lane 0 alone.
// Two accumulator slots of 256 columns (R tiles x N columns each) let the
// MMAs of one item run while the epilogue drains the previous one.
//
// Each CTA owns a contiguous range of input samples and runs, in input
// order, the items of every merge set that start in it, so the split input
// is read from HBM about once and every group reuses it from L2.
//
// Every mbarrier wait is bounded (TcLaunch::poll); a wait that runs out sets
// the error flag (mapped host memory, read by fdsp_channelizer_status),
// drains the copies and MMAs this CTA issued and exits.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cmath>
#include <cstring>
#include <vector>

#include "fdsp_internal.h"
#include "fdsp_nco.cuh"
#include "fdsp_tc.cuh"

namespace fdsp {

constexpr int kTcEpiWarps = 16;                       // kTcEpiPerQ per TMEM lane quarter
constexpr int kTcEpiPerQ = kTcEpiWarps / 4;
constexpr int kTcEpiOwn = 8 / kTcEpiPerQ;             // most column chunks a warp reads per item (R NS <= 64)
constexpr int kTcSchedWarp = 2 + kTcEpiWarps;         // the item scheduler (after the epilogue warps)
constexpr int kTcThreads = 96 + 32 * kTcEpiWarps;     // producer, MMA, epilogue and scheduler warps
constexpr int kTcRing = 16;                           // items announced ahead (> stages + 2)
constexpr int kTcQueue = 64;                          // items the scheduler warp finds ahead
constexpr uint32_t kTmemCols = 512;

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
template <int FMT>
__device__ __forceinline__ void split2(float2 x, uint32_t& hi, uint32_t& lo) {
  if constexpr (FMT == 0) {
    const __half2 h = __float22half2_rn(x);
    const float2 hf = __half22float2(h);
    const __half2 l = __float22half2_rn(make_float2(x.x - hf.x, x.y - hf.y));
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  } else {
    const __nv_bfloat162 h = __float22bfloat162_rn(x);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __float22bfloat162_rn(make_float2(x.x - hf.x, x.y - hf.y));
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  }
}

__device__ __forceinline__ float2 tc_load_x(const TcLaunch& L, int64_t v) {
  if (v < 0) {
    const int64_t hv = v + L.H;
    return hv >= 0 ? L.hist[hv] : make_float2(0.f, 0.f);
  }
  if (v >= L.N) return make_float2(0.f, 0.f);
  if (L.block16 != nullptr) {
    const short2 s = L.block16[v];
    return make_float2((float)s.x, (float)s.y);
  }
  return __ldg(L.block + v);
}

// Shared-memory matrix descriptor, K-major, 128-byte swizzle: 8-row atoms of
// 128-byte rows 1024 bytes apart (stride byte offset), version 1, layout 2.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1u << 16) | ((uint64_t)(1024u >> 4) << 32) |
         ((uint64_t)1u << 46) | ((uint64_t)2u << 61);
}

__device__ __forceinline__ void mma_f16_ss(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                           uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int32_t x, int32_t y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
          dst),
      "l"(map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(tc::smem_u32(bar)), "r"(bytes)
               : "memory");
}

// The sequence of items (merge set, item index) a CTA runs, walked by the
// producer warp and announced to the MMA and epilogue warps through a ring of
// (merge set, item) entries.  Items of merge set m start at input sample
// a + t P; the next item is the earliest start (ties: the lower merge set).
// Lane l keeps merge sets l and l + 32 in registers: its next start u, its
// item range [cur, end) and P; a butterfly reduction picks the next item.
struct TcCursor {
  int64_t u[2], P[2];
  int32_t cur[2], end[2];
  __device__ void init(const TcMset* ms, const TcGroup* groups, int nmsets, int64_t Lc, int G, int b, int lane) {
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int m = lane + 32 * i;
      cur[i] = end[i] = 0;
      u[i] = P[i] = 0;
      if (m >= nmsets) continue;
      const TcMset& M = ms[m];
      P[i] = (int64_t)M.R * kTcRows * groups[M.group].D;
      int64_t f, l;
      tc_item_range(M.a, P[i], M.items, Lc, b, G, &f, &l);
      cur[i] = (int32_t)f;
      end[i] = (int32_t)l;
      u[i] = (int64_t)M.a + f * P[i];
    }
  }
  // (whole warp; every lane returns the same item)
  __device__ __forceinline__ bool next(int lane, int* m_out, int* t_out) {
    int64_t bu = INT64_MAX;
    int bm = INT32_MAX;
#pragma unroll
    for (int i = 0; i < 2; ++i)
      if (cur[i] < end[i] && u[i] < bu) {
        bu = u[i];
        bm = lane + 32 * i;
      }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const int64_t u2 = __shfl_xor_sync(0xffffffffu, bu, o);
      const int m2 = __shfl_xor_sync(0xffffffffu, bm, o);
      if (u2 < bu || (u2 == bu && m2 < bm)) {
        bu = u2;
        bm = m2;
      }
    }
    if (bm == INT32_MAX) return false;
    int t = 0;
    if ((bm & 31) == lane) {
      const int i = bm >> 5;
      t = i ? cur[1] : cur[0];
      if (i) {
        cur[1]++;
        u[1] += P[1];
      } else {
        cur[0]++;
        u[0] += P[0];
      }
    }
    *m_out = bm;
    *t_out = __shfl_sync(0xffffffffu, t, bm & 31);
    return true;
  }
};

// Position in the stage ring: stage s of round r (chunk r * stages + s),
// advanced without a division per chunk.
struct TcRing {
  int s = 0, r = 0;
  __device__ __forceinline__ void next(int stages) {
    if (++s == stages) {
      s = 0;
      ++r;
    }
  }
};

// ---------------------------------------------------------------------------
// prep: split [history | block] into {hi, lo} parts and build the B images
// ---------------------------------------------------------------------------
// B image of merge set m, chunk c: N = 4 NS rows (columns of B) of 128
// bytes, the 16-byte piece q of row n (taps 2q, 2q + 1 of the chunk) at
// (q ^ (n & 7)) 16, the 128-byte swizzle of a 1024-byte-aligned atom.
// Column n: hi/lo half h = n / (2 NS), slot s = (n mod 2 NS) / 2, part
// p = n & 1 (Re, Im).  For the input elements (x_re, x_im) of either half
// (hi or lo) the Re column holds (g_re, -g_im) and the Im column (g_im, g_re)
// of the tap's hi or lo part.
template <int FMT>
__global__ void __launch_bounds__(256) tc_prep_kernel(const __grid_constant__ TcLaunch L, int nb_build) {
  if (blockIdx.x == 0) {  // the record, for the filter-bank kernel
    const uint4* src = reinterpret_cast<const uint4*>(&L);
    uint4* dst = reinterpret_cast<uint4*>(L.rec_out);
    for (int i = (int)threadIdx.x; i < (int)(sizeof(TcLaunch) / 16); i += 256) dst[i] = src[i];
  }
  if ((int)blockIdx.x < nb_build) {
    const int total = L.bprefix[L.nmsets];
    for (int p = (int)blockIdx.x * 256 + (int)threadIdx.x; p < total; p += nb_build * 256) {
      int lo = 0, hi = L.nmsets;  // largest m with bprefix[m] <= p
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (L.bprefix[mid] <= p) lo = mid;
        else hi = mid;
      }
      const TcMset& M = L.ms[lo];
      const int NS = M.NS, N = 4 * NS;
      const int lp = p - L.bprefix[lo];
      const int c = lp / (N * 8);
      const int rem = lp - c * N * 8;
      const int n = rem >> 3, q = rem & 7;
      const int h = n / (2 * NS);
      const int s = (n - h * 2 * NS) >> 1, part = n & 1;
      const TcSlot& S = L.slots[M.slot0 + s];
      uint32_t w[4] = {0u, 0u, 0u, 0u};
      if (S.J > 0) {
        const float2* g = L.ctaps[S.ch] + (size_t)S.phi * S.T;
        for (int u = 0; u < 2; ++u) {
          const int t = c * kTcChunkTaps + 2 * q + u - (int)S.o;
          if (t < 0 || t >= (int)S.T) continue;
          uint32_t gh, gl;
          split2<FMT>(__ldg(g + t), gh, gl);
          const uint32_t v = h ? gl : gh;  // {re, im} of the tap's hi or lo part
          const uint32_t re = v & 0xFFFFu, im = v >> 16;
          const uint32_t e0 = part ? (im | (re << 16)) : (re | ((im ^ 0x8000u) << 16));
          w[2 * u] = e0;       // x_hi elements
          w[2 * u + 1] = e0;   // x_lo elements
        }
      }
      uint8_t* dst = L.bbuf + M.b + ((size_t)c * N + n) * 128 + (size_t)((q ^ (n & 7)) * 16);
      *reinterpret_cast<uint4*>(dst) = make_uint4(w[0], w[1], w[2], w[3]);
    }
    return;
  }
  const int64_t stride = (int64_t)(gridDim.x - nb_build) * 256;
  const int64_t NH = L.N + L.H;
  for (int64_t u = (int64_t)(blockIdx.x - nb_build) * 256 + threadIdx.x; u < L.xhl_n; u += stride) {
    float2 x = make_float2(0.f, 0.f);
    if (u < L.H) {
      x = L.hist[u];
    } else if (u < NH) {
      if (L.block16 != nullptr) {
        const short2 s = L.block16[u - L.H];
        x = make_float2((float)s.x, (float)s.y);
      } else {
        x = L.block[u - L.H];
      }
    }
    uint2 hl;
    split2<FMT>(x, hl.x, hl.y);
    L.xhl[u] = hl;
  }
}

// ---------------------------------------------------------------------------
// epilogue constants and the exact NCO path
// ---------------------------------------------------------------------------
// Per-slot epilogue constants, staged in shared memory at CTA start (read
// with warp-uniform addresses: broadcasts, no constant-cache traffic).
struct TcEpiSlot {
  uint64_t out;   // float2*: output of row 0
  uint64_t om;    // NCO turns per sample (2^-64 units); 0: no rotation
  uint64_t fm;    // ceil(2^64 / R): (a mod R) as one multiply-high (Lemire et al. 2019)
  int64_t x0;     // NCO counter argument of row 0's window start (base + w0, unreduced)
  uint32_t R;     // counter rollover; 0: every output takes the exact path
  int32_t J;      // rows with an output
  uint16_t U;     // output stride
  uint16_t Tm1;   // taps - 1
  uint32_t pair;  // 1: the next slot holds this channel's next output (one 16-byte store)
};
static_assert(sizeof(TcEpiSlot) == kTcEpiSlotBytes, "epilogue slot table layout");
static_assert(offsetof(TcEpiSlot, om) == 8 && offsetof(TcEpiSlot, R) == 32 && offsetof(TcEpiSlot, J) == 36 &&
                  offsetof(TcEpiSlot, U) == 40 && offsetof(TcEpiSlot, Tm1) == 42 && offsetof(TcEpiSlot, pair) == 44,
              "the epilogue reads a slot record as two 16-byte halves");

// Outputs whose window crosses the NCO rollover (or whose counter leaves the
// fast path's 32-bit range) were stored unrotated; rotate_prep/rotate_apply
// split the window sum at the rollover exactly, from the FP32 modulated taps.
__device__ __noinline__ void tc_fix_exact(const TcLaunch& L, int slot, int64_t j, int64_t D, float2* dst) {
  const TcSlot& S = L.slots[slot];
  const NcoConst nc = L.nco[S.ch];
  OutMeta cm;
  cm.omega64 = nc.omega64;
  cm.wrap64 = nc.wrap64;
  cm.fastmod = nc.fastmod;
  cm.out = nullptr;
  cm.rollover = nc.rollover;
  cm.base = L.nco_base[S.ch];
  cm.enabled = nc.enabled;
  cm.pad_ = 0;
  const int64_t w0 = (int64_t)S.w0 + j * D;
  const ExactRot er = rotate_prep(cm, w0, S.T);
  float2 B = make_float2(0.f, 0.f);
  if (er.straddle) {
    const float2* g = L.ctaps[S.ch] + (size_t)S.phi * S.T;
    for (int k = er.k0; k < (int)S.T; ++k) {
      const float2 x = tc_load_x(L, w0 + k);
      const float2 gk = __ldg(g + k);
      B.x = fmaf(gk.x, x.x, B.x);
      B.x = fmaf(-gk.y, x.y, B.x);
      B.y = fmaf(gk.x, x.y, B.y);
      B.y = fmaf(gk.y, x.x, B.y);
    }
  }
  *dst = rotate_apply(er, *dst, B);
}

// Row stride D' of the merge set that holds slot s.
__device__ __forceinline__ int64_t tc_slot_stride(const TcLaunch& L, int s) {
  for (int m = 0; m < L.nmsets; ++m)
    if (s >= L.ms[m].slot0 && s < L.ms[m].slot0 + L.ms[m].NS) return L.groups[L.ms[m].group].D;
  return 0;
}

// Whether the filter-bank epilogue rotates slot S's rows itself (its fast
// path); when not, every row of the slot was stored unrotated.
__device__ __forceinline__ bool tc_slot_fast(const TcLaunch& L, const NcoConst& nc, int64_t Dp, int T) {
  return !L.exact_all && nc.rollover < 0x80000000u && (int64_t)31 * Dp + T < (int64_t)nc.rollover;
}

// Exact rotation of the rows that the filter-bank kernel stored unrotated:
// windows that straddle the NCO rollover (the phase restarts inside the
// window, so the product splits into the taps before and after it), or every
// row of a slot whose rollover is too short (or too long) for the epilogue's
// 32-bit counters.  Blocks (slot, y): the gridDim.y blocks of a slot take its
// rollover points (or its rows) in turn.  Runs after the filter-bank launch
// on the same stream.
__global__ void __launch_bounds__(128) tc_fix_kernel(const __grid_constant__ TcLaunch L) {
  const int s = blockIdx.x;
  if (s >= L.nslots) return;
  const TcSlot& S = L.slots[s];
  if (S.J <= 0 || S.T == 0) return;
  const NcoConst nc = L.nco[S.ch];
  if (!nc.enabled || nc.omega64 == 0 || nc.rollover == 0) return;
  const int64_t Dp = tc_slot_stride(L, s);
  if (Dp <= 0) return;
  float2* out = reinterpret_cast<float2*>(S.out);
  const int64_t J = S.J, T = S.T, R = nc.rollover;
  const int64_t t0 = (int64_t)blockIdx.y * blockDim.x + threadIdx.x, tstep = (int64_t)gridDim.y * blockDim.x;
  if (!tc_slot_fast(L, nc, Dp, (int)T)) {
    for (int64_t j = t0; j < J; j += tstep) tc_fix_exact(L, s, j, Dp, out + (uint64_t)S.U * (uint64_t)j);
    return;
  }
  // rollover points n (block relative): (nco_base + n) mod R == 0; row j's
  // window [w0 + j D', w0 + j D' + T - 1] straddles n when it holds n - 1 and n
  const int64_t w0 = S.w0;
  const int64_t base = L.nco_base[S.ch];
  const int64_t first = w0 + 1;                            // smallest n a window can straddle
  const int64_t last = w0 + (J - 1) * Dp + T - 1;          // largest
  int64_t r0 = (base + first) % R;
  if (r0 < 0) r0 += R;
  const int64_t n0 = first + (r0 == 0 ? 0 : R - r0);
  for (int64_t n = n0 + t0 * R; n <= last; n += tstep * R) {
    // rows with n - T + 1 <= w0 + j D' <= n - 1
    const int64_t lo = n - T + 1 - w0, hi = n - 1 - w0;
    int64_t j0 = lo <= 0 ? 0 : (lo + Dp - 1) / Dp;
    int64_t j1 = hi < 0 ? -1 : hi / Dp;
    if (j1 > J - 1) j1 = J - 1;
    for (int64_t j = j0; j <= j1; ++j) tc_fix_exact(L, s, j, Dp, out + (uint64_t)S.U * (uint64_t)j);
  }
}

// 16-byte shared-memory load (one instruction for four fields of a slot record).
__device__ __forceinline__ uint4 lds128(uint32_t addr) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];\n" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(addr));
  return v;
}

// ---------------------------------------------------------------------------
// the filter-bank kernel
// ---------------------------------------------------------------------------
template <int FMT>
__global__ void __launch_bounds__(kTcThreads, 1) tc_filter_kernel(const __grid_constant__ TcFilterParams P) {
  const TcLaunch& L = *P.rec;
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[kTcMaxStages];
  __shared__ __align__(8) uint64_t empty_bar[kTcMaxStages];
  __shared__ __align__(8) uint64_t acc_full[2];
  __shared__ __align__(8) uint64_t acc_empty[2];
  __shared__ __align__(8) uint64_t drain_bar;
  __shared__ uint32_t tmem_base_s;
  __shared__ int2 ring[kTcRing];       // item k: (merge set, item index); merge set -1 ends the sequence
  __shared__ int2 q_items[kTcQueue];   // scheduler -> producer: item i at i % kTcQueue
  __shared__ int q_prod, q_cons;       // items written / taken
  __shared__ TcMset s_ms[kTcMaxMsets];       // merge sets and groups of the launch (read per item)
  __shared__ TcGroup s_groups[kTcMaxGroups];
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;
  const uint32_t sbase = (tc::smem_u32(smem_raw) + 1023u) & ~1023u;
  // launch constants in registers (L lives in device memory, and the inline
  // PTX's memory clobbers would otherwise reload them every chunk)
  const int stages = L.stages;
  const uint32_t poll = L.poll;
  const uint32_t stage_bytes = (uint32_t)L.stage_bytes;
  const bool hold = L.hold != 0;
  const uint8_t* const bbuf = L.bbuf;

  if (warp == 0) {
    tc::tmem_alloc(&tmem_base_s, kTmemCols);
    tc::tmem_relinquish();
  }
  if (tid == 0) q_prod = q_cons = 0;
  if (tid == 32) {
    for (int i = 0; i < stages; ++i) {
      tc::mbar_init(&full_bar[i], 1);
      tc::mbar_init(&empty_bar[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&acc_full[i], 1);
      tc::mbar_init(&acc_empty[i], kTcEpiWarps);
    }
    tc::mbar_init(&drain_bar, 1);
    tc::mbar_fence_init();
  }
  for (int i = tid; i < L.nmsets; i += kTcThreads) s_ms[i] = L.ms[i];
  for (int i = tid; i < L.ngroups; i += kTcThreads) s_groups[i] = L.groups[i];
  // epilogue constants of every slot of the launch (after the stages)
  TcEpiSlot* etab =
      reinterpret_cast<TcEpiSlot*>(smem_raw + (sbase - tc::smem_u32(smem_raw)) + (size_t)stages * L.stage_bytes);
  for (int s = tid; s < L.nslots; s += kTcThreads) {
    const TcSlot& S = L.slots[s];
    int64_t D = 2;
    for (int m = 0; m < L.nmsets; ++m)
      if (s >= L.ms[m].slot0 && s < L.ms[m].slot0 + L.ms[m].NS) D = L.groups[L.ms[m].group].D;
    TcEpiSlot e;
    e.out = S.out;
    e.J = S.J;
    e.U = S.U;
    e.pair = S.flags & 1u;
    e.Tm1 = (uint16_t)(S.T > 0 ? S.T - 1u : 0u);
    e.om = 0;
    e.fm = 0;
    e.x0 = 0;
    e.R = 0xFFFFFFFFu;
    if (S.J > 0) {
      const NcoConst nc = L.nco[S.ch];
      if (nc.enabled) {
        // fast path: row counters (P0 + lane D) stay below 2 R < 2^32 with one
        // conditional subtraction; otherwise every output goes exact (R = 0)
        const bool fast = tc_slot_fast(L, nc, D, S.T);
        e.om = nc.omega64;
        e.fm = nc.fastmod;
        e.x0 = (int64_t)L.nco_base[S.ch] + S.w0;
        e.R = fast ? nc.rollover : 0u;
      }
    }
    etab[s] = e;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tmem_base_s;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    // Lane 0 alone waits and issues the copies (keeping the other lanes in
    // warp-synchronous calls around every wait slowed the MMA stream to less
    // than half its rate); its items come from the scheduler warp's queue.
    if (lane == 0) {
      int64_t ci = 0;  // chunks issued
      TcRing rg;       // their stage and round
      int64_t k = 0;   // items announced
      bool failed = false;
      while (!hold && !failed) {
        // item k from the scheduler (bounded wait)
        uint32_t polls = 0;
        while (*reinterpret_cast<volatile int*>(&q_prod) <= k) {
          if (++polls > poll) {
            failed = true;
            break;
          }
          __nanosleep(32);
        }
        if (failed) break;
        __threadfence_block();  // the item was written before the count
        const volatile int* qi = reinterpret_cast<volatile int*>(&q_items[k % kTcQueue]);
        const int2 item = make_int2(qi[0], qi[1]);
        __threadfence_block();
        *reinterpret_cast<volatile int*>(&q_cons) = (int)(k + 1);
        const bool more = item.x >= 0;
        // announce item k (or the end of the sequence) with its first stage
        if (rg.r > 0 && !tc::mbar_wait_bounded_fast(&empty_bar[rg.s], (uint32_t)((rg.r - 1) & 1), poll)) {
          failed = true;
          break;
        }
        ring[k % kTcRing] = item;
        ++k;
        if (!more) {
          tc::mbar_arrive(&full_bar[rg.s]);  // no copies: the consumers read the end marker
          ++ci;
          rg.next(stages);
          break;
        }
        const int m = item.x, t = item.y;
        const TcMset& M = s_ms[m];
        const int D = s_groups[M.group].D;
        const CUtensorMap* map = &P.maps[M.group];
        const int R = M.R;
        const uint32_t bbytes = (uint32_t)(4 * M.NS * 128);
        const uint32_t tx = (uint32_t)R * kTcTileBytes + bbytes;
        const int32_t x0 = 4 * (M.a % D);
        const int32_t y0 = t * R * kTcRows + M.a / D;
        const uint8_t* bsrc = bbuf + M.b;
        const int nchunks = M.nchunks;
        for (int c = 0; c < nchunks; ++c, ++ci, rg.next(stages)) {
          const int s = rg.s;
          // (the first chunk's stage was claimed with the announcement)
          if (c > 0 && rg.r > 0 && !tc::mbar_wait_bounded_fast(&empty_bar[s], (uint32_t)((rg.r - 1) & 1), poll)) {
            failed = true;
            break;
          }
          const uint32_t st = sbase + (uint32_t)s * stage_bytes;
          const uint32_t fb = tc::smem_u32(&full_bar[s]);
          mbar_expect_tx(&full_bar[s], tx);
          for (int r = 0; r < R; ++r)
            tma_load_2d(st + (uint32_t)r * kTcTileBytes, map, x0 + 64 * c, y0 + r * kTcRows, fb);
          bulk_load(st + (uint32_t)R * kTcTileBytes, bsrc + (size_t)c * bbytes, bbytes, fb);
        }
      }
      // every copy issued lands before the CTA can exit
      for (int64_t i = (ci > stages ? ci - stages : 0); i < ci; ++i)
        if (!tc::mbar_wait_bounded_fast(&full_bar[i % stages], (uint32_t)((i / stages) & 1), poll)) failed = true;
      if (failed) atomicExch(L.err, 1);
    }
  } else if (warp == kTcSchedWarp) {
    // ------------------------------------------------------------ scheduler
    // The CTA's item sequence (warp-parallel cursor), kTcQueue items ahead of
    // the producer; an item with merge set -1 ends it.
    TcCursor cur;
    cur.init(s_ms, s_groups, L.nmsets, L.Lc, L.G, blockIdx.x, lane);
    bool failed = false;
    for (int i = 0; !hold; ++i) {
      int m = -1, t = 0;
      const bool more = cur.next(lane, &m, &t);
      if (lane == 0) {
        uint32_t polls = 0;
        while (i - *reinterpret_cast<volatile int*>(&q_cons) >= kTcQueue) {  // room in the queue
          if (++polls > poll) {
            failed = true;
            break;
          }
          __nanosleep(64);
        }
        if (!failed) {
          volatile int* qi = reinterpret_cast<volatile int*>(&q_items[i % kTcQueue]);
          qi[0] = more ? m : -1;
          qi[1] = more ? t : 0;
          __threadfence_block();
          *reinterpret_cast<volatile int*>(&q_prod) = i + 1;
        }
      }
      failed = __shfl_sync(0xffffffffu, failed ? 1 : 0, 0) != 0;
      if (!more || failed) break;
    }
    if (failed && lane == 0) atomicExch(L.err, 1);
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    // (lane 0 alone, for the same reason)
    if (lane == 0) {
      int64_t ci = 0;
      TcRing rg;
      int k = 0;
      bool failed = false, issued = false;
      auto wait1 = [&](uint64_t* bar, uint32_t parity) {
        const bool ok = tc::mbar_wait_bounded_fast(bar, parity, poll);
        tc::fence_after_sync();
        return ok;
      };
      while (true) {
        // the first stage of item k also announces it (ring entry k)
        if (!wait1(&full_bar[rg.s], (uint32_t)(rg.r & 1))) {
          failed = true;
          break;
        }
        const int2 it = ring[k % kTcRing];
        const int a = k & 1;
        if (k >= 2 && !wait1(&acc_empty[a], (uint32_t)(((k >> 1) - 1) & 1))) {
          failed = true;
          break;
        }
        if (it.x < 0) {  // end of the sequence: pass it on through the accumulator slot
          tc::mbar_arrive(&acc_full[a]);
          break;
        }
        const TcMset& M = s_ms[it.x];
        const int R = M.R, N = 4 * M.NS, nchunks = M.nchunks;
        const uint32_t idesc = tc::idesc_f16(FMT, 128, (uint32_t)N);
        const uint32_t dcol = tbase + (uint32_t)a * 256u;
        const uint32_t rstep = R == 2 ? 128u : 256u;  // accumulator columns of a tile
        for (int c = 0; c < nchunks; ++c, ++ci, rg.next(stages)) {
          const int s = rg.s;
          if (c > 0 && !wait1(&full_bar[s], (uint32_t)(rg.r & 1))) {
            failed = true;
            break;
          }
          const uint32_t st = sbase + (uint32_t)s * stage_bytes;
          const uint64_t bdesc = desc_sw128(st + (uint32_t)R * kTcTileBytes);
          for (int r = 0; r < R; ++r) {
            const uint64_t adesc = desc_sw128(st + (uint32_t)r * kTcTileBytes);
            const uint32_t d = dcol + (uint32_t)r * rstep;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              mma_f16_ss(d, adesc + (uint64_t)(2 * kk), bdesc + (uint64_t)(2 * kk), idesc, (c | kk) != 0 ? 1u : 0u);
          }
          tc::mma_commit(&empty_bar[s]);
          issued = true;
        }
        if (failed) break;
        tc::mma_commit(&acc_full[a]);
        ++k;
      }
      // every MMA this CTA issued completes before its TMEM is released
      if (issued) {
        tc::mma_commit(&drain_bar);
        if (!tc::mbar_wait_bounded(&drain_bar, 0u, poll)) failed = true;
      }
      if (failed) atomicExch(L.err, 1);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;           // TMEM lane quarter this warp may read
    const int h = (warp - 2) >> 2;    // which of the item's column chunks (every kTcEpiPerQ-th)
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    bool failed = false;
    for (int k = 0;; ++k) {
      const int a = k & 1;
      bool ok = true;
      if (lane == 0) ok = tc::mbar_wait_bounded(&acc_full[a], (uint32_t)((k >> 1) & 1), poll);
      if (!__shfl_sync(0xffffffffu, ok ? 1 : 0, 0)) {
        failed = true;
        break;
      }
      tc::fence_after_sync();
      const int2 it = ring[k % kTcRing];
      if (it.x < 0) break;
      const int m = it.x, t = it.y;
      const TcMset& M = s_ms[m];
      const int R = M.R, NS = M.NS, nch = NS >> 3;
      const int64_t D = s_groups[M.group].D;
      const uint32_t laneD = (uint32_t)lane * (uint32_t)D;
      // every column chunk this warp owns (at most kTcEpiOwn: R * NS <= 64)
      // is read out of tensor memory first and the accumulator slot
      // released, so the MMAs of a later item run while this warp rotates
      // and stores
      const int n_own = (R * nch - h + kTcEpiPerQ - 1) / kTcEpiPerQ;  // chunks h, h + kTcEpiPerQ, ...
      float yv[kTcEpiOwn][16];                                       // (hi + lo) sums of those chunks
#pragma unroll
      for (int u = 0; u < kTcEpiOwn; ++u) {
        if (u < n_own) {
          const int idx = h + kTcEpiPerQ * u;
          const int r = idx / nch, cc = idx - r * nch;
          const uint32_t col = tbase + lane_off + (uint32_t)a * 256u + (uint32_t)(r * (256 / R) + 16 * cc);
          uint32_t vh[16], vl[16];
          tc::tmem_ld16(col, vh);
          tc::tmem_ld16(col + (uint32_t)(2 * NS), vl);
          tc::tmem_wait_ld();
#pragma unroll
          for (int i = 0; i < 16; ++i) yv[u][i] = __uint_as_float(vh[i]) + __uint_as_float(vl[i]);
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&acc_empty[a]);
      // one copy of the chunk code (kept small: the warps of every role share
      // the SM's instruction cache); the chunks move down into yv[0] in turn
#pragma unroll 1
      for (int u = 0; u < n_own; ++u) {
        if (u > 0) {
#pragma unroll
          for (int w = 0; w + 1 < kTcEpiOwn; ++w)
#pragma unroll
            for (int i = 0; i < 16; ++i) yv[w][i] = yv[w + 1][i];
        }
        const int idx = h + kTcEpiPerQ * u;
        const int r = idx / nch, cc = idx - r * nch;
        const int64_t row0 = ((int64_t)t * R + r) * kTcRows + q * 32;  // row of lane 0
        const int64_t j = row0 + lane;
        const TcEpiSlot* E8 = etab + M.slot0 + cc * 8;
        // NCO counter of lane 0's window start for slot e (lane e computes it):
        // (x0 + row0 D) mod R, once per chunk; 0 <= x0 + row0 D < 2^32 or
        // > -R on the fast path
        uint32_t p0 = 0;
        if (lane < 8) {
          const TcEpiSlot& E = E8[lane];
          if (E.om != 0 && E.R != 0) {
            const int64_t v = E.x0 + row0 * D;
            p0 = v < 0 ? (uint32_t)(v + (int64_t)E.R)
                       : (uint32_t)__umul64hi(E.fm * (uint64_t)(uint32_t)v, (uint64_t)E.R);
          }
        }
        // per pair of slots: their constants as two 16-byte shared loads each
        // ({out, om} and {R, J, U | Tm1 << 16, pair}), the rotation, and one
        // 16-byte store where a slot and the next hold the same channel's
        // consecutive outputs (contiguous across the lanes when the outputs
        // interleave by two)
        const uint32_t e8 = tc::smem_u32(E8);
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
          const uint4 b0 = lds128(e8 + (uint32_t)e * kTcEpiSlotBytes + 32u);
          const uint4 b1 = lds128(e8 + (uint32_t)(e + 1) * kTcEpiSlotBytes + 32u);
          if ((int32_t)b0.y <= 0 && (int32_t)b1.y <= 0) continue;  // two padding slots (no rows): nothing to do
          const uint4 a0 = lds128(e8 + (uint32_t)e * kTcEpiSlotBytes);
          const uint4 a1 = lds128(e8 + (uint32_t)(e + 1) * kTcEpiSlotBytes);
          float2 o[2];
#pragma unroll
          for (int k2 = 0; k2 < 2; ++k2) {
            const uint4 A = k2 ? a1 : a0, Bv = k2 ? b1 : b0;
            const uint32_t Rr = Bv.x, Tm1 = Bv.z >> 16, om_lo = A.z, om_hi = A.w;
            const uint32_t P0 = __shfl_sync(0xffffffffu, p0, e + k2);
            const float2 y0 = make_float2(yv[0][2 * (e + k2)], yv[0][2 * (e + k2) + 1]);
            uint32_t pc = P0 + laneD;
            pc = pc >= Rr ? pc - Rr : pc;
            const bool fast = pc + Tm1 < Rr || (om_lo | om_hi) == 0u;
            const uint32_t turns = __umulhi(pc, om_lo) + pc * om_hi;  // bits 32..63 of pc * om: 2^-32 turns
            float sn, cs;
            __sincosf((float)(int32_t)turns * 1.4629180792671596e-09f, &sn, &cs);  // 2 pi / 2^32
            const float2 y = cmul_nco(y0, make_float2(cs, sn));
            o[k2] = fast ? y : y0;  // windows across the NCO rollover: unrotated, for tc_fix_kernel
          }
          float2* d0 = reinterpret_cast<float2*>((uint64_t)a0.x | ((uint64_t)a0.y << 32)) +
                       (uint64_t)(b0.z & 0xFFFFu) * (uint64_t)j;
          const bool v0 = j < (int64_t)(int32_t)b0.y, v1 = j < (int64_t)(int32_t)b1.y;
          if (b0.w != 0u && v0 && v1 && (reinterpret_cast<uintptr_t>(d0) & 15u) == 0) {
            __stcs(reinterpret_cast<float4*>(d0), make_float4(o[0].x, o[0].y, o[1].x, o[1].y));
          } else {
            if (v0) __stcs(d0, o[0]);
            if (v1)
              __stcs(reinterpret_cast<float2*>((uint64_t)a1.x | ((uint64_t)a1.y << 32)) +
                         (uint64_t)(b1.z & 0xFFFFu) * (uint64_t)j,
                     o[1]);
          }
        }
      }
    }
    if (failed && lane == 0) atomicExch(L.err, 1);
  }

  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, kTmemCols);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

void PolyEngine::free_tc() {
  if (d_ctaps_) dfree(d_ctaps_);
  if (d_ctab_) dfree(d_ctab_);
  if (d_xhl_) dfree(d_xhl_);
  if (d_bbuf_) dfree(d_bbuf_);
  if (d_tcrec_) dfree(d_tcrec_);
  for (cudaEvent_t e : pack_ev_) cudaEventDestroy(e);
  pack_ev_.clear();
  for (cudaStream_t q : side_) cudaStreamDestroy(q);
  side_.clear();
  if (h_err_) cudaFreeHost(h_err_);
  d_ctaps_ = nullptr;
  d_ctab_ = nullptr;
  d_xhl_ = nullptr;
  d_bbuf_ = nullptr;
  d_tcrec_ = nullptr;
  h_err_ = nullptr;
  d_err_ = nullptr;
  xhl_cap_ = 0;
  bbuf_cap_ = 0;
}

// FP32 NCO-modulated taps of every channel, [U][T] per channel, and the
// per-channel pointer table the kernels read; the error flag in mapped host
// memory.
int PolyEngine::build_tc(int fmt) {
  free_tc();
  tc_fmt_ = fmt;
  std::vector<size_t> off(chans_.size());
  size_t total = 0;
  for (size_t c = 0; c < chans_.size(); ++c) {
    off[c] = total;
    total += (size_t)chans_[c].up * chans_[c].T;
  }
  std::vector<float2> g(total);
  for (size_t c = 0; c < chans_.size(); ++c) {
    const EngineChannel& e = chans_[c];
    int64_t fm = 0;
    if (e.nco.enabled) {
      fm = (int64_t)e.shift_hz % (int64_t)fs_;
      if (fm < 0) fm += fs_;
    }
    for (uint32_t ph = 0; ph < e.up; ++ph) {
      for (uint32_t k = 0; k < e.T; ++k) {
        const float2 h = e.flipped[(size_t)ph * e.T + k];
        double gr = h.x, gi = h.y;
        if (e.nco.enabled) {
          // e^{j w k}, w k reduced exactly: 2 pi ((f mod fs) k mod fs) / fs
          const uint64_t red = (uint64_t)(((unsigned __int128)(uint64_t)fm * (uint64_t)k) % fs_);
          const double ang = 2.0 * M_PI * (double)red / (double)fs_;
          const double cs = std::cos(ang), sn = std::sin(ang);
          gr = (double)h.x * cs - (double)h.y * sn;
          gi = (double)h.x * sn + (double)h.y * cs;
        }
        g[off[c] + (size_t)ph * e.T + k] = make_float2((float)gr, (float)gi);
      }
    }
  }
  cudaError_t err = dalloc(reinterpret_cast<void**>(&d_ctaps_), total * sizeof(float2));
  if (err == cudaSuccess) err = cudaMemcpy(d_ctaps_, g.data(), total * sizeof(float2), cudaMemcpyHostToDevice);
  std::vector<const float2*> tab(chans_.size());
  for (size_t c = 0; c < chans_.size(); ++c) tab[c] = d_ctaps_ + off[c];
  if (err == cudaSuccess) err = dalloc(reinterpret_cast<void**>(&d_ctab_), tab.size() * sizeof(float2*));
  if (err == cudaSuccess) err = cudaMemcpy(d_ctab_, tab.data(), tab.size() * sizeof(float2*), cudaMemcpyHostToDevice);
  // one device record per launch pack (packs <= groups)
  if (err == cudaSuccess) err = dalloc(reinterpret_cast<void**>(&d_tcrec_), kTcMaxGroups * sizeof(TcLaunch));
  for (int i = 0; i < kTcSideStreams && err == cudaSuccess; ++i) {
    cudaStream_t q = nullptr;
    err = cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking);
    if (err == cudaSuccess) side_.push_back(q);
  }
  for (int i = 0; i <= kTcSideStreams && err == cudaSuccess; ++i) {
    cudaEvent_t e = nullptr;
    err = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (err == cudaSuccess) pack_ev_.push_back(e);
  }
  if (err == cudaSuccess) err = cudaHostAlloc(&h_err_, sizeof(int), cudaHostAllocMapped);
  if (err == cudaSuccess) {
    *h_err_ = 0;
    err = cudaHostGetDevicePointer(reinterpret_cast<void**>(&d_err_), h_err_, 0);
  }
  if (err != cudaSuccess) return cuda_status(err);
  if (!tensor_map_encoder()) return FDSP_ERR_UNSUPPORTED;
  return FDSP_OK;
}

int PolyEngine::tc_error() {
  if (!h_err_) return 0;
  const int v = *reinterpret_cast<volatile int*>(h_err_);
  *reinterpret_cast<volatile int*>(h_err_) = 0;
  return v;
}

// Plans and enqueues the tensor-core form of the groups in `tc_groups`
// (engine group indices).  Groups are packed greedily into launches whose
// records fit the kernel parameter block; per pack one prep (the first also
// splits the input, which every pack then reads), one filter-bank launch and
// the exact rotation pass.  Each pack has its own device record and B-image
// region, so the packs run at the same time: pack 0 on the caller's stream,
// pack k > 0 on side stream (k - 1) mod kTcSideStreams once the split is
// done, and a pack's filter-bank CTAs take the SMs that the earlier packs'
// CTAs leave as they finish (one launch's tail instead of one per pack).
// With kernel timing on (each launch timed alone), or with a completion hook
// (apply_host: the first packs' device-to-host copies then start while the
// later packs compute, where concurrent packs would all end together), the
// packs run one after another on the caller's stream.  Groups no launch can
// hold are returned in `fallback` for the FP32 kernel.
int PolyEngine::launch_tc(const float2* d_in, uint64_t n, float2* const* out, const std::vector<int>& tc_groups,
                          std::vector<int>& fallback, cudaStream_t stream) {
  fallback.clear();
  std::vector<TcGroupIn> gin;
  std::vector<int> gmap;
  for (int gi : tc_groups) {
    const EngineGroup& g = groups_[gi];
    TcGroupIn in;
    in.D = (int)g.D;
    in.max_split = std::max(1, g.tc_split);
    for (size_t ki = 0; ki < classes_.size(); ++ki) {
      const EngineClass& k = classes_[ki];
      if (k.down != g.D) continue;
      const uint32_t U = k.up;
      for (uint32_t r = 0; r < U; ++r) {
        if (k.M <= r) continue;
        const uint64_t tt = (uint64_t)k.phase + (uint64_t)r * g.D;
        for (int c : k.chans) {
          TcSlotIn s;
          s.ch = c;
          s.T = (int)chans_[c].T;
          s.U = (int)U;
          s.r = (int)r;
          s.phi = (int)(tt % U);
          s.delta = (int64_t)(k.xoffset + tt / U);
          s.J = (int64_t)((k.M - r + U - 1) / U);
          in.slots.push_back(s);
        }
      }
    }
    if (!in.slots.empty()) {
      gin.push_back(in);
      gmap.push_back(gi);
    }
  }
  if (gin.empty()) return FDSP_OK;
  if (num_sms_ == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev);
    if (num_sms_ <= 0) num_sms_ = 1;
  }
  // pack groups into launches
  std::vector<std::vector<int>> packs;  // indices into gin
  std::vector<TcPlan> plans;
  {
    std::vector<int> cur;
    TcPlan cur_plan;
    auto plan_of = [&](const std::vector<int>& idx, TcPlan& p) {
      std::vector<TcGroupIn> sub;
      for (int i : idx) sub.push_back(gin[i]);
      return tc_plan(sub, (int64_t)n, H_, num_sms_, p) == 0;
    };
    for (int i = 0; i < (int)gin.size(); ++i) {
      std::vector<int> trial = cur;
      trial.push_back(i);
      TcPlan p;
      if (plan_of(trial, p)) {
        cur = trial;
        cur_plan = std::move(p);
        continue;
      }
      if (!cur.empty()) {
        packs.push_back(cur);
        plans.push_back(std::move(cur_plan));
      }
      cur.assign(1, i);
      if (!plan_of(cur, cur_plan)) {
        fallback.push_back(gmap[i]);
        cur.clear();
      }
    }
    if (!cur.empty()) {
      packs.push_back(cur);
      plans.push_back(std::move(cur_plan));
    }
  }
  if (plans.empty()) return FDSP_OK;
  if (plans.size() > (size_t)kTcMaxGroups) return FDSP_ERR_UNSUPPORTED;
  // scratch (grow only): the split input, which every pack reads, and the B
  // images of every pack (a 1 KB aligned region each)
  int64_t xhl_need = 0;
  size_t b_need = 0;
  std::vector<size_t> boff(plans.size());
  for (size_t li = 0; li < plans.size(); ++li) {
    xhl_need = std::max(xhl_need, plans[li].xhl_samples);
    boff[li] = b_need;
    b_need += (plans[li].b_bytes + 1023u) & ~(size_t)1023u;
  }
  if ((size_t)xhl_need > xhl_cap_) {
    if (d_xhl_) dfree(d_xhl_);
    d_xhl_ = nullptr;
    xhl_cap_ = 0;
    FDSP_TRY(cuda_status(dalloc(reinterpret_cast<void**>(&d_xhl_), (size_t)xhl_need * sizeof(uint2))));
    xhl_cap_ = (size_t)xhl_need;
  }
  if (b_need > bbuf_cap_) {
    if (d_bbuf_) dfree(d_bbuf_);
    d_bbuf_ = nullptr;
    bbuf_cap_ = 0;
    FDSP_TRY(cuda_status(dalloc(reinterpret_cast<void**>(&d_bbuf_), b_need)));
    bbuf_cap_ = b_need;
  }
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return FDSP_ERR_UNSUPPORTED;
  // (side streams and events made by build_tc, outside any stream capture)
  if (side_.empty() || pack_ev_.size() < side_.size() + 1) return FDSP_ERR_UNSUPPORTED;
  const bool concurrent = !kprof_ && !done_fn_ && plans.size() > 1;
  std::vector<char> side_used(side_.size(), 0);
  static thread_local TcLaunch L;
  for (size_t li = 0; li < plans.size(); ++li) {
    const TcPlan& plan = plans[li];
    cudaStream_t ps = stream;  // this pack's stream
    if (concurrent && li > 0) {
      const size_t si = (li - 1) % side_.size();
      ps = side_[si];
      if (!side_used[si]) {  // after the split (recorded below by pack 0)
        FDSP_TRY(cuda_status(kwait(ps, pack_ev_[0])));
        side_used[si] = 1;
      }
    }
    std::memset(&L, 0, sizeof(L));
    L.block = in16_ ? nullptr : d_in;
    L.block16 = in16_;
    L.hist = d_hist_[hist_cur_];
    L.nco = d_nco_;
    L.ctaps = d_ctab_;
    L.xhl = d_xhl_;
    L.bbuf = d_bbuf_ + boff[li];
    L.err = d_err_;
    L.rec_out = d_tcrec_ + li;
    L.N = (int64_t)n;
    L.Lc = plan.Lc;
    L.xhl_n = xhl_need;
    L.H = H_;
    L.G = plan.G;
    L.nmsets = (int32_t)plan.ms.size();
    L.ngroups = (int32_t)plan.groups.size();
    L.stages = plan.stages;
    L.stage_bytes = plan.stage_bytes;
    L.nslots = (int32_t)plan.slots.size();
    L.poll = tc_poll_;
    L.hold = tc_hold_;
    L.exact_all = tc_exact_all_;
    for (size_t c = 0; c < chans_.size(); ++c) {
      const uint32_t R = chans_[c].nco.rollover;
      L.nco_base[c] = R ? (uint32_t)(abs0_ % R) : 0u;
    }
    int pieces = 0;
    for (size_t m = 0; m < plan.ms.size(); ++m) {
      L.ms[m] = plan.ms[m];
      L.bprefix[m] = pieces;
      pieces += plan.ms[m].nchunks * 4 * plan.ms[m].NS * 8;
    }
    L.bprefix[plan.ms.size()] = pieces;
    for (size_t s = 0; s < plan.slots.size(); ++s) {
      L.slots[s] = plan.slots[s];
      if (plan.slots[s].J > 0)
        L.slots[s].out = (uint64_t)(uintptr_t)(out[plan.slots[s].ch] + plan.slot_r[s]);
    }
    for (size_t g = 0; g < plan.groups.size(); ++g) {
      const TcPlanGroup& pg = plan.groups[g];
      L.groups[g].D = pg.D;
      L.groups[g].S = pg.S;
      groups_[gmap[packs[li][g]]].tc_split_used = pg.S;
      // rows of D' samples; a row spans Wx samples (4 16-bit elements each);
      // (rows - 1) D' + Wx <= xhl_samples keeps every address inside xhl
      const cuuint64_t rows = (cuuint64_t)((plan.xhl_samples - pg.Wx) / pg.D + 1);
      const cuuint64_t dims[2] = {(cuuint64_t)(4 * pg.Wx), rows};
      const cuuint64_t strides[1] = {(cuuint64_t)pg.D * 8u};
      const cuuint32_t box[2] = {64u, (cuuint32_t)kTcRows};
      const cuuint32_t estr[2] = {1u, 1u};
      const CUresult r = enc(&L.maps[g], CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, d_xhl_, dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r != CUDA_SUCCESS) return FDSP_ERR_UNSUPPORTED;
    }
    // prep: B images (few blocks), then, for the first launch, the split
    const int nb_build = std::max(1, std::min(num_sms_, (pieces + 255) / 256));
    const int64_t nb_split = li == 0 ? std::min<int64_t>((xhl_need + 255) / 256, (int64_t)num_sms_ * 8) : 0;
    auto prep = tc_fmt_ == 0 ? tc_prep_kernel<0> : tc_prep_kernel<1>;
    int nbb = nb_build;
    cudaError_t e = klaunch(reinterpret_cast<const void*>(prep), dim3((unsigned)(nb_build + nb_split)), dim3(256), 0,
                            ps, L, nbb);
    if (e != cudaSuccess) return cuda_status(e);
    launches_last_++;
    if (concurrent && li == 0) FDSP_TRY(cuda_status(krecord(pack_ev_[0], stream)));
    auto kern = tc_fmt_ == 0 ? tc_filter_kernel<0> : tc_filter_kernel<1>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, plan.smem);
    if (e != cudaSuccess) return cuda_status(e);
    if (kprof_) cudaEventRecord(kprof_event(), ps);
    static thread_local TcFilterParams FP;
    std::memcpy(FP.maps, L.maps, sizeof(FP.maps));
    FP.rec = d_tcrec_ + li;
    e = klaunch(reinterpret_cast<const void*>(kern), dim3((unsigned)plan.G), dim3(kTcThreads), (size_t)plan.smem, ps,
                FP);
    if (kprof_) cudaEventRecord(kprof_event(), ps);
    if (e != cudaSuccess) return cuda_status(e);
    launches_last_++;
    // exact pass: blocks per slot for the most rows (or rollover points) a
    // slot of this launch has to fix, one per thread (the pass is latency
    // bound: each point is a serial T-tap sum, and the last pack's pass ends
    // the step)
    int64_t work = 1;
    for (size_t si = 0; si < plan.slots.size(); ++si) {
      const TcSlot& S = plan.slots[si];
      if (S.J <= 0) continue;
      const NcoConst& nc = chans_[S.ch].nco;
      if (!nc.enabled || nc.omega64 == 0 || nc.rollover == 0) continue;
      int64_t Dp = 0;
      for (const TcMset& m : plan.ms)
        if ((int)si >= m.slot0 && (int)si < m.slot0 + m.NS) Dp = plan.groups[m.group].D;
      const bool fast = !tc_exact_all_ && nc.rollover < 0x80000000u && 31 * Dp + S.T < (int64_t)nc.rollover;
      work = std::max<int64_t>(work, fast ? ((int64_t)S.J * Dp + S.T) / nc.rollover + 1 : (int64_t)S.J);
    }
    const unsigned fix_y = (unsigned)std::min<int64_t>(4096, (work + 127) / 128);
    e = klaunch(reinterpret_cast<const void*>(tc_fix_kernel), dim3((unsigned)plan.slots.size(), fix_y), dim3(128), 0,
                ps, L);
    if (e != cudaSuccess) return cuda_status(e);
    launches_last_++;
    tc_groups_last_ += (int)packs[li].size();
    if (done_fn_) {
      std::vector<int> egs;
      for (int gi : packs[li]) egs.push_back(gmap[gi]);
      notify_done(egs, ps);
    }
  }
  // the side streams join the caller's stream (before the history update)
  for (size_t si = 0; si < side_.size(); ++si) {
    if (!side_used[si]) continue;
    FDSP_TRY(cuda_status(krecord(pack_ev_[1 + si], side_[si])));
    FDSP_TRY(cuda_status(kwait(stream, pack_ev_[1 + si])));
  }
  return FDSP_OK;
}

}  // namespace fdsp
