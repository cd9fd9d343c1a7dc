// Tensor-core form of the polyphase engine (tcgen05, sm_103a).
//
// The fused shift + polyphase contraction of one decimation group is recast
// as dense matrix products over 128-row tiles:
//
//     Y[j][c] = sum_k X[j][k] * G[k][c]
//
//   j  output row of the tile (window end delta + j D),   M = 128
//   k  tap of the window,                                 K = 8 x taps
//   c  Re / Im column of each channel,                    N <= 128
//
// X[j][k] is input sample (j D + k + offset): a Hankel matrix over the input
// de-interleaved by D.  Each sample is held in shared memory as one 16-byte
// record of its hi and lo 16-bit parts, {hi(re,im), lo(re,im), hi, lo}, so
// that the K-major core matrix of 8 rows x 16 bytes for rows j..j+7 and tap k
// is 8 consecutive records of phase (k mod D): the MMA reads every window of
// the tile straight from the staged input through its descriptor (leading
// byte offset = one phase array, stride byte offset = 8 records), with no
// per-row copy.  The matching B record of a tap holds the NCO-modulated tap's
// hi and lo parts ordered so that the 8 products sum to the full
// (hi + lo) x (hi + lo) complex product with FP32 accumulation in tensor
// memory (~2^-22 relative, far above the 60 dB target).
//
// For even D the records are pairs instead: record (v, q) holds samples
// q D + 2v and q D + 2v + 1 as {hi(re,im), lo(re,im)} each, so only phases
// 0, 2, .., D are staged (half the bytes).  One MMA then covers four taps and
// is issued twice, against a B of the hi taps and a B of the lo taps, into
// the same accumulator columns; merged windows start on an even sample and
// span a multiple of four taps.
//
// Work sets (class x output phase) of a group whose windows end close
// together are merged into one product (a merge set): each one's taps sit at
// its own offset of a common window (zeros elsewhere) and its channels side by
// side along N, so one MMA chain serves up to 64 channels.  The offsets follow
// the streaming state, so every CTA assembles the merged B in shared memory at
// start from per-phase blocks precomputed on the host.
//
// Persistent warp-specialised CTA, one per SM (all 512 TMEM columns):
//   warps 0-2   producers: assemble B and the channel constants once, then
//               per tile stage the de-interleaved input records (cp.async,
//               zero-filled outside the data) into one of up to four buffers,
//               several tiles in flight;
//   warp 3      MMA issuer: per (tile, merge set) waits for the staged tile
//               and a drained accumulator slot, issues Kw/2 MMAs, commits;
//   warps 4-19  epilogue, four groups of four warps (one per TMEM lane
//               quarter); group g drains items g, g+4, ... (accumulator slot
//               g): rotates by the NCO phase of each window start (one
//               phasor per 8-row group from the exact integer counter times
//               a per-slot row-step table), fixes windows that straddle the
//               NCO rollover with an exact FP32 split sum, and stores.
// Every mbarrier wait is bounded and reports through an error flag.
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fdsp_internal.h"
#include "fdsp_nco.cuh"
#include "fdsp_tc.cuh"
#include "fdsp_tc_plan.h"

namespace fdsp {

constexpr int kTcThreads = 672;       // 3 producer warps + 2 MMA warps (3, 20) + 16 epilogue warps
constexpr int kTcProdThreads = 96;    // (20 warps: 5 per SM sub-partition, up to 96 registers each)
constexpr int kTcDSlots = 4;          // accumulator slots = epilogue groups (items in flight)
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kWaitPolls = 1u << 20;
constexpr int kTcChunk = 32;          // channels per chunk (64 columns)
constexpr int kTcMaxTaps = 64;        // taps per phase of a chunk

// Constants of one channel slot (Re/Im column pair) of a merge set, staged
// in shared memory: read once per item (row-0 counter) and on the exact
// path; the per-output constants are in the kernel parameters (TcSlotHot).
struct SlotMeta {
  uint32_t om_lo, om_hi;  // NCO turns per sample (2^-64 units; 0: no shift)
  float2* out;            // output base of the channel
  uint32_t R;             // counter rollover (0x7fffffff: no shift or general)
  uint32_t Tm1;           // taps - 1 (0x7fffffff: general, every output exact)
  int32_t U, r;           // output m = r + U j
  int32_t J;              // rows with an output (0: padding slot)
  uint32_t pad0_;
  uint64_t fastmod;       // ceil(2^64 / R)
  int32_t delta;          // window end of row 0
  int32_t T;
  OutMeta nco;            // full NCO constants (row-0 counter, exact path)
  const float2* taps32;   // FP32 modulated taps [T][tstride] of the work set
  int32_t tstride, tidx;
  int32_t pad_[2];
};
static_assert(sizeof(SlotMeta) == 128, "slot constants layout");

__device__ __forceinline__ float2 load_x(const TcLaunch& L, int64_t v) {
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

// [history | block] -> packed {hi, lo} 16-bit pairs, once per apply: every
// sample is used by many windows, so the split is not repeated per use.
template <int FMT>
__global__ void split_input_kernel(const float2* __restrict__ block, const short2* __restrict__ block16,
                                   const float2* __restrict__ hist, int64_t N, int H, uint2* __restrict__ xhl) {
  const int64_t total = N + H;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
    float2 x;
    if (u < H) {
      x = hist[u];
    } else if (block16 != nullptr) {  // int16 front end
      const short2 s = block16[u - H];
      x = make_float2((float)s.x, (float)s.y);
    } else {
      x = block[u - H];
    }
    uint2 hl;
    split2<FMT>(x, hl.x, hl.y);
    xhl[u] = hl;
  }
}

// Asynchronous copy of input sample v (block relative), its 8-byte
// pre-split {hi, lo} pair, into one half of a 16-byte record (zero outside
// the data).  Two lanes fill the two halves of a record, so a warp writes 256
// contiguous bytes of shared memory per instruction.
__device__ __forceinline__ void stage_half(const TcLaunch& L, int64_t v, uint32_t dst) {
  const int64_t u = v + L.H;
  const uint2* src = L.xhl;
  uint32_t bytes = 0;
  if (u >= 0 && u < L.N + L.H) {
    src = L.xhl + u;
    bytes = 8;
  }
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}

// Tile schedule shared by every role.  With two or more input buffers two
// MMA warps issue alternate tiles (one issuing thread does not keep the
// tensor pipe busy with MMAs this narrow): tile t goes to warp w = t % 2 as
// its (t / 2)-th tile, and warp w owns input buffers [w nbw, (w + 1) nbw)
// and accumulator slots {2w, 2w + 1}.  Every barrier then has one waiter,
// which consumes its phases in order (parity waits never alias).
struct TcSched {
  int nw;   // MMA warps in use (1 or 2)
  int nbw;  // input buffers per MMA warp
  int spw;  // accumulator slots per MMA warp
};
__device__ __forceinline__ TcSched tc_sched(int nbuf) {
  TcSched s;
  s.nw = nbuf >= 2 ? 2 : 1;
  s.nbw = nbuf / s.nw;
  s.spw = kTcDSlots / s.nw;
  return s;
}
// input buffer of tile t and how many earlier tiles used it
__device__ __forceinline__ int tc_buf(const TcSched& s, int t, int* use) {
  const int w = t % s.nw, k = t / s.nw;
  *use = k / s.nbw;
  return w * s.nbw + k % s.nbw;
}

// Bulk copy (one TMA transfer) of the {hi, lo} pairs of absolute samples
// [u0, u0 + raw_span) that exist (0 <= u < N + H) into the raw buffer, whose
// element i holds sample (u0 & ~1) + i; completion is counted on `bar`.  The
// copy starts and ends on even samples (16-byte aligned; the scratch array
// has one spare pair past its end); a span with no data only arrives.
__device__ __forceinline__ void raw_issue(const TcLaunch& L, int64_t u0, uint32_t raw_s, uint64_t* bar) {
  const int64_t total = L.N + L.H;
  const int64_t base = u0 & ~1LL;
  const int64_t c0 = (u0 < 0 ? 0 : u0) & ~1LL;
  int64_t hi = u0 + L.raw_span;
  if (hi > total) hi = total;
  const int64_t c1 = (hi + 1) & ~1LL;
  const uint32_t bar_s = tc::smem_u32(bar);
  if (c1 > c0) {
    const uint32_t bytes = (uint32_t)((c1 - c0) * 8);
    const uint32_t dst = raw_s + (uint32_t)((c0 - base) * 8);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar_s), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
                 "l"(L.xhl + c0), "r"(bytes), "r"(bar_s)
                 : "memory");
  } else {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar_s) : "memory");
  }
}

// Constants of channel slot s (columns 2s, 2s + 1) of merge set M: from the
// work set that owns the slot, else a padding slot (J = 0).  Built once per
// slot at CTA start (row-0 counter inputs) and again on the exact path.
__device__ __noinline__ SlotMeta slot_meta(const TcLaunch& L, const TcMset& M, int s, int D) {
  SlotMeta sm;
  std::memset(&sm, 0, sizeof(sm));
  sm.R = 0x7fffffffu;
  for (int wi = M.ws_begin; wi < M.ws_end; ++wi) {
    const TcWorkSet& W = L.ws[wi];
    const int i = s - W.s0;
    if (i < 0 || i >= W.n) continue;
    const int c = W.ch[i];
    const NcoConst nc = L.nco[c];
    sm.nco.omega64 = nc.omega64;
    sm.nco.wrap64 = nc.wrap64;
    sm.nco.fastmod = nc.fastmod;
    sm.nco.out = L.out[c];
    sm.nco.rollover = nc.rollover;
    sm.nco.base = L.nco_base[c];
    sm.nco.enabled = nc.enabled;
    // fast path: R < 2^31 (row counters in 32 bits) and 127 D + T < R, so
    // the counter of row `row` is row 0's plus row D, past the rollover at
    // most once (R >= 1e5 by construction, so this holds for D up to ~780);
    // otherwise ("general") every output takes the exact path
    const bool general = nc.enabled && (nc.rollover >= 0x80000000u || 127LL * D + W.T >= (int64_t)nc.rollover);
    sm.fastmod = nc.fastmod;
    sm.om_lo = nc.enabled && !general ? (uint32_t)nc.omega64 : 0u;
    sm.om_hi = nc.enabled && !general ? (uint32_t)(nc.omega64 >> 32) : 0u;
    sm.out = L.out[c];
    sm.R = nc.enabled && !general ? nc.rollover : 0x7fffffffu;
    sm.taps32 = W.taps32;
    sm.delta = W.delta;
    sm.T = W.T;
    sm.Tm1 = general ? 0x7fffffffu : (uint32_t)(W.T - 1);
    sm.U = W.U;
    sm.r = W.r;
    sm.J = W.J;
    sm.tstride = W.n;
    sm.tidx = i;
    break;
  }
  return sm;
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_ss(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
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

template <int FMT>
__global__ void __launch_bounds__(kTcThreads, 1) poly_tc_kernel(const __grid_constant__ TcLaunch L) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ uint32_t tmem_base_s;
  __shared__ __align__(8) uint64_t bar_in_full[kTcMaxBuf];   // tile staged        (one arrival per producer warp)
  __shared__ __align__(8) uint64_t bar_in_empty[kTcMaxBuf];  // tile's MMAs done   (commit)
  __shared__ __align__(8) uint64_t bar_d_full[kTcDSlots];    // accumulator ready  (commit)
  __shared__ __align__(8) uint64_t bar_d_empty[kTcDSlots];   // accumulator drained (one arrival per group warp)
  __shared__ __align__(8) uint64_t bar_b_full;               // B + slot constants (one arrival per producer warp)
  __shared__ __align__(8) uint64_t bar_raw[2];               // raw span landed    (bulk copy)
  __shared__ __align__(16) float2 epi_ph[16 * 32];           // epilogue: one phasor per (slot, 8-row group) of a chunk
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane_id = tid & 31;
  const int D = L.D;
  const int nms = L.nmsets;

  if (warp == 0) {
    tc::tmem_alloc(&tmem_base_s, kTmemCols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < kTcMaxBuf; ++i) {
      tc::mbar_init(&bar_in_full[i], kTcProdThreads / 32);
      tc::mbar_init(&bar_in_empty[i], 1);
    }
    for (int i = 0; i < kTcDSlots; ++i) {
      tc::mbar_init(&bar_d_full[i], 1);
      tc::mbar_init(&bar_d_empty[i], 16 / L.epi_groups);
    }
    tc::mbar_init(&bar_b_full, kTcProdThreads / 32);
    tc::mbar_init(&bar_raw[0], 1);
    tc::mbar_init(&bar_raw[1], 1);
    tc::mbar_fence_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tmem_base_s;
  bool failed = false;

  if (warp < 3) {
    // ------------------------------------------------------------ producers
    // B of every merge set: column pair s (slot s) of core row k comes from
    // the work set that owns slot s and tap k (its channel i = s - s0 sits in
    // column group i / 4, pair i % 4 of the chunk's packed B), else it is zero.
    for (int mi = 0; mi < nms; ++mi) {
      const TcMset& M = L.ms[mi];
      const int ncores = (M.N / 8) * M.Kw;
      if (L.pair) {
        // pair records: two matrices (hi taps, then lo taps) of cores
        // (cg, m) of 8 columns x taps 2m, 2m + 1 at byte (cg Kw/2 + m) 128;
        // column c at c 16, tap 2m + u at u 8 (the hi or lo half of the
        // tap's 16-byte record)
        const int half_k = M.Kw / 2;
        const size_t mbytes = (size_t)(M.N / 8) * half_k * 128;
        for (int p = tid; p < ncores * 16; p += kTcProdThreads) {
          const int u = p & 1, c = (p >> 1) & 7;
          const int rest = p >> 4;  // (h, cg, m)
          const int m = rest % half_k;
          const int hc = rest / half_k;
          const int cg = hc % (M.N / 8), h = hc / (M.N / 8);
          const int k = 2 * m + u;
          const int slot = (cg * 8 + c) >> 1, part = c & 1;
          uint8_t* dst = smem + M.boff + (size_t)h * mbytes + ((size_t)cg * half_k + m) * 128 + c * 16 + u * 8;
          const uint8_t* src = nullptr;
          for (int wi = M.ws_begin; wi < M.ws_end; ++wi) {
            const TcWorkSet& W = L.ws[wi];
            const int i = slot - W.s0;
            if (i >= 0 && i < W.n && k >= W.o && k < W.o + W.T) {
              src = W.b + ((size_t)(i >> 2) * W.T + (k - W.o)) * 128 + (2 * (i & 3) + part) * 16 + h * 8;
              break;
            }
          }
          if (src)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(tc::smem_u32(dst)), "l"(src) : "memory");
          else
            *reinterpret_cast<uint2*>(dst) = make_uint2(0u, 0u);
        }
      }
      for (int p = tid; p < (L.pair ? 0 : ncores * 8); p += kTcProdThreads) {
        const int core = p >> 3, piece = p & 7;
        const int cg = core / M.Kw, k = core - cg * M.Kw;
        const int slot = (cg * 8 + piece) >> 1, half = piece & 1;
        uint8_t* dst = smem + M.boff + (size_t)core * 128 + piece * 16;
        const uint8_t* src = nullptr;
        for (int wi = M.ws_begin; wi < M.ws_end; ++wi) {
          const TcWorkSet& W = L.ws[wi];
          const int i = slot - W.s0;
          if (i >= 0 && i < W.n && k >= W.o && k < W.o + W.T) {
            src = W.b + ((size_t)(i >> 2) * W.T + (k - W.o)) * 128 + (2 * (i & 3) + half) * 16;
            break;
          }
        }
        if (src)
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(tc::smem_u32(dst)), "l"(src) : "memory");
        else
          *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
      }
      // channel slot s = columns 2s, 2s+1
      for (int s = tid; s < M.N / 2; s += kTcProdThreads) {
        const SlotMeta sm = slot_meta(L, M, s, D);
        // the slot's row-0 counter inputs, one array per field (lanes of the
        // epilogue read consecutive slots without bank conflicts): window
        // start of row 0 in samples since reset, R, the fast-modulo constant,
        // whether the slot rotates on the fast path, its NCO step and T - 1
        const int NS = M.N >> 1;
        float2* rtab = reinterpret_cast<float2*>(smem + M.poff);
        uint32_t* P0in = reinterpret_cast<uint32_t*>(smem + M.poff + (size_t)NS * 64);
        const int64_t x0 = (int64_t)sm.nco.base + sm.delta - sm.T + 1;
        P0in[s] = (uint32_t)(uint64_t)x0;
        P0in[NS + s] = (uint32_t)((uint64_t)x0 >> 32);
        P0in[2 * NS + s] = sm.R;
        P0in[3 * NS + s] = (uint32_t)sm.fastmod;
        P0in[4 * NS + s] = (uint32_t)(sm.fastmod >> 32);
        P0in[5 * NS + s] = (sm.om_lo | sm.om_hi) ? 1u : 0u;
        P0in[6 * NS + s] = sm.om_lo;
        P0in[7 * NS + s] = sm.om_hi;
        P0in[8 * NS + s] = sm.Tm1;
        // rotation of row i of an 8-row group relative to the group's first
        // row: e^{j 2 pi ((i D omega64) mod 2^64) / 2^64}, i = 0..7
        for (int i = 0; i < 8; ++i) {
          const uint32_t iD = (uint32_t)(i * D);
          const uint32_t turns = __umulhi(iD, sm.om_lo) + iD * sm.om_hi;
          float sn, cs;
          sincospif((float)(int32_t)turns * 4.656612873077393e-10f, &sn, &cs);  // 2^-31
          rtab[s * 8 + i] = make_float2(cs, sn);
        }
      }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    tc::fence_proxy_async_smem();
    __syncwarp();
    if (lane_id == 0) tc::mbar_arrive(&bar_b_full);

    if (L.raw_span > 0) {
      // tiles through the raw buffers: one bulk copy brings the tile's whole
      // input span; the three producer warps then write the records (v, q)
      // (phase D = phase 0 one row on) from shared memory, phases fastest
      // across threads (Qp is odd, so 8 consecutive records hit 8 distinct
      // bank groups).  With two raw buffers the copy of tile t + 2 is issued
      // once tile t's span has been read, so copies stay one tile ahead of
      // the record writes.
      const uint32_t raw_s = tc::smem_u32(smem + L.raw_off);
      const int nraw = L.nraw;
      const int64_t total = L.N + L.H;
      const int V = L.V, Qp = L.Qp;
      const bool pair = L.pair != 0;
      const TcSched S = tc_sched(L.nbuf);
      const int nrec = V * Qp;
      const int step_q = kTcProdThreads / V, step_v = kTcProdThreads % V;
      int issued[2] = {0, 0}, landed[2] = {0, 0};  // copies per raw buffer
      for (int i = 0; i < nraw; ++i) {
        const int t = (int)blockIdx.x + i * (int)gridDim.x;
        if (t < L.ntiles) {
          if (tid == 0) raw_issue(L, (int64_t)t * 128 * D + L.B0 + L.H, raw_s + (uint32_t)(i * L.raw_stride), &bar_raw[i]);
          issued[i]++;
        }
      }
      int tile_ord = 0;
      for (int tile = blockIdx.x; tile < L.ntiles; tile += gridDim.x, ++tile_ord) {
        int use = 0;
        const int buf = tc_buf(S, tile_ord, &use);
        const int rb = tile_ord % nraw;
        const int64_t u0 = (int64_t)tile * 128 * D + L.B0 + L.H;
        const int64_t base = u0 & ~1LL;
        bool ok = tc::mbar_wait_bounded(&bar_raw[rb], (uint32_t)(landed[rb] & 1), kWaitPolls);
        if (ok) landed[rb]++;
        if (ok && use >= 1) ok = tc::mbar_wait_bounded(&bar_in_empty[buf], (uint32_t)((use - 1) & 1), kWaitPolls);
        if (tc::named_bar_red_or(1, kTcProdThreads, !ok)) {
          failed = true;
          break;
        }
        const uint2* raw = reinterpret_cast<const uint2*>(smem + L.raw_off + (size_t)rb * L.raw_stride);
        uint8_t* A = smem + L.in_off + (size_t)buf * L.in_bytes;
        int q = tid / V, v = tid - (tid / V) * V;
        for (int idx = tid; idx < nrec; idx += kTcProdThreads) {
          // phase D is phase 0 one row on; pair records hold samples 2v, 2v + 1
          const int64_t u = u0 + (int64_t)q * D + (pair ? 2 * v : v);
          uint2 x = make_uint2(0u, 0u), y = make_uint2(0u, 0u);
          if (u >= 0 && u < total) x = raw[u - base];
          if (!pair)
            y = x;
          else if (u + 1 >= 0 && u + 1 < total)
            y = raw[u + 1 - base];
          *reinterpret_cast<uint4*>(A + ((size_t)v * Qp + q) * 16) = make_uint4(x.x, x.y, y.x, y.y);
          v += step_v;
          q += step_q;
          if (v >= V) {
            v -= V;
            ++q;
          }
        }
        tc::named_bar_sync(1, kTcProdThreads);  // every read of raw buffer rb is done
        const int next = tile + nraw * (int)gridDim.x;
        if (next < L.ntiles) {
          if (tid == 0) {
            tc::fence_proxy_async_smem();
            raw_issue(L, (int64_t)next * 128 * D + L.B0 + L.H, raw_s + (uint32_t)(rb * L.raw_stride), &bar_raw[rb]);
          }
          issued[rb]++;
        }
        tc::fence_proxy_async_smem();  // the records are visible to the tensor core
        __syncwarp();
        if (lane_id == 0) tc::mbar_arrive(&bar_in_full[buf]);
      }
      if (failed) {
        // copies still in flight land before the CTA can exit
        for (int i = 0; i < nraw; ++i)
          for (; landed[i] < issued[i]; ++landed[i])
            if (!tc::mbar_wait_bounded(&bar_raw[i], (uint32_t)(landed[i] & 1), kWaitPolls)) break;
        if (lane_id == 0) atomicExch(L.err, 1);
      }
    } else {
    // tiles: record (v, q) of tile t = input sample 128 t D + B0 + q D + v.
    // Up to nbuf - 1 tiles' copies stay in flight; the oldest is announced
    // once its copy group is complete, before the next tile's copies are
    // issued (the buffer of tile t is reused for tile t + nbuf after the
    // MMAs of tile t are done).
    const TcSched S = tc_sched(L.nbuf);
    const int lag = S.nw * S.nbw - 1;  // buffers in use - 1
    int tile_ord = 0;
    int announced = 0;
    // staging map: lanes 2i, 2i+1 write the two halves of record (v, q),
    // records of one phase in consecutive lanes (q fastest)
    const int V = L.V;
    const uint32_t half = (uint32_t)(tid & 1) * 8u;
    const int rsub = tid >> 1;  // 0..47
    // record (v, q): sample q D + v in both halves, or (pair records) samples
    // q D + 2 v and q D + 2 v + 1
    const int vmul = L.pair ? 2 : 1;
    const int hadd = L.pair ? (tid & 1) : 0;
    for (int tile = blockIdx.x; tile < L.ntiles; tile += gridDim.x, ++tile_ord) {
      int use = 0;
      const int buf = tc_buf(S, tile_ord, &use);
      if (tile_ord >= lag && lag > 0) {
        switch (lag) {  // all but the lag - 1 most recent groups
          case 1: asm volatile("cp.async.wait_group 0;\n" ::: "memory"); break;
          case 2: asm volatile("cp.async.wait_group 1;\n" ::: "memory"); break;
          default: asm volatile("cp.async.wait_group 2;\n" ::: "memory"); break;
        }
        tc::fence_proxy_async_smem();
        __syncwarp();
        int ua = 0;
        if (lane_id == 0) tc::mbar_arrive(&bar_in_full[tc_buf(S, announced, &ua)]);
        ++announced;
      }
      if (use >= 1) {  // the buffer's previous tile has been consumed
        const bool ok = tc::mbar_wait_bounded(&bar_in_empty[buf], (uint32_t)((use - 1) & 1), kWaitPolls);
        if (__any_sync(0xffffffffu, !ok)) {
          failed = true;
          break;
        }
      }
      const uint32_t xb = tc::smem_u32(smem + L.in_off + buf * L.in_bytes);
      const int64_t tb = (int64_t)tile * 128 * D + L.B0;
      for (int v = 0; v < V; ++v)
        for (int q = rsub; q < L.Qp; q += kTcProdThreads / 2)
          stage_half(L, tb + (int64_t)q * D + vmul * v + hadd, xb + (uint32_t)(v * L.Qp + q) * 16u + half);
      asm volatile("cp.async.commit_group;\n" ::: "memory");
      if (lag == 0) {
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        tc::fence_proxy_async_smem();
        __syncwarp();
        if (lane_id == 0) tc::mbar_arrive(&bar_in_full[buf]);
        ++announced;
      }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    if (!failed) {
      tc::fence_proxy_async_smem();
      __syncwarp();
      for (; announced < tile_ord; ++announced) {
        int ua = 0;
        if (lane_id == 0) tc::mbar_arrive(&bar_in_full[tc_buf(S, announced, &ua)]);
      }
    }
    if (failed && lane_id == 0) atomicExch(L.err, 1);
    }
  } else if (warp == 3 || warp == kTcThreads / 32 - 1) {
    // ------------------------------------------------------------ MMA issuer
    // A-offset table of every merge set: entry kp = record index (v Qp + q)
    // of the first tap of MMA kp in a staged tile (taps 2kp, 2kp+1; with
    // pair records taps 4kp .. 4kp+3, record phase v = tap phase / 2), i.e.
    // the A descriptor's address field relative to the buffer (computed once,
    // by all 32 lanes)
    const TcSched S = tc_sched(L.nbuf);
    const int mw = warp == 3 ? 0 : 1;
    const int tpm = L.pair ? 4 : 2;  // taps per MMA
    uint32_t* tab = reinterpret_cast<uint32_t*>(smem + L.tab_off);
    for (int mi = 0; mi < nms && mw == 0; ++mi) {
      const TcMset& M = L.ms[mi];
      const int nkp = M.Kw / tpm;
      for (int kp = lane_id; kp < ((nkp + 3) & ~3); kp += 32) {
        uint32_t e = 0;
        if (kp < nkp) {
          const int s = M.a + tpm * kp;
          const int q = L.wrap ? s / D : 0;
          e = (uint32_t)(((s - q * D) / (tpm / 2)) * L.Qp + q);
        }
        tab[M.toff + kp] = e;
      }
    }
    tc::named_bar_sync(2, 64);  // both MMA warps: the table is written before it is read
    bool ok = tc::mbar_wait_bounded(&bar_b_full, 0u, kWaitPolls);
    if (__any_sync(0xffffffffu, !ok)) failed = true;
    if (mw >= S.nw) failed = true;  // second MMA warp unused: one input buffer
    // descriptor words: low = address >> 4 | (leading byte offset >> 4) << 16,
    // high = (stride byte offset >> 4) | version 1 (bit 46)
    const uint32_t a_hi = (128u >> 4) | (1u << 14);
    int tile_ord = mw;
    for (int tile = blockIdx.x + mw * (int)gridDim.x; !failed && tile < L.ntiles;
         tile += S.nw * (int)gridDim.x, tile_ord += S.nw) {
      int use = 0;
      const int buf = tc_buf(S, tile_ord, &use);
      ok = tc::mbar_wait_bounded(&bar_in_full[buf], (uint32_t)(use & 1), kWaitPolls);
      if (__any_sync(0xffffffffu, !ok)) {
        failed = true;
        break;
      }
      tc::fence_after_sync();
      const uint32_t xb = tc::smem_u32(smem + L.in_off + buf * L.in_bytes);
      const uint32_t a_lo0 = ((xb >> 4) & 0x3FFFu) | ((((uint32_t)L.Qp * 16u) >> 4) << 16);
      for (int mi = 0; mi < nms; ++mi) {
        const int jw = (tile_ord / S.nw) * nms + mi;  // this warp's item number
        const uint32_t ds = (uint32_t)(mw * S.spw + jw % S.spw);
        const int suse = jw / S.spw;
        if (suse >= 1) {
          ok = tc::mbar_wait_bounded(&bar_d_empty[ds], (uint32_t)((suse - 1) & 1), kWaitPolls);
          if (__any_sync(0xffffffffu, !ok)) {
            failed = true;
            break;
          }
          tc::fence_after_sync();
        }
        if (lane_id == 0) {
          // taps 2kp, 2kp+1 read records (v, q) and (v + 1, q) of the tile
          // (phase D is phase 0 one row on): A address = buffer + tab[kp];
          // B advances one 256-byte pair of cores per MMA
          const TcMset& M = L.ms[mi];
          const uint32_t idesc = tc::idesc_f16(FMT, 128, (uint32_t)M.N);
          const uint32_t bb = tc::smem_u32(smem + M.boff);
          const uint32_t b_lo0 = ((bb >> 4) & 0x3FFFu) | ((128u >> 4) << 16);
          const uint32_t b_hi = (((uint32_t)M.Kw * 128u) >> 4) | (1u << 14);
          const uint32_t d_tm = tbase + ds * kTcDCols;
          const uint4* t4 = reinterpret_cast<const uint4*>(tab + M.toff);
          if (L.pair) {
            // pair records: MMA kp covers taps 4kp .. 4kp+3 (two records of
            // two samples), once against the hi taps and once against the lo
            // taps (B matrices of (N / 8) x (Kw / 2) cores, one after the
            // other); both accumulate into the same columns
            const uint32_t sbo = (((uint32_t)M.Kw / 2u * 128u) >> 4) | (1u << 14);
            const uint32_t lo_off = ((uint32_t)M.N * (uint32_t)M.Kw * 8u) >> 4;
            const int nkp = M.Kw / 4;
            for (int kp = 0; kp < nkp; kp += 4) {
              const uint4 o = t4[kp >> 2];
              const uint32_t ao[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                if (kp + i < nkp) {
                  const uint64_t da = ((uint64_t)a_hi << 32) | (a_lo0 + ao[i]);
                  const uint32_t bl = b_lo0 + (uint32_t)(kp + i) * 16u;
                  mma_ss(d_tm, da, ((uint64_t)sbo << 32) | bl, idesc, (kp + i) > 0 ? 1u : 0u);
                  mma_ss(d_tm, da, ((uint64_t)sbo << 32) | (bl + lo_off), idesc, 1u);
                }
              }
            }
            tc::mma_commit(&bar_d_full[ds]);
          }
          const int nkp = L.pair ? 0 : M.Kw / 2;
          for (int kp = 0; kp < nkp; kp += 4) {
            // the four descriptor pairs are ready before the first MMA issues
            const uint4 o = t4[kp >> 2];
            const uint32_t bl = b_lo0 + (uint32_t)kp * 16u;
            const uint64_t da0 = ((uint64_t)a_hi << 32) | (a_lo0 + o.x);
            const uint64_t da1 = ((uint64_t)a_hi << 32) | (a_lo0 + o.y);
            const uint64_t da2 = ((uint64_t)a_hi << 32) | (a_lo0 + o.z);
            const uint64_t da3 = ((uint64_t)a_hi << 32) | (a_lo0 + o.w);
            const uint64_t db0 = ((uint64_t)b_hi << 32) | bl;
            const uint64_t db1 = ((uint64_t)b_hi << 32) | (bl + 16u);
            const uint64_t db2 = ((uint64_t)b_hi << 32) | (bl + 32u);
            const uint64_t db3 = ((uint64_t)b_hi << 32) | (bl + 48u);
            mma_ss(d_tm, da0, db0, idesc, kp > 0 ? 1u : 0u);
            if (kp + 1 < nkp) mma_ss(d_tm, da1, db1, idesc, 1u);
            if (kp + 2 < nkp) mma_ss(d_tm, da2, db2, idesc, 1u);
            if (kp + 3 < nkp) mma_ss(d_tm, da3, db3, idesc, 1u);
          }
          if (!L.pair) tc::mma_commit(&bar_d_full[ds]);
        }
        __syncwarp();
      }
      if (failed) break;
      if (lane_id == 0) tc::mma_commit(&bar_in_empty[buf]);
      __syncwarp();
    }
    if (failed && mw < S.nw && lane_id == 0) atomicExch(L.err, 1);
  } else {
    // ------------------------------------------------------------ epilogue
    // The 16 epilogue warps form NG groups (L.epi_groups: 4 for narrow merge
    // sets, 1 for wide ones).  Group g owns the accumulator slots s with
    // s % NG == g and drains their items in tile order (item = tile_ord *
    // nmsets + merge set), so every slot keeps one in-order consumer.  Warp w
    // covers TMEM lanes 32 (w % 4) .. +31 (the lanes it may read) and the
    // 8-slot chunks cp, cp + 4/NG, ... of an item: with one group all 16
    // warps share each item and a slot is free again after a quarter of its
    // epilogue work; with four, each group's 4 warps drain whole items side
    // by side.  Each warp runs on its own (a slot is released once the 16/NG
    // warps of its group arrived), so a stop decision only has to be uniform
    // over a warp.
    const int NG = L.epi_groups;
    const int mrow = (warp - 4) >> 2;
    const int eg_own = mrow % NG;
    const int cp = mrow / NG;
    const int cstep = 4 / NG;
    const int quarter = warp & 3;
    const uint32_t lane = (uint32_t)(quarter * 32) << 16;
    const int row = quarter * 32 + lane_id;
    bool ok = tc::mbar_wait_bounded(&bar_b_full, 0u, kWaitPolls);
    if (__any_sync(0xffffffffu, !ok)) failed = true;
    const TcSched S = tc_sched(L.nbuf);
    for (int itg = 0; !failed; ++itg) {
      const int tile_ord = itg / nms;
      const int mi = itg - tile_ord * nms;
      const int tile = blockIdx.x + tile_ord * gridDim.x;
      if (tile >= L.ntiles) break;
      // the accumulator slot of this item (the issuing warp's schedule)
      const int ew = tile_ord % S.nw;
      const int jw = (tile_ord / S.nw) * nms + mi;
      const int eg = ew * S.spw + jw % S.spw;
      if (eg % NG != eg_own) continue;  // another group's slot
      ok = tc::mbar_wait_bounded(&bar_d_full[eg], (uint32_t)((jw / S.spw) & 1), kWaitPolls);
      if (__any_sync(0xffffffffu, !ok)) {
        failed = true;
        break;
      }
      tc::fence_after_sync();
      const TcMset& M = L.ms[mi];
      const int nslots = M.N >> 1;
      const float2* rtab = reinterpret_cast<const float2*>(smem + M.poff);
      const uint32_t* P0in = reinterpret_cast<const uint32_t*>(smem + M.poff + (size_t)nslots * 64);
      const int64_t j0 = (int64_t)tile * 128;
      const int64_t j = j0 + row;
      const uint32_t rowD = (uint32_t)(row * D);
      const int32_t j32 = (int32_t)j;
      const uint32_t dcol = (uint32_t)eg * kTcDCols;
      const int nch = M.N >> 4;  // 8-slot chunks (16 columns)
      // the warps sharing an item take its chunks round robin, starting one
      // column group further on every item, so the extra chunks of an item
      // whose chunk count is not a multiple of four rotate over the warps
      const int cpi = (cp + itg) % cstep;
      if (cpi >= nch) {  // no chunk of this item for this warp: release at once
        tc::fence_before_sync();
        __syncwarp();
        if (lane_id == 0) tc::mbar_arrive(&bar_d_empty[eg]);
      }
      for (int cc = cpi; cc < nch; cc += cstep) {
        uint32_t v[16];
        tc::tmem_ld16(tbase + lane + dcol + 16 * cc, v);
        tc::tmem_wait_ld();
        if (cc + cstep >= nch) {
          // the slot is free for the MMAs once every warp holds its last part
          tc::fence_before_sync();
          __syncwarp();
          if (lane_id == 0) tc::mbar_arrive(&bar_d_empty[eg]);
        }
        // row-0 NCO counter of the chunk's 8 slots (lane e + 8 g computes
        // slot cc * 8 + e): P0 = (samples since reset at the window start of
        // row 0) mod R; row `row` then starts at (P0 + row D) mod R
        const int e_l = lane_id & 7;
        const int si_l = cc * 8 + e_l;
        uint32_t p0 = 0;
        const uint32_t R_l = P0in[2 * nslots + si_l];
        if (P0in[5 * nslots + si_l]) {
          // x < R + 2^31 < 2^32 on the fast path; x >= -(T - 1) > -R
          const int64_t x0 = (int64_t)(((uint64_t)P0in[nslots + si_l] << 32) | P0in[si_l]);
          const int64_t x = x0 + j0 * D;
          const uint64_t fm = ((uint64_t)P0in[4 * nslots + si_l] << 32) | P0in[3 * nslots + si_l];
          p0 = x < 0 ? (uint32_t)(x + R_l) : (uint32_t)__umul64hi(fm * (uint64_t)x, (uint64_t)R_l);
        }
        const TcSlotHot* hot = L.slot + M.slot0 + cc * 8;
        // Grouped rotation: when no row of an 8-row group wraps the counter or
        // has its window cross the rollover, the phase of row 8 g + i of the
        // warp is the group's first-row phase plus i D omega (mod 1 turn), so
        // the group needs one phasor (lane e + 8 g computes it for slot e) and
        // the slot's table of the eight i D omega phasors.  Chunks where every
        // group of every slot qualifies take this path.
        {
          const uint32_t Tm1_l = P0in[8 * nslots + si_l];
          const uint32_t rg = (uint32_t)(quarter * 32 + (lane_id & ~7)) * (uint32_t)D;  // first row of the group x D
          uint32_t pg = p0 + rg;  // < R + 127 D < 2^32 on the fast path
          pg = pg >= R_l ? pg - R_l : pg;
          const bool fast_l = Tm1_l != 0x7fffffffu && pg + 7u * (uint32_t)D + Tm1_l < R_l;
          if (__all_sync(0xffffffffu, fast_l)) {
            const uint32_t turns = __umulhi(pg, P0in[6 * nslots + si_l]) + pg * P0in[7 * nslots + si_l];
            float sn, cs;
            __sincosf((float)(int32_t)turns * 1.4629180792671596e-09f, &sn, &cs);  // 2 pi / 2^32
            float2* gph = epi_ph + (warp - 4) * 32;
            gph[lane_id] = make_float2(cs, sn);
            __syncwarp();
            const float4* g4 = reinterpret_cast<const float4*>(gph + (lane_id & ~7));
            const float2* rt = rtab + cc * 64 + (lane_id & 7);
#pragma unroll
            for (int e = 0; e < 8; ++e) {
              const float4 a2 = g4[e >> 1];
              const float2 A = (e & 1) ? make_float2(a2.z, a2.w) : make_float2(a2.x, a2.y);
              const TcSlotHot& sh = hot[e];
              const float2 y0 = make_float2(__uint_as_float(v[2 * e]), __uint_as_float(v[2 * e + 1]));
              const float2 y = cmul_nco(y0, cmul_nco(A, rt[e * 8]));
              float2* dst = reinterpret_cast<float2*>(((uint64_t)sh.out_hi << 32) | sh.out_lo) +
                            (uint64_t)sh.U * (uint32_t)j32;
              if (j32 < sh.J) *dst = y;
            }
            __syncwarp();  // every lane has read the phasors before the next chunk writes them
            continue;
          }
        }
        // per-row rotation (a group wraps the counter or crosses the
        // rollover, or a slot takes the exact path): outputs whose window
        // crosses the NCO rollover are written unrotated and fixed from that
        // value below
        uint32_t slow = 0;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const TcSlotHot sh = hot[e];
          const uint32_t P0 = __shfl_sync(0xffffffffu, p0, e);
          const uint32_t R = sh.R;
          // (P0 + row D) mod R: P0 < R and row D < R - T on the fast path,
          // so one conditional subtraction
          const uint32_t a = P0 + rowD;
          const uint32_t pc = a >= R ? a - R : a;
          const bool okr = pc + sh.Tm1 < R;
          // bits 32..63 of pc * omega64: the phase in 2^-32 turns
          const uint32_t turns = __umulhi(pc, sh.om_lo) + pc * sh.om_hi;
          const float ang = (float)(int32_t)turns * 1.4629180792671596e-09f;  // 2 pi / 2^32
          float sn, cs;
          __sincosf(ang, &sn, &cs);
          const float2 y0 = make_float2(__uint_as_float(v[2 * e]), __uint_as_float(v[2 * e + 1]));
          const float2 y = cmul_nco(y0, make_float2(cs, sn));
          const bool valid = j32 < sh.J;
          float2* dst = reinterpret_cast<float2*>(((uint64_t)sh.out_hi << 32) | sh.out_lo) +
                        (uint64_t)sh.U * (uint32_t)j32;
          if (valid) *dst = okr ? y : y0;
          slow |= (valid && !okr) ? (1u << e) : 0u;
        }
        while (slow) {
          const int e = __ffs(slow) - 1;
          slow &= slow - 1;
          const SlotMeta sm = slot_meta(L, M, cc * 8 + e, D);
          const int64_t w0 = (int64_t)sm.delta + j * D - sm.T + 1;
          float2* dst = sm.nco.out + ((int64_t)sm.r + (int64_t)sm.U * j);
          const ExactRot er = rotate_prep(sm.nco, w0, sm.T);
          float2 B = make_float2(0.f, 0.f);
          if (er.straddle) {
            for (int k = er.k0; k < sm.T; ++k) {
              const float2 x = load_x(L, w0 + k);
              const float2 gk = __ldg(sm.taps32 + (size_t)k * sm.tstride + sm.tidx);
              B.x = fmaf(gk.x, x.x, B.x);
              B.x = fmaf(-gk.y, x.y, B.x);
              B.y = fmaf(gk.x, x.y, B.y);
              B.y = fmaf(gk.y, x.x, B.y);
            }
          }
          *dst = rotate_apply(er, *dst, B);
        }
      }
    }
    if (failed && lane_id == 0) atomicExch(L.err, 1);
  }

  // teardown: once every role has left its loop, every MMA this CTA issued
  // has been drained by the epilogue (after a failure, bounded waits have
  // already given the tensor core time)
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, kTmemCols);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static uint16_t to16(float v, int fmt) {
  if (fmt == 0) {
    const __half h = __float2half_rn(v);
    return *reinterpret_cast<const uint16_t*>(&h);
  }
  const __nv_bfloat16 b = __float2bfloat16_rn(v);
  return *reinterpret_cast<const uint16_t*>(&b);
}
static float from16(uint16_t u, int fmt) {
  if (fmt == 0) {
    __half h;
    std::memcpy(&h, &u, 2);
    return __half2float(h);
  }
  __nv_bfloat16 b;
  std::memcpy(&b, &u, 2);
  return __bfloat162float(b);
}

void PolyEngine::free_tc() {
  if (d_xhl_) cudaFree(d_xhl_);
  d_xhl_ = nullptr;
  xhl_cap_ = 0;
  for (auto& c : tc_chunks_) {
    if (c.d_b) cudaFree(c.d_b);
    if (c.d_taps32) cudaFree(c.d_taps32);
    if (c.d_ch) cudaFree(c.d_ch);
  }
  tc_chunks_.clear();
  if (d_err_) cudaFree(d_err_);
  d_err_ = nullptr;
}

// Chunks of <= 32 channels per class (sorted by taps per phase).  For every
// phase, B records in the K-major no-swizzle core layout: core (cg, t) of 8
// columns x 1 tap at byte (cg T + t) 128, column c of the core at c 16,
// element e at e 2.  Column 2i is Re, 2i+1 Im of channel i; with the input
// record [xr_h, xi_h, xr_l, xi_l, xr_h, xi_h, xr_l, xi_l] the elements are
//     Re: [gr_h, -gi_h, gr_h, -gi_h, gr_l, -gi_l, gr_l, -gi_l]
//     Im: [gi_h,  gr_h, gi_h,  gr_h, gi_l,  gr_l, gi_l,  gr_l]
// so each column sums (xh + xl)(gh + gl) over re/im.  Also the FP32
// modulated taps for the rollover correction.
int PolyEngine::build_tc(int fmt) {
  free_tc();
  tc_fmt_ = fmt;
  for (size_t ki = 0; ki < classes_.size(); ++ki) {
    const EngineClass& k = classes_[ki];
    std::vector<int> cs = k.chans;
    std::stable_sort(cs.begin(), cs.end(), [&](int a, int b) { return chans_[a].T > chans_[b].T; });
    for (size_t i0 = 0; i0 < cs.size(); i0 += kTcChunk) {
      TcChunk ch;
      ch.cls = (int)ki;
      ch.chans.assign(cs.begin() + i0, cs.begin() + std::min(cs.size(), i0 + (size_t)kTcChunk));
      const int n = (int)ch.chans.size();
      const int tmax = (int)chans_[ch.chans[0]].T;
      ch.T = (tmax + 1) & ~1;
      ch.supported = ch.T <= kTcMaxTaps;
      ch.ng = (2 * n + 7) / 8;
      ch.bbytes = (size_t)ch.ng * ch.T * 128;
      ch.d_b = nullptr;
      ch.d_taps32 = nullptr;
      ch.d_ch = nullptr;
      if (!ch.supported) {
        tc_chunks_.push_back(ch);
        continue;
      }
      const uint32_t U = k.up;
      std::vector<uint8_t> bh((size_t)U * ch.bbytes, 0);
      std::vector<float2> t32((size_t)U * ch.T * n, make_float2(0.f, 0.f));
      for (int ci = 0; ci < n; ++ci) {
        const EngineChannel& e = chans_[ch.chans[ci]];
        const int pad = ch.T - (int)e.T;
        int64_t fm = 0;
        if (e.nco.enabled) {
          fm = (int64_t)e.shift_hz % (int64_t)fs_;
          if (fm < 0) fm += fs_;
        }
        for (uint32_t ph = 0; ph < U; ++ph) {
          uint8_t* bp = bh.data() + (size_t)ph * ch.bbytes;
          for (int kk = pad; kk < ch.T; ++kk) {
            const float2 h = e.flipped[(size_t)ph * e.T + (kk - pad)];
            double gr = h.x, gi = h.y;
            if (e.nco.enabled) {
              const uint64_t red = (uint64_t)(((unsigned __int128)(uint64_t)fm * (uint64_t)kk) % fs_);
              const double ang = 2.0 * M_PI * (double)red / (double)fs_;
              const double c = std::cos(ang), s = std::sin(ang);
              gr = (double)h.x * c - (double)h.y * s;
              gi = (double)h.x * s + (double)h.y * c;
            }
            const float fr = (float)gr, fi = (float)gi;
            t32[((size_t)ph * ch.T + kk) * n + ci] = make_float2(fr, fi);
            const uint16_t rh = to16(fr, fmt), ih = to16(fi, fmt);
            const uint16_t rl = to16(fr - from16(rh, fmt), fmt), il = to16(fi - from16(ih, fmt), fmt);
            const uint16_t sgn = 0x8000u;
            const uint16_t re_col[8] = {rh, (uint16_t)(ih ^ sgn), rh, (uint16_t)(ih ^ sgn),
                                        rl, (uint16_t)(il ^ sgn), rl, (uint16_t)(il ^ sgn)};
            const uint16_t im_col[8] = {ih, rh, ih, rh, il, rl, il, rl};
            for (int part = 0; part < 2; ++part) {
              const int col = 2 * ci + part;
              uint8_t* core = bp + ((size_t)(col / 8) * ch.T + kk) * 128 + (col % 8) * 16;
              std::memcpy(core, part ? im_col : re_col, 16);
            }
          }
        }
      }
      std::vector<int16_t> ids(ch.chans.begin(), ch.chans.end());
      cudaError_t err = cudaMalloc(&ch.d_b, bh.size());
      if (err == cudaSuccess) err = cudaMemcpy(ch.d_b, bh.data(), bh.size(), cudaMemcpyHostToDevice);
      if (err == cudaSuccess) err = cudaMalloc(&ch.d_taps32, t32.size() * sizeof(float2));
      if (err == cudaSuccess)
        err = cudaMemcpy(ch.d_taps32, t32.data(), t32.size() * sizeof(float2), cudaMemcpyHostToDevice);
      if (err == cudaSuccess) err = cudaMalloc(&ch.d_ch, ids.size() * sizeof(int16_t));
      if (err == cudaSuccess)
        err = cudaMemcpy(ch.d_ch, ids.data(), ids.size() * sizeof(int16_t), cudaMemcpyHostToDevice);
      tc_chunks_.push_back(ch);
      if (err != cudaSuccess) return cuda_status(err);
    }
  }
  cudaError_t err = cudaMalloc(&d_err_, sizeof(int));
  if (err == cudaSuccess) err = cudaMemset(d_err_, 0, sizeof(int));
  if (err != cudaSuccess) return cuda_status(err);
  return FDSP_OK;
}

bool PolyEngine::group_tc_ok(int gi) const {
  for (const auto& ch : tc_chunks_) {
    if (groups_idx_of_class(ch.cls) == gi && !ch.supported) return false;
  }
  return true;
}

int PolyEngine::groups_idx_of_class(int cls) const {
  for (size_t gi = 0; gi < groups_.size(); ++gi)
    if (groups_[gi].D == classes_[cls].down) return (int)gi;
  return -1;
}

// Pre-split [history | block] into packed {hi, lo} pairs (scratch buffer
// owned by the engine, grown on demand).
int PolyEngine::prepare_tc_input(const float2* d_in, uint64_t n, cudaStream_t stream) {
  const size_t need = (size_t)(n + H_) + 2;  // one spare pair: bulk copies end on an even sample
  if (need > xhl_cap_) {
    if (d_xhl_) cudaFree(d_xhl_);
    d_xhl_ = nullptr;
    xhl_cap_ = 0;
    cudaError_t e = cudaMalloc(&d_xhl_, need * sizeof(uint2));
    if (e != cudaSuccess) return cuda_status(e);
    xhl_cap_ = need;
  }
  if (num_sms_ == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev);
    if (num_sms_ <= 0) num_sms_ = 1;
  }
  const int64_t blocks = std::min<int64_t>((int64_t)(need + 255) / 256, (int64_t)num_sms_ * 8);
  if (tc_fmt_ == 0)
    split_input_kernel<0><<<(unsigned)blocks, 256, 0, stream>>>(in16_ ? nullptr : d_in, in16_, d_hist_[hist_cur_],
                                                                 (int64_t)n, H_, d_xhl_);
  else
    split_input_kernel<1><<<(unsigned)blocks, 256, 0, stream>>>(in16_ ? nullptr : d_in, in16_, d_hist_[hist_cur_],
                                                                 (int64_t)n, H_, d_xhl_);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e);
  launches_last_++;
  return FDSP_OK;
}

int PolyEngine::launch_tc_group(int gi, const float2* d_in, uint64_t n, float2* const* out, cudaStream_t stream) {
  const EngineGroup& g = groups_[gi];
  const uint32_t Dg = g.D;
  // Row split: a group with few channel columns wastes most of each MMA's N.
  // Its work sets' rows j = S i + b (b < S) become S work sets whose rows
  // are S D samples apart and whose windows end b D later; merged, one
  // staged tile then feeds S x the columns (the window grows by (S - 1) D
  // taps, the MMAs per output drop by about S, B grows S-fold).  S is the
  // largest split up to the group's limit (autotuned) whose columns and
  // window still fit one merge set.
  int cols = 0, tmax = 0;
  for (const auto& ch : tc_chunks_) {
    const EngineClass& k = classes_[ch.cls];
    if (k.down != Dg || !ch.supported) continue;
    cols += 2 * (int)ch.chans.size() * (int)k.up;
    tmax = std::max(tmax, ch.T);
  }
  const uint32_t split = tc_row_split(cols, tmax, Dg, g.tc_split);
  const uint32_t D = Dg * split;
  groups_[gi].tc_split_used = (int)split;
  // ---- work sets of this apply (chunk x output phase r x row class b)
  std::vector<TcWsPlan> wl;
  for (const auto& ch : tc_chunks_) {
    const EngineClass& k = classes_[ch.cls];
    if (k.down != Dg) continue;
    const uint32_t U = k.up;
    for (uint32_t r = 0; r < U; ++r) {
      if (k.M <= r) continue;
      const uint64_t t = (uint64_t)k.phase + (uint64_t)r * Dg;
      const int64_t J = (int64_t)((k.M - r + U - 1) / U);
      for (uint32_t b = 0; b < split; ++b) {
        if (J <= (int64_t)b) continue;
        TcWsPlan w;
        w.ch = &ch;
        w.T = ch.T;
        w.n = (int)ch.chans.size();
        w.phi = (uint32_t)(t % U);
        w.delta = (int64_t)(k.xoffset + t / U) + (int64_t)b * Dg;
        w.J = (J - (int64_t)b + split - 1) / split;
        w.U = U * split;
        w.r = r + b * U;
        wl.push_back(w);
      }
    }
  }
  if (wl.empty()) return FDSP_OK;
  std::vector<int> order(wl.size());
  for (size_t i = 0; i < wl.size(); ++i) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return wl[a].delta < wl[b].delta; });
  // ---- merge sets and launches; narrower merge sets when a wide one's B
  // and input tile do not fit in shared memory together
  std::vector<TcMsetPlan> msets;
  std::vector<TcLaunchPlan> plans;
  const int pair = (D % 2 == 0) ? 1 : 0;  // records of two samples: half the staged bytes
  bool fits = false;
  for (int cap = (int)kTcDCols; cap >= 16 && !fits; cap /= 2) {
    msets = tc_merge(wl, order, cap);
    if (pair) tc_pair_windows(msets);
    fits = tc_pack(msets, D, pair, plans);
  }
  if (!fits) return FDSP_ERR_UNSUPPORTED;
  if (num_sms_ == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev);
    if (num_sms_ <= 0) num_sms_ = 1;
  }
  // ---- fill and launch
  static thread_local TcLaunch L;
  for (const auto& p : plans) {
    std::memset(&L, 0, sizeof(L));
    L.block = in16_ ? nullptr : d_in;
    L.block16 = in16_;
    L.hist = d_hist_[hist_cur_];
    L.xhl = d_xhl_;
    L.nco = d_nco_;
    L.err = d_err_;
    L.N = (int64_t)n;
    L.H = H_;
    L.D = (int32_t)D;
    for (size_t c = 0; c < chans_.size(); ++c) {
      L.out[c] = out[c];
      const uint32_t R = chans_[c].nco.rollover;
      L.nco_base[c] = R ? (uint32_t)(abs0_ % R) : 0u;
    }
    size_t off = 0;
    int nws = 0;
    int64_t rows = 0;
    L.nmsets = (int32_t)p.ms.size();
    // wide merge sets (5 or more 8-slot chunks): all epilogue warps share
    // each item; narrow ones: four groups drain whole items side by side
    int max_n = 0;
    for (int m : p.ms) max_n = std::max(max_n, ((msets[m].cols + 15) / 16) * 16);
    L.epi_groups = (max_n / 16 >= 5) ? 1 : 4;
    for (size_t q = 0; q < p.ms.size(); ++q) {
      const TcMsetPlan& m = msets[p.ms[q]];
      TcMset& M = L.ms[q];
      M.Kw = m.Kw;
      M.N = ((m.cols + 15) / 16) * 16;
      M.a = (int32_t)(m.S - p.B0);
      M.boff = (int32_t)off;
      off += (size_t)M.N * M.Kw * 16;
      M.ws_begin = nws;
      int s0 = 0;
      for (int wi : m.ws) {
        const TcWsPlan& w = wl[wi];
        TcWorkSet& W = L.ws[nws++];
        W.b = w.ch->d_b + (size_t)w.phi * w.ch->bbytes;
        W.taps32 = w.ch->d_taps32 + (size_t)w.phi * w.ch->T * w.ch->chans.size();
        W.ch = w.ch->d_ch;
        W.T = w.ch->T;
        W.n = (int32_t)w.ch->chans.size();
        W.ng = w.ch->ng;
        W.delta = (int32_t)w.delta;
        W.J = (int32_t)w.J;
        W.U = (int32_t)w.U;
        W.r = (int32_t)w.r;
        W.o = (int32_t)((w.delta - w.ch->T + 1) - m.S);
        W.s0 = s0;
        s0 += W.n;
        rows = std::max(rows, w.J);
      }
      M.ws_end = nws;
    }
    // per-output slot constants (the same rules as the kernel's slot table)
    int nslot = 0;
    for (size_t q = 0; q < p.ms.size(); ++q) {
      TcMset& M = L.ms[q];
      M.slot0 = nslot;
      for (int sI = 0; sI < M.N / 2; ++sI) {
        TcSlotHot& h = L.slot[nslot++];
        h.R = 0x7fffffffu;
        for (int wi = M.ws_begin; wi < M.ws_end; ++wi) {
          const TcWorkSet& W = L.ws[wi];
          const int i = sI - W.s0;
          if (i < 0 || i >= W.n) continue;
          {
            const TcWsPlan& w = wl[msets[p.ms[q]].ws[wi - M.ws_begin]];
            const int c = w.ch->chans[i];
            const NcoConst& nc = chans_[c].nco;
            const bool general =
                nc.enabled && (nc.rollover >= 0x80000000u || 127LL * D + W.T >= (int64_t)nc.rollover);
            h.om_lo = nc.enabled && !general ? (uint32_t)nc.omega64 : 0u;
            h.om_hi = nc.enabled && !general ? (uint32_t)(nc.omega64 >> 32) : 0u;
            const uintptr_t o = (uintptr_t)(out[c] + W.r);
            h.out_lo = (uint32_t)o;
            h.out_hi = (uint32_t)(o >> 32);
            h.R = nc.enabled && !general ? nc.rollover : 0x7fffffffu;
            h.Tm1 = general ? 0x7fffffffu : (uint32_t)(W.T - 1);
            h.U = (uint32_t)W.U;
            h.J = W.J;
          }
          break;
        }
      }
    }
    for (size_t q = 0; q < p.ms.size(); ++q) {
      L.ms[q].poff = (int32_t)off;
      off += (size_t)(L.ms[q].N / 2) * (8 * sizeof(float2) + 9 * sizeof(uint32_t));
    }
    L.tab_off = (int32_t)off;
    int toff = 0;
    for (size_t q = 0; q < p.ms.size(); ++q) {
      L.ms[q].toff = toff;
      toff += (L.ms[q].Kw / (p.pair ? 4 : 2) + 3) & ~3;
    }
    off += (size_t)toff * 4;
    off = (off + 127) & ~(size_t)127;
    L.raw_off = (int32_t)off;
    L.raw_span = p.raw_span;
    L.nraw = p.nraw;
    L.raw_stride = (int32_t)p.raw_stride;
    off += p.raw_bytes;
    L.in_off = (int32_t)off;
    L.in_bytes = (int32_t)p.in_bytes;
    L.nbuf = p.nbuf;
    L.V = p.V;
    L.Qp = p.Qp;
    L.wrap = p.wrap;
    L.pair = p.pair;
    L.B0 = (int32_t)p.B0;
    L.ntiles = (int32_t)((rows + 127) / 128);
    if (L.ntiles == 0) continue;
    const size_t smem = off + (size_t)p.nbuf * p.in_bytes;
    if (smem > kTcSmemMax) return FDSP_ERR_UNSUPPORTED;
    const int grid = std::max(1, std::min(num_sms_, (int)L.ntiles));
    void (*kern)(const TcLaunch) = tc_fmt_ == 0 ? poly_tc_kernel<0> : poly_tc_kernel<1>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e);
    kern<<<(unsigned)grid, kTcThreads, smem, stream>>>(L);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e);
    launches_last_++;
  }
  tc_groups_last_++;
  return FDSP_OK;
}

int PolyEngine::tc_error() const {
  if (!d_err_) return 0;
  int v = 0;
  cudaMemcpy(&v, d_err_, sizeof(int), cudaMemcpyDeviceToHost);
  return v;
}

}  // namespace fdsp
