// Tensor-core form of the polyphase engine (tcgen05, sm_103a).
//
// The fused shift + polyphase contraction of one decimation group is recast
// as a dense matrix product per (tap chunk, output class r):
//
//     Y[j][c] = sum_k X[j][k] * G[k][c]
//
//   j  output row (window end delta_r + j*D),           M = 128 rows per CTA
//   k  tap index of the padded window (T_pad <= 64),    K = 2*T_pad (re/im)
//   c  channel of the chunk (<= 64), re and im columns, N = 2*n padded to 16
//
// X rows are the raw (unshifted) input windows, G the NCO-modulated taps of
// phase phi_r (the same folding as the FP32 engine).  Both are split into
// hi + lo 16-bit parts and the product is taken as hi*hi + hi*lo + lo*hi with
// FP32 accumulation in tensor memory, which keeps ~2^-21 relative accuracy
// (far above the 60 dB SNR target) at tensor-core throughput.
//
//   * A (X) lives in TMEM: thread j of the CTA owns TMEM lane j and writes its
//     window as packed 16-bit (re, im) pairs, one 32-bit column per sample,
//     with tcgen05.st -- no shared-memory traffic for the large operand.
//   * B (G) is staged in shared memory in the K-major no-swizzle layout
//     (8 x 16-byte core matrices), precomputed on the host per phase.
//   * One thread issues 3 MMAs per K-step of 16 and commits to an mbarrier;
//     every wait is bounded and reports through an error flag.
//   * The epilogue loads each row's accumulators (tcgen05.ld), rotates them by
//     the exact integer NCO phase of the window start, applies the exact FP32
//     split-sum correction for windows that straddle the NCO rollover, and
//     stores each channel's output sample.
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fdsp_internal.h"
#include "fdsp_nco.cuh"
#include "fdsp_tc.cuh"

namespace fdsp {

constexpr int kTcThreads = 672;         // 4 producer warps + 1 MMA warp + 16 epilogue warps
constexpr int kTcProdThreads = 128;     // one producer warp per TMEM lane quarter
constexpr int kTcEpiThreads = 512;      // four epilogue warps per TMEM lane quarter
constexpr uint32_t kTmemCols = 512;     // [A slot 0 | A slot 1 | D slot 0 | D slot 1], 128 columns each
constexpr uint32_t kWaitPolls = 1u << 20;

using TcMeta = OutMeta;

__device__ __forceinline__ float2 cmul_tc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ float2 phasor64_tc(uint64_t turns64) {
  const int32_t top = (int32_t)(turns64 >> 32);
  const float a = (float)top * 1.4629180792671596e-09f;  // 2 pi / 2^32
  float s, c;
  __sincosf(a, &s, &c);
  return make_float2(c, s);
}

__device__ __forceinline__ float2 load_x(const TcLaunch& L, int64_t v) {
  if (v < 0) {
    const int64_t hv = v + L.H;
    return hv >= 0 ? L.hist[hv] : make_float2(0.f, 0.f);
  }
  return v < L.N ? __ldg(L.block + v) : make_float2(0.f, 0.f);
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

// Item sequence of one persistent CTA, tile-major: tiles blockIdx.x,
// blockIdx.x + gridDim.x, ... and within a tile every work set of the group
// that has rows there.  Producers and the epilogue walk it independently.
struct ItemIter {
  int tile, wi;
};

__device__ __forceinline__ void item_settle(const TcLaunch& L, const TcGroup& G, ItemIter& t) {
  while (t.tile < G.ntiles) {
    while (t.wi < G.ws_end && t.tile >= L.ws[t.wi].ntiles) ++t.wi;
    if (t.wi < G.ws_end) return;
    t.tile += gridDim.x;
    t.wi = G.ws_begin;
  }
}
__device__ __forceinline__ ItemIter item_first(const TcLaunch& L, const TcGroup& G) {
  ItemIter t{(int)blockIdx.x, G.ws_begin};
  item_settle(L, G, t);
  return t;
}
__device__ __forceinline__ ItemIter item_next(const TcLaunch& L, const TcGroup& G, ItemIter t) {
  ++t.wi;
  item_settle(L, G, t);
  return t;
}

// Asynchronous 8-byte copy of pre-split input sample v (block relative,
// v >= -H; {hi, lo} packed 16-bit pairs; zero-fill outside the data) into
// shared memory.
__device__ __forceinline__ void stage_sample(const TcLaunch& L, int64_t v, uint2* dst) {
  const int64_t u = v + L.H;
  const uint2* src = L.xhl;
  uint32_t bytes = 0;
  if (u >= 0 && u < L.N + L.H) {
    src = L.xhl + u;
    bytes = 8;
  }
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(tc::smem_u32(dst)), "l"(src), "r"(bytes)
               : "memory");
}

// [history | block] -> packed {hi, lo} 16-bit pairs, once per apply: every
// sample is used by many windows, so the split is not repeated per use.
template <int FMT>
__global__ void split_input_kernel(const float2* __restrict__ block, const float2* __restrict__ hist, int64_t N,
                                   int H, uint2* __restrict__ xhl) {
  const int64_t total = N + H;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
    const float2 x = u < H ? hist[u] : block[u - H];
    uint2 hl;
    split2<FMT>(x, hl.x, hl.y);
    xhl[u] = hl;
  }
}

// Persistent warp-specialised CTA (one per SM, all 512 TMEM columns):
//   warps 0-3   producers (TMEM lane quarter = warp): stage the B operands of
//               every work set once, then per tile stage the input (kDeint:
//               the whole tile de-interleaved by D in a double buffer, shared
//               by all work sets; otherwise each thread prefetches its own
//               row's window one item ahead) and build A for each work set into
//               one of two TMEM A slots;
//   warp 4      MMA issuer: waits for a built A slot and a drained accumulator
//               slot, issues the 3 x (T/8) MMAs, commits;
//   warps 5-20  epilogue (four warps per lane quarter, splitting the channels):
//               drain an accumulator slot (tcgen05.ld), rotate, fix rollover
//               straddles, store, release the slot.
// Shared memory: [B hi|lo of every work set][channel constants][input].
template <int FMT, bool kDeint>
__global__ void __launch_bounds__(kTcThreads, 1) poly_tc_kernel(const __grid_constant__ TcLaunch L, int g) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ uint32_t tmem_base_s;
  __shared__ __align__(8) uint64_t bar_a_full[2];    // A slot built                  (128 producer arrivals)
  __shared__ __align__(8) uint64_t bar_a_empty[2];   // MMA done reading A slot       (commit)
  __shared__ __align__(8) uint64_t bar_d_full[2];    // accumulator slot ready        (commit)
  __shared__ __align__(8) uint64_t bar_d_empty[2];   // epilogue drained accumulator  (512 arrivals)
  __shared__ __align__(8) uint64_t bar_b_full;       // B operands + constants staged (128 arrivals)
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const TcGroup& G = L.groups[g];
  const int D = G.D;
  uint2* xin = reinterpret_cast<uint2*>(smem + G.in_off);

  if (warp == 0) {
    tc::tmem_alloc(&tmem_base_s, kTmemCols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&bar_a_full[i], kTcProdThreads);
      tc::mbar_init(&bar_a_empty[i], 1);
      tc::mbar_init(&bar_d_full[i], 1);
      tc::mbar_init(&bar_d_empty[i], kTcEpiThreads);
    }
    tc::mbar_init(&bar_b_full, kTcProdThreads);
    tc::mbar_fence_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tmem_base_s;
  bool failed = false;

  if (warp < 4) {
    // ------------------------------------------------------------ producers
    // Every decision to stop is taken jointly (bar.red.or over the 128
    // producer threads) so no producer is ever left alone at a barrier.
    const uint32_t lane = (uint32_t)(warp * 32) << 16;
    const int row = tid;  // 0..127 = TMEM lane
    for (int wi = G.ws_begin; wi < G.ws_end; ++wi) {
      const TcWorkSet& W = L.ws[wi];
      uint8_t* bhi_s = smem + W.boff;
      for (int i = tid; i < W.bbytes / 16; i += kTcProdThreads) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(tc::smem_u32(bhi_s + 16 * i)),
                     "l"(W.bhi + 16 * i)
                     : "memory");
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(tc::smem_u32(bhi_s + W.bbytes + 16 * i)),
                     "l"(W.blo + 16 * i)
                     : "memory");
      }
      if (tid < W.n) {
        const int c = W.ch[tid];
        const NcoConst nc = L.nco[c];
        OutMeta m;
        m.omega64 = nc.omega64;
        m.wrap64 = nc.wrap64;
        m.fastmod = nc.fastmod;
        m.out = L.out[c];
        m.rollover = nc.rollover;
        m.base = L.nco_base[c];
        m.enabled = nc.enabled;
        m.pad_ = 0;
        reinterpret_cast<OutMeta*>(smem + W.moff)[tid] = m;
      }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    tc::fence_proxy_async_smem();
    tc::mbar_arrive(&bar_b_full);

    ItemIter itr = item_first(L, G);
    int it = 0;
    int cur_tile = -1;
    int tile_ord = 0;            // tiles begun by this CTA (tile buffer = tile_ord & 1)
    const int wp = G.win_pitch;  // window mode: uint2 per staged row
    auto stage_tile = [&](int tile, int buf) {
      const int64_t sb = (int64_t)tile * 128 * D + G.delta_min - G.tmax + 1;
      const int len = 127 * D + G.delta_span + G.tmax;
      uint2* dst = xin + buf * G.tile_elems;
      for (int t = tid; t < len; t += kTcProdThreads) {
        const int q = t / D;
        stage_sample(L, sb + t, dst + (t - q * D) * G.P + q);
      }
    };
    auto stage_window = [&](const ItemIter& t, int buf) {
      const TcWorkSet& WT = L.ws[t.wi];
      const int64_t w0 = (int64_t)WT.delta + ((int64_t)t.tile * 128 + row) * D - WT.T + 1;
      uint2* dst = xin + (buf * 128 + row) * wp;
      for (int k = 0; k < WT.T; ++k) stage_sample(L, w0 + k, dst + k);
    };
    if (itr.tile < G.ntiles) {
      if constexpr (kDeint)
        stage_tile(itr.tile, 0);
      else
        stage_window(itr, 0);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");

    while (itr.tile < G.ntiles) {
      const TcWorkSet& W = L.ws[itr.wi];
      const int T = W.T;
      const ItemIter nx = item_next(L, G, itr);
      if constexpr (kDeint) {
        if (itr.tile != cur_tile) {
          // this tile's copies (issued one tile ago) complete, then a producer
          // barrier: every copy is visible and every producer has finished
          // reading the previous tile, whose buffer now takes the prefetch of
          // this CTA's next tile
          asm volatile("cp.async.wait_group 0;\n" ::: "memory");
          tc::named_bar_sync(1, kTcProdThreads);
          const int nt = itr.tile + (int)gridDim.x;
          if (nt < G.ntiles) stage_tile(nt, (tile_ord + 1) & 1);
          asm volatile("cp.async.commit_group;\n" ::: "memory");
          cur_tile = itr.tile;
          ++tile_ord;
        }
      } else {
        // prefetch the next item's window (own row), then wait for this item's
        if (nx.tile < G.ntiles) stage_window(nx, (it + 1) & 1);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
      }
      const uint32_t slot = (uint32_t)(it & 1);
      // A slot free once the MMAs of item it-2 are done
      bool ok = true;
      if (it >= 2) ok = tc::mbar_wait_bounded(&bar_a_empty[slot], (uint32_t)(((it - 2) >> 1) & 1), kWaitPolls);
      if (tc::named_bar_red_or(2, kTcProdThreads, !ok || failed)) {
        failed = true;
        break;
      }
      // build A from shared memory: this row's window, hi and lo parts
      const uint32_t acol = slot * 128u;
      if constexpr (kDeint) {
        const int a0 = (W.delta - G.delta_min) + (G.tmax - T);
        const uint2* xt = xin + ((tile_ord - 1) & 1) * G.tile_elems;
        int q0 = a0 / D;
        int b0 = a0 - q0 * D;
        const uint2* xp = xt + b0 * G.P + q0 + row;
        const int wrap = 1 - D * G.P;
        for (int kc = 0; kc < T; kc += 8) {
          uint32_t hi[8], lo[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            const uint2 hl = *xp;
            hi[e] = hl.x;
            lo[e] = hl.y;
            xp += G.P;
            if (++b0 == D) {
              b0 = 0;
              xp += wrap;
            }
          }
          tc::tmem_st8(tbase + lane + acol + kc, hi);
          tc::tmem_st8(tbase + lane + acol + 64 + kc, lo);
        }
      } else {
        const uint2* xr = xin + ((it & 1) * 128 + row) * wp;
        for (int kc = 0; kc < T; kc += 8) {
          uint32_t hi[8], lo[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            const uint2 hl = xr[kc + e];
            hi[e] = hl.x;
            lo[e] = hl.y;
          }
          tc::tmem_st8(tbase + lane + acol + kc, hi);
          tc::tmem_st8(tbase + lane + acol + 64 + kc, lo);
        }
      }
      tc::tmem_wait_st();
      tc::fence_before_sync();
      tc::mbar_arrive(&bar_a_full[slot]);
      itr = nx;
      ++it;
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    if (failed && tid == 0) atomicExch(L.err, 1);
  } else if (warp == 4) {
    // ------------------------------------------------------------ MMA issuer
    bool ok = tc::mbar_wait_bounded(&bar_b_full, 0u, kWaitPolls);
    if (__any_sync(0xffffffffu, !ok)) failed = true;
    ItemIter itr = item_first(L, G);
    int it = 0;
    while (!failed && itr.tile < G.ntiles) {
      const TcWorkSet& W = L.ws[itr.wi];
      const int T = W.T;
      const uint32_t slot = (uint32_t)(it & 1);
      ok = tc::mbar_wait_bounded(&bar_a_full[slot], (uint32_t)((it >> 1) & 1), kWaitPolls);
      if (ok && it >= 2) ok = tc::mbar_wait_bounded(&bar_d_empty[slot], (uint32_t)(((it - 2) >> 1) & 1), kWaitPolls);
      if (__any_sync(0xffffffffu, !ok)) {
        failed = true;
        break;
      }
      tc::fence_after_sync();
      if ((tid & 31) == 0) {
        const uint32_t idesc = tc::idesc_f16(FMT, 128, W.N_pad);
        const uint32_t sbo = 16u * (2u * T);
        const uint32_t bh = tc::smem_u32(smem + W.boff);
        const uint32_t bl = bh + W.bbytes;
        const uint32_t acol = slot * 128u;
        const uint32_t dcol = 256u + slot * 128u;
        for (int s2 = 0; s2 < T / 8; ++s2) {
          const uint64_t dh = tc::smem_desc(bh + 256u * s2, 128u, sbo);
          const uint64_t dl = tc::smem_desc(bl + 256u * s2, 128u, sbo);
          tc::mma_ts(tbase + dcol, tbase + acol + 8 * s2, dh, idesc, s2 > 0 ? 1u : 0u);
          tc::mma_ts(tbase + dcol, tbase + acol + 8 * s2, dl, idesc, 1u);
          tc::mma_ts(tbase + dcol, tbase + acol + 64 + 8 * s2, dh, idesc, 1u);
        }
        tc::mma_commit(&bar_a_empty[slot]);
        tc::mma_commit(&bar_d_full[slot]);
      }
      __syncwarp();
      itr = item_next(L, G, itr);
      ++it;
    }
    if (failed && (tid & 31) == 0) atomicExch(L.err, 1);
  } else {
    // ------------------------------------------------------------ epilogue
    const int ew = warp - 5;                 // 0..15
    const int quarter = warp & 3;            // TMEM lanes this warp may access
    const int part = ew >> 2;                // which quarter of the channels
    const uint32_t lane = (uint32_t)(quarter * 32) << 16;
    const int row = quarter * 32 + (tid & 31);
    // stop decisions are uniform over all epilogue threads (bar.red.or)
    bool ok = tc::mbar_wait_bounded(&bar_b_full, 0u, kWaitPolls);
    if (tc::named_bar_red_or(4, kTcEpiThreads, !ok)) failed = true;
    ItemIter itr = item_first(L, G);
    int it = 0;
    while (!failed && itr.tile < G.ntiles) {
      const TcWorkSet& W = L.ws[itr.wi];
      const uint32_t slot = (uint32_t)(it & 1);
      ok = tc::mbar_wait_bounded(&bar_d_full[slot], (uint32_t)((it >> 1) & 1), kWaitPolls);
      if (tc::named_bar_red_or(4, kTcEpiThreads, !ok)) {
        failed = true;
        break;
      }
      tc::fence_after_sync();
      const OutMeta* meta = reinterpret_cast<const OutMeta*>(smem + W.moff);
      const int T = W.T;
      const int64_t j = (int64_t)itr.tile * 128 + row;
      const int64_t w0 = (int64_t)W.delta + j * D - T + 1;
      const bool row_ok = j < W.J;
      const int64_t m = (int64_t)W.r + (int64_t)W.U * j;
      const uint32_t dcol = 256u + slot * 128u;
      // the four warps of a lane quarter split the channels in 8-channel
      // chunks: this warp takes chunks [c_lo, c_hi) (at most 2 for n <= 64)
      const int nch = (W.n + 7) >> 3;
      const int c_lo = (nch * part) >> 2, c_hi = (nch * (part + 1)) >> 2;
      const int n_lo = c_lo * 8, n_hi = min(W.n, c_hi * 8);
      uint32_t vv[2][16];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int cc = c_lo + q;
        if (cc < c_hi) tc::tmem_ld16(tbase + lane + dcol + 16 * cc, vv[q]);
      }
      tc::tmem_wait_ld();
      // the accumulator slot is free for the next MMAs as soon as it is in
      // registers
      tc::fence_before_sync();
      tc::mbar_arrive(&bar_d_empty[slot]);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int cc = c_lo + q;
        if (cc >= c_hi) break;
        const uint32_t* v = vv[q];
        // 8 channels branch free (so their phase chains interleave); outputs
        // whose window crosses the NCO rollover are written unrotated and
        // fixed from that value below (nothing extra stays live)
        uint32_t slow = 0;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int n = cc * 8 + e;
          const bool valid = row_ok && n < n_hi;
          const OutMeta& cm = meta[valid ? n : n_lo];
          const float2 y0 = make_float2(__uint_as_float(v[2 * e]), __uint_as_float(v[2 * e + 1]));
          float2 y = y0;
          const bool okr = rotate_fast(cm, w0, T, y);
          if (valid) cm.out[m] = okr ? y : y0;
          slow |= (valid && !okr) ? (1u << e) : 0u;
        }
        while (slow) {
          const int e = __ffs(slow) - 1;
          slow &= slow - 1;
          const int n = cc * 8 + e;
          const OutMeta& cm = meta[n];
          const ExactRot er = rotate_prep(cm, w0, T);
          float2 B = make_float2(0.f, 0.f);
          if (er.straddle) {
            for (int k = er.k0; k < T; ++k) {
              const float2 x = load_x(L, w0 + k);
              const float2 gk = __ldg(W.taps32 + (size_t)k * W.n + n);
              B.x = fmaf(gk.x, x.x, B.x);
              B.x = fmaf(-gk.y, x.y, B.x);
              B.y = fmaf(gk.x, x.y, B.y);
              B.y = fmaf(gk.y, x.x, B.y);
            }
          }
          cm.out[m] = rotate_apply(er, cm.out[m], B);
        }
      }
      itr = item_next(L, G, itr);
      ++it;
    }
    if (failed && tid == 160) atomicExch(L.err, 1);
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

// Chunks of <= 64 channels per class (sorted by taps per phase), B operands in
// the tcgen05 K-major no-swizzle layout for every phase, FP32 modulated taps
// for the rollover correction.
int PolyEngine::build_tc(int fmt) {
  free_tc();
  tc_fmt_ = fmt;
  for (size_t ki = 0; ki < classes_.size(); ++ki) {
    const EngineClass& k = classes_[ki];
    std::vector<int> cs = k.chans;
    std::stable_sort(cs.begin(), cs.end(), [&](int a, int b) { return chans_[a].T > chans_[b].T; });
    for (size_t i0 = 0; i0 < cs.size(); i0 += 64) {
      TcChunk ch;
      ch.cls = (int)ki;
      ch.chans.assign(cs.begin() + i0, cs.begin() + std::min(cs.size(), i0 + 64));
      const int n = (int)ch.chans.size();
      const int tmax = (int)chans_[ch.chans[0]].T;
      ch.T = (tmax + 7) & ~7;
      ch.supported = ch.T <= 64;
      ch.N_pad = ((2 * n + 15) / 16) * 16;
      const int Kp = 2 * ch.T;
      ch.bbytes = ch.N_pad * Kp * 2;
      ch.d_b = nullptr;
      ch.d_taps32 = nullptr;
      ch.d_ch = nullptr;
      if (!ch.supported) {
        tc_chunks_.push_back(ch);
        continue;
      }
      const uint32_t U = k.up;
      std::vector<uint8_t> bh((size_t)U * 2 * ch.bbytes, 0);
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
          uint8_t* bhi = bh.data() + (size_t)ph * 2 * ch.bbytes;
          uint8_t* blo = bhi + ch.bbytes;
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
            // columns: 2ci -> Re(y) = sum gr*xr - gi*xi ; 2ci+1 -> Im(y) = sum gi*xr + gr*xi
            const float col[2][2] = {{fr, -fi}, {fi, fr}};
            for (int part = 0; part < 2; ++part) {
              const int nn = 2 * ci + part;
              for (int ri = 0; ri < 2; ++ri) {
                const int kp = 2 * kk + ri;
                const size_t off = (size_t)(nn / 8) * (16 * Kp) + (size_t)(kp / 8) * 128 + (nn % 8) * 16 + (kp % 8) * 2;
                const float v = col[part][ri];
                const uint16_t hv = to16(v, fmt);
                const uint16_t lv = to16(v - from16(hv, fmt), fmt);
                std::memcpy(bhi + off, &hv, 2);
                std::memcpy(blo + off, &lv, 2);
              }
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
  const size_t need = (size_t)(n + H_);
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
    split_input_kernel<0><<<(unsigned)blocks, 256, 0, stream>>>(d_in, d_hist_[hist_cur_], (int64_t)n, H_, d_xhl_);
  else
    split_input_kernel<1><<<(unsigned)blocks, 256, 0, stream>>>(d_in, d_hist_[hist_cur_], (int64_t)n, H_, d_xhl_);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e);
  launches_last_++;
  return FDSP_OK;
}

int PolyEngine::launch_tc_group(int gi, const float2* d_in, uint64_t n, float2* const* out, cudaStream_t stream) {
  static thread_local TcLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.block = d_in;
  L.hist = d_hist_[hist_cur_];
  L.xhl = d_xhl_;
  L.N = (int64_t)n;
  L.H = H_;
  L.nco = d_nco_;
  L.err = d_err_;
  for (size_t c = 0; c < chans_.size(); ++c) {
    L.out[c] = out[c];
    const uint32_t R = chans_[c].nco.rollover;
    L.nco_base[c] = R ? (uint32_t)(abs0_ % R) : 0u;
  }
  const EngineGroup& g = groups_[gi];
  TcGroup& gd = L.groups[0];
  gd.D = (int32_t)g.D;
  gd.ws_begin = 0;
  int nws = 0;
  int64_t rows = 0;
  int dmin = INT32_MAX, dmax = INT32_MIN, tmax = 8;
  size_t off = 0;  // shared-memory layout: B of every work set, then constants, then input
  for (const auto& ch : tc_chunks_) {
    const EngineClass& k = classes_[ch.cls];
    if (k.down != g.D) continue;
    const uint32_t U = k.up;
    for (uint32_t r = 0; r < U; ++r) {
      if (k.M <= r) continue;
      const uint64_t J = (k.M - r + U - 1) / U;
      const uint64_t t = (uint64_t)k.phase + (uint64_t)r * g.D;
      const uint64_t delta = k.xoffset + t / U;
      const uint32_t phi = (uint32_t)(t % U);
      if (nws >= kMaxTcWorkSets) return FDSP_ERR_UNSUPPORTED;
      TcWorkSet& W = L.ws[nws++];
      W.bhi = ch.d_b + (size_t)phi * 2 * ch.bbytes;
      W.blo = W.bhi + ch.bbytes;
      W.taps32 = ch.d_taps32 + (size_t)phi * ch.T * ch.chans.size();
      W.ch = ch.d_ch;
      W.T = ch.T;
      W.N_pad = ch.N_pad;
      W.n = (int32_t)ch.chans.size();
      W.delta = (int32_t)delta;
      W.J = (int32_t)J;
      W.U = (int32_t)U;
      W.r = (int32_t)r;
      W.bbytes = ch.bbytes;
      W.ntiles = (int32_t)((J + 127) / 128);
      W.boff = (int32_t)off;
      off += (size_t)2 * ch.bbytes;
      rows = std::max<int64_t>(rows, (int64_t)J);
      dmin = std::min(dmin, (int)delta);
      dmax = std::max(dmax, (int)delta);
      tmax = std::max(tmax, ch.T);
    }
  }
  gd.ws_end = nws;
  L.ngroups = 1;
  if (nws == 0) return FDSP_OK;
  for (int wi = 0; wi < nws; ++wi) {
    L.ws[wi].moff = (int32_t)off;
    off += (size_t)L.ws[wi].n * sizeof(TcMeta);
  }
  off = (off + 127) & ~(size_t)127;
  gd.in_off = (int32_t)off;
  gd.ntiles = (int32_t)((rows + 127) / 128);
  gd.tmax = tmax;
  gd.delta_min = dmin;
  gd.delta_span = dmax - dmin;
  // input staging: the whole tile de-interleaved by D when it is small (dense
  // decimation, windows overlap), else each row's window in a double buffer
  const int64_t len = 127LL * g.D + gd.delta_span + tmax;
  int64_t P = (len + g.D - 1) / g.D;
  if ((P & 1) == 0) P++;
  gd.P = (int32_t)P;
  gd.win_pitch = tmax + 1;  // odd pitch: two-way (minimal) bank use for 8-byte rows
  gd.tile_elems = (int32_t)(((int64_t)g.D * P + 15) & ~15LL);  // one tile buffer (uint2), 128-byte multiple
  const size_t deint_bytes = (size_t)2 * gd.tile_elems * sizeof(uint2);  // double buffered
  const size_t win_bytes = (size_t)2 * 128 * gd.win_pitch * sizeof(float2);
  const bool deint = deint_bytes <= win_bytes;
  const size_t smem = std::max<size_t>(off + (deint ? deint_bytes : win_bytes), 120 * 1024);
  if (smem > 225 * 1024) return FDSP_ERR_UNSUPPORTED;
  // persistent: one CTA per SM (at least 120 KB of shared memory and all 512
  // TMEM columns each, so two never share an SM), tiles strided over CTAs
  if (num_sms_ == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev);
    if (num_sms_ <= 0) num_sms_ = 1;
  }
  const int grid = std::max(1, std::min(num_sms_, (int)gd.ntiles));
  void (*kern)(const TcLaunch, int);
  if (tc_fmt_ == 0)
    kern = deint ? poly_tc_kernel<0, true> : poly_tc_kernel<0, false>;
  else
    kern = deint ? poly_tc_kernel<1, true> : poly_tc_kernel<1, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  kern<<<(unsigned)grid, kTcThreads, smem, stream>>>(L, 0);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e);
  launches_last_++;
  return FDSP_OK;
}

int PolyEngine::tc_error() const {
  if (!d_err_) return 0;
  int v = 0;
  cudaMemcpy(&v, d_err_, sizeof(int), cudaMemcpyDeviceToHost);
  return v;
}

}  // namespace fdsp
