// Polyphase engine: fused per-channel NCO shift + polyphase up/down resampling
// for any number of channels sharing one input stream (plain FP32 form).
//
// Reference behaviour reproduced (paths relative to the reference project):
//   shift      src/transform/falcon_dsp_freq_shift.cc:164-192, :194-235
//   resample   src/transform/falcon_dsp_polyphase_resampler.cc:114-162, :256-346
//   channelize src/transform/falcon_dsp_multi_rate_channelizer.cc:146-164
//
// Design (GB300-first, not a translation of the Jetson kernels):
//  * Channels are grouped by decimation factor D.  For one group, one CTA owns
//    a tile of Qt output rows and stages the RAW input span the tile needs in
//    shared memory exactly once, de-interleaved by D (sample s at
//    [s mod D][s div D]) so that 32 lanes computing 32 consecutive rows read
//    32 consecutive words: no bank conflicts, whatever D is.
//  * The NCO is folded into the taps.  For a window starting at input s with
//    no counter rollover inside it,
//        sum_k h[k] x[s+k] e^{j w ((s+k) mod R)} = e^{j w (s mod R)} sum_k g[k] x[s+k]
//    with g[k] = h[k] e^{j w k}.  All channels of a group therefore read the
//    same unshifted samples, and each output pays one rotation by an exact
//    integer phase (64-bit fixed point turns).  A window that straddles a
//    rollover (the reference's phase jump) is corrected exactly by splitting
//    its sum at the rollover.
//  * Channels with the same (up, down) share streaming state, so their outputs
//    sit at the same input positions.  They are packed NB at a time into tap
//    batches: one shared-memory load of x feeds NB complex MACs, which keeps
//    the kernel FMA-bound instead of shared-memory bound.
//  * All per-launch parameters ride in the kernel parameter block; the launch
//    needs no host->device copy and is safe to capture in a CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>

#include "fdsp_internal.h"
#include "fdsp_nco.cuh"

namespace fdsp {

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// (pv mod R) for 0 <= pv < 2^32 with a precomputed M = ceil(2^64 / R)
// (Lemire, Kaser & Kurz, "Faster remainder by direct computation", 2019).
__device__ __forceinline__ uint32_t fastmod_u32(uint32_t a, uint64_t M, uint32_t R) {
  return (uint32_t)__umul64hi(M * (uint64_t)a, (uint64_t)R);
}

// Counter value (n mod R) of the sample at block-relative index w.
__device__ __forceinline__ uint32_t nco_counter(const NcoConst& nc, uint32_t base, int64_t w) {
  const int64_t pv = (int64_t)base + w;
  if (pv < 0) return (uint32_t)(pv + (int64_t)nc.rollover);
  if (pv < 0x100000000LL) return fastmod_u32((uint32_t)pv, nc.fastmod, nc.rollover);
  return (uint32_t)((uint64_t)pv % nc.rollover);
}

// e^{j 2 pi t} for t in 2^-64 turns, on the SFU: the reduced argument lies in
// [-pi, pi), where __sincosf is accurate to ~4e-7 absolute.
__device__ __forceinline__ float2 phasor64_fast(uint64_t turns64) {
  const int32_t top = (int32_t)(turns64 >> 32);
  const float a = (float)top * 1.4629180792671596e-09f;  // 2 pi / 2^32
  float s, c;
  __sincosf(a, &s, &c);
  return make_float2(c, s);
}

using ChanMeta = OutMeta;

// One row of one work set with NB live channels: T complex MACs per channel
// (taps and samples from shared memory), then rotation and store.  Taps are
// stored [T][NBS] with NBS = NB rounded up to even, so every row of taps
// starts on a 16-byte boundary for the float4 loads.
template <int NB>
__device__ __forceinline__ void process_row(const float2* __restrict__ xs, const float2* __restrict__ tp,
                                            const ChanMeta* __restrict__ meta, int T, int D, int P, int a0, int jl,
                                            int64_t j, int U, int r, int delta) {
  constexpr int NBS = (NB + 1) & ~1;  // tap row stride (even: 16-byte aligned rows)
  int bq = a0 / D;
  int b = a0 - bq * D;
  const float2* xp = xs + b * P + bq + jl;
  const int wrap = 1 - D * P;
  // Narrow batches keep the two products of each complex MAC in separate
  // accumulators so the FMA dependency chains stay short.
  constexpr bool kSplit = NB <= 4;
  float2 acc[NB], acc2[kSplit ? NB : 1];
#pragma unroll
  for (int n = 0; n < NB; ++n) acc[n] = make_float2(0.f, 0.f);
#pragma unroll
  for (int n = 0; n < (kSplit ? NB : 1); ++n) acc2[n] = make_float2(0.f, 0.f);
#pragma unroll 2
  for (int k = 0; k < T; ++k) {
    const float2 x = *xp;
    float2 gk[NB];
    const float4* q4 = reinterpret_cast<const float4*>(tp + k * NBS);
#pragma unroll
    for (int i = 0; i < NB / 2; ++i) {
      const float4 v = q4[i];
      gk[2 * i] = make_float2(v.x, v.y);
      gk[2 * i + 1] = make_float2(v.z, v.w);
    }
    if constexpr (NB & 1) gk[NB - 1] = tp[k * NBS + NB - 1];
#pragma unroll
    for (int n = 0; n < NB; ++n) {
      if constexpr (kSplit) {
        acc[n].x = fmaf(gk[n].x, x.x, acc[n].x);
        acc2[n].x = fmaf(-gk[n].y, x.y, acc2[n].x);
        acc[n].y = fmaf(gk[n].x, x.y, acc[n].y);
        acc2[n].y = fmaf(gk[n].y, x.x, acc2[n].y);
      } else {
        acc[n].x = fmaf(gk[n].x, x.x, acc[n].x);
        acc[n].x = fmaf(-gk[n].y, x.y, acc[n].x);
        acc[n].y = fmaf(gk[n].x, x.y, acc[n].y);
        acc[n].y = fmaf(gk[n].y, x.x, acc[n].y);
      }
    }
    xp += P;
    if (++b == D) {
      b = 0;
      xp += wrap;
    }
  }

  if constexpr (kSplit) {
#pragma unroll
    for (int n = 0; n < NB; ++n) {
      acc[n].x += acc2[n].x;
      acc[n].y += acc2[n].y;
    }
  }

  // Epilogue: rotate by the NCO phase of the window start (branch free, so
  // the channels' phase chains interleave), store; windows that straddle the
  // NCO rollover take the exact split-sum path.
  const int64_t m = (int64_t)r + (int64_t)U * j;
  const int64_t w = (int64_t)delta + j * D - T + 1;  // window start, block relative
  // The rare outputs that need the exact path (window across the NCO
  // rollover) are first written unrotated, then fixed from that value, so no
  // accumulator stays live through the fix-up.
  uint32_t slow = 0;
#pragma unroll
  for (int n = 0; n < NB; ++n) {
    float2 y = acc[n];
    const bool ok = rotate_fast(meta[n], w, T, y);
    meta[n].out[m] = ok ? y : acc[n];
    slow |= ok ? 0u : (1u << n);
  }
  while (slow) {
    const int n = __ffs(slow) - 1;
    slow &= slow - 1;
    const OutMeta& cm = meta[n];
    const ExactRot er = rotate_prep(cm, w, T);
    float2 B = make_float2(0.f, 0.f);
    if (er.straddle) {
      const int kb = a0 + er.k0;
      int qq = kb / D;
      int bb = kb - qq * D;
      qq += jl;
      for (int k = er.k0; k < T; ++k) {
        const float2 x = xs[bb * P + qq];
        const float2 gk = tp[k * NBS + n];
        B.x = fmaf(gk.x, x.x, B.x);
        B.x = fmaf(-gk.y, x.y, B.x);
        B.y = fmaf(gk.x, x.y, B.y);
        B.y = fmaf(gk.y, x.x, B.y);
        if (++bb == D) {
          bb = 0;
          ++qq;
        }
      }
    }
    cm.out[m] = rotate_apply(er, cm.out[m], B);
  }
}

// Single-channel work sets with long filters: each thread computes kWinRows
// consecutive output rows.  Taps are visited phase by phase (k = v, v + D,
// ...), where the samples of consecutive taps and consecutive rows are
// consecutive in the de-interleaved tile, so the rows share one sliding
// window of samples held in registers: one shared-memory load per tap step
// serves kWinRows outputs (the per-row path loads a sample per tap and
// output).  kWinRows is odd so the lanes of a warp (row blocks kWinRows
// apart) read distinct bank pairs.  Real taps (no NCO shift, resampler
// semantics) take 2 FMAs per tap instead of 4.
constexpr int kWinRows = 7;

template <bool kReal>
__device__ __forceinline__ void win_mac(float2& acc, float2 g, float2 x) {
  if constexpr (kReal) {
    acc.x = fmaf(g.x, x.x, acc.x);
    acc.y = fmaf(g.x, x.y, acc.y);
  } else {
    acc.x = fmaf(g.x, x.x, acc.x);
    acc.x = fmaf(-g.y, x.y, acc.x);
    acc.y = fmaf(g.x, x.y, acc.y);
    acc.y = fmaf(g.y, x.x, acc.y);
  }
}

// Rotation and store of one single-channel output (the per-row epilogue
// for NB = 1, taps at stride 2 float2).
__device__ __forceinline__ void win_finish(float2 acc, const ChanMeta& cm, const float2* __restrict__ xs,
                                           const float2* __restrict__ tp, int T, int D, int P, int a0, int jl,
                                           int64_t j, int U, int r, int delta) {
  const int64_t m = (int64_t)r + (int64_t)U * j;
  const int64_t w = (int64_t)delta + j * D - T + 1;
  float2 y = acc;
  if (rotate_fast(cm, w, T, y)) {
    cm.out[m] = y;
    return;
  }
  const ExactRot er = rotate_prep(cm, w, T);
  float2 B = make_float2(0.f, 0.f);
  if (er.straddle) {
    const int kb = a0 + er.k0;
    int qq = kb / D;
    int bb = kb - qq * D;
    qq += jl;
    for (int k = er.k0; k < T; ++k) {
      const float2 x = xs[bb * P + qq];
      const float2 gk = tp[k * 2];
      B.x = fmaf(gk.x, x.x, B.x);
      B.x = fmaf(-gk.y, x.y, B.x);
      B.y = fmaf(gk.x, x.y, B.y);
      B.y = fmaf(gk.y, x.x, B.y);
      if (++bb == D) {
        bb = 0;
        ++qq;
      }
    }
  }
  cm.out[m] = rotate_apply(er, acc, B);
}

template <bool kReal>
__device__ __forceinline__ void process_rows_win(const float2* __restrict__ xs, const float2* __restrict__ tp,
                                                 const ChanMeta* __restrict__ meta, int T, int D, int P, int a0,
                                                 int jl0, int64_t j0, int64_t J, int U, int r, int delta) {
  float2 acc[kWinRows];
#pragma unroll
  for (int q = 0; q < kWinRows; ++q) acc[q] = make_float2(0.f, 0.f);
  const int bq = a0 / D, b0 = a0 - bq * D;
  const int nv = T < D ? T : D;
  for (int vp = 0; vp < nv; ++vp) {
    int ph = b0 + vp, q0 = bq + jl0;
    if (ph >= D) {
      ph -= D;
      ++q0;
    }
    const float2* xr = xs + ph * P + q0;  // row jl0 + q, tap vp + m D: xr[m + q]
    const float2* tk = tp + 2 * vp;       // tap k at tp[2 k]
    const int tstep = 2 * D;
    const int nm = (T - 1 - vp) / D + 1;
    float2 w[kWinRows];
#pragma unroll
    for (int q = 0; q < kWinRows - 1; ++q) w[q] = xr[q];
    int m = 0;
    for (; m + kWinRows <= nm; m += kWinRows) {
      // circular window: sample m + u + q sits in slot (u + q) % kWinRows
#pragma unroll
      for (int u = 0; u < kWinRows; ++u) {
        w[(u + kWinRows - 1) % kWinRows] = xr[m + u + kWinRows - 1];
        const float2 g = tk[(m + u) * tstep];
#pragma unroll
        for (int q = 0; q < kWinRows; ++q) win_mac<kReal>(acc[q], g, w[(u + q) % kWinRows]);
      }
    }
    for (; m < nm; ++m) {
      w[kWinRows - 1] = xr[m + kWinRows - 1];
      const float2 g = tk[m * tstep];
#pragma unroll
      for (int q = 0; q < kWinRows; ++q) win_mac<kReal>(acc[q], g, w[q]);
#pragma unroll
      for (int q = 0; q < kWinRows - 1; ++q) w[q] = w[q + 1];
    }
  }
#pragma unroll
  for (int q = 0; q < kWinRows; ++q)
    if (j0 + q < J) win_finish(acc[q], meta[0], xs, tp, T, D, P, a0, jl0 + q, j0 + q, U, r, delta);
}

// One CTA = one tile of Qt output rows of decimation group g.  Shared memory:
// [input tile, de-interleaved: D x P float2][taps of every work set of the
// group, packed [T][nb]][ChanMeta per (work set, channel)].
template <int NBMAX, bool kTapsSmem, bool kWin>
__global__ void __launch_bounds__(kThreads, 3) poly_fp32_kernel(const __grid_constant__ PolyLaunch<NBMAX> L, int g) {
  extern __shared__ __align__(16) float2 xs[];
  // g < 0: one launch over several groups (small blocks), group =
  // fuse_map[blockIdx.y + (-g - 1)]
  const GroupDesc& G = L.groups[g >= 0 ? g : (int)L.fuse_map[(int)blockIdx.y - g - 1]];
  const int tile = blockIdx.x;
  if (tile >= G.ntiles) return;  // uniform over the CTA, before any barrier
  const int D = G.D, Qt = G.Qt, P = G.P;
  const int64_t row0 = (int64_t)tile * Qt;
  const int64_t sb = row0 * D + G.delta_min - G.tmax + 1;  // first staged input (block relative)
  const int len = Qt * D + G.delta_span + G.tmax - 1;
  float2* taps_s = xs + G.taps_off;
  ChanMeta* meta_s = reinterpret_cast<ChanMeta*>(xs + G.meta_off);
  const int nws = G.ws_end - G.ws_begin;

  // Stage the raw input span, de-interleaved by D, with asynchronous 8-byte
  // copies (every copy of the tile in flight at once).  Negative indices come
  // from the history (the H samples before the block); past the block end the
  // copy reads 0 bytes and zero-fills.
  if (L.block16 == nullptr) {
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
      const int64_t v = sb + t;
      const float2* src = L.block;
      uint32_t bytes = 0;
      if (v < 0) {
        const int64_t hv = v + L.H;
        if (hv >= 0) {
          src = L.hist + hv;
          bytes = 8;
        }
      } else if (v < L.N) {
        src = L.block + v;
        bytes = 8;
      }
      const int q = t / D;
      const uint32_t dst = (uint32_t)__cvta_generic_to_shared(xs + (t - q * D) * P + q);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
    }
  } else {
    // int16 front end: block samples are converted on the way in (the
    // history is already float)
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
      const int64_t v = sb + t;
      const int q = t / D;
      float2 x = make_float2(0.f, 0.f);
      if (v < 0) {
        const int64_t hv = v + L.H;
        if (hv >= 0) x = L.hist[hv];
      } else if (v < L.N) {
        const short2 s = L.block16[v];
        x = make_float2((float)s.x, (float)s.y);
      }
      xs[(t - q * D) * P + q] = x;
    }
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  // Stage the taps of every work set (when they fit) and the per-channel NCO
  // constants.
  for (int wi = 0; wi < nws; ++wi) {
    const WorkSet<NBMAX>& W = L.ws[G.ws_begin + wi];
    if constexpr (kTapsSmem) {
      const int cnt = W.T * ((W.nb + 1) & ~1);
      for (int i = threadIdx.x; i < cnt; i += blockDim.x) taps_s[W.soff + i] = __ldg(W.taps + i);
    }
    if (threadIdx.x < W.nb) {
      const int c = W.ch[threadIdx.x];
      const NcoConst nc = L.nco[c];
      ChanMeta m;
      m.omega64 = nc.omega64;
      m.wrap64 = nc.wrap64;
      m.fastmod = nc.fastmod;
      m.out = L.out[c];
      m.rollover = nc.rollover;
      m.base = L.nco_base[c];
      m.enabled = nc.enabled;
      m.pad_ = 0;
      meta_s[wi * NBMAX + threadIdx.x] = m;
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();

  if constexpr (kWin) {
    // single-channel work sets: items are (work set, block of kWinRows rows),
    // blocks fastest (Qt is a multiple of 32 kWinRows)
    const int nblk = Qt / kWinRows;
    const int nitems = nws * nblk;
    for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
      const int wq = it / nblk;
      const int jl0 = (it - wq * nblk) * kWinRows;
      const WorkSet<NBMAX>& W = L.ws[G.ws_begin + wq];
      const int64_t j0 = row0 + jl0;
      if (j0 >= W.J) continue;
      const int T = W.T;
      const int a0 = (W.delta - G.delta_min) + (G.tmax - T);
      const float2* tp = kTapsSmem ? taps_s + W.soff : W.taps;
      const ChanMeta* mt = meta_s + wq * NBMAX;
      if (G.real_taps)
        process_rows_win<true>(xs, tp, mt, T, D, P, a0, jl0, j0, W.J, W.U, W.r, W.delta);
      else
        process_rows_win<false>(xs, tp, mt, T, D, P, a0, jl0, j0, W.J, W.U, W.r, W.delta);
    }
    return;
  }

  // Items are (work set, row) with rows fastest; Qt is a multiple of 32 so a
  // warp never mixes work sets and every tap load is a broadcast.
  const int nitems = nws * Qt;
  for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
    const int wq = it / Qt;
    const int jl = it - wq * Qt;
    const WorkSet<NBMAX>& W = L.ws[G.ws_begin + wq];
    const int64_t j = row0 + jl;
    if (j >= W.J) continue;
    const int T = W.T;
    const int a0 = (W.delta - G.delta_min) + (G.tmax - T);
    const float2* tp = kTapsSmem ? taps_s + W.soff : W.taps;
    const ChanMeta* mt = meta_s + wq * NBMAX;
    switch (W.nb) {
      case 1: process_row<1>(xs, tp, mt, T, D, P, a0, jl, j, W.U, W.r, W.delta); break;
      case 2: if constexpr (NBMAX >= 2) process_row<2>(xs, tp, mt, T, D, P, a0, jl, j, W.U, W.r, W.delta); break;
      case 3: if constexpr (NBMAX >= 3) process_row<3>(xs, tp, mt, T, D, P, a0, jl, j, W.U, W.r, W.delta); break;
      case 4: if constexpr (NBMAX >= 4) process_row<4>(xs, tp, mt, T, D, P, a0, jl, j, W.U, W.r, W.delta); break;
      case 5: if constexpr (NBMAX >= 5) process_row<5>(xs, tp, mt, T, D, P, a0, jl, j, W.U, W.r, W.delta); break;
      case 6: if constexpr (NBMAX >= 6) process_row<6>(xs, tp, mt, T, D, P, a0, jl, j, W.U, W.r, W.delta); break;
      case 7: if constexpr (NBMAX >= 7) process_row<7>(xs, tp, mt, T, D, P, a0, jl, j, W.U, W.r, W.delta); break;
      default: if constexpr (NBMAX >= 8) process_row<NBMAX>(xs, tp, mt, T, D, P, a0, jl, j, W.U, W.r, W.delta); break;
    }
  }
}

// History after a block: the last H samples of [old history | block].
__global__ void hist_update_kernel(const float2* __restrict__ old_hist, const float2* __restrict__ block,
                                   const short2* __restrict__ block16, int64_t N, int H, float2* __restrict__ new_hist) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= H) return;
  const int64_t v = N + i;
  if (v < H) {
    new_hist[i] = old_hist[v];
  } else if (block16 != nullptr) {
    const short2 s = block16[v - H];
    new_hist[i] = make_float2((float)s.x, (float)s.y);
  } else {
    new_hist[i] = block[v - H];
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
NcoConst make_nco(uint32_t fs, int32_t f) {
  NcoConst n;
  std::memset(&n, 0, sizeof(n));
  if (f == 0 || fs == 0) return n;
  // rollover index: falcon_dsp_freq_shift.cc:216-229
  double r = (double)fs / (double)std::llabs((long long)f);
  while (r < 1e5) r *= 10.0;
  const uint32_t R = (uint32_t)std::round(r);
  int64_t fm = (int64_t)f % (int64_t)fs;
  if (fm < 0) fm += fs;
  const unsigned __int128 num = ((unsigned __int128)(uint64_t)fm << 64) + (fs / 2);
  const uint64_t w = (uint64_t)(num / fs);
  n.omega64 = w;
  n.wrap64 = (uint64_t)R * w;
  n.rollover = R;
  n.fastmod = R ? (~0ull / R + 1) : 0;
  n.enabled = (R != 0) ? 1u : 0u;
  return n;
}

PolyEngine::~PolyEngine() {
  if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
  if (graph_) cudaGraphDestroy(graph_);
  for (auto e : kprof_ev_)
    if (e) cudaEventDestroy(e);
  free_tc();
  for (auto& b : batches_) {
    if (b.d_taps) dfree(b.d_taps);
  }
  if (d_nco_) dfree(d_nco_);
  for (auto& h : d_hist_) {
    if (h) dfree(h);
  }
}

// ---------------------------------------------------------------------------
// device memory: the engine's own buffers come from its pool when it has one
// ---------------------------------------------------------------------------
cudaError_t PolyEngine::dalloc(void** p, size_t bytes) {
  if (!pool_) return cudaMalloc(p, bytes);
  *p = pool_->alloc(bytes);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}

void PolyEngine::dfree(void* p) {
  if (!p) return;
  if (pool_) pool_->release(p);
  else cudaFree(p);
}

DevPool::~DevPool() {
  if (base_) cudaFree(base_);
}

int DevPool::init(size_t bytes) {
  std::lock_guard<std::mutex> lk(mu_);
  if (base_ || bytes < RangePool::kAlign) return FDSP_ERR_INVALID_ARG;
  bytes &= ~(RangePool::kAlign - 1);
  const cudaError_t e = cudaMalloc(&base_, bytes);
  if (e != cudaSuccess) {
    base_ = nullptr;
    return cuda_status(e);
  }
  ranges_.init(bytes);
  return FDSP_OK;
}

void* DevPool::alloc(size_t bytes) {
  std::lock_guard<std::mutex> lk(mu_);
  if (!base_) return nullptr;
  const size_t off = ranges_.alloc(bytes);
  return off == RangePool::kNone ? nullptr : base_ + off;
}

void DevPool::release(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(mu_);
  if (base_) ranges_.release((size_t)(static_cast<char*>(p) - base_));
}

static int choose_qt(uint32_t D, int tmax) {
  // ~4K input samples per tile (three CTAs per SM), at least one warp of rows,
  // shared memory (tile + halo + offset spread, de-interleaved) under ~200 KB.
  int qt = (int)((4096 / D) & ~31u);
  if (qt < 32) qt = 32;
  auto bytes = [&](int q) {
    const int64_t len = (int64_t)q * D + 3LL * D + tmax;
    const int64_t P = len / D + 2;
    return (int64_t)D * P * 8;
  };
  while (qt > 32 && bytes(qt) > 200 * 1024) qt -= 32;
  if (bytes(qt) > 200 * 1024) return -1;
  return qt;
}

int PolyEngine::init(uint32_t fs, const fdsp_channel_cfg* ch, uint32_t nch, bool complex_taps, cudaStream_t stream) {
  if (nch == 0 || ch == nullptr) return FDSP_ERR_INVALID_ARG;
  if (nch > (uint32_t)kMaxChannels) return FDSP_ERR_UNSUPPORTED;
  fs_ = fs;
  complex_taps_ = complex_taps;
  chans_.resize(nch);
  cls_of_.assign(nch, -1);
  int tmax_all = 1;
  for (uint32_t c = 0; c < nch; ++c) {
    const fdsp_channel_cfg& cc = ch[c];
    if (cc.up_rate == 0 || cc.down_rate == 0 || cc.num_coeffs == 0 || cc.resample_filter_coeffs == nullptr)
      return FDSP_ERR_INVALID_ARG;
    EngineChannel& e = chans_[c];
    e.up = cc.up_rate;
    e.down = cc.down_rate;
    // polyphase_resampler.cc:131-157 -- pad to a multiple of up, transpose, flip
    uint32_t padded = cc.num_coeffs;
    while (padded % e.up) padded++;
    e.T = padded / e.up;
    e.flipped.assign((size_t)padded, make_float2(0.f, 0.f));
    for (uint32_t ph = 0; ph < e.up; ++ph) {
      for (uint32_t jj = 0; jj < e.T; ++jj) {
        const uint64_t src = (uint64_t)jj * e.up + ph;
        if (src < cc.num_coeffs) {
          const fdsp_cf32 v = cc.resample_filter_coeffs[src];
          e.flipped[(size_t)ph * e.T + (e.T - 1 - jj)] = make_float2(v.re, complex_taps ? v.im : 0.f);
        }
      }
    }
    e.shift_hz = (int32_t)cc.freq_shift_in_hz;  // initialize(uint32_t, int32_t) truncation
    e.nco = make_nco(fs, e.shift_hz);
    if (e.nco.enabled && e.T > e.nco.rollover) return FDSP_ERR_UNSUPPORTED;
    tmax_all = std::max(tmax_all, (int)e.T);
    // class by (up, down)
    int k = -1;
    for (size_t i = 0; i < classes_.size(); ++i) {
      if (classes_[i].up == e.up && classes_[i].down == e.down) k = (int)i;
    }
    if (k < 0) {
      EngineClass nc;
      nc.up = e.up;
      nc.down = e.down;
      nc.phase = 0;
      nc.xoffset = 0;
      nc.M = 0;
      classes_.push_back(nc);
      k = (int)classes_.size() - 1;
    }
    classes_[k].chans.push_back((int)c);
    cls_of_[c] = k;
  }
  H_ = tmax_all - 1;

  // NB: channels per tap batch (largest class decides, power of two <= 8)
  size_t maxcls = 1;
  for (auto& k : classes_) maxcls = std::max(maxcls, k.chans.size());
  nb_ = maxcls >= 8 ? 8 : maxcls >= 4 ? 4 : maxcls >= 2 ? 2 : 1;

  // decimation groups
  std::map<uint32_t, int> gidx;
  for (auto& k : classes_) {
    if (!gidx.count(k.down)) {
      gidx[k.down] = (int)groups_.size();
      EngineGroup g;
      g.D = k.down;
      g.Qt = 0;
      groups_.push_back(g);
    }
  }
  if (groups_.size() > (size_t)kMaxGroups) return FDSP_ERR_UNSUPPORTED;

  // batches: within a class, channels sorted by taps per phase (descending)
  for (size_t ki = 0; ki < classes_.size(); ++ki) {
    std::vector<int> cs = classes_[ki].chans;
    std::stable_sort(cs.begin(), cs.end(), [&](int a, int b) { return chans_[a].T > chans_[b].T; });
    for (size_t i = 0; i < cs.size(); i += nb_) {
      EngineBatch bt;
      bt.cls = (int)ki;
      bt.group = gidx[classes_[ki].down];
      bt.chans.assign(cs.begin() + i, cs.begin() + std::min(cs.size(), i + nb_));
      bt.T = (int)chans_[bt.chans[0]].T;
      bt.d_taps = nullptr;
      groups_[bt.group].batches.push_back((int)batches_.size());
      batches_.push_back(bt);
    }
  }
  for (size_t gi = 0; gi < groups_.size(); ++gi) group_of_d_[groups_[gi].D] = (int)gi;
  for (auto& g : groups_) {
    int tmax = 1;
    for (int b : g.batches) tmax = std::max(tmax, batches_[b].T);
    g.Qt = choose_qt(g.D, tmax);
    if (g.Qt < 0) return FDSP_ERR_UNSUPPORTED;
    g.Qt_default = g.Qt;
    // sliding-window form: every batch of the group holds one channel and
    // the filter is long enough for row blocks to pay; tiles of a multiple
    // of 32 x kWinRows rows within the same shared-memory budget
    bool single = true, real = true;
    for (int b : g.batches) {
      single = single && batches_[b].chans.size() == 1;
      for (int c : batches_[b].chans) {
        real = real && !chans_[c].nco.enabled;
        for (const float2& h : chans_[c].flipped) real = real && h.y == 0.f;
      }
    }
    const int unit = 32 * kWinRows;
    if (single && tmax >= 16) {
      auto bytes = [&](int q) {
        const int64_t len = (int64_t)q * g.D + 3LL * g.D + tmax;
        return (int64_t)g.D * (len / g.D + 2) * 8;
      };
      // enough row blocks for every thread of the CTA: kThreads blocks of
      // kWinRows rows spread over the group's work sets (U output phases each
      // class), as far as shared memory allows
      size_t nws = 0;
      for (int b : g.batches) nws += classes_[batches_[b].cls].up;
      const int want = (int)((kThreads + std::max<size_t>(nws, 1) - 1) / std::max<size_t>(nws, 1)) * kWinRows;
      int q = std::max(unit, (want + unit - 1) / unit * unit);
      while (q > unit && bytes(q) > 200 * 1024) q -= unit;
      if (bytes(q) <= 200 * 1024) {
        g.win = 1;
        g.real_taps = real ? 1 : 0;
        g.Qt_win = q;
      }
    }
  }

  // modulated, padded taps of every batch: [up][T][NB]
  for (auto& bt : batches_) {
    const uint32_t U = classes_[bt.cls].up;
    const size_t nb = (bt.chans.size() + 1) & ~(size_t)1;  // tap rows padded to an even width
    std::vector<float2> host((size_t)U * bt.T * nb, make_float2(0.f, 0.f));
    for (size_t n = 0; n < bt.chans.size(); ++n) {
      const EngineChannel& e = chans_[bt.chans[n]];
      const int pad = bt.T - (int)e.T;
      int64_t fm = 0;
      if (e.nco.enabled) {
        fm = (int64_t)e.shift_hz % (int64_t)fs;
        if (fm < 0) fm += fs;
      }
      for (uint32_t ph = 0; ph < U; ++ph) {
        for (int k = pad; k < bt.T; ++k) {
          const float2 h = e.flipped[(size_t)ph * e.T + (k - pad)];
          double gr = h.x, gi = h.y;
          if (e.nco.enabled) {
            // e^{j w k} with w k reduced exactly: 2 pi ((f mod fs) k mod fs) / fs
            const uint64_t red = (uint64_t)(((unsigned __int128)(uint64_t)fm * (uint64_t)k) % fs);
            const double ang = 2.0 * M_PI * (double)red / (double)fs;
            const double c = std::cos(ang), s = std::sin(ang);
            gr = (double)h.x * c - (double)h.y * s;
            gi = (double)h.x * s + (double)h.y * c;
          }
          host[((size_t)ph * bt.T + k) * nb + n] = make_float2((float)gr, (float)gi);
        }
      }
    }
    cudaError_t e = dalloc(reinterpret_cast<void**>(&bt.d_taps), host.size() * sizeof(float2));
    if (e != cudaSuccess) return cuda_status(e);
    e = cudaMemcpy(bt.d_taps, host.data(), host.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_status(e);
  }

  std::vector<NcoConst> nco(nch);
  for (uint32_t c = 0; c < nch; ++c) nco[c] = chans_[c].nco;
  cudaError_t e = dalloc(reinterpret_cast<void**>(&d_nco_), nch * sizeof(NcoConst));
  if (e != cudaSuccess) return cuda_status(e);
  e = cudaMemcpy(d_nco_, nco.data(), nch * sizeof(NcoConst), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_status(e);
  if (H_ > 0) {
    for (auto& h : d_hist_) {
      e = dalloc(reinterpret_cast<void**>(&h), (size_t)H_ * sizeof(float2));
      if (e != cudaSuccess) return cuda_status(e);
      e = stream ? cudaMemsetAsync(h, 0, (size_t)H_ * sizeof(float2), stream)
                 : cudaMemset(h, 0, (size_t)H_ * sizeof(float2));
      if (e != cudaSuccess) return cuda_status(e);
    }
  }
  // with a stream the engine's applies on it follow the fill; without one
  // every later stream must see it
  if (!stream) {
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_status(e);
  }
  return FDSP_OK;
}

// Outputs the reference loop emits for n inputs from (phase, xoffset):
// the m >= 0 with xoffset + floor((phase + m*down)/up) < n.
uint64_t polyphase_out_count(uint32_t up, uint32_t down, uint32_t phase, uint64_t xoffset, uint64_t n) {
  if (xoffset >= n) return 0;
  const unsigned __int128 lim = (unsigned __int128)up * (n - xoffset);  // > phase
  return (uint64_t)((lim - phase + down - 1) / down);
}

// State after M outputs of an apply of n inputs (polyphase_resampler.cc:303-312).
void polyphase_advance(uint32_t up, uint32_t down, uint32_t& phase, uint64_t& xoffset, uint64_t n, uint64_t M) {
  if (xoffset >= n) {
    xoffset -= n;
    return;
  }
  const unsigned __int128 t = (unsigned __int128)phase + (unsigned __int128)M * down;
  const uint64_t x_new = xoffset + (uint64_t)(t / up);
  phase = (uint32_t)(t % up);
  xoffset = x_new - n;
}

static uint64_t class_out_count(const EngineClass& k, uint64_t n) {
  return polyphase_out_count(k.up, k.down, k.phase, k.xoffset, n);
}

int PolyEngine::out_counts(uint64_t n_in, uint64_t* n_out) const {
  if (!n_out) return FDSP_ERR_INVALID_ARG;
  for (size_t c = 0; c < chans_.size(); ++c) n_out[c] = class_out_count(classes_[cls_of_[c]], n_in);
  return FDSP_OK;
}

int PolyEngine::set_precision(int mode) {
  if (mode == precision_) return FDSP_OK;
  if (mode == FDSP_PRECISION_FP32) {
    precision_ = mode;
    return FDSP_OK;
  }
  if (mode != FDSP_PRECISION_FP16X3 && mode != FDSP_PRECISION_BF16X3) return FDSP_ERR_INVALID_ARG;
  const int st = build_tc(mode == FDSP_PRECISION_FP16X3 ? 0 : 1);
  if (st != FDSP_OK) return st;
  precision_ = mode;
  return FDSP_OK;
}

void PolyEngine::notify_done(const std::vector<int>& egroups, cudaStream_t stream) {
  if (!done_fn_ || egroups.empty()) return;
  std::vector<int> ch;
  for (int eg : egroups)
    for (const EngineClass& k : classes_)
      if (k.down == groups_[eg].D && k.M > 0) ch.insert(ch.end(), k.chans.begin(), k.chans.end());
  if (!ch.empty()) done_fn_(done_ctx_, ch.data(), (int)ch.size(), stream);
}

void PolyEngine::set_graph(bool on) {
  use_graph_ = on;
  graph_replays_ = 0;
  if (!on) {
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    graph_exec_ = nullptr;
    if (graph_) cudaGraphDestroy(graph_);
    graph_ = nullptr;
    knodes_.clear();
  }
}

void PolyEngine::set_profile(bool on) {
  kprof_ = on;
  kprof_used_ = 0;
}

cudaEvent_t PolyEngine::kprof_event() {
  if (kprof_used_ == kprof_ev_.size()) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    kprof_ev_.push_back(e);
  }
  return kprof_ev_[kprof_used_++];
}

int PolyEngine::read_profile(double* ms, uint32_t* launches) {
  if (!ms || !launches) return FDSP_ERR_INVALID_ARG;
  *ms = 0.0;
  *launches = 0;
  for (size_t i = 0; i + 1 < kprof_used_; i += 2) {
    if (!kprof_ev_[i] || !kprof_ev_[i + 1]) continue;
    FDSP_TRY(cuda_status(cudaEventSynchronize(kprof_ev_[i + 1])));
    float t = 0.f;
    FDSP_TRY(cuda_status(cudaEventElapsedTime(&t, kprof_ev_[i], kprof_ev_[i + 1])));
    *ms += t;
    ++*launches;
  }
  return FDSP_OK;
}

bool PolyEngine::use_tc_for(int eg) const {
  if (precision_ == FDSP_PRECISION_FP32 || force_ == 0) return false;
  return force_ == 1 || groups_[eg].use_tc != 0;
}

int PolyEngine::autotune(uint64_t n, cudaStream_t stream) {
  if (n == 0 || n >= (1ull << 31)) return FDSP_ERR_INVALID_ARG;
  const size_t ng = groups_.size();
  float2* d_in = nullptr;
  std::vector<float2*> outs(chans_.size(), nullptr);
  int st = cuda_status(cudaMalloc(&d_in, n * sizeof(float2)));
  if (st == FDSP_OK) st = cuda_status(cudaMemsetAsync(d_in, 0, n * sizeof(float2), stream));
  for (size_t c = 0; c < chans_.size() && st == FDSP_OK; ++c) {
    const uint64_t cap = (n * chans_[c].up + chans_[c].down - 1) / chans_[c].down + 2;
    st = cuda_status(cudaMalloc(&outs[c], cap * sizeof(float2)));
  }
  prof_ev_.assign(2 * ng, nullptr);
  prof_hit_.assign(ng, 0);
  for (size_t i = 0; i < prof_ev_.size() && st == FDSP_OK; ++i) st = cuda_status(cudaEventCreate(&prof_ev_[i]));
  std::vector<uint64_t> counts(chans_.size());
  // minimum over 3 timed applies (after one untimed) of each group's time
  auto run = [&](int force, std::vector<float>& t) -> int {
    t.assign(ng, 3.4e38f);
    reset();
    force_ = force;
    for (int rep = 0; rep < 4; ++rep) {
      std::fill(prof_hit_.begin(), prof_hit_.end(), 0);
      int s2 = apply(d_in, n, outs.data(), nullptr, counts.data(), stream);
      if (s2 == FDSP_OK) s2 = cuda_status(cudaStreamSynchronize(stream));
      if (s2 != FDSP_OK) return s2;
      if (rep == 0) continue;
      for (size_t g = 0; g < ng; ++g) {
        if (!prof_hit_[g]) continue;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, prof_ev_[2 * g], prof_ev_[2 * g + 1]) == cudaSuccess) t[g] = std::min(t[g], ms);
      }
    }
    return FDSP_OK;
  };
  std::vector<float> best(ng, 3.4e38f), t;
  std::vector<int> best_qt(ng);
  for (size_t g = 0; g < ng; ++g) best_qt[g] = groups_[g].Qt_default;
  // FP32 tile height: the default, half, double and four times where shared memory allows
  // (large decimations start from small default tiles, where staging the
  // input span and taps dominates: four times the default is tried too)
  const int factor_num[4] = {1, 1, 2, 4}, factor_den[4] = {1, 2, 1, 1};
  for (int ci = 0; ci < 4 && st == FDSP_OK; ++ci) {
    std::vector<char> valid(ng, 0);
    for (size_t g = 0; g < ng; ++g) {
      EngineGroup& eg = groups_[g];
      const int q = (eg.Qt_default * factor_num[ci] / factor_den[ci]) & ~31;
      const int64_t len = (int64_t)q * eg.D + 3LL * eg.D + 64;
      valid[g] = q >= 32 && (int64_t)eg.D * (len / eg.D + 2) * 8 <= 200 * 1024;
      eg.Qt = valid[g] ? q : eg.Qt_default;
    }
    st = run(0, t);
    for (size_t g = 0; g < ng && st == FDSP_OK; ++g)
      if (valid[g] && t[g] < best[g]) {
        best[g] = t[g];
        best_qt[g] = groups_[g].Qt;
      }
  }
  for (size_t g = 0; g < ng; ++g) groups_[g].Qt = best_qt[g];
  force_ = -1;
  for (auto ev : prof_ev_)
    if (ev) cudaEventDestroy(ev);
  prof_ev_.clear();
  cudaStreamSynchronize(stream);
  if (d_in) cudaFree(d_in);
  for (auto p : outs)
    if (p) cudaFree(p);
  reset();
  return st;
}

void PolyEngine::reset() {
  if (d_err_) cudaMemset(d_err_, 0, sizeof(int));
  for (auto& k : classes_) {
    k.phase = 0;
    k.xoffset = 0;
  }
  abs0_ = 0;
  cudaDeviceSynchronize();
  for (auto& h : d_hist_) {
    if (h) cudaMemset(h, 0, (size_t)H_ * sizeof(float2));
  }
  hist_cur_ = 0;
  cudaDeviceSynchronize();
}

template <int NB>
int PolyEngine::launch(const float2* d_in, uint64_t n, float2* const* out, cudaStream_t stream) {
  static thread_local PolyLaunch<NB> L;  // ~20 KB: keep it off the stack
  std::memset(&L, 0, sizeof(L));
  if (num_sms_ == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev);
    if (num_sms_ <= 0) num_sms_ = 1;
  }
  L.block = in16_ ? nullptr : d_in;
  L.block16 = in16_;
  L.hist = d_hist_[hist_cur_];
  L.N = (int64_t)n;
  L.H = H_;
  L.nco = d_nco_;
  for (size_t c = 0; c < chans_.size(); ++c) {
    L.out[c] = out[c];
    const uint32_t R = chans_[c].nco.rollover;
    L.nco_base[c] = R ? (uint32_t)(abs0_ % R) : 0u;
  }
  int ng = 0, nws = 0, max_tiles = 0;
  size_t smem_max = 0;
  for (auto& g : groups_) {
    GroupDesc& gd = L.groups[ng];
    gd.D = (int32_t)g.D;
    gd.ws_begin = nws;
    int dmin = INT32_MAX, dmax = INT32_MIN, tmax = 1;
    int64_t rows = 0;
    for (int bi : g.batches) {
      const EngineBatch& bt = batches_[bi];
      const EngineClass& k = classes_[bt.cls];
      const uint32_t U = k.up;
      for (uint32_t r = 0; r < U; ++r) {
        if (k.M <= r) continue;
        const uint64_t J = (k.M - r + U - 1) / U;
        const uint64_t t = (uint64_t)k.phase + (uint64_t)r * g.D;
        const uint64_t delta = k.xoffset + t / U;
        const uint32_t phi = (uint32_t)(t % U);
        if (nws >= kMaxWorkSets) return FDSP_ERR_UNSUPPORTED;
        WorkSet<NB>& W = L.ws[nws++];
        W.taps = bt.d_taps + (size_t)phi * bt.T * ((bt.chans.size() + 1) & ~(size_t)1);
        W.T = bt.T;
        W.delta = (int32_t)delta;
        W.J = (int32_t)J;
        W.U = (int32_t)U;
        W.r = (int32_t)r;
        W.nb = (int32_t)bt.chans.size();
        for (size_t i = 0; i < bt.chans.size(); ++i) W.ch[i] = (int16_t)bt.chans[i];
        dmin = std::min(dmin, (int)delta);
        dmax = std::max(dmax, (int)delta);
        tmax = std::max(tmax, bt.T);
        rows = std::max<int64_t>(rows, (int64_t)J);
      }
    }
    gd.ws_end = nws;
    if (gd.ws_end == gd.ws_begin) continue;
    gd.tmax = tmax;
    gd.delta_min = dmin;
    gd.delta_span = dmax - dmin;
    // the sliding-window form where it fills the GPU with its larger tiles
    // (short blocks keep the per-row form, whose smaller tiles spread wider)
    const bool win = g.win && rows >= (int64_t)g.Qt_win * num_sms_;
    const int Qt = win ? g.Qt_win : g.Qt;
    gd.Qt = Qt;
    gd.win = win ? 1 : 0;
    gd.real_taps = g.real_taps;
    gd.ntiles = (int32_t)((rows + Qt - 1) / Qt);
    const int64_t len = (int64_t)Qt * g.D + gd.delta_span + tmax - 1;
    int64_t P = (len + g.D - 1) / g.D;
    if ((P & 1) == 0) P++;  // odd pitch: the staging scatter spreads over banks
    gd.P = (int32_t)P;
    // shared-memory layout: input tile | taps of each work set | channel constants
    int64_t off = ((int64_t)g.D * P + 1) & ~1LL;  // float2 units, 16-byte aligned
    gd.taps_off = (int32_t)off;
    int64_t toff = 0;
    for (int wi = gd.ws_begin; wi < gd.ws_end; ++wi) {
      L.ws[wi].soff = (int32_t)toff;
      toff += (int64_t)L.ws[wi].T * ((L.ws[wi].nb + 1) & ~1);
    }
    const int64_t meta_bytes = (int64_t)(gd.ws_end - gd.ws_begin) * NB * 48;
    // taps go to shared memory unless they would push the CTA past ~150 KB
    // (long filters of many phases); those groups read taps through L1
    gd.taps_smem = ((off + toff) * (int64_t)sizeof(float2) + meta_bytes <= 150 * 1024) ? 1 : 0;
    if (gd.taps_smem) off += toff;
    gd.meta_off = (int32_t)off;
    const int64_t bytes = off * (int64_t)sizeof(float2) + meta_bytes;
    if (bytes > 227 * 1024) return FDSP_ERR_UNSUPPORTED;
    gd.smem_bytes = (int32_t)bytes;
    smem_max = std::max(smem_max, (size_t)bytes);
    max_tiles = std::max(max_tiles, gd.ntiles);
    ng++;
  }
  L.ngroups = ng;
  L.max_tiles = max_tiles;
  L.nws = nws;
  if (num_sms_ == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev);
    if (num_sms_ <= 0) num_sms_ = 1;
  }
  // tensor-core groups: one prep launch and one filter-bank launch for all of
  // them; groups the tensor-core plan cannot hold stay on the FP32 kernel
  std::vector<char> on_tc(ng, 0);
  {
    std::vector<int> tcg, fallback;
    for (int gi = 0; gi < ng; ++gi) {
      const int eg = group_of_d_[L.groups[gi].D];
      if (L.groups[gi].ntiles > 0 && use_tc_for(eg)) tcg.push_back(eg);
    }
    if (!tcg.empty()) {
      FDSP_TRY(launch_tc(d_in, n, out, tcg, fallback, stream));
      for (int gi = 0; gi < ng; ++gi) {
        const int eg = group_of_d_[L.groups[gi].D];
        on_tc[gi] = std::find(tcg.begin(), tcg.end(), eg) != tcg.end() &&
                    std::find(fallback.begin(), fallback.end(), eg) == fallback.end();
      }
    }
  }
  // small blocks: the FP32 groups in at most four launches (by way of
  // staging taps and tile form; grid = tiles x groups, shared memory of the
  // largest group of the launch); the per-launch cost then stops dominating
  // short blocks
  {
    int nfp = 0;
    int64_t tiles = 0;
    for (int gi = 0; gi < ng; ++gi) {
      if (on_tc[gi] || L.groups[gi].ntiles <= 0) continue;
      ++nfp;
      tiles += L.groups[gi].ntiles;
    }
    if (nfp > 1 && prof_ev_.empty() && tiles <= 3LL * num_sms_) {
      int nm = 0;
      for (int pass = 0; pass < 4; ++pass) {  // (taps in shared memory?, sliding window?)
        const int first = nm;
        size_t fsmem = 0;
        int ftiles = 0;
        const int want_smem = (pass & 1) == 0 ? 1 : 0, want_win = pass >> 1;
        for (int gi = 0; gi < ng; ++gi) {
          const GroupDesc& gd = L.groups[gi];
          if (on_tc[gi] || gd.taps_smem != want_smem || gd.win != want_win || gd.ntiles <= 0) continue;
          L.fuse_map[nm++] = (int8_t)gi;
          fsmem = std::max(fsmem, (size_t)gd.smem_bytes);
          ftiles = std::max(ftiles, (int)gd.ntiles);
        }
        if (nm == first) continue;
        auto kern = want_win ? (want_smem ? poly_fp32_kernel<NB, true, true> : poly_fp32_kernel<NB, false, true>)
                             : (want_smem ? poly_fp32_kernel<NB, true, false> : poly_fp32_kernel<NB, false, false>);
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem);
        if (e != cudaSuccess) return cuda_status(e);
        if (kprof_) cudaEventRecord(kprof_event(), stream);
        int garg = -1 - first;
        e = klaunch(reinterpret_cast<const void*>(kern), dim3((unsigned)ftiles, (unsigned)(nm - first)),
                    dim3(kThreads), fsmem, stream, L, garg);
        if (kprof_) cudaEventRecord(kprof_event(), stream);
        if (e != cudaSuccess) return cuda_status(e);
        launches_last_++;
        if (done_fn_) {
          std::vector<int> egs;
          for (int i = first; i < nm; ++i) egs.push_back(group_of_d_[L.groups[L.fuse_map[i]].D]);
          notify_done(egs, stream);
        }
      }
      for (int gi = 0; gi < ng; ++gi) on_tc[gi] = 1;  // nothing left for the per-group loop
    }
  }
  // one launch per remaining FP32 group, each with its own tile shape and
  // shared-memory size (all on `stream`, so they run back to back)
  for (int gi = 0; gi < ng; ++gi) {
    const GroupDesc& gd = L.groups[gi];
    if (gd.ntiles <= 0 || on_tc[gi]) continue;
    const int eg = group_of_d_[gd.D];
    if (!prof_ev_.empty()) {
      cudaEventRecord(prof_ev_[2 * eg], stream);
      prof_hit_[eg] = 1;
    }
    const size_t smem = (size_t)gd.smem_bytes;
    auto kern = gd.win ? (gd.taps_smem ? poly_fp32_kernel<NB, true, true> : poly_fp32_kernel<NB, false, true>)
                       : (gd.taps_smem ? poly_fp32_kernel<NB, true, false> : poly_fp32_kernel<NB, false, false>);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e);
    if (kprof_) cudaEventRecord(kprof_event(), stream);
    int garg = gi;
    e = klaunch(reinterpret_cast<const void*>(kern), dim3((unsigned)gd.ntiles), dim3(kThreads), smem, stream, L, garg);
    if (kprof_) cudaEventRecord(kprof_event(), stream);
    if (e != cudaSuccess) return cuda_status(e);
    launches_last_++;
    if (!prof_ev_.empty()) cudaEventRecord(prof_ev_[2 * eg + 1], stream);
    if (done_fn_) notify_done(std::vector<int>(1, eg), stream);
  }
  if (H_ > 0) {
    const float2* a0 = d_hist_[hist_cur_];
    const float2* a1 = in16_ ? nullptr : d_in;
    const short2* a2 = in16_;
    int64_t a3 = (int64_t)n;
    int a4 = H_;
    float2* a5 = d_hist_[hist_cur_ ^ 1];
    cudaError_t e = klaunch(reinterpret_cast<const void*>(hist_update_kernel), dim3((unsigned)((H_ + 255) / 256)),
                            dim3(256), 0, stream, a0, a1, a2, a3, a4, a5);
    if (e != cudaSuccess) return cuda_status(e);
    hist_cur_ ^= 1;
    launches_last_++;
  }
  return FDSP_OK;
}

int PolyEngine::apply_ci16(const int16_t* d_in, uint64_t n, float2* const* out, const uint64_t* cap,
                           uint64_t* n_out, cudaStream_t stream) {
  in16_ = reinterpret_cast<const short2*>(d_in);
  // the float pointer is only checked for NULL; every kernel reads in16_
  const int st = apply(reinterpret_cast<const float2*>(d_in), n, out, cap, n_out, stream);
  in16_ = nullptr;
  return st;
}

int PolyEngine::apply(const float2* d_in, uint64_t n, float2* const* out, const uint64_t* cap, uint64_t* n_out,
                      cudaStream_t stream) {
  launches_last_ = 0;
  tc_groups_last_ = 0;
  if (n > 0 && d_in == nullptr) return FDSP_ERR_INVALID_ARG;
  if (n >= (1ull << 31)) return FDSP_ERR_UNSUPPORTED;
  for (auto& k : classes_) k.M = class_out_count(k, n);
  for (size_t c = 0; c < chans_.size(); ++c) {
    const uint64_t M = classes_[cls_of_[c]].M;
    if (n_out) n_out[c] = M;
    if (M > 0 && (out == nullptr || out[c] == nullptr)) return FDSP_ERR_INVALID_ARG;
    if (cap && cap[c] < M) return FDSP_ERR_CAPACITY;
  }
  if (n == 0) return FDSP_OK;
  cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
  const bool graph = use_graph_ && !kprof_ && !done_fn_ && stream != nullptr &&
                     cudaStreamIsCapturing(stream, &capturing) == cudaSuccess &&
                     capturing == cudaStreamCaptureStatusNone;
  auto run = [&]() {
    switch (nb_) {
      case 1: return launch<1>(d_in, n, out, stream);
      case 2: return launch<2>(d_in, n, out, stream);
      case 4: return launch<4>(d_in, n, out, stream);
      default: return launch<8>(d_in, n, out, stream);
    }
  };
  int st = FDSP_OK;
  bool done = false;
  if (graph && graph_exec_ && !knodes_.empty()) {
    // replay: the same launch sequence with this apply's arguments written
    // into the recorded kernel nodes (no capture)
    const int hist_save = hist_cur_;
    kmode_ = 2;
    kcur_ = 0;
    kshape_ok_ = true;
    st = run();
    kmode_ = 0;
    if (st != FDSP_OK) return st;
    if (kshape_ok_ && kcur_ == knodes_.size()) {
      const cudaError_t e = cudaGraphLaunch(graph_exec_, stream);
      if (e != cudaSuccess) return cuda_status(e);
      graph_replays_++;
      done = true;
    } else {  // another launch sequence: capture it afresh
      hist_cur_ = hist_save;
      launches_last_ = 0;
      tc_groups_last_ = 0;
    }
  }
  if (!done && graph) {
    cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return cuda_status(e);
    kmode_ = 1;
    knodes_.clear();
    kfuncs_.clear();
    kshape_ok_ = true;
    st = run();
    kmode_ = 0;
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(stream, &g);
    if (st == FDSP_OK && e != cudaSuccess) st = cuda_status(e);
    if (st == FDSP_OK && kshape_ok_) {
      // a fresh executable graph whose kernel nodes the next applies update
      if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
      graph_exec_ = nullptr;
      if (graph_) cudaGraphDestroy(graph_);
      graph_ = g;
      g = nullptr;
      e = cudaGraphInstantiate(&graph_exec_, graph_, 0);
      if (e != cudaSuccess) {
        graph_exec_ = nullptr;
        knodes_.clear();
        st = cuda_status(e);
      }
    } else if (st == FDSP_OK) {
      // nodes not recorded: update the executable graph from each capture
      knodes_.clear();
      if (graph_exec_) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(graph_exec_, g, &info) != cudaSuccess) {
          cudaGetLastError();
          cudaGraphExecDestroy(graph_exec_);
          graph_exec_ = nullptr;
        }
      }
      if (!graph_exec_) {
        e = cudaGraphInstantiate(&graph_exec_, g, 0);
        if (e != cudaSuccess) {
          graph_exec_ = nullptr;
          st = cuda_status(e);
        }
      }
    }
    if (st == FDSP_OK) {
      e = cudaGraphLaunch(graph_exec_, stream);
      if (e != cudaSuccess) st = cuda_status(e);
      else graph_replays_++;
    }
    if (g) cudaGraphDestroy(g);
    done = true;
  }
  if (!done) st = run();
  if (st != FDSP_OK) return st;
  // advance the streaming state (polyphase_resampler.cc:303-312)
  for (auto& k : classes_) polyphase_advance(k.up, k.down, k.phase, k.xoffset, n, k.M);
  abs0_ += n;
  return FDSP_OK;
}

}  // namespace fdsp
