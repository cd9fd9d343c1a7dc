// Output-side NCO rotation shared by the FP32 and tensor-core engines.
//
// Every output of a channel is the filter sum over a window of raw samples
// starting at block-relative index w0, rotated by the channel's NCO phase at
// w0: angle = 2 pi f/fs * ((n0 + w0) mod R), the reference's counter rule
// (falcon_dsp_freq_shift.cc:164-192).  The common case is computed branch
// free so the outputs of a chunk interleave; windows that straddle the
// counter rollover (and counters beyond 32 bits) return false and go through
// rotate_exact, which splits the window sum at the rollover.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fdsp {

// Per (work set, channel) constants, staged in shared memory by each CTA.
struct OutMeta {
  uint64_t omega64;   // turns per sample, 2^-64 units
  uint64_t wrap64;    // R * omega64 mod 2^64
  uint64_t fastmod;   // ceil(2^64 / R)
  float2* out;        // output base of the channel for this launch
  uint32_t rollover;  // R
  uint32_t base;      // counter of block sample 0 (mod R)
  uint32_t enabled;   // 0: no shift (phasor 1)
  uint32_t pad_;
};

__device__ __forceinline__ float2 cmul_nco(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// e^{j 2 pi t} for t in 2^-64 turns; the SFU argument lies in [-pi, pi),
// where __sincosf is accurate to ~4e-7 absolute.
__device__ __forceinline__ float2 phasor64_sfu(uint64_t turns64) {
  const int32_t top = (int32_t)(turns64 >> 32);
  const float a = (float)top * 1.4629180792671596e-09f;  // 2 pi / 2^32
  float s, c;
  __sincosf(a, &s, &c);
  return make_float2(c, s);
}

// Fast path: y <- y * e^{j phase(w0)}.  Returns false (y untouched in that
// case is not guaranteed) when the exact path is needed: the window of T
// samples crosses the rollover, or the counter argument leaves 32 bits.
__device__ __forceinline__ bool rotate_fast(const OutMeta& cm, int64_t w0, int T, float2& y) {
  const uint32_t R = cm.rollover;
  const int64_t pv = (int64_t)cm.base + w0;
  const bool neg = pv < 0;
  const uint32_t p_pos = (uint32_t)__umul64hi(cm.fastmod * (uint64_t)(uint32_t)pv, (uint64_t)R);
  const uint32_t p_neg = (uint32_t)(pv + (int64_t)R);
  const uint32_t p = neg ? p_neg : p_pos;
  const bool in32 = neg || (pv >> 32) == 0;
  const bool ok = !cm.enabled || (in32 && (uint64_t)p + (uint64_t)T - 1 < (uint64_t)R);
  float2 e = phasor64_sfu((uint64_t)p * cm.omega64);
  e = cm.enabled ? e : make_float2(1.f, 0.f);
  y = cmul_nco(y, e);
  return ok;
}

// Exact path, in two steps around the caller's partial sum: rotate_prep
// reduces the counter with a full 64-bit modulo and tells whether the window
// crosses the rollover (then the caller sums taps k0..T-1 into B); rotate_apply
// combines y (the unrotated full window sum) with B.
struct ExactRot {
  float2 e, e2;   // phasors before / after the rollover
  int k0;         // first tap past the rollover
  bool straddle;
  bool enabled;
};

__device__ __forceinline__ ExactRot rotate_prep(const OutMeta& cm, int64_t w0, int T) {
  ExactRot r;
  r.enabled = cm.enabled != 0;
  r.straddle = false;
  r.k0 = T;
  r.e = make_float2(1.f, 0.f);
  r.e2 = r.e;
  if (!r.enabled) return r;
  const uint32_t R = cm.rollover;
  const int64_t pv = (int64_t)cm.base + w0;
  const uint32_t p = pv < 0 ? (uint32_t)(pv + (int64_t)R) : (uint32_t)((uint64_t)pv % R);
  const uint64_t ph = (uint64_t)p * cm.omega64;
  r.e = phasor64_sfu(ph);
  if ((uint64_t)p + (uint64_t)T - 1 >= (uint64_t)R) {
    // samples from k0 on use angle w (p + k - R) instead of w (p + k)
    r.straddle = true;
    r.k0 = (int)(R - p);
    r.e2 = phasor64_sfu(ph - cm.wrap64);
  }
  return r;
}

__device__ __forceinline__ float2 rotate_apply(const ExactRot& r, float2 y, float2 B) {
  if (!r.enabled) return y;
  if (!r.straddle) return cmul_nco(y, r.e);
  const float2 ya = cmul_nco(make_float2(y.x - B.x, y.y - B.y), r.e), yb = cmul_nco(B, r.e2);
  return make_float2(ya.x + yb.x, ya.y + yb.y);
}

}  // namespace fdsp
