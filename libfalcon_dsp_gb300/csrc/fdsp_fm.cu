// FM mono demodulator on the GPU: falcon_dsp_fm_demodulator_cuda
// (hdr/signals/falcon_dsp_fm_demod_cuda.h:83-104,
// src/signals/falcon_dsp_fm_demod_cuda.cu) with every stage on the device.
//
//   input (fs) -> channelizer, one channel: NCO to the station, resample to
//   228 kS/s with the predefined REMEZ-64 filter
//   -> polar discriminator + de-emphasis (one-pole IIR), one fused kernel
//   -> mono decimator to 45.6 kS/s (REMEZ-64)
//   -> max |x| over the call, x * (10000 / max) truncated to int16.
//
// The reference runs the last four stages on the CPU (demod_mono,
// src/signals/falcon_dsp_fm_demod_cuda.cu:215-262).  Streaming state (the
// discriminator's last sample, the de-emphasis output, the resamplers'
// history and phase, the NCO counter) stays on the device between calls.
#include <cstring>
#include <new>
#include <vector>

#include "fdsp_internal.h"

namespace fdsp {
namespace {

constexpr int kFmThreads = 128;
constexpr int kFmPer = 32;                        // outputs per thread
constexpr int kFmTile = kFmThreads * kFmPer;      // outputs per block
// The de-emphasis recurrence y[n] = b0 x[n] + c y[n-1] (0 < c < 0.94) forgets
// its start: after W steps a different start state has shrunk by c^W <
// 1e-14, far below FP32 resolution.  A thread therefore starts W samples
// before its first output from y = 0 (or, within W of the call start, from
// the carried y[-1] at the call start, which is exact).
constexpr int kFmWarm = 512;

struct FmLaunch {
  const float2* iso;    // channelized samples of this call
  int64_t n_pol;        // discriminator outputs of this call
  int s0;               // 1 on the very first call (its first sample only seeds x[-1])
  const float2* state;  // [0] = x[-1] of the discriminator, [1].x = y[-1] of the de-emphasis
  float b0, c;          // y = b0 x - a1 y[-1], c = -a1
  float2* out;          // (y, 0): the mono decimator's complex input
};

// atan2 of a * conj(b), with the polar discriminator's arithmetic
__device__ __forceinline__ float polar_of(float2 a, float2 b) {
  const float re = a.x * b.x + a.y * b.y;
  const float im = a.y * b.x - a.x * b.y;
  return atan2f(im, re);
}

// one de-emphasis step rounded like the reference's complex<float> IIR
// (products rounded, then the difference): fl(fl(x b0) - fl(y a1))
__device__ __forceinline__ float deemph_step(float x, float y, float b0, float c) {
  return __fadd_rn(__fmul_rn(x, b0), __fmul_rn(y, c));
}

__global__ void __launch_bounds__(kFmThreads) fm_polar_deemph_kernel(const FmLaunch L) {
  __shared__ float pol[kFmWarm + kFmTile];
  __shared__ float res[kFmTile];
  const int64_t t0 = (int64_t)blockIdx.x * kFmTile;
  const int64_t h0 = t0 - kFmWarm;  // discriminator output held in pol[0]
  for (int i = threadIdx.x; i < kFmWarm + kFmTile; i += kFmThreads) {
    const int64_t j = h0 + i;
    float v = 0.f;
    if (j >= 0 && j < L.n_pol) {
      const int64_t ia = j + L.s0;
      v = polar_of(L.iso[ia], ia > 0 ? L.iso[ia - 1] : L.state[0]);
    }
    pol[i] = v;
  }
  __syncthreads();
  const int64_t c0 = t0 + (int64_t)threadIdx.x * kFmPer;
  if (c0 < L.n_pol) {
    int64_t w = c0 - kFmWarm;
    float y = 0.f;
    if (w <= 0) {
      w = 0;
      y = L.state[1].x;
    }
    for (; w < c0; ++w) y = deemph_step(pol[w - h0], y, L.b0, L.c);
#pragma unroll 4
    for (int k = 0; k < kFmPer; ++k) {
      y = deemph_step(pol[c0 + k - h0], y, L.b0, L.c);
      res[threadIdx.x * kFmPer + k] = y;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kFmTile; i += kFmThreads) {
    const int64_t j = t0 + i;
    if (j < L.n_pol) L.out[j] = make_float2(res[i], 0.f);
  }
}

// the discriminator's x[-1] and the de-emphasis y[-1] for the next call
__global__ void fm_state_kernel(const float2* iso, int64_t n_iso, const float2* out, int64_t n_pol, float2* state) {
  if (n_iso > 0) state[0] = iso[n_iso - 1];
  if (n_pol > 0) state[1] = make_float2(out[n_pol - 1].x, 0.f);
}

// max |x| over the call (non-negative floats order like their bit patterns)
__global__ void fm_absmax_kernel(const float2* m, int64_t n, unsigned* amax) {
  float v = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v = fmaxf(v, fabsf(m[i].x));
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMax(amax, __float_as_uint(v));
}

// out = x * (10000 / max), the quotient in double then float, the product in
// float, truncated to int16 (src/signals/falcon_dsp_fm_demod_cuda.cu:246-259)
__global__ void fm_scale_kernel(const float2* m, int64_t n, const unsigned* amax, int16_t* out) {
  const float scale = (float)(10000.0 / (double)__uint_as_float(*amax));
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int16_t)__float2int_rz(__fmul_rn(m[i].x, scale));
}

// de-emphasis taps of falcon_dsp_fm_demod.cc:119-133 (b0, a1; a0 = 1)
constexpr float kAmericasTau = 75e-6f;
constexpr float kEuropeTau = 50e-6f;

}  // namespace
}  // namespace fdsp

using namespace fdsp;

struct fdsp_fm_demod {
  fdsp_channelizer* iso = nullptr;
  fdsp_resampler* mono = nullptr;
  float b0 = 0.f, c = 0.f;
  bool have_prev = false;
  float2* d_state = nullptr;  // [0] x[-1], [1] y[-1], [2] max |x| (as bits)
  DevBuf iso_buf, iir_buf, mono_buf, in, out;
  ~fdsp_fm_demod() {
    if (iso) fdsp_channelizer_destroy(iso);
    if (mono) fdsp_resampler_destroy(mono);
    if (d_state) cudaFree(d_state);
  }
};

namespace {

struct FmCounts {
  uint64_t iso = 0, pol = 0, mono = 0;
};

int fm_counts(const fdsp_fm_demod* h, uint64_t n_in, FmCounts* c) {
  FDSP_TRY(fdsp_channelizer_out_count(h->iso, n_in, &c->iso));
  c->pol = c->iso == 0 ? 0 : (h->have_prev ? c->iso : c->iso - 1);
  FDSP_TRY(fdsp_resampler_out_count(h->mono, c->pol, &c->mono));
  return FDSP_OK;
}

// a filter of the predefined table as complex taps
int table_taps(uint32_t in_sps, uint32_t out_sps, uint32_t* up, uint32_t* down, std::vector<fdsp_cf32>& h) {
  uint32_t n = 0;
  int st = fdsp_get_resample_fir_params(in_sps, out_sps, 64, 0, up, down, nullptr, 0, &n);
  if (st != FDSP_ERR_CAPACITY && st != FDSP_OK) return st;
  h.resize(n);
  return fdsp_get_resample_fir_params(in_sps, out_sps, 64, 0, up, down, h.data(), n, &n);
}

}  // namespace

extern "C" {

int fdsp_fm_demod_create(uint32_t input_sample_rate, int32_t signal_offset_hz, float deemphasis_tau,
                         fdsp_fm_demod** out) {
  if (!out) return FDSP_ERR_INVALID_ARG;
  *out = nullptr;
  float b0, a1;
  if (deemphasis_tau == kAmericasTau) {
    b0 = 0.064493014968382223f;
    a1 = -0.93550698503161778f;
  } else if (deemphasis_tau == kEuropeTau) {
    b0 = 0.095162581964040482f;
    a1 = -0.90483741803595952f;
  } else {
    return FDSP_ERR_INVALID_ARG;  // the reference accepts only these two
  }
  uint32_t up = 0, down = 0, mup = 0, mdown = 0;
  std::vector<fdsp_cf32> taps, mtaps;
  FDSP_TRY(table_taps(input_sample_rate, FDSP_FM_RADIO_SAMPLE_RATE, &up, &down, taps));
  FDSP_TRY(table_taps(FDSP_FM_RADIO_SAMPLE_RATE, FDSP_FM_AUDIO_SAMPLE_RATE, &mup, &mdown, mtaps));
  fdsp_fm_demod* h = new (std::nothrow) fdsp_fm_demod();
  if (!h) return FDSP_ERR_ALLOC;
  h->b0 = b0;
  h->c = -a1;
  fdsp_channel_cfg cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.output_sample_rate_in_sps = FDSP_FM_RADIO_SAMPLE_RATE;
  cfg.freq_shift_in_hz = signal_offset_hz;
  cfg.up_rate = up;
  cfg.down_rate = down;
  cfg.resample_filter_coeffs = taps.data();
  cfg.num_coeffs = (uint32_t)taps.size();
  int st = fdsp_channelizer_create(input_sample_rate, &cfg, 1, &h->iso);
  if (st == FDSP_OK) st = fdsp_resampler_create(mup, mdown, mtaps.data(), (uint32_t)mtaps.size(), &h->mono);
  if (st == FDSP_OK) st = cuda_status(cudaMalloc(&h->d_state, 3 * sizeof(float2)));
  if (st == FDSP_OK) st = cuda_status(cudaMemset(h->d_state, 0, 3 * sizeof(float2)));
  if (st != FDSP_OK) {
    delete h;
    return st;
  }
  *out = h;
  return FDSP_OK;
}

int fdsp_fm_demod_destroy(fdsp_fm_demod* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  delete h;
  return FDSP_OK;
}

int fdsp_fm_demod_reset(fdsp_fm_demod* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  FDSP_TRY(fdsp_channelizer_reset(h->iso));
  FDSP_TRY(fdsp_resampler_reset(h->mono));
  h->have_prev = false;
  return cuda_status(cudaMemset(h->d_state, 0, 3 * sizeof(float2)));
}

int fdsp_fm_demod_out_count(const fdsp_fm_demod* h, uint64_t n_in, uint64_t* n_out) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!n_out) return FDSP_ERR_INVALID_ARG;
  FmCounts c;
  FDSP_TRY(fm_counts(h, n_in, &c));
  *n_out = c.mono;
  return FDSP_OK;
}

int fdsp_fm_demod_apply(fdsp_fm_demod* h, const fdsp_cf32* d_in, uint64_t n_in, int16_t* d_out, uint64_t out_cap,
                        uint64_t* n_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  FmCounts c;
  FDSP_TRY(fm_counts(h, n_in, &c));
  if (n_out) *n_out = c.mono;
  if (n_in == 0) return FDSP_OK;
  if (!d_in || (c.mono > 0 && !d_out)) return FDSP_ERR_INVALID_ARG;
  if (out_cap < c.mono) return FDSP_ERR_CAPACITY;
  if (c.iso >= (1ull << 31)) return FDSP_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  FDSP_TRY(h->iso_buf.ensure((c.iso + 1) * sizeof(float2)));
  FDSP_TRY(h->iir_buf.ensure((c.pol + 1) * sizeof(float2)));
  FDSP_TRY(h->mono_buf.ensure((c.mono + 1) * sizeof(float2)));
  float2* iso = static_cast<float2*>(h->iso_buf.p);
  float2* iir = static_cast<float2*>(h->iir_buf.p);
  float2* mono = static_cast<float2*>(h->mono_buf.p);
  fdsp_cf32* iso_ptr[1] = {reinterpret_cast<fdsp_cf32*>(iso)};
  const uint64_t iso_cap[1] = {c.iso + 1};
  uint64_t got[1] = {0};
  FDSP_TRY(fdsp_channelizer_apply(h->iso, d_in, n_in, iso_ptr, iso_cap, got, stream));
  if (c.pol > 0) {
    FmLaunch L;
    L.iso = iso;
    L.n_pol = (int64_t)c.pol;
    L.s0 = h->have_prev ? 0 : 1;
    L.state = h->d_state;
    L.b0 = h->b0;
    L.c = h->c;
    L.out = iir;
    const int64_t blocks = ((int64_t)c.pol + kFmTile - 1) / kFmTile;
    fm_polar_deemph_kernel<<<(unsigned)blocks, kFmThreads, 0, s>>>(L);
    FDSP_TRY(cuda_status(cudaGetLastError()));
  }
  if (c.iso > 0) {
    fm_state_kernel<<<1, 1, 0, s>>>(iso, (int64_t)c.iso, iir, (int64_t)c.pol, h->d_state);
    FDSP_TRY(cuda_status(cudaGetLastError()));
    h->have_prev = true;
  }
  uint64_t nm = 0;
  FDSP_TRY(fdsp_resampler_apply(h->mono, reinterpret_cast<const fdsp_cf32*>(iir), c.pol,
                                reinterpret_cast<fdsp_cf32*>(mono), c.mono + 1, &nm, stream));
  if (c.mono > 0) {
    unsigned* amax = reinterpret_cast<unsigned*>(h->d_state + 2);
    FDSP_TRY(cuda_status(cudaMemsetAsync(amax, 0, sizeof(unsigned), s)));
    const int64_t blocks = std::min<int64_t>(((int64_t)c.mono + 255) / 256, 1024);
    fm_absmax_kernel<<<(unsigned)blocks, 256, 0, s>>>(mono, (int64_t)c.mono, amax);
    FDSP_TRY(cuda_status(cudaGetLastError()));
    fm_scale_kernel<<<(unsigned)blocks, 256, 0, s>>>(mono, (int64_t)c.mono, amax, d_out);
    FDSP_TRY(cuda_status(cudaGetLastError()));
  }
  return FDSP_OK;
}

int fdsp_fm_demod_apply_host(fdsp_fm_demod* h, const fdsp_cf32* h_in, uint64_t n_in, int16_t* h_out,
                             uint64_t out_cap, uint64_t* n_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  FmCounts c;
  FDSP_TRY(fm_counts(h, n_in, &c));
  if (n_out) *n_out = c.mono;
  if (n_in == 0) return FDSP_OK;
  if (!h_in || (c.mono > 0 && !h_out)) return FDSP_ERR_INVALID_ARG;
  if (out_cap < c.mono) return FDSP_ERR_CAPACITY;
  cudaStream_t s = (cudaStream_t)stream;
  FDSP_TRY(h->in.ensure(n_in * sizeof(float2) + 16));
  FDSP_TRY(h->out.ensure(c.mono * sizeof(int16_t) + 16));
  FDSP_TRY(cuda_status(cudaMemcpyAsync(h->in.p, h_in, n_in * sizeof(float2), cudaMemcpyHostToDevice, s)));
  FDSP_TRY(fdsp_fm_demod_apply(h, static_cast<const fdsp_cf32*>(h->in.p), n_in, static_cast<int16_t*>(h->out.p),
                               c.mono, nullptr, stream));
  if (c.mono)
    FDSP_TRY(cuda_status(cudaMemcpyAsync(h_out, h->out.p, c.mono * sizeof(int16_t), cudaMemcpyDeviceToHost, s)));
  return cuda_status(cudaStreamSynchronize(s));
}

}  // extern "C"
