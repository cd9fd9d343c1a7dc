// Elementwise stages of the path: the multi-channel NCO frequency shift and
// the polar discriminator.  Both are HBM-bound: the input block is read once
// and each output is written once.
//
// Reference behaviour:
//   shift   src/transform/falcon_dsp_freq_shift.cc:164-192 (CPU),
//           src/transform/falcon_dsp_freq_shift_cuda.cu:166-216, :355-488 (CUDA)
//   polar   src/transform/falcon_dsp_polar_discriminator.cc:134-171 (CPU only)
#include <cstring>

#include "fdsp_internal.h"
#include "fdsp_shift_polar.h"

namespace fdsp {

// e^{j 2 pi t} for t in 2^-64 turns; the argument handed to the SFU lies in
// [-pi, pi), where __sincosf is accurate to ~4e-7 absolute.
__device__ __forceinline__ float2 phasor64_sp(uint64_t turns64) {
  const int32_t top = (int32_t)(turns64 >> 32);
  const float a = (float)top * 1.4629180792671596e-09f;  // 2 pi / 2^32
  float s, c;
  __sincosf(a, &s, &c);
  return make_float2(c, s);
}

// One CTA owns kShiftTile consecutive input samples and writes them, shifted,
// for every channel.  Each thread keeps its kShiftPer samples in registers, so
// the input is read from HBM once however many channels there are.
constexpr int kShiftThreads = 256;
constexpr int kShiftPer = 8;
constexpr int kShiftTile = kShiftThreads * kShiftPer;

__global__ void __launch_bounds__(kShiftThreads)
    freq_shift_kernel(const __grid_constant__ ShiftLaunch L) {
  const int64_t t0 = (int64_t)blockIdx.x * kShiftTile;
  float2 x[kShiftPer];
#pragma unroll
  for (int u = 0; u < kShiftPer; ++u) {
    const int64_t i = t0 + threadIdx.x + (int64_t)u * kShiftThreads;
    if (L.i16) {
      const short2 s = i < L.N ? reinterpret_cast<const short2*>(L.in)[i] : make_short2(0, 0);
      x[u] = make_float2((float)s.x, (float)s.y);
    } else {
      x[u] = i < L.N ? L.in[i] : make_float2(0.f, 0.f);
    }
  }
  for (int c = 0; c < L.nch; ++c) {
    const NcoConst nc = L.nco[c];
    float2* __restrict__ out = L.out[c];
    if (!nc.enabled) {
#pragma unroll
      for (int u = 0; u < kShiftPer; ++u) {
        const int64_t i = t0 + threadIdx.x + (int64_t)u * kShiftThreads;
        if (i >= L.N) continue;
        if (L.i16)
          reinterpret_cast<short2*>(out)[i] = make_short2((short)__float2int_rz(x[u].x), (short)__float2int_rz(x[u].y));
        else
          out[i] = x[u];
      }
      continue;
    }
    const uint32_t R = nc.rollover;
    // counter of this thread's first sample, then step by kShiftThreads
    uint64_t p = ((uint64_t)L.nco_base[c] + (uint64_t)(t0 + threadIdx.x)) % R;
    const uint32_t step = kShiftThreads % R;
#pragma unroll
    for (int u = 0; u < kShiftPer; ++u) {
      const int64_t i = t0 + threadIdx.x + (int64_t)u * kShiftThreads;
      const float2 e = phasor64_sp(p * nc.omega64);
      if (i < L.N) {
        const float2 v = x[u];
        const float2 y = make_float2(fmaf(v.x, e.x, -v.y * e.y), fmaf(v.x, e.y, v.y * e.x));
        if (L.i16)
          reinterpret_cast<short2*>(out)[i] = make_short2((short)__float2int_rz(y.x), (short)__float2int_rz(y.y));
        else
          out[i] = y;
      }
      p += step;
      if (p >= R) p -= R;
    }
  }
}

int launch_freq_shift(const ShiftLaunch& L, cudaStream_t stream) {
  if (L.N <= 0) return FDSP_OK;
  const int64_t nblocks = (L.N + kShiftTile - 1) / kShiftTile;
  if (nblocks > 0x7fffffffLL) return FDSP_ERR_UNSUPPORTED;
  freq_shift_kernel<<<(unsigned)nblocks, kShiftThreads, 0, stream>>>(L);
  return cuda_status(cudaGetLastError());
}

__global__ void cf32_to_ci16_kernel(const float2* __restrict__ in, int64_t n, short2* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = in[i];
    out[i] = make_short2((short)__float2int_rz(v.x), (short)__float2int_rz(v.y));
  }
}

int launch_cf32_to_ci16(const float2* in, int64_t n, short2* out, cudaStream_t stream) {
  if (n <= 0) return FDSP_OK;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, 4096);
  cf32_to_ci16_kernel<<<(unsigned)blocks, 256, 0, stream>>>(in, n, out);
  return cuda_status(cudaGetLastError());
}

// out[i - start] = atan2(Im, Re) of x[i] * conj(x[i-1]); x[-1] is the sample
// saved by the previous apply (polar_discriminator.cc:150-165).
__global__ void polar_kernel(const float2* __restrict__ in, int64_t N, const float2* __restrict__ prev, int start,
                             float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x + start;
  if (i >= N) return;
  const float2 a = in[i];
  const float2 b = i > 0 ? in[i - 1] : *prev;
  // a * conj(b), rounded like the reference's complex<float> product
  const float re = a.x * b.x + a.y * b.y;
  const float im = a.y * b.x - a.x * b.y;
  out[i - start] = atan2f(im, re);
}

__global__ void polar_save_kernel(const float2* __restrict__ in, int64_t N, float2* __restrict__ prev) {
  *prev = in[N - 1];
}

int launch_polar(const float2* in, int64_t N, float2* d_prev, int start, float* out, cudaStream_t stream) {
  if (N <= 0) return FDSP_OK;
  const int64_t n_out = N - start;
  if (n_out > 0) {
    const int64_t nblocks = (n_out + 255) / 256;
    if (nblocks > 0x7fffffffLL) return FDSP_ERR_UNSUPPORTED;
    polar_kernel<<<(unsigned)nblocks, 256, 0, stream>>>(in, N, d_prev, start, out);
    int st = cuda_status(cudaGetLastError());
    if (st != FDSP_OK) return st;
  }
  polar_save_kernel<<<1, 1, 0, stream>>>(in, N, d_prev);
  return cuda_status(cudaGetLastError());
}

}  // namespace fdsp
