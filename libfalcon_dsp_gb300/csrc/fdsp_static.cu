// fdsp_resample_static: one-shot polyphase resampling that allocates nothing.
//
// The resampler handle (fdsp_resampler_create) owns device buffers for its
// transposed taps and filter history.  This variant keeps the caller's taps
// in a fixed, file-scope device array instead, so a call makes no device or
// host allocation: it is one copy of the taps into that array and one kernel
// launch.  Output m of a fresh resampler (phase 0, xOffset 0) is
//     y[m] = sum_{jj < T} Re(h[jj U + ph]) x[i - jj],   i = floor(m D / U),
//     ph = (m D) mod U,  T = ceil(num_coeffs / U),  x[< 0] = 0,
// the polyphase loop of src/transform/falcon_dsp_polyphase_resampler.cc:256-319
// written per output; taps past num_coeffs are the zero padding of
// src/transform/falcon_dsp_polyphase_resampler.cc:131-157.
#include <mutex>

#include "fdsp_internal.h"

namespace fdsp {

// Fixed scratch for the taps: FDSP_RESAMPLE_STATIC_MAX_COEFFS complex values
// (64 KiB) per device.  Entries past the current call's num_coeffs are never
// read, so nothing in it has to be cleared between calls.
static __device__ __align__(256) float2 g_static_taps[FDSP_RESAMPLE_STATIC_MAX_COEFFS];

namespace {

constexpr int kMaxStaticDevices = 64;

struct StaticSlot {
  float2* taps = nullptr;  // device address of g_static_taps on this device
  int num_sms = 0;
};

std::mutex g_static_mu;
StaticSlot g_static_slots[kMaxStaticDevices];

// Per-device set-up, done once on the first call made with that device
// current: look up the array's device address and the SM count.
int static_slot(StaticSlot* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e);
  if (dev < 0 || dev >= kMaxStaticDevices) return FDSP_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_static_mu);
  StaticSlot& s = g_static_slots[dev];
  if (!s.taps) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_taps);
    if (e != cudaSuccess) return cuda_status(e);
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_status(e);
    s.num_sms = sms > 0 ? sms : 1;
    s.taps = static_cast<float2*>(p);
  }
  *out = s;
  return FDSP_OK;
}

__global__ void __launch_bounds__(256) resample_static_kernel(const float2* __restrict__ taps, uint32_t ncoeffs,
                                                             uint32_t U, uint32_t D, uint32_t T,
                                                             const float2* __restrict__ x, int64_t n_in,
                                                             float2* __restrict__ y, int64_t n_out) {
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < n_out; m += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t t = (uint64_t)m * D;
    const int64_t i = (int64_t)(t / U);
    const uint32_t ph = (uint32_t)(t - (uint64_t)i * U);
    float2 acc = make_float2(0.f, 0.f);
    for (uint32_t jj = 0; jj < T; ++jj) {
      const uint64_t src = (uint64_t)jj * U + ph;
      const int64_t xi = i - (int64_t)jj;
      if (src >= ncoeffs || xi < 0) break;  // both only grow with jj
      const float h = taps[src].x;
      const float2 v = x[xi];
      acc.x = fmaf(h, v.x, acc.x);
      acc.y = fmaf(h, v.y, acc.y);
    }
    y[m] = acc;
  }
}

}  // namespace
}  // namespace fdsp

using namespace fdsp;

extern "C" int fdsp_resample_static(uint32_t up_rate, uint32_t down_rate, const fdsp_cf32* coeffs,
                                    uint32_t num_coeffs, const fdsp_cf32* d_in, uint64_t n_in, fdsp_cf32* d_out,
                                    uint64_t out_cap, uint64_t* n_out, fdsp_stream_t stream) {
  if (!n_out) return FDSP_ERR_INVALID_ARG;
  *n_out = 0;
  if (up_rate == 0 || down_rate == 0 || !coeffs || num_coeffs == 0) return FDSP_ERR_INVALID_ARG;
  if (num_coeffs > FDSP_RESAMPLE_STATIC_MAX_COEFFS) return FDSP_ERR_UNSUPPORTED;
  if (n_in > (1ull << 62) / up_rate) return FDSP_ERR_UNSUPPORTED;
  const uint64_t cnt = polyphase_out_count(up_rate, down_rate, 0, 0, n_in);
  if (cnt > out_cap) return FDSP_ERR_CAPACITY;
  if (cnt > 0 && (!d_in || !d_out)) return FDSP_ERR_INVALID_ARG;
  StaticSlot slot;
  int st = static_slot(&slot);
  if (st != FDSP_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  st = cuda_status(cudaMemcpyAsync(slot.taps, coeffs, (size_t)num_coeffs * sizeof(float2), cudaMemcpyDefault, s));
  if (st != FDSP_OK) return st;
  if (cnt > 0) {
    // taps per phase, in 64 bits: up_rate near 2^32 must not wrap the sum
    const uint32_t T = (uint32_t)(((uint64_t)num_coeffs + up_rate - 1) / up_rate);
    const int64_t blocks = std::min<int64_t>((int64_t)((cnt + 255) / 256), (int64_t)slot.num_sms * 8);
    resample_static_kernel<<<(unsigned)blocks, 256, 0, s>>>(slot.taps, num_coeffs, up_rate, down_rate, T,
                                                            reinterpret_cast<const float2*>(d_in), (int64_t)n_in,
                                                            reinterpret_cast<float2*>(d_out), (int64_t)cnt);
    st = cuda_status(cudaGetLastError());
    if (st != FDSP_OK) return st;
  }
  *n_out = cnt;
  return FDSP_OK;
}
