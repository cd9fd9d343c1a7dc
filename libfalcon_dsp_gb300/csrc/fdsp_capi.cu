// The C ABI (include/fdsp_c.h): opaque handles over the polyphase engine and
// the elementwise stages.  No entry point prints, throws across the boundary
// or exits; every failure is a negative status code.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "fdsp_internal.h"
#include "fdsp_shift_polar.h"

namespace fdsp {

static thread_local int g_last_cuda_error = 0;

void set_last_cuda_error(int code) { g_last_cuda_error = code; }

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return FDSP_OK;
  g_last_cuda_error = (int)e;
  if (e == cudaErrorMemoryAllocation) return FDSP_ERR_ALLOC;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return FDSP_ERR_NO_DEVICE;
  return FDSP_ERR_CUDA;
}

}  // namespace fdsp

using namespace fdsp;

struct fdsp_channelizer {
  PolyEngine eng;
  DevBuf in;
  DevBuf arena;  // apply_host: device outputs of every channel, back to back
  // apply_host: device-to-host copies on their own stream, each group's
  // started as soon as the launches that write it are enqueued
  cudaStream_t copy = nullptr;
  std::vector<cudaEvent_t> ev;
  size_t ev_used = 0;
  fdsp_cf32* const* h_out = nullptr;
  const float2* const* d_out = nullptr;
  const uint64_t* n_out = nullptr;
  int copy_err = 0;
  ~fdsp_channelizer() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    if (copy) cudaStreamDestroy(copy);
  }
};

namespace {
cudaEvent_t next_event(fdsp_channelizer* h) {
  if (h->ev_used == h->ev.size()) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    h->ev.push_back(e);
  }
  return h->ev[h->ev_used++];
}

// PolyEngine completion hook: the listed channels' outputs are complete once
// `stream` reaches this point; copy them back on the copy stream.
void channelizer_copy_back(void* ctx, const int* chans, int count, cudaStream_t stream) {
  fdsp_channelizer* h = static_cast<fdsp_channelizer*>(ctx);
  cudaEvent_t e = next_event(h);
  if (!e || cudaEventRecord(e, stream) != cudaSuccess || cudaStreamWaitEvent(h->copy, e, 0) != cudaSuccess) {
    h->copy_err = 1;
    return;
  }
  for (int i = 0; i < count; ++i) {
    const int c = chans[i];
    if (h->n_out[c] && cudaMemcpyAsync(h->h_out[c], h->d_out[c], h->n_out[c] * sizeof(float2),
                                       cudaMemcpyDeviceToHost, h->copy) != cudaSuccess)
      h->copy_err = 1;
  }
}

// Device outputs of an apply_host call: one allocation (grown when a block
// needs more), channel regions back to back at 256-byte boundaries.
int channel_arena(fdsp_channelizer* h, const std::vector<uint64_t>& cnt, std::vector<float2*>& dptr) {
  std::vector<size_t> off(cnt.size());
  size_t total = 0;
  for (size_t c = 0; c < cnt.size(); ++c) {
    off[c] = total;
    total += (cnt[c] * sizeof(float2) + 16 + 255) & ~(size_t)255;
  }
  FDSP_TRY(h->arena.ensure(total + 256));
  for (size_t c = 0; c < cnt.size(); ++c)
    dptr[c] = reinterpret_cast<float2*>(static_cast<uint8_t*>(h->arena.p) + off[c]);
  return FDSP_OK;
}

// apply (float or int16 input) with the outputs copied back group by group
// while the later groups compute; the caller's stream waits for every copy.
template <class ApplyFn>
int apply_with_copy_back(fdsp_channelizer* h, fdsp_cf32* const* h_out, float2* const* dptr, uint64_t* n_out,
                         cudaStream_t s, ApplyFn&& fn) {
  if (!h->copy) FDSP_TRY(cuda_status(cudaStreamCreateWithFlags(&h->copy, cudaStreamNonBlocking)));
  h->ev_used = 0;
  h->copy_err = 0;
  h->h_out = h_out;
  h->d_out = dptr;
  h->n_out = n_out;
  h->eng.set_done_hook(channelizer_copy_back, h);
  const int st = fn();
  h->eng.set_done_hook(nullptr, nullptr);
  cudaEvent_t e = next_event(h);
  if (!e) return FDSP_ERR_CUDA;
  FDSP_TRY(cuda_status(cudaEventRecord(e, h->copy)));
  FDSP_TRY(cuda_status(cudaStreamWaitEvent(s, e, 0)));
  if (st != FDSP_OK) return st;
  return h->copy_err ? FDSP_ERR_CUDA : FDSP_OK;
}
}  // namespace

struct fdsp_resampler {
  PolyEngine eng;
  uint32_t up = 1, down = 1;
  DevBuf in, out;
};

struct fdsp_fir {
  PolyEngine eng;  // y[n] = sum_k h[k] x[n-k]: one channel, up = down = 1
  DevBuf in, out;
  PolyEngine& active() { return eng; }
};

struct fdsp_freq_shift {
  uint32_t fs = 0;
  std::vector<NcoConst> nco;
  NcoConst* d_nco = nullptr;
  uint64_t abs0 = 0;
  DevBuf in;
  std::vector<DevBuf> out;
  ~fdsp_freq_shift() {
    if (d_nco) cudaFree(d_nco);
  }
};

struct fdsp_polar {
  float2* d_prev = nullptr;
  bool have_prev = false;
  DevBuf in, out;
  ~fdsp_polar() {
    if (d_prev) cudaFree(d_prev);
  }
};

// Status of the applies enqueued on `stream` so far: CUDA errors, then the
// tensor-core kernel's bounded-wait record (cleared by the read).
static int engine_status(PolyEngine& e, cudaStream_t s) {
  const int st = cuda_status(cudaStreamSynchronize(s));
  if (st != FDSP_OK) return st;
  return e.tc_error() ? FDSP_ERR_TIMEOUT : FDSP_OK;
}

extern "C" {

const char* fdsp_status_string(int status) {
  switch (status) {
    case FDSP_OK: return "ok";
    case FDSP_ERR_INVALID_ARG: return "invalid argument";
    case FDSP_ERR_NOT_INITIALIZED: return "handle not initialized";
    case FDSP_ERR_ALLOC: return "allocation failed";
    case FDSP_ERR_CUDA: return "CUDA runtime error";
    case FDSP_ERR_CAPACITY: return "output buffer too small";
    case FDSP_ERR_UNSUPPORTED: return "configuration outside this build's limits";
    case FDSP_ERR_NO_DEVICE: return "no CUDA device";
    case FDSP_ERR_NOT_FOUND: return "no predefined filter for this key";
    case FDSP_ERR_TIMEOUT: return "a tensor-core kernel's bounded wait gave up (outputs incomplete)";
    default: return "unknown status";
  }
}

int fdsp_last_cuda_error(void) { return g_last_cuda_error; }

int fdsp_version(void) { return 100; }

int fdsp_freq_shift_params(uint32_t fs, int32_t f, uint32_t* rollover, double* omega) {
  if (!rollover || !omega) return FDSP_ERR_INVALID_ARG;
  // falcon_dsp_freq_shift.cc:194-235 (abs(0) gives an infinite ratio whose
  // integer conversion is undefined in the reference; 0 is reported here)
  double r = (double)fs / (double)std::llabs((long long)f);
  while (r < 1e5) r *= 10.0;
  *rollover = (f == 0) ? 0u : (uint32_t)std::round(r);
  *omega = ((double)f / (double)fs) * 2.0 * M_PI;
  return FDSP_OK;
}

int fdsp_rat_approx(double f, int64_t md, int64_t* num, int64_t* den) {
  if (!num || !den) return FDSP_ERR_INVALID_ARG;
  // Continued-fraction convergents with a denominator cap
  // (falcon_dsp_utils.cc:231-294).
  int64_t h[3] = {0, 1, 0}, k[3] = {1, 0, 0};
  int64_t n = 1;
  bool neg = false;
  if (md <= 1) {
    *den = 1;
    *num = (int64_t)f;
    return FDSP_OK;
  }
  if (f < 0) {
    neg = true;
    f = -f;
  }
  while (f != std::floor(f)) {
    n <<= 1;
    f *= 2;
  }
  int64_t d = (int64_t)f;
  for (int i = 0; i < 64; i++) {
    const int64_t a = n ? d / n : 0;
    if (i && !a) break;
    int64_t x = d;
    d = n;
    n = x % n;
    x = a;
    if (k[1] * a + k[0] >= md) {
      x = (md - k[0]) / k[1];
      if (x * 2 >= a || k[1] >= md)
        i = 65;
      else
        break;
    }
    h[2] = x * h[1] + h[0];
    h[0] = h[1];
    h[1] = h[2];
    k[2] = x * k[1] + k[0];
    k[0] = k[1];
    k[1] = k[2];
  }
  *den = k[1];
  *num = neg ? -h[1] : h[1];
  return FDSP_OK;
}

int fdsp_polyphase_advance(uint32_t up, uint32_t down, uint32_t phase, uint64_t xoffset, uint64_t n_in,
                           uint64_t* n_out, uint32_t* phase_out, uint64_t* xoffset_out) {
  if (up == 0 || down == 0 || phase >= up) return FDSP_ERR_INVALID_ARG;
  const uint64_t M = polyphase_out_count(up, down, phase, xoffset, n_in);
  polyphase_advance(up, down, phase, xoffset, n_in, M);
  if (n_out) *n_out = M;
  if (phase_out) *phase_out = phase;
  if (xoffset_out) *xoffset_out = xoffset;
  return FDSP_OK;
}

/* ---------------- channelizer ---------------- */
int fdsp_channelizer_create(uint32_t fs, const fdsp_channel_cfg* ch, uint32_t nch, fdsp_channelizer** out) {
  if (!out) return FDSP_ERR_INVALID_ARG;
  *out = nullptr;
  if (fs == 0 || nch == 0 || !ch) return FDSP_ERR_INVALID_ARG;
  fdsp_channelizer* h = new (std::nothrow) fdsp_channelizer();
  if (!h) return FDSP_ERR_ALLOC;
  int st = h->eng.init(fs, ch, nch, false);
  if (st != FDSP_OK) {
    delete h;
    return st;
  }
  *out = h;
  return FDSP_OK;
}

int fdsp_channelizer_destroy(fdsp_channelizer* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  delete h;
  return FDSP_OK;
}

int fdsp_channelizer_reset(fdsp_channelizer* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  h->eng.reset();
  return FDSP_OK;
}

int fdsp_channelizer_num_channels(const fdsp_channelizer* h, uint32_t* n) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!n) return FDSP_ERR_INVALID_ARG;
  *n = h->eng.num_channels();
  return FDSP_OK;
}

int fdsp_channelizer_out_count(const fdsp_channelizer* h, uint64_t n_in, uint64_t* n_out) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return h->eng.out_counts(n_in, n_out);
}

int fdsp_channelizer_apply(fdsp_channelizer* h, const fdsp_cf32* d_in, uint64_t n_in, fdsp_cf32* const* d_out,
                           const uint64_t* out_cap, uint64_t* n_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return h->eng.apply(reinterpret_cast<const float2*>(d_in), n_in, reinterpret_cast<float2* const*>(d_out), out_cap,
                      n_out, (cudaStream_t)stream);
}

int fdsp_channelizer_status(fdsp_channelizer* h, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return engine_status(h->eng, (cudaStream_t)stream);
}

int fdsp_channelizer_set_tc_exact_all(fdsp_channelizer* h, int on) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  h->eng.set_tc_exact_all(on != 0 ? 1 : 0);
  return FDSP_OK;
}

int fdsp_channelizer_set_tc_wait(fdsp_channelizer* h, uint32_t max_polls, int withhold_copies) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (max_polls == 0) return FDSP_ERR_INVALID_ARG;
  h->eng.set_tc_wait(max_polls, withhold_copies != 0 ? 1 : 0);
  return FDSP_OK;
}

int fdsp_channelizer_profile(fdsp_channelizer* h, int enable) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  h->eng.set_profile(enable != 0);
  return FDSP_OK;
}

int fdsp_channelizer_profile_read(fdsp_channelizer* h, double* ms, uint32_t* launches) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return h->eng.read_profile(ms, launches);
}

int fdsp_channelizer_apply_ci16(fdsp_channelizer* h, const int16_t* d_in, uint64_t n_in, fdsp_cf32* const* d_out,
                                const uint64_t* out_cap, uint64_t* n_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return h->eng.apply_ci16(d_in, n_in, reinterpret_cast<float2* const*>(d_out), out_cap, n_out, (cudaStream_t)stream);
}

int fdsp_channelizer_set_precision(fdsp_channelizer* h, int precision) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return h->eng.set_precision(precision);
}

int fdsp_channelizer_kernel_launches(const fdsp_channelizer* h, uint32_t* n) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!n) return FDSP_ERR_INVALID_ARG;
  *n = (uint32_t)h->eng.kernel_launches_last();
  return FDSP_OK;
}

int fdsp_channelizer_tc_groups(const fdsp_channelizer* h, uint32_t* n) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!n) return FDSP_ERR_INVALID_ARG;
  *n = (uint32_t)h->eng.tc_groups_last();
  return FDSP_OK;
}

int fdsp_channelizer_autotune(fdsp_channelizer* h, uint64_t n_in, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return h->eng.autotune(n_in, (cudaStream_t)stream);
}

int fdsp_channelizer_set_graph(fdsp_channelizer* h, int enable) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  h->eng.set_graph(enable != 0);
  return FDSP_OK;
}

int fdsp_channelizer_graph_replays(const fdsp_channelizer* h, uint32_t* replays) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!replays) return FDSP_ERR_INVALID_ARG;
  *replays = (uint32_t)h->eng.graph_replays();
  return FDSP_OK;
}

int fdsp_channelizer_num_groups(const fdsp_channelizer* h, uint32_t* n) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!n) return FDSP_ERR_INVALID_ARG;
  *n = (uint32_t)h->eng.num_groups();
  return FDSP_OK;
}

int fdsp_channelizer_group_info(const fdsp_channelizer* h, uint32_t group, uint32_t* down_rate, uint32_t* tile_rows,
                                int* tensor_core) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!down_rate || !tile_rows || !tensor_core || group >= (uint32_t)h->eng.num_groups()) return FDSP_ERR_INVALID_ARG;
  int qt = 0;
  h->eng.group_info((int)group, down_rate, &qt, tensor_core);
  *tile_rows = (uint32_t)qt;
  return FDSP_OK;
}

int fdsp_channelizer_set_tc_split(fdsp_channelizer* h, uint32_t max_split) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return h->eng.set_tc_split((int)max_split);
}

int fdsp_channelizer_group_tc_split(const fdsp_channelizer* h, uint32_t group, uint32_t* split) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!split || group >= (uint32_t)h->eng.num_groups()) return FDSP_ERR_INVALID_ARG;
  *split = (uint32_t)h->eng.group_tc_split((int)group);
  return FDSP_OK;
}

int fdsp_channelizer_apply_host(fdsp_channelizer* h, const fdsp_cf32* h_in, uint64_t n_in, fdsp_cf32* const* h_out,
                                const uint64_t* out_cap, uint64_t* n_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if ((n_in > 0 && !h_in) || !n_out) return FDSP_ERR_INVALID_ARG;
  const uint32_t nch = h->eng.num_channels();
  std::vector<uint64_t> cnt(nch);
  FDSP_TRY(h->eng.out_counts(n_in, cnt.data()));
  for (uint32_t c = 0; c < nch; ++c) {
    if (out_cap && out_cap[c] < cnt[c]) return FDSP_ERR_CAPACITY;
    if (cnt[c] > 0 && (!h_out || !h_out[c])) return FDSP_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  FDSP_TRY(h->in.ensure(n_in * sizeof(float2) + 16));
  std::vector<float2*> dptr(nch);
  FDSP_TRY(channel_arena(h, cnt, dptr));
  if (n_in) FDSP_TRY(cuda_status(cudaMemcpyAsync(h->in.p, h_in, n_in * sizeof(float2), cudaMemcpyHostToDevice, s)));
  FDSP_TRY(apply_with_copy_back(h, h_out, dptr.data(), n_out, s, [&] {
    return h->eng.apply(static_cast<const float2*>(h->in.p), n_in, dptr.data(), nullptr, n_out, s);
  }));
  return engine_status(h->eng, s);
}

int fdsp_channelizer_apply_ci16_host(fdsp_channelizer* h, const int16_t* h_in, uint64_t n_in, fdsp_cf32* const* h_out,
                                     const uint64_t* out_cap, uint64_t* n_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if ((n_in > 0 && !h_in) || !n_out) return FDSP_ERR_INVALID_ARG;
  const uint32_t nch = h->eng.num_channels();
  std::vector<uint64_t> cnt(nch);
  FDSP_TRY(h->eng.out_counts(n_in, cnt.data()));
  for (uint32_t c = 0; c < nch; ++c) {
    if (out_cap && out_cap[c] < cnt[c]) return FDSP_ERR_CAPACITY;
    if (cnt[c] > 0 && (!h_out || !h_out[c])) return FDSP_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  FDSP_TRY(h->in.ensure(n_in * 2 * sizeof(int16_t) + 16));
  std::vector<float2*> dptr(nch);
  FDSP_TRY(channel_arena(h, cnt, dptr));
  if (n_in)
    FDSP_TRY(cuda_status(cudaMemcpyAsync(h->in.p, h_in, n_in * 2 * sizeof(int16_t), cudaMemcpyHostToDevice, s)));
  FDSP_TRY(apply_with_copy_back(h, h_out, dptr.data(), n_out, s, [&] {
    return h->eng.apply_ci16(static_cast<const int16_t*>(h->in.p), n_in, dptr.data(), nullptr, n_out, s);
  }));
  return engine_status(h->eng, s);
}

/* ---------------- resampler ---------------- */
int fdsp_resampler_create(uint32_t up, uint32_t down, const fdsp_cf32* coeffs, uint32_t ncoeffs,
                          fdsp_resampler** out) {
  if (!out) return FDSP_ERR_INVALID_ARG;
  *out = nullptr;
  if (up == 0 || down == 0 || !coeffs || ncoeffs == 0) return FDSP_ERR_INVALID_ARG;
  fdsp_resampler* h = new (std::nothrow) fdsp_resampler();
  if (!h) return FDSP_ERR_ALLOC;
  fdsp_channel_cfg c;
  c.output_sample_rate_in_sps = 0;
  c.freq_shift_in_hz = 0;
  c.up_rate = up;
  c.down_rate = down;
  c.resample_filter_coeffs = coeffs;
  c.num_coeffs = ncoeffs;
  int st = h->eng.init(1, &c, 1, false);
  if (st != FDSP_OK) {
    delete h;
    return st;
  }
  h->up = up;
  h->down = down;
  *out = h;
  return FDSP_OK;
}

int fdsp_resampler_destroy(fdsp_resampler* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  delete h;
  return FDSP_OK;
}

int fdsp_resampler_reset(fdsp_resampler* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  h->eng.reset();
  return FDSP_OK;
}

int fdsp_resampler_coeffs_per_phase(const fdsp_resampler* h, uint32_t* cpp) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!cpp) return FDSP_ERR_INVALID_ARG;
  *cpp = h->eng.coeffs_per_phase(0);
  return FDSP_OK;
}

int fdsp_resampler_out_count(const fdsp_resampler* h, uint64_t n_in, uint64_t* n_out) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return h->eng.out_counts(n_in, n_out);
}

int fdsp_resampler_needed_out_count(const fdsp_resampler* h, uint32_t n_in, uint32_t* n_out) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!n_out) return FDSP_ERR_INVALID_ARG;
  // polyphase_resampler.cc:216-228, in its own uint32 arithmetic
  const uint64_t np = (uint64_t)n_in * (uint64_t)h->up;
  uint32_t need = (uint32_t)(np / h->down);
  const uint32_t ph = h->eng.phase_of(0);
  const uint32_t xo = (uint32_t)h->eng.xoffset_of(0);
  if ((uint32_t)(ph + h->up * xo) < (np % h->down)) need++;
  *n_out = need;
  return FDSP_OK;
}

int fdsp_resampler_state(const fdsp_resampler* h, uint32_t* coeff_phase, uint64_t* x_offset) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (coeff_phase) *coeff_phase = h->eng.phase_of(0);
  if (x_offset) *x_offset = h->eng.xoffset_of(0);
  return FDSP_OK;
}

int fdsp_resampler_apply(fdsp_resampler* h, const fdsp_cf32* d_in, uint64_t n_in, fdsp_cf32* d_out,
                         uint64_t out_cap, uint64_t* n_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  float2* o = reinterpret_cast<float2*>(d_out);
  return h->eng.apply(reinterpret_cast<const float2*>(d_in), n_in, &o, &out_cap, n_out, (cudaStream_t)stream);
}

int fdsp_resampler_apply_ci16(fdsp_resampler* h, const int16_t* d_in, uint64_t n_in, fdsp_cf32* d_out,
                              uint64_t out_cap, uint64_t* n_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  float2* o = reinterpret_cast<float2*>(d_out);
  return h->eng.apply_ci16(d_in, n_in, &o, &out_cap, n_out, (cudaStream_t)stream);
}

int fdsp_resampler_apply_host(fdsp_resampler* h, const fdsp_cf32* h_in, uint64_t n_in, fdsp_cf32* h_out,
                              uint64_t out_cap, uint64_t* n_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if ((n_in > 0 && !h_in) || !n_out) return FDSP_ERR_INVALID_ARG;
  uint64_t cnt = 0;
  FDSP_TRY(h->eng.out_counts(n_in, &cnt));
  if (out_cap < cnt) return FDSP_ERR_CAPACITY;
  if (cnt > 0 && !h_out) return FDSP_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  FDSP_TRY(h->in.ensure(n_in * sizeof(float2) + 16));
  FDSP_TRY(h->out.ensure(cnt * sizeof(float2) + 16));
  if (n_in) FDSP_TRY(cuda_status(cudaMemcpyAsync(h->in.p, h_in, n_in * sizeof(float2), cudaMemcpyHostToDevice, s)));
  float2* o = static_cast<float2*>(h->out.p);
  FDSP_TRY(h->eng.apply(static_cast<const float2*>(h->in.p), n_in, &o, nullptr, n_out, s));
  if (*n_out)
    FDSP_TRY(cuda_status(cudaMemcpyAsync(h_out, o, *n_out * sizeof(float2), cudaMemcpyDeviceToHost, s)));
  return engine_status(h->eng, s);
}

int fdsp_resampler_set_precision(fdsp_resampler* h, int precision) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return h->eng.set_precision(precision);
}

int fdsp_resampler_tc_groups(const fdsp_resampler* h, uint32_t* n) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!n) return FDSP_ERR_INVALID_ARG;
  *n = (uint32_t)h->eng.tc_groups_last();
  return FDSP_OK;
}

int fdsp_resampler_status(fdsp_resampler* h, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return engine_status(h->eng, (cudaStream_t)stream);
}

/* ---------------- FIR ---------------- */
int fdsp_fir_create(const fdsp_cf32* coeffs, uint32_t ncoeffs, fdsp_fir** out) {
  if (!out) return FDSP_ERR_INVALID_ARG;
  *out = nullptr;
  if (!coeffs || ncoeffs == 0) return FDSP_ERR_INVALID_ARG;
  fdsp_fir* h = new (std::nothrow) fdsp_fir();
  if (!h) return FDSP_ERR_ALLOC;
  fdsp_channel_cfg c;
  c.output_sample_rate_in_sps = 0;
  c.freq_shift_in_hz = 0;
  c.up_rate = 1;
  c.down_rate = 1;
  c.resample_filter_coeffs = coeffs;
  c.num_coeffs = ncoeffs;
  int st = h->eng.init(1, &c, 1, true);
  if (st != FDSP_OK) {
    delete h;
    return st;
  }
  *out = h;
  return FDSP_OK;
}

// Tensor-core FIR: the one-channel engine under a tensor-core precision.
// The planner splits its outputs into 32 interleaved streams (output
// m = b + 32 i, windows starting b samples apart), the 32 output streams of
// one product: a Toeplitz matrix product that reads each input row once for
// 32 outputs.
int fdsp_fir_set_precision(fdsp_fir* h, int precision) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return h->eng.set_precision(precision);
}

int fdsp_fir_tc_groups(const fdsp_fir* h, uint32_t* n) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!n) return FDSP_ERR_INVALID_ARG;
  *n = (uint32_t)h->eng.tc_groups_last();
  return FDSP_OK;
}

int fdsp_fir_status(fdsp_fir* h, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  return engine_status(h->eng, (cudaStream_t)stream);
}

int fdsp_fir_destroy(fdsp_fir* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  delete h;
  return FDSP_OK;
}

int fdsp_fir_reset(fdsp_fir* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  h->active().reset();
  return FDSP_OK;
}

int fdsp_fir_apply(fdsp_fir* h, const fdsp_cf32* d_in, uint64_t n_in, fdsp_cf32* d_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  float2* o = reinterpret_cast<float2*>(d_out);
  uint64_t cnt = 0;
  return h->active().apply(reinterpret_cast<const float2*>(d_in), n_in, &o, nullptr, &cnt, (cudaStream_t)stream);
}

int fdsp_fir_apply_host(fdsp_fir* h, const fdsp_cf32* h_in, uint64_t n_in, fdsp_cf32* h_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (n_in > 0 && (!h_in || !h_out)) return FDSP_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  FDSP_TRY(h->in.ensure(n_in * sizeof(float2) + 16));
  FDSP_TRY(h->out.ensure(n_in * sizeof(float2) + 16));
  if (n_in) FDSP_TRY(cuda_status(cudaMemcpyAsync(h->in.p, h_in, n_in * sizeof(float2), cudaMemcpyHostToDevice, s)));
  float2* o = static_cast<float2*>(h->out.p);
  uint64_t cnt = 0;
  FDSP_TRY(h->active().apply(static_cast<const float2*>(h->in.p), n_in, &o, nullptr, &cnt, s));
  if (cnt) FDSP_TRY(cuda_status(cudaMemcpyAsync(h_out, o, cnt * sizeof(float2), cudaMemcpyDeviceToHost, s)));
  return engine_status(h->eng, s);
}

int fdsp_fir_apply_ci16(fdsp_fir* h, const int16_t* d_in, uint64_t n_in, int16_t* d_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (n_in == 0) return FDSP_OK;
  if (!d_in || !d_out) return FDSP_ERR_INVALID_ARG;
  FDSP_TRY(h->out.ensure(n_in * sizeof(float2) + 16));
  float2* o = static_cast<float2*>(h->out.p);
  uint64_t cnt = 0;
  FDSP_TRY(h->active().apply_ci16(d_in, n_in, &o, nullptr, &cnt, (cudaStream_t)stream));
  return launch_cf32_to_ci16(o, (int64_t)cnt, reinterpret_cast<short2*>(d_out), (cudaStream_t)stream);
}

int fdsp_fir_apply_ci16_host(fdsp_fir* h, const int16_t* h_in, uint64_t n_in, int16_t* h_out, fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (n_in == 0) return FDSP_OK;
  if (!h_in || !h_out) return FDSP_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  FDSP_TRY(h->in.ensure(n_in * 4 * sizeof(int16_t) + 16));  // int16 input, then int16 output
  int16_t* din = static_cast<int16_t*>(h->in.p);
  int16_t* dout = din + 2 * n_in;
  FDSP_TRY(cuda_status(cudaMemcpyAsync(din, h_in, n_in * 2 * sizeof(int16_t), cudaMemcpyHostToDevice, s)));
  FDSP_TRY(fdsp_fir_apply_ci16(h, din, n_in, dout, stream));
  FDSP_TRY(cuda_status(cudaMemcpyAsync(h_out, dout, n_in * 2 * sizeof(int16_t), cudaMemcpyDeviceToHost, s)));
  return engine_status(h->eng, s);
}

/* ---------------- frequency shift ---------------- */
int fdsp_freq_shift_create(uint32_t fs, const int32_t* shifts, uint32_t nch, fdsp_freq_shift** out) {
  if (!out) return FDSP_ERR_INVALID_ARG;
  *out = nullptr;
  if (fs == 0 || nch == 0 || !shifts) return FDSP_ERR_INVALID_ARG;
  if (nch > (uint32_t)kMaxChannels) return FDSP_ERR_UNSUPPORTED;
  fdsp_freq_shift* h = new (std::nothrow) fdsp_freq_shift();
  if (!h) return FDSP_ERR_ALLOC;
  h->fs = fs;
  h->nco.resize(nch);
  for (uint32_t c = 0; c < nch; ++c) h->nco[c] = make_nco(fs, shifts[c]);
  cudaError_t e = cudaMalloc(&h->d_nco, nch * sizeof(NcoConst));
  if (e == cudaSuccess) e = cudaMemcpy(h->d_nco, h->nco.data(), nch * sizeof(NcoConst), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete h;
    return cuda_status(e);
  }
  h->out.resize(nch);
  *out = h;
  return FDSP_OK;
}

int fdsp_freq_shift_destroy(fdsp_freq_shift* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  delete h;
  return FDSP_OK;
}

int fdsp_freq_shift_reset(fdsp_freq_shift* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  h->abs0 = 0;
  return FDSP_OK;
}

int fdsp_freq_shift_num_channels(const fdsp_freq_shift* h, uint32_t* n) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!n) return FDSP_ERR_INVALID_ARG;
  *n = (uint32_t)h->nco.size();
  return FDSP_OK;
}

int fdsp_freq_shift_counter(const fdsp_freq_shift* h, uint32_t c, uint64_t* counter) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!counter || c >= h->nco.size()) return FDSP_ERR_INVALID_ARG;
  const uint32_t R = h->nco[c].rollover;
  *counter = R ? h->abs0 % R : 0;
  return FDSP_OK;
}

int fdsp_freq_shift_apply(fdsp_freq_shift* h, const fdsp_cf32* d_in, uint64_t n_in, fdsp_cf32* const* d_out,
                          fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (n_in == 0) return FDSP_OK;
  if (!d_in || !d_out) return FDSP_ERR_INVALID_ARG;
  static thread_local ShiftLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.in = reinterpret_cast<const float2*>(d_in);
  L.N = (int64_t)n_in;
  L.nch = (int32_t)h->nco.size();
  L.nco = h->d_nco;
  for (size_t c = 0; c < h->nco.size(); ++c) {
    if (!d_out[c]) return FDSP_ERR_INVALID_ARG;
    L.out[c] = reinterpret_cast<float2*>(d_out[c]);
    const uint32_t R = h->nco[c].rollover;
    L.nco_base[c] = R ? (uint32_t)(h->abs0 % R) : 0u;
  }
  FDSP_TRY(launch_freq_shift(L, (cudaStream_t)stream));
  h->abs0 += n_in;
  return FDSP_OK;
}

int fdsp_freq_shift_apply_ci16(fdsp_freq_shift* h, const int16_t* d_in, uint64_t n_in, int16_t* const* d_out,
                               fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (n_in == 0) return FDSP_OK;
  if (!d_in || !d_out) return FDSP_ERR_INVALID_ARG;
  static thread_local ShiftLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.in = reinterpret_cast<const float2*>(d_in);
  L.i16 = 1;
  L.N = (int64_t)n_in;
  L.nch = (int32_t)h->nco.size();
  L.nco = h->d_nco;
  for (size_t c = 0; c < h->nco.size(); ++c) {
    if (!d_out[c]) return FDSP_ERR_INVALID_ARG;
    L.out[c] = reinterpret_cast<float2*>(d_out[c]);
    const uint32_t R = h->nco[c].rollover;
    L.nco_base[c] = R ? (uint32_t)(h->abs0 % R) : 0u;
  }
  FDSP_TRY(launch_freq_shift(L, (cudaStream_t)stream));
  h->abs0 += n_in;
  return FDSP_OK;
}

int fdsp_freq_shift_apply_ci16_host(fdsp_freq_shift* h, const int16_t* h_in, uint64_t n_in, int16_t* const* h_out,
                                    fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (n_in == 0) return FDSP_OK;
  if (!h_in || !h_out) return FDSP_ERR_INVALID_ARG;
  const size_t nch = h->nco.size();
  cudaStream_t s = (cudaStream_t)stream;
  FDSP_TRY(h->in.ensure(n_in * 2 * sizeof(int16_t) + 16));
  std::vector<int16_t*> d(nch);
  for (size_t c = 0; c < nch; ++c) {
    FDSP_TRY(h->out[c].ensure(n_in * 2 * sizeof(int16_t) + 16));
    d[c] = static_cast<int16_t*>(h->out[c].p);
  }
  FDSP_TRY(cuda_status(cudaMemcpyAsync(h->in.p, h_in, n_in * 2 * sizeof(int16_t), cudaMemcpyHostToDevice, s)));
  FDSP_TRY(fdsp_freq_shift_apply_ci16(h, static_cast<const int16_t*>(h->in.p), n_in, d.data(), stream));
  for (size_t c = 0; c < nch; ++c)
    FDSP_TRY(cuda_status(cudaMemcpyAsync(h_out[c], d[c], n_in * 2 * sizeof(int16_t), cudaMemcpyDeviceToHost, s)));
  return cuda_status(cudaStreamSynchronize(s));
}

int fdsp_freq_shift_apply_host(fdsp_freq_shift* h, const fdsp_cf32* h_in, uint64_t n_in, fdsp_cf32* const* h_out,
                               fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (n_in == 0) return FDSP_OK;
  if (!h_in || !h_out) return FDSP_ERR_INVALID_ARG;
  const size_t nch = h->nco.size();
  cudaStream_t s = (cudaStream_t)stream;
  FDSP_TRY(h->in.ensure(n_in * sizeof(float2) + 16));
  std::vector<fdsp_cf32*> d(nch);
  for (size_t c = 0; c < nch; ++c) {
    FDSP_TRY(h->out[c].ensure(n_in * sizeof(float2) + 16));
    d[c] = static_cast<fdsp_cf32*>(h->out[c].p);
  }
  FDSP_TRY(cuda_status(cudaMemcpyAsync(h->in.p, h_in, n_in * sizeof(float2), cudaMemcpyHostToDevice, s)));
  FDSP_TRY(fdsp_freq_shift_apply(h, static_cast<const fdsp_cf32*>(h->in.p), n_in, d.data(), stream));
  for (size_t c = 0; c < nch; ++c)
    FDSP_TRY(cuda_status(cudaMemcpyAsync(h_out[c], d[c], n_in * sizeof(float2), cudaMemcpyDeviceToHost, s)));
  return cuda_status(cudaStreamSynchronize(s));
}

/* ---------------- polar discriminator ---------------- */
int fdsp_polar_create(fdsp_polar** out) {
  if (!out) return FDSP_ERR_INVALID_ARG;
  *out = nullptr;
  fdsp_polar* h = new (std::nothrow) fdsp_polar();
  if (!h) return FDSP_ERR_ALLOC;
  cudaError_t e = cudaMalloc(&h->d_prev, sizeof(float2));
  if (e == cudaSuccess) e = cudaMemset(h->d_prev, 0, sizeof(float2));
  if (e != cudaSuccess) {
    delete h;
    return cuda_status(e);
  }
  *out = h;
  return FDSP_OK;
}

int fdsp_polar_destroy(fdsp_polar* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  delete h;
  return FDSP_OK;
}

int fdsp_polar_reset(fdsp_polar* h) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  h->have_prev = false;
  return FDSP_OK;
}

int fdsp_polar_out_count(const fdsp_polar* h, uint64_t n_in, uint64_t* n_out) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  if (!n_out) return FDSP_ERR_INVALID_ARG;
  *n_out = n_in == 0 ? 0 : (h->have_prev ? n_in : n_in - 1);
  return FDSP_OK;
}

int fdsp_polar_apply(fdsp_polar* h, const fdsp_cf32* d_in, uint64_t n_in, float* d_out, uint64_t* n_out,
                     fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  uint64_t cnt = 0;
  fdsp_polar_out_count(h, n_in, &cnt);
  if (n_out) *n_out = cnt;
  if (n_in == 0) return FDSP_OK;
  if (!d_in || (cnt > 0 && !d_out)) return FDSP_ERR_INVALID_ARG;
  FDSP_TRY(launch_polar(reinterpret_cast<const float2*>(d_in), (int64_t)n_in, h->d_prev, h->have_prev ? 0 : 1, d_out,
                        (cudaStream_t)stream));
  h->have_prev = true;
  return FDSP_OK;
}

int fdsp_polar_apply_host(fdsp_polar* h, const fdsp_cf32* h_in, uint64_t n_in, float* h_out, uint64_t* n_out,
                          fdsp_stream_t stream) {
  if (!h) return FDSP_ERR_NOT_INITIALIZED;
  uint64_t cnt = 0;
  fdsp_polar_out_count(h, n_in, &cnt);
  if (n_out) *n_out = cnt;
  if (n_in == 0) return FDSP_OK;
  if (!h_in || (cnt > 0 && !h_out)) return FDSP_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  FDSP_TRY(h->in.ensure(n_in * sizeof(float2) + 16));
  FDSP_TRY(h->out.ensure(n_in * sizeof(float) + 16));
  FDSP_TRY(cuda_status(cudaMemcpyAsync(h->in.p, h_in, n_in * sizeof(float2), cudaMemcpyHostToDevice, s)));
  FDSP_TRY(fdsp_polar_apply(h, static_cast<const fdsp_cf32*>(h->in.p), n_in, static_cast<float*>(h->out.p), nullptr,
                            stream));
  if (cnt) FDSP_TRY(cuda_status(cudaMemcpyAsync(h_out, h->out.p, cnt * sizeof(float), cudaMemcpyDeviceToHost, s)));
  return cuda_status(cudaStreamSynchronize(s));
}

}  // extern "C"

int fdsp::channelizer_create_pooled(uint32_t fs, const fdsp_channel_cfg* ch, uint32_t nch, DevPool* pool,
                                    cudaStream_t stream, fdsp_channelizer** out) {
  if (!out) return FDSP_ERR_INVALID_ARG;
  *out = nullptr;
  if (fs == 0 || nch == 0 || !ch) return FDSP_ERR_INVALID_ARG;
  fdsp_channelizer* h = new (std::nothrow) fdsp_channelizer();
  if (!h) return FDSP_ERR_ALLOC;
  h->eng.set_pool(pool);
  int st = h->eng.init(fs, ch, nch, false, stream);
  if (st != FDSP_OK) {
    delete h;
    return st;
  }
  *out = h;
  return FDSP_OK;
}
