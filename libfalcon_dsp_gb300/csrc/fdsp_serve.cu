// Streaming channelizer server: many concurrent streams (jobs) on one GPU.
//
// Each admitted stream owns a channelizer (its filter history, resampler
// phase and NCO counter stay on the device between blocks), a CUDA stream,
// one device input buffer of its maximum block length and one device output
// buffer per channel.  A submitted block is enqueued on the stream's CUDA
// stream as host->device copy, channelizer apply and device->host copies,
// followed by a host function that stamps the completion time; blocks of
// different streams overlap on the GPU.  Streams are admitted while their
// device footprint fits the server's memory budget and the active-stream
// limit, so new work starts as soon as earlier streams close.
//
// Device memory: the server takes its budget as one pool when it is created
// (csrc/fdsp_engine.cu DevPool); every stream's channelizer (taps, NCO
// constants, history), input buffer and output arena come from it, and the
// CUDA streams of closed streams are kept for the next ones, so opening and
// closing streams call neither cudaMalloc/cudaFree nor a device-wide
// synchronisation (only the closing stream is synchronised).
//
// The reference has no server; its channelizer classes are one blocking
// apply() per object (hdr/transform/falcon_dsp_multi_rate_channelizer_cuda.h:113).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <vector>

#include "fdsp_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct DoneQueue {  // tickets completed on the GPU, in completion order
  std::mutex mu;
  std::condition_variable cv;
  std::deque<uint64_t> ids;
};

struct Ticket {
  uint32_t sid = 0;
  uint64_t id = 0;
  DoneQueue* q = nullptr;
  Clock::time_point t_submit;
  std::atomic<int64_t> t_done_ns{0};  // completion, ns since t_submit (set by the host function)
  std::atomic<int> done{0};
  bool reported = false;
  std::vector<uint64_t> n_out;
};

struct ServeStream {
  fdsp_channelizer* ch = nullptr;
  cudaStream_t cs = nullptr;
  float2* d_in = nullptr;
  float2* d_arena = nullptr;     // every channel's output, back to back (capacity each)
  std::vector<float2*> d_out;    // channel c's part of the arena
  std::vector<uint64_t> cap;
  uint64_t max_block = 0;
  uint64_t footprint = 0;
  uint32_t nch = 0;
  std::vector<uint64_t> up, down;
};

void CUDART_CB on_block_done(void* p) {
  Ticket* t = static_cast<Ticket*>(p);
  const int64_t ns = std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t->t_submit).count();
  t->t_done_ns.store(ns > 0 ? ns : 1, std::memory_order_relaxed);
  t->done.store(1, std::memory_order_release);
  {
    std::lock_guard<std::mutex> lk(t->q->mu);
    t->q->ids.push_back(t->id);
  }
  t->q->cv.notify_one();
}

// Returns the stream's memory to the pool and its CUDA stream to `spare`.
void free_stream(ServeStream& s, fdsp::DevPool& pool, std::vector<cudaStream_t>& spare) {
  if (s.cs) cudaStreamSynchronize(s.cs);
  if (s.ch) fdsp_channelizer_destroy(s.ch);
  pool.release(s.d_in);
  pool.release(s.d_arena);
  if (s.cs) spare.push_back(s.cs);
  s = ServeStream();
}

}  // namespace

struct fdsp_server {
  uint64_t budget = 0, used = 0;
  uint32_t max_active = 0;
  uint32_t next_sid = 1;
  uint64_t next_ticket = 1;
  std::map<uint32_t, ServeStream> streams;
  std::map<uint64_t, std::unique_ptr<Ticket>> tickets;
  std::vector<double> lat_ms;
  uint64_t outputs = 0;
  std::mutex mu;
  DoneQueue done;
  fdsp::DevPool pool;                   // the budget's device memory
  std::vector<cudaStream_t> spare;      // CUDA streams of closed streams
  ~fdsp_server() {
    for (cudaStream_t c : spare) cudaStreamDestroy(c);
  }
};

using namespace fdsp;

// Device bytes a stream holds: input and output buffers, the channelizer's
// taps, history and (tensor-core precisions) its split-input scratch.
static uint64_t stream_footprint(const fdsp_channel_cfg* ch, uint32_t nch, uint64_t max_block, int precision) {
  uint64_t b = 8 * max_block + (1u << 20);
  uint64_t hist = 0;
  for (uint32_t c = 0; c < nch; ++c) {
    b += 8 * ((max_block * ch[c].up_rate + ch[c].down_rate - 1) / ch[c].down_rate + 2);
    b += 16ull * ch[c].num_coeffs + 64ull * ch[c].num_coeffs;  // FP32 and tensor-core tap tables
    hist = std::max<uint64_t>(hist, ch[c].num_coeffs / std::max(1u, ch[c].up_rate) + 1);
  }
  b += 16 * hist;
  if (precision != FDSP_PRECISION_FP32) b += 8 * (max_block + hist);
  return b;
}

extern "C" int fdsp_server_create(uint64_t budget_bytes, uint32_t max_active, fdsp_server** out) {
  if (!out || budget_bytes == 0 || max_active == 0) return FDSP_ERR_INVALID_ARG;
  fdsp_server* s = new (std::nothrow) fdsp_server();
  if (!s) return FDSP_ERR_ALLOC;
  s->budget = budget_bytes;
  s->max_active = max_active;
  // the pool: the budget, or what the device has free less 1 GiB
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    delete s;
    return FDSP_ERR_CUDA;
  }
  const size_t reserve = (size_t)1 << 30;
  const size_t pool_b = std::min<uint64_t>(budget_bytes, free_b > reserve ? free_b - reserve : free_b / 2);
  const int rc = s->pool.init(pool_b);
  if (rc != FDSP_OK) {
    delete s;
    return rc;
  }
  s->budget = std::min<uint64_t>(budget_bytes, s->pool.size());
  *out = s;
  return FDSP_OK;
}

extern "C" int fdsp_server_destroy(fdsp_server* s) {
  if (!s) return FDSP_ERR_NOT_INITIALIZED;
  for (auto& kv : s->streams) free_stream(kv.second, s->pool, s->spare);
  s->streams.clear();
  delete s;
  return FDSP_OK;
}

extern "C" int fdsp_server_open(fdsp_server* s, uint32_t fs, const fdsp_channel_cfg* ch, uint32_t nch,
                                uint64_t max_block, int precision, uint32_t* sid) {
  if (!s) return FDSP_ERR_NOT_INITIALIZED;
  if (!ch || nch == 0 || max_block == 0 || !sid) return FDSP_ERR_INVALID_ARG;
  const uint64_t fp = stream_footprint(ch, nch, max_block, precision);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->streams.size() >= s->max_active || s->used + fp > s->budget) return FDSP_ERR_CAPACITY;
    s->used += fp;  // reserved while the stream is set up
  }
  ServeStream st;
  st.max_block = max_block;
  st.footprint = fp;
  st.nch = nch;
  int rc = FDSP_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->spare.empty()) {
      st.cs = s->spare.back();
      s->spare.pop_back();
    }
  }
  if (!st.cs) rc = cuda_status(cudaStreamCreateWithFlags(&st.cs, cudaStreamNonBlocking));
  if (rc == FDSP_OK) rc = fdsp::channelizer_create_pooled(fs, ch, nch, &s->pool, st.cs, &st.ch);
  if (rc == FDSP_OK && precision != FDSP_PRECISION_FP32) rc = fdsp_channelizer_set_precision(st.ch, precision);
  if (rc == FDSP_OK) {
    st.d_in = static_cast<float2*>(s->pool.alloc(8 * max_block));
    if (!st.d_in) rc = FDSP_ERR_CAPACITY;
  }
  st.d_out.assign(nch, nullptr);
  st.cap.assign(nch, 0);
  uint64_t total = 0;
  for (uint32_t c = 0; c < nch; ++c) {
    st.cap[c] = (max_block * ch[c].up_rate + ch[c].down_rate - 1) / ch[c].down_rate + 2;
    total += st.cap[c];
  }
  if (rc == FDSP_OK) {
    st.d_arena = static_cast<float2*>(s->pool.alloc(8 * total));
    if (!st.d_arena) rc = FDSP_ERR_CAPACITY;
  }
  for (uint32_t c = 0, off = 0; c < nch && rc == FDSP_OK; off += (uint32_t)st.cap[c], ++c) st.d_out[c] = st.d_arena + off;
  std::lock_guard<std::mutex> lk(s->mu);
  if (rc != FDSP_OK) {
    free_stream(st, s->pool, s->spare);
    s->used -= fp;
    return rc;
  }
  const uint32_t id = s->next_sid++;
  s->streams.emplace(id, std::move(st));
  *sid = id;
  return FDSP_OK;
}

extern "C" int fdsp_server_submit(fdsp_server* s, uint32_t sid, const fdsp_cf32* h_in, uint64_t n_in,
                                  fdsp_cf32* const* h_out, const uint64_t* out_cap, uint64_t* ticket) {
  if (!s) return FDSP_ERR_NOT_INITIALIZED;
  if (!h_in || n_in == 0 || !h_out || !ticket) return FDSP_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->streams.find(sid);
  if (it == s->streams.end()) return FDSP_ERR_INVALID_ARG;
  ServeStream& st = it->second;
  if (n_in > st.max_block) return FDSP_ERR_CAPACITY;
  std::unique_ptr<Ticket> t(new (std::nothrow) Ticket());
  if (!t) return FDSP_ERR_ALLOC;
  t->sid = sid;
  t->id = s->next_ticket;
  t->q = &s->done;
  t->n_out.assign(st.nch, 0);
  t->t_submit = Clock::now();
  int rc = cuda_status(cudaMemcpyAsync(st.d_in, h_in, 8 * n_in, cudaMemcpyHostToDevice, st.cs));
  if (rc == FDSP_OK)
    rc = fdsp_channelizer_apply(st.ch, reinterpret_cast<const fdsp_cf32*>(st.d_in), n_in,
                                reinterpret_cast<fdsp_cf32* const*>(st.d_out.data()), st.cap.data(), t->n_out.data(),
                                (fdsp_stream_t)st.cs);
  // host outputs laid out like the device arena (each channel's region at
  // least the device capacity, back to back): one copy for the whole block
  bool one_copy = out_cap != nullptr;
  for (uint32_t c = 0; c < st.nch && one_copy; ++c)
    one_copy = out_cap[c] >= st.cap[c] && h_out[c] == h_out[0] + (st.d_out[c] - st.d_arena);
  if (one_copy && rc == FDSP_OK) {
    const uint64_t n = (uint64_t)(st.d_out[st.nch - 1] - st.d_arena) + t->n_out[st.nch - 1];
    rc = cuda_status(cudaMemcpyAsync(h_out[0], st.d_arena, 8 * n, cudaMemcpyDeviceToHost, st.cs));
  }
  for (uint32_t c = 0; c < st.nch && rc == FDSP_OK && !one_copy; ++c) {
    if (out_cap && out_cap[c] < t->n_out[c]) rc = FDSP_ERR_CAPACITY;
    if (rc == FDSP_OK && t->n_out[c])
      rc = cuda_status(cudaMemcpyAsync(h_out[c], st.d_out[c], 8 * t->n_out[c], cudaMemcpyDeviceToHost, st.cs));
  }
  if (rc == FDSP_OK) rc = cuda_status(cudaLaunchHostFunc(st.cs, on_block_done, t.get()));
  if (rc != FDSP_OK) {
    cudaStreamSynchronize(st.cs);  // nothing of this ticket may still reference it
    return rc;
  }
  const uint64_t id = s->next_ticket++;
  s->tickets.emplace(id, std::move(t));
  *ticket = id;
  return FDSP_OK;
}

extern "C" int fdsp_server_poll(fdsp_server* s, uint64_t ticket, int* done, uint64_t* n_out, double* latency_ms) {
  if (!s) return FDSP_ERR_NOT_INITIALIZED;
  if (!done) return FDSP_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return FDSP_ERR_INVALID_ARG;
  Ticket& t = *it->second;
  *done = t.done.load(std::memory_order_acquire);
  if (!*done) return FDSP_OK;
  const double ms = (double)t.t_done_ns.load(std::memory_order_relaxed) / 1e6;
  if (latency_ms) *latency_ms = ms;
  if (n_out) std::copy(t.n_out.begin(), t.n_out.end(), n_out);
  uint64_t tot = 0;
  for (auto v : t.n_out) tot += v;
  s->lat_ms.push_back(ms);
  s->outputs += tot;
  s->tickets.erase(it);  // a completed ticket is reported once
  return FDSP_OK;
}

extern "C" int fdsp_server_wait_any(fdsp_server* s, uint32_t timeout_us, uint64_t* ticket) {
  if (!s) return FDSP_ERR_NOT_INITIALIZED;
  if (!ticket) return FDSP_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->done.mu);
  if (s->done.ids.empty() && timeout_us)
    s->done.cv.wait_for(lk, std::chrono::microseconds(timeout_us), [&] { return !s->done.ids.empty(); });
  if (s->done.ids.empty()) {
    *ticket = 0;
    return FDSP_OK;
  }
  *ticket = s->done.ids.front();
  s->done.ids.pop_front();
  return FDSP_OK;
}

extern "C" int fdsp_server_close(fdsp_server* s, uint32_t sid) {
  if (!s) return FDSP_ERR_NOT_INITIALIZED;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->streams.find(sid);
  if (it == s->streams.end()) return FDSP_ERR_INVALID_ARG;
  s->used -= it->second.footprint;
  free_stream(it->second, s->pool, s->spare);  // waits for the stream's blocks
  s->streams.erase(it);
  return FDSP_OK;
}

extern "C" int fdsp_server_stats(fdsp_server* s, double* p50_ms, double* p99_ms, double* p999_ms, uint64_t* blocks,
                                 uint64_t* outputs, uint64_t* used_bytes, uint32_t* active) {
  if (!s) return FDSP_ERR_NOT_INITIALIZED;
  std::lock_guard<std::mutex> lk(s->mu);
  std::vector<double> v = s->lat_ms;
  std::sort(v.begin(), v.end());
  auto q = [&](double p) { return v.empty() ? 0.0 : v[std::min(v.size() - 1, (size_t)(p * (double)(v.size() - 1) + 0.5))]; };
  if (p50_ms) *p50_ms = q(0.5);
  if (p99_ms) *p99_ms = q(0.99);
  if (p999_ms) *p999_ms = q(0.999);
  if (blocks) *blocks = v.size();
  if (outputs) *outputs = s->outputs;
  if (used_bytes) *used_bytes = s->used;
  if (active) *active = (uint32_t)s->streams.size();
  return FDSP_OK;
}

extern "C" int fdsp_server_reset_stats(fdsp_server* s) {
  if (!s) return FDSP_ERR_NOT_INITIALIZED;
  std::lock_guard<std::mutex> lk(s->mu);
  s->lat_ms.clear();
  s->outputs = 0;
  return FDSP_OK;
}
