// Internal declarations shared by the CUDA translation units of
// libfalcon_dsp_gb300.  Nothing here is part of the public C ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "fdsp_c.h"
#include "fdsp_pool.h"
#include "fdsp_tc_plan.h"

#define FDSP_TRY(expr)              \
  do {                              \
    int st_ = (expr);               \
    if (st_ != FDSP_OK) return st_; \
  } while (0)

namespace fdsp {

// ---------------------------------------------------------------------------
// Limits of one polyphase-engine launch.  Every field of the launch travels in
// the kernel parameter block (CUDA allows up to 32 764 bytes on sm_70+), so a
// launch needs no host->device copy and can be captured into a CUDA graph.
// ---------------------------------------------------------------------------
constexpr int kMaxChannels = 512;   // output channels per engine
constexpr int kMaxGroups = 16;      // distinct decimation factors per engine
constexpr int kMaxWorkSets = 256;   // (tap batch, output class) pairs per launch
constexpr int kThreads = 256;       // threads per CTA of the FP32 engine kernel

// Per-channel NCO constants (device array, written once at create time).
// The reference's angle for input sample n of a channel is
//   omega * (n mod R),  omega = 2*pi*f/fs          (falcon_dsp_freq_shift.cc:164-192)
// Here the angle is carried as a 64-bit fixed-point fraction of a turn:
//   turns(p) = p * omega64 mod 2^64, omega64 = round(2^64 * (f mod fs) / fs)
// which is exact to ~1e-9 rad for every p < R.
struct NcoConst {
  uint64_t omega64;   // turns per sample, 2^-64 units
  uint64_t wrap64;    // R * omega64 mod 2^64 (phase that the rollover drops)
  uint64_t fastmod;   // ceil(2^64 / R): n mod R as one 64-bit multiply-high
  uint32_t rollover;  // R; 0 when the channel has no shift
  uint32_t enabled;   // 0: phasor is exactly 1 (shift of 0 Hz)
};

// One decimation-factor group of an engine launch (one CTA per tile of it).
struct GroupDesc {
  int32_t D;          // down rate shared by every channel of the group
  int32_t Qt;         // output rows per tile (multiple of 32)
  int32_t P;          // shared-memory pitch (float2) of the de-interleaved tile
  int32_t tmax;       // longest padded window (taps) of the group
  int32_t delta_min;  // smallest window-end offset of any active output class
  int32_t delta_span; // delta_max - delta_min
  int32_t ntiles;     // tiles of Qt rows in this launch
  int32_t ws_begin;   // work sets [ws_begin, ws_end) belong to this group
  int32_t ws_end;
  int32_t taps_off;   // shared-memory offset (float2) of the staged taps
  int32_t meta_off;   // shared-memory offset (float2) of the staged channel constants
  int32_t smem_bytes; // dynamic shared memory of one CTA
  int32_t taps_smem;  // 1: taps staged in shared memory; 0: read through L1
  int32_t win;        // 1: single-channel work sets, sliding-window rows (Qt multiple of 32 x kWinRows)
  int32_t real_taps;  // 1: every tap of the group is real (2 FMAs per tap)
};

// One (tap batch, output class r) pair of a launch.  Output j of the class is
// output index m = r + U*j of every channel in the batch; its window is
// [delta + j*D - T + 1, delta + j*D] in block-relative input indices.
template <int NB>
struct WorkSet {
  const float2* taps;   // [T][nb] modulated taps of phase phi_r (device)
  int32_t T;            // padded taps per phase of the batch
  int32_t soff;         // shared-memory offset (float2) of these taps in the CTA
  int32_t delta;        // window end of row j = 0 (block relative)
  int32_t J;            // rows that have an output in this launch
  int32_t U;            // up rate of the batch's channels
  int32_t r;            // output class (m mod U)
  int32_t nb;           // live channels in the batch (<= NB)
  int16_t ch[NB];       // channel ids
};

template <int NB>
struct PolyLaunch {
  const float2* block;      // device input block (N samples)
  const short2* block16;    // or, when set, the block as complex int16 (converted on load)
  const float2* hist;       // device history (H samples preceding block)
  int64_t N;
  int32_t H;
  int32_t ngroups;
  int32_t max_tiles;
  int32_t nws;
  const NcoConst* nco;      // [nch]
  int8_t fuse_map[kMaxGroups];  // fused launches: group of blockIdx.y + offset
  GroupDesc groups[kMaxGroups];
  WorkSet<NB> ws[kMaxWorkSets];
  float2* out[kMaxChannels];         // output base of each channel for this launch
  uint32_t nco_base[kMaxChannels];   // (samples since reset at block[0]) mod R
};

// ---------------------------------------------------------------------------
// Tensor-core launch: the decimation groups of one launch pack computed on
// the tensor cores, planned by tc_plan (fdsp_tc_plan.h).  The record is the
// parameter block of tc_prep_kernel and tc_fix_kernel (no host->device copy
// per apply); tc_prep_kernel copies it into device memory for the filter-bank
// kernel, which takes only the tensor maps and a pointer (TcFilterParams).
// ---------------------------------------------------------------------------
struct TcLaunch {
  CUtensorMap maps[kTcMaxGroups];    // A operand of each group: rows D' samples apart over xhl
  const float2* block;               // input block (exact rollover path)
  const short2* block16;             // or, when set, the block as complex int16
  const float2* hist;                // history (H samples preceding the block)
  const NcoConst* nco;               // [channels]
  const float2* const* ctaps;        // per channel: FP32 modulated taps [U][T]
  uint2* xhl;                        // [history | block | zeros] as {hi, lo} 16-bit parts (prep writes it)
  uint8_t* bbuf;                     // B images of the merge sets (prep writes them)
  int* err;                          // bounded-wait failures (mapped host memory)
  TcLaunch* rec_out;                 // device copy of this record (the prep kernel writes it)
  int64_t N;                         // block samples
  int64_t Lc;                        // samples of the time range each CTA owns
  int64_t xhl_n;                     // samples of xhl the prep writes
  int32_t H, G, nmsets, ngroups, stages, stage_bytes, nslots;
  uint32_t poll;                     // polls before a wait gives up (each suspends up to ~2 us)
  int32_t hold;                      // test hook: the producer issues nothing (every wait runs out)
  int32_t exact_all;                 // test hook: every output takes the exact rotation pass
  int32_t bprefix[kTcMaxMsets + 1];  // 16-byte pieces of the B images before merge set m
  TcGroup groups[kTcMaxGroups];
  TcMset ms[kTcMaxMsets];
  TcSlot slots[kTcMaxSlots];
  uint32_t nco_base[kMaxChannels];   // (samples since reset at block[0]) mod R per channel
};

static_assert(sizeof(TcLaunch) <= 32764, "tensor-core launch must fit the kernel parameter block");
static_assert(sizeof(TcLaunch) % 16 == 0, "tensor-core launch record is copied in 16-byte pieces");

// Parameters of the filter-bank kernel: the tensor maps (TMA reads them from
// the parameter space) and the launch record, which the prep kernel copied
// into device memory -- a 2 KB parameter block instead of the 32 KB record.
struct TcFilterParams {
  CUtensorMap maps[kTcMaxGroups];
  const TcLaunch* rec;
};

// CUDA error -> status, remembering the CUDA code for fdsp_last_cuda_error().
int cuda_status(cudaError_t e);

// Grow-only device buffer (scratch of the *_apply_host entry points and of
// multi-stage pipelines).
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) {
    o.p = nullptr;
    o.bytes = 0;
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  int ensure(size_t want) {
    if (want <= bytes) return FDSP_OK;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) return cuda_status(e);
    bytes = want;
    return FDSP_OK;
  }
};
void set_last_cuda_error(int code);

// ---------------------------------------------------------------------------
// Polyphase engine: the shared machinery behind the channelizer, the
// standalone resampler and the FIR filter.
// ---------------------------------------------------------------------------
struct EngineChannel {
  uint32_t up, down;
  uint32_t T;                  // taps per phase (reference coeffs_per_phase)
  int32_t shift_hz;            // int32 shift, as the reference's NCO stores it
  std::vector<float2> flipped; // [up][T] transposed & flipped taps
  NcoConst nco;
};

// Device memory pool: one cudaMalloc'd region handed out by a RangePool
// (fdsp_pool.h: first fit, 256-byte aligned, neighbours coalesced) under a
// mutex.  The stream server gives it to its channelizers so that opening,
// closing and resetting streams allocate nothing from the driver.
class DevPool {
 public:
  ~DevPool();
  int init(size_t bytes);            // the one cudaMalloc
  void* alloc(size_t bytes);         // nullptr when no free range fits
  void release(void* p);
  size_t size() const { return ranges_.size(); }

 private:
  char* base_ = nullptr;
  RangePool ranges_;
  std::mutex mu_;
};

// A channelizer whose device memory comes from `pool` and whose initial
// history fill is enqueued on `stream` (no allocation from the driver and no
// device synchronisation: the stream server's open path).
int channelizer_create_pooled(uint32_t fs, const fdsp_channel_cfg* ch, uint32_t nch, DevPool* pool,
                              cudaStream_t stream, fdsp_channelizer** out);

struct EngineClass {   // channels with identical (up, down) share streaming state
  uint32_t up, down;
  uint32_t phase;      // reference coeff_phase
  uint64_t xoffset;    // reference xOffset
  uint64_t M;          // outputs of the current launch
  std::vector<int> chans;
};

struct EngineBatch {
  int cls;             // class index
  int group;           // decimation group index
  int T;               // padded taps per phase
  std::vector<int> chans;
  float2* d_taps;      // [up][T][nb] on the device
};

struct EngineGroup {
  uint32_t D;
  int Qt;
  int Qt_default = 0;  // tile rows chosen from the shapes alone
  int use_tc = 1;      // tensor-core form when the precision asks for it (autotuned)
  int tc_split = 32;   // largest row split of the tensor-core form (1 = none)
  int tc_split_used = 1;  // row split of its last tensor-core launch
  int win = 0;         // single-channel long filters: the FP32 kernel's sliding-window form applies
  int Qt_win = 0;      // its tile rows (multiple of 32 x kWinRows)
  int real_taps = 0;   // every channel of the group has real taps
  std::vector<int> batches;
};

class PolyEngine {
 public:
  // complex_taps: FIR semantics (taps used as complex numbers);
  // otherwise resampler semantics (only the real part of each tap is used,
  // falcon_dsp_polyphase_resampler.cc:286-299).
  // stream: where the initial history fill is enqueued (the engine's applies
  // on that stream follow it); nullptr: filled and synchronised on the device
  int init(uint32_t fs, const fdsp_channel_cfg* ch, uint32_t nch, bool complex_taps, cudaStream_t stream = nullptr);
  // device memory of later allocations from `pool` (set before init)
  void set_pool(DevPool* pool) { pool_ = pool; }
  cudaError_t dalloc(void** p, size_t bytes);
  void dfree(void* p);
  ~PolyEngine();

  int out_counts(uint64_t n_in, uint64_t* n_out) const;
  // Enqueue one streaming block on `stream`; outputs of channel c go to out[c]
  // (device pointers, capacity checked against cap[c] when cap != nullptr).
  // complex int16 input, converted to float inside the first kernel that
  // reads it (the staging of the FP32 kernel, the {hi, lo} split of the
  // tensor-core path, the history update)
  int apply_ci16(const int16_t* d_in, uint64_t n, float2* const* out, const uint64_t* cap, uint64_t* n_out,
                 cudaStream_t stream);
  int apply(const float2* d_in, uint64_t n, float2* const* out, const uint64_t* cap, uint64_t* n_out,
            cudaStream_t stream);
  void reset();

  uint32_t num_channels() const { return (uint32_t)chans_.size(); }
  uint32_t coeffs_per_phase(int c) const { return chans_[c].T; }
  uint32_t phase_of(int c) const { return classes_[cls_of_[c]].phase; }
  uint64_t xoffset_of(int c) const { return classes_[cls_of_[c]].xoffset; }
  uint64_t samples_since_reset() const { return abs0_; }
  int history_len() const { return H_; }
  int nb() const { return nb_; }
  // Kernel launches enqueued by the most recent apply.
  int kernel_launches_last() const { return launches_last_; }
  // Decimation groups computed by the tensor-core kernel in the most recent
  // apply (the others took the FP32 kernel).
  int tc_groups_last() const { return tc_groups_last_; }

  // Arithmetic of the filter-bank contraction: FDSP_PRECISION_FP32 (SIMT FP32)
  // or one of the split-precision tensor-core forms.
  int set_precision(int mode);
  int precision() const { return precision_; }
  // 1 when a tensor-core kernel hit its bounded wait since the last check
  // (after the caller has synchronised with the apply); clears the flag.
  int tc_error();
  // Polls before a tensor-core wait gives up (each suspends up to ~2 us), and
  // a test hook that makes the next launches' producer issue nothing.
  // Kernel timing (diagnostics): while on, applies launch directly (no graph)
  // and every filter-bank launch (tensor-core or FP32) is bracketed by CUDA
  // events on the apply's stream; read_profile synchronises and returns the
  // summed milliseconds and the launch count since profiling was enabled.
  void set_profile(bool on);
  int read_profile(double* ms, uint32_t* launches);
  void set_tc_exact_all(int on) { tc_exact_all_ = on; }
  void set_tc_wait(uint32_t polls, int hold) {
    tc_poll_ = polls ? polls : 1u;
    tc_hold_ = hold;
  }
  // Time every decimation group on an n-sample block and keep, per group,
  // the fastest FP32 tile height among {1/2, 1, 2, 4} x the default (the
  // tensor-core form runs every group of an apply in one launch and plans its
  // own tiles).  Resets the stream.
  int autotune(uint64_t n, cudaStream_t stream);
  int num_groups() const { return (int)groups_.size(); }
  // CUDA-graph replay of each apply's launch sequence (captured on the
  // caller's stream, the instantiated graph updated in place while the
  // sequence keeps its shape).  Applies on the legacy default stream, or on a
  // stream the caller is capturing, launch directly.
  void set_graph(bool on);
  // Completion hook of the next applies: after the last launch that writes
  // the outputs of some decimation groups, fn(ctx, channels, count, stream)
  // runs on the host with the channels whose outputs are then enqueued
  // complete on `stream` (the apply_host entry points start their
  // device-to-host copies from it while later groups compute).  Applies
  // launch directly (no graph) while a hook is set.
  using DoneFn = void (*)(void* ctx, const int* chans, int count, cudaStream_t stream);
  void set_done_hook(DoneFn fn, void* ctx) {
    done_fn_ = fn;
    done_ctx_ = ctx;
  }
  int graph_replays() const { return graph_replays_; }
  void group_info(int g, uint32_t* D, int* Qt, int* use_tc) const {
    *D = groups_[g].D;
    *Qt = groups_[g].Qt;
    *use_tc = use_tc_for(g) ? 1 : 0;
  }
  int group_tc_split(int g) const { return groups_[g].tc_split_used; }
  // Largest row split of every group's tensor-core form (1..32).
  int set_tc_split(int s) {
    if (s < 1 || s > 32) return FDSP_ERR_INVALID_ARG;
    for (auto& g : groups_) g.tc_split = s;
    return FDSP_OK;
  }

 private:
  template <int NB>
  int launch(const float2* d_in, uint64_t n, float2* const* out, cudaStream_t stream);
  int build_tc(int fmt);
  void free_tc();
  int launch_tc(const float2* d_in, uint64_t n, float2* const* out, const std::vector<int>& tc_groups,
                std::vector<int>& fallback, cudaStream_t stream);
  int precision_ = FDSP_PRECISION_FP32;
  int tc_fmt_ = 0;
  float2* d_ctaps_ = nullptr;          // FP32 modulated taps of every channel, [U][T] each
  const float2** d_ctab_ = nullptr;    // per channel: its taps in d_ctaps_
  uint2* d_xhl_ = nullptr;             // scratch: split input of the current apply
  size_t xhl_cap_ = 0;                 // samples
  uint8_t* d_bbuf_ = nullptr;          // scratch: B images of the current apply (a region per launch pack)
  TcLaunch* d_tcrec_ = nullptr;        // device copies of the launch records, one per pack (kTcMaxGroups)
  std::vector<cudaStream_t> side_;     // launch packs 1.. (beside pack 0 on the caller's stream)
  std::vector<cudaEvent_t> pack_ev_;   // [0]: the split is done; [1 + i]: side stream i joins
  size_t bbuf_cap_ = 0;
  int* h_err_ = nullptr;               // bounded-wait failures, mapped host memory
  int* d_err_ = nullptr;               // its device address
  uint32_t tc_poll_ = 1u << 20;
  int tc_hold_ = 0;
  int tc_exact_all_ = 0;
  int num_sms_ = 0;

  uint32_t fs_ = 0;
  bool complex_taps_ = false;
  int nb_ = 1;
  int H_ = 0;                       // history length (max T - 1)
  std::vector<EngineChannel> chans_;
  std::vector<EngineClass> classes_;
  std::vector<int> cls_of_;
  std::vector<EngineBatch> batches_;
  std::vector<EngineGroup> groups_;
  std::map<uint32_t, int> group_of_d_;
  NcoConst* d_nco_ = nullptr;
  float2* d_hist_[2] = {nullptr, nullptr};
  int hist_cur_ = 0;
  const short2* in16_ = nullptr;  // set for the duration of apply_ci16
  uint64_t abs0_ = 0;               // samples since reset at the next block
  int launches_last_ = 0;
  int tc_groups_last_ = 0;
  int force_ = -1;                     // autotuning: -1 chosen forms, 0 all FP32, 1 all tensor cores
  bool use_graph_ = false;
  cudaGraph_t graph_ = nullptr;        // the captured launch sequence behind graph_exec_
  cudaGraphExec_t graph_exec_ = nullptr;
  int graph_replays_ = 0;              // applies replayed as a graph since set_graph(true)
  // Kernel launches of an apply go through klaunch: direct (kmode_ 0), or
  // while the sequence is captured (1: each kernel node is recorded in
  // launch order), or for a replay (2: each launch's arguments are written
  // into its recorded node of graph_exec_ instead: no capture per apply).
  int kmode_ = 0;
  std::vector<cudaGraphNode_t> knodes_;
  std::vector<const void*> kfuncs_;    // the kernel of each recorded node (a replay needs the same sequence)
  size_t kcur_ = 0;
  bool kshape_ok_ = true;
 public:
  template <class... A>
  cudaError_t klaunch(const void* func, dim3 grid, dim3 block, size_t smem, cudaStream_t s, A&... args) {
    void* ptrs[] = {static_cast<void*>(&args)...};
    if (kmode_ == 2) {
      if (kcur_ >= knodes_.size() || kfuncs_[kcur_] != func) {
        kshape_ok_ = false;
        return cudaSuccess;
      }
      cudaKernelNodeParams p = {};
      p.func = const_cast<void*>(func);
      p.gridDim = grid;
      p.blockDim = block;
      p.sharedMemBytes = (unsigned)smem;
      p.kernelParams = ptrs;
      if (cudaGraphExecKernelNodeSetParams(graph_exec_, knodes_[kcur_++], &p) != cudaSuccess) {
        cudaGetLastError();
        kshape_ok_ = false;
      }
      return cudaSuccess;
    }
    cudaError_t e = cudaLaunchKernel(func, grid, block, ptrs, smem, s);
    if (e == cudaSuccess && kmode_ == 1) {
      cudaStreamCaptureStatus cs;
      const cudaGraphNode_t* deps = nullptr;
      size_t nd = 0;
      e = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &deps, nullptr, &nd);
      if (e == cudaSuccess && nd == 1) {
        knodes_.push_back(deps[0]);
        kfuncs_.push_back(func);
      } else {
        kshape_ok_ = false;  // (the replay needs one node per launch)
      }
      e = cudaSuccess;
    }
    return e;
  }
  // stream-order edges of an apply (skipped in a replay: they are graph edges)
  cudaError_t krecord(cudaEvent_t ev, cudaStream_t s) { return kmode_ == 2 ? cudaSuccess : cudaEventRecord(ev, s); }
  cudaError_t kwait(cudaStream_t s, cudaEvent_t ev) { return kmode_ == 2 ? cudaSuccess : cudaStreamWaitEvent(s, ev, 0); }
 private:
  bool use_tc_for(int eg) const;
  std::vector<cudaEvent_t> prof_ev_;   // autotuning: [2 g] / [2 g + 1] around group g
  std::vector<int> prof_hit_;          // group g launched in the timed apply
  bool kprof_ = false;                 // kernel timing on
  DoneFn done_fn_ = nullptr;           // completion hook (apply_host overlap)
  DevPool* pool_ = nullptr;            // device memory source (nullptr: cudaMalloc)
  void* done_ctx_ = nullptr;
  void notify_done(const std::vector<int>& egroups, cudaStream_t stream);
  std::vector<cudaEvent_t> kprof_ev_;  // (start, end) pairs of the timed launches
  size_t kprof_used_ = 0;
  cudaEvent_t kprof_event();           // next free event of the pool
};

// NCO constants of a (fs, f) pair, following falcon_dsp_freq_shift.cc:194-235.
NcoConst make_nco(uint32_t fs, int32_t f);

// Closed-form index bookkeeping of the reference's resampler loop.
uint64_t polyphase_out_count(uint32_t up, uint32_t down, uint32_t phase, uint64_t xoffset, uint64_t n);
void polyphase_advance(uint32_t up, uint32_t down, uint32_t& phase, uint64_t& xoffset, uint64_t n, uint64_t M);

static_assert(sizeof(PolyLaunch<8>) <= 32764, "engine launch must fit the kernel parameter block");

}  // namespace fdsp
