/*
 * fdsp_c.h -- C ABI of libfalcon_dsp_gb300, the GB300 (sm_103a) implementation
 * of libfalcon_dsp's multi-rate channelizer path.
 *
 * Conventions
 *   - Every entry point returns an int status: FDSP_OK (0) or a negative
 *     fdsp_status code.  Nothing here prints or calls exit(); the reference's
 *     convention of gpuAssert -> exit(code)
 *     (src/utilities/falcon_dsp_cuda_utils.cu:84-94) is replaced by codes.
 *   - Complex samples are fdsp_cf32 {re, im}: the memory layout of
 *     std::complex<float>, cuFloatComplex and float2.
 *   - *_apply functions take DEVICE pointers and a CUDA stream, enqueue their
 *     kernels on that stream and return without synchronising.  All streaming
 *     state (filter history, NCO counter, resampler phase and offset) lives
 *     in the handle and on the device, so consecutive applies on one stream
 *     continue the stream exactly as the reference's apply/apply/... does.
 *   - *_apply_host functions take HOST pointers (pinned or pageable) and do
 *     the host->device copy, the kernels and the device->host copy on the
 *     given stream, then synchronise it: the drop-in for the reference's
 *     std::vector in / std::vector out apply().
 *   - Output counts are computed on the host with exact integer arithmetic
 *     and equal, sample for sample, what the reference CPU loop emits
 *     (src/transform/falcon_dsp_polyphase_resampler.cc:256-319).
 *   - A handle is not thread safe; use one per host thread (the reference's
 *     per-object mutex never locked anything, see
 *     src/transform/falcon_dsp_polyphase_resampler.cc:258).
 */
#ifndef FDSP_C_H
#define FDSP_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *fdsp_stream_t; /* same type as cudaStream_t; NULL = legacy default stream */

typedef struct {
    float re;
    float im;
} fdsp_cf32;

enum fdsp_status {
    FDSP_OK = 0,
    FDSP_ERR_INVALID_ARG = -1,     /* bad pointer, size or configuration */
    FDSP_ERR_NOT_INITIALIZED = -2, /* NULL handle */
    FDSP_ERR_ALLOC = -3,           /* host or device allocation failed */
    FDSP_ERR_CUDA = -4,            /* a CUDA runtime call failed; see fdsp_last_cuda_error() */
    FDSP_ERR_CAPACITY = -5,        /* an output buffer is smaller than the output count */
    FDSP_ERR_UNSUPPORTED = -6,     /* configuration outside this build's limits */
    FDSP_ERR_NO_DEVICE = -7,       /* no CUDA device is visible */
    FDSP_ERR_NOT_FOUND = -8,       /* no predefined filter for the requested key */
    FDSP_ERR_TIMEOUT = -9          /* a tensor-core kernel's bounded wait gave up: the outputs of the
                                      applies since the last status check are incomplete */
};

/* Short text for a status code (static storage). */
const char *fdsp_status_string(int status);
/* cudaError_t value behind the last FDSP_ERR_CUDA returned on this thread. */
int fdsp_last_cuda_error(void);
/* Library version, major*10000 + minor*100 + patch. */
int fdsp_version(void);

/* ------------------------------------------------------------------------
 * Helpers (host only, no GPU needed)
 * ---------------------------------------------------------------------- */

/* Replaces falcon_dsp_freq_shift::get_freq_shift_params
 * (src/transform/falcon_dsp_freq_shift.cc:194-235): rollover index R and
 * angular frequency omega of a shift of f Hz at fs samples/s. */
int fdsp_freq_shift_params(uint32_t fs, int32_t f, uint32_t *rollover, double *omega);

/* Replaces falcon_dsp::rat_approx (src/utilities/falcon_dsp_utils.cc:231-294). */
int fdsp_rat_approx(double f, int64_t max_denom, int64_t *num, int64_t *den);

/* ------------------------------------------------------------------------
 * FM mono demodulator: falcon_dsp_fm_demodulator_cuda
 * (hdr/signals/falcon_dsp_fm_demod_cuda.h:83-104,
 * src/signals/falcon_dsp_fm_demod_cuda.cu) with every stage on the device:
 * channelizer (NCO to signal_offset_hz, resample to 228 kS/s with the
 * predefined REMEZ-64 filter) -> polar discriminator -> de-emphasis
 * (one-pole IIR, 75 us or 50 us taps of src/signals/falcon_dsp_fm_demod.cc)
 * -> mono decimator to 45.6 kS/s (REMEZ-64) -> x * (10000 / max |x| of the
 * call) truncated to int16.
 *   - create: deemphasis_tau must be 75e-6f or 50e-6f (else
 *     FDSP_ERR_INVALID_ARG) and the table must hold input_sample_rate ->
 *     228000 (else FDSP_ERR_NOT_FOUND), as the reference's initialize().
 *   - apply: int16 audio for the call; the discriminator's first call emits
 *     one sample less, and every stage's state carries to the next call.
 * ---------------------------------------------------------------------- */
#define FDSP_FM_RADIO_SAMPLE_RATE 228000u
#define FDSP_FM_AUDIO_SAMPLE_RATE 45600u
typedef struct fdsp_fm_demod fdsp_fm_demod;

int fdsp_fm_demod_create(uint32_t input_sample_rate, int32_t signal_offset_hz, float deemphasis_tau,
                         fdsp_fm_demod **out);
int fdsp_fm_demod_destroy(fdsp_fm_demod *h);
int fdsp_fm_demod_reset(fdsp_fm_demod *h);
int fdsp_fm_demod_out_count(const fdsp_fm_demod *h, uint64_t n_in, uint64_t *n_out);
int fdsp_fm_demod_apply(fdsp_fm_demod *h, const fdsp_cf32 *d_in, uint64_t n_in, int16_t *d_out, uint64_t out_cap,
                        uint64_t *n_out, fdsp_stream_t stream);
int fdsp_fm_demod_apply_host(fdsp_fm_demod *h, const fdsp_cf32 *h_in, uint64_t n_in, int16_t *h_out,
                             uint64_t out_cap, uint64_t *n_out, fdsp_stream_t stream);

/* ------------------------------------------------------------------------
 * Resampling filter design (host only: no device, no stream).
 *
 * fdsp_get_resample_fir_params replaces falcon_dsp::get_resample_fir_params
 * (src/transform/falcon_dsp_fir_filter.cc:111-130): the predefined
 * anti-alias lowpass for (input rate, output rate, taps, source), with its
 * up/down rates.  taps: 16, 32, 64, 128, 256 or -1 (FILTER_TAPS_OPTIMAL);
 * source: 0 REMEZ, 1 FIRLS (hdr/transform/falcon_dsp_predefined_fir_filter.h:
 * 63-78).  The table is built with the library, by the reference's published
 * recipe; a missing key returns FDSP_ERR_NOT_FOUND (the reference returns
 * false).  *n_coeffs is always set; coeffs NULL or cap < *n_coeffs returns
 * FDSP_ERR_CAPACITY, so a first call with coeffs NULL sizes the buffer.
 *
 * fdsp_design_resample_firls designs the same FIRLS lowpass for ANY rate
 * pair: up/down from out/in, num_taps made odd, least-squares lowpass with
 * edge 1/max(up, down) of Nyquist (closed form), scaled by up, Kaiser window
 * (beta; the table uses 5).  Coefficients at full float precision (the table
 * rounds them to 8 decimals).
 * ---------------------------------------------------------------------- */
int fdsp_get_resample_fir_params(uint32_t in_sps, uint32_t out_sps, int32_t taps, uint32_t source, uint32_t *up_rate,
                                 uint32_t *down_rate, fdsp_cf32 *coeffs, uint32_t cap, uint32_t *n_coeffs);
int fdsp_design_resample_firls(uint32_t in_sps, uint32_t out_sps, uint32_t num_taps, double kaiser_beta,
                               uint32_t *up_rate, uint32_t *down_rate, fdsp_cf32 *coeffs, uint32_t cap,
                               uint32_t *n_coeffs);

/* Index bookkeeping of one resampler apply, in closed form: for n_in inputs
 * from state (phase, x_offset), the number of outputs the reference loop
 * emits and the state it leaves (the recurrence of
 * src/transform/falcon_dsp_polyphase_resampler.cc:267-312).  Host only. */
int fdsp_polyphase_advance(uint32_t up_rate, uint32_t down_rate, uint32_t phase, uint64_t x_offset, uint64_t n_in,
                           uint64_t *n_out, uint32_t *phase_out, uint64_t *x_offset_out);

/* ------------------------------------------------------------------------
 * Multi-rate channelizer: per channel NCO shift then polyphase resampling,
 * fused in one kernel launch over all channels.
 * Replaces falcon_dsp_multi_rate_channelizer_cuda
 * (hdr/transform/falcon_dsp_multi_rate_channelizer_cuda.h:73-167,
 *  src/transform/falcon_dsp_multi_rate_channelizer_cuda.cu:87-576) and its
 * CPU twin (hdr/transform/falcon_dsp_multi_rate_channelizer.h:70-134).
 * ---------------------------------------------------------------------- */

/* Field for field multi_rate_channelizer_channel_s
 * (hdr/transform/falcon_dsp_multi_rate_channelizer.h:70-77), with the tap
 * vector as a host pointer + count. */
typedef struct {
    uint32_t output_sample_rate_in_sps; /* informational, as in the reference */
    int64_t freq_shift_in_hz;           /* truncated to int32 like the reference's NCO */
    uint32_t up_rate;
    uint32_t down_rate;
    const fdsp_cf32 *resample_filter_coeffs; /* host pointer; only the real parts are used */
    uint32_t num_coeffs;
} fdsp_channel_cfg;

typedef struct fdsp_channelizer fdsp_channelizer;

/* Arithmetic of the channelizer's filter-bank contraction. */
enum fdsp_precision {
    FDSP_PRECISION_FP32 = 0,     /* plain FP32 complex arithmetic on the SIMT cores (default) */
    FDSP_PRECISION_FP16X3 = 1,   /* tensor cores: FP16 hi+lo split of data and taps, (hi+lo)(hi+lo), FP32 accumulate */
    FDSP_PRECISION_BF16X3 = 2    /* tensor cores: BF16 hi+lo split, (hi+lo)(hi+lo), FP32 accumulate */
};

/* initialize(input_sample_rate, channels)
 * (src/transform/falcon_dsp_multi_rate_channelizer_cuda.cu:320-372). */
int fdsp_channelizer_create(uint32_t input_sample_rate, const fdsp_channel_cfg *channels, uint32_t num_channels,
                            fdsp_channelizer **out);
int fdsp_channelizer_destroy(fdsp_channelizer *h);
/* reset_state() (src/transform/falcon_dsp_multi_rate_channelizer.cc:166-173). */
int fdsp_channelizer_reset(fdsp_channelizer *h);
int fdsp_channelizer_num_channels(const fdsp_channelizer *h, uint32_t *n);
/* Output count of every channel for the next block of n_in samples. */
int fdsp_channelizer_out_count(const fdsp_channelizer *h, uint64_t n_in, uint64_t *n_out);
/* apply(in, out) on device buffers: d_out[c] (capacity out_cap[c], may be
 * NULL to skip the check) receives n_out[c] samples. */
int fdsp_channelizer_apply(fdsp_channelizer *h, const fdsp_cf32 *d_in, uint64_t n_in, fdsp_cf32 *const *d_out,
                           const uint64_t *out_cap, uint64_t *n_out, fdsp_stream_t stream);
/* Select the arithmetic of later applies (fdsp_precision).  Under a
 * tensor-core precision every decimation group runs in one persistent
 * tensor-core launch (any taps per phase); groups beyond that launch's record
 * limits keep the FP32 form. */
int fdsp_channelizer_set_precision(fdsp_channelizer *h, int precision);
/* Error status of the applies enqueued so far (no counterpart in the
 * reference, whose CUDA errors exit the process,
 * src/utilities/falcon_dsp_cuda_utils.cu:84-94): synchronises `stream`, then
 * returns FDSP_ERR_TIMEOUT when a tensor-core kernel's bounded wait gave up
 * since the last check (and clears that record), a CUDA error as
 * FDSP_ERR_CUDA, else FDSP_OK.  The *_apply_host entry points check it
 * themselves before returning. */
int fdsp_channelizer_status(fdsp_channelizer *h, fdsp_stream_t stream);
/* Bounded waits of the tensor-core kernel: a wait gives up after max_polls
 * polls (each suspends the waiting thread for up to ~2 us; default 2^20).
 * withhold_copies != 0 makes later launches issue no operand copies, so every
 * wait runs out: a test hook for the timeout path, never for production. */
int fdsp_channelizer_set_tc_wait(fdsp_channelizer *h, uint32_t max_polls, int withhold_copies);
/* Test hook of the tensor-core kernel's exact rotation pass: on != 0 makes
 * every output of later applies take it (as slots whose row stride spans
 * more than the NCO rollover do), instead of only the windows that straddle
 * the rollover.  Results stay within the tensor-core bound; slower. */
int fdsp_channelizer_set_tc_exact_all(fdsp_channelizer *h, int on);
/* Kernel timing (diagnostics, no counterpart in the reference): while
 * enabled, applies launch directly (no graph) and each filter-bank launch
 * (tensor-core or FP32 kernel) is bracketed by CUDA events on the apply's
 * stream (the tensor-core launch packs, concurrent otherwise, then run one
 * after another on that stream); enabling restarts the record.  read:
 * synchronises and returns the summed milliseconds and the number of timed
 * launches. */
int fdsp_channelizer_profile(fdsp_channelizer *h, int enable);
int fdsp_channelizer_profile_read(fdsp_channelizer *h, double *ms, uint32_t *launches);
/* Kernel launches the most recent apply enqueued (diagnostics, profiling). */
int fdsp_channelizer_kernel_launches(const fdsp_channelizer *h, uint32_t *n);
/* Decimation groups that the most recent apply computed on the tensor-core
 * kernel; the rest of the groups took the FP32 kernel (configurations outside
 * the tensor-core kernel's limits, or precision FP32).  No counterpart in the
 * reference, which has one arithmetic path. */
int fdsp_channelizer_tc_groups(const fdsp_channelizer *h, uint32_t *n);
/* Autotuner (no counterpart in the reference): times every decimation group
 * (channels sharing a down rate) on an n_in-sample block on `stream` and keeps,
 * per group, the fastest FP32 tile height.  It allocates scratch for the
 * trial, synchronises the stream and resets the streaming state; call it
 * before the first apply. */
int fdsp_channelizer_autotune(fdsp_channelizer *h, uint64_t n_in, fdsp_stream_t stream);
/* Decimation groups of the channelizer and, per group, its down rate, FP32
 * tile height (output rows per CTA) and whether applies ask for the
 * tensor-core form for it. */
int fdsp_channelizer_num_groups(const fdsp_channelizer *h, uint32_t *n);
/* CUDA-graph replay of every later apply (no counterpart in the reference):
 * the first apply's launches are captured on the caller's stream and
 * instantiated once; later applies write their kernels' arguments into that
 * graph's nodes (no capture) and replay it, and a different launch sequence
 * is captured afresh.  Applies on the legacy default stream (NULL), or on a
 * stream the caller is itself capturing, launch directly.  `replays` (may be
 * NULL) receives the applies replayed since graphs were enabled. */
int fdsp_channelizer_set_graph(fdsp_channelizer *h, int enable);
int fdsp_channelizer_graph_replays(const fdsp_channelizer *h, uint32_t *replays);
int fdsp_channelizer_group_info(const fdsp_channelizer *h, uint32_t group, uint32_t *down_rate, uint32_t *tile_rows,
                                int *tensor_core);
/* Row split S of a group's last tensor-core launch (1 = none): rows
 * j = S i + b run as S output streams whose rows are S x down_rate apart, so
 * one tile of input rows feeds S times the channel columns (odd down rates
 * always split by 2 or more: the input rows of a tile must start 16 bytes
 * apart). */
int fdsp_channelizer_group_tc_split(const fdsp_channelizer *h, uint32_t group, uint32_t *split);
/* Largest row split (1..32, default 32) of every group's tensor-core form;
 * the split used is the largest power of two up to it whose streams still
 * fit one 32-stream product and whose windows grow by at most a quarter. */
int fdsp_channelizer_set_tc_split(fdsp_channelizer *h, uint32_t max_split);
/* apply(in, out) on host buffers (copies in, computes, copies out, syncs). */
int fdsp_channelizer_apply_host(fdsp_channelizer *h, const fdsp_cf32 *h_in, uint64_t n_in, fdsp_cf32 *const *h_out,
                                const uint64_t *out_cap, uint64_t *n_out, fdsp_stream_t stream);
/* int16 front end: n_in complex int16 samples (interleaved I, Q: the layout
 * of std::complex<int16_t> and of the reference's "<2h" sample files,
 * src/utilities/falcon_dsp_utils.cc:534-742), converted to float inside the
 * first kernel that reads them, so the block crosses HBM (and PCIe) at 4
 * bytes a sample.  Outputs as fdsp_channelizer_apply; equal to converting
 * first, as the reference's int16 overloads do (freq_shift.cc:133-162). */
int fdsp_channelizer_apply_ci16(fdsp_channelizer *h, const int16_t *d_in, uint64_t n_in, fdsp_cf32 *const *d_out,
                                const uint64_t *out_cap, uint64_t *n_out, fdsp_stream_t stream);
int fdsp_channelizer_apply_ci16_host(fdsp_channelizer *h, const int16_t *h_in, uint64_t n_in,
                                     fdsp_cf32 *const *h_out, const uint64_t *out_cap, uint64_t *n_out,
                                     fdsp_stream_t stream);

/* ------------------------------------------------------------------------
 * Polyphase resampler (single channel, no shift).
 * Replaces falcon_dsp_polyphase_resampler_cuda
 * (hdr/transform/falcon_dsp_polyphase_resampler_cuda.h:187-226) and the CPU
 * class it derives from (hdr/transform/falcon_dsp_polyphase_resampler.h:168-195).
 * Semantics are the CPU loop's (carried xOffset and phase across blocks).
 * ---------------------------------------------------------------------- */
typedef struct fdsp_resampler fdsp_resampler;

int fdsp_resampler_create(uint32_t up_rate, uint32_t down_rate, const fdsp_cf32 *coeffs, uint32_t num_coeffs,
                          fdsp_resampler **out);
int fdsp_resampler_destroy(fdsp_resampler *h);
int fdsp_resampler_reset(fdsp_resampler *h);
/* coeffs_per_phase() (hdr/transform/falcon_dsp_polyphase_resampler.h:185). */
int fdsp_resampler_coeffs_per_phase(const fdsp_resampler *h, uint32_t *cpp);
/* Exact output count of the next apply of n_in samples. */
int fdsp_resampler_out_count(const fdsp_resampler *h, uint64_t n_in, uint64_t *n_out);
/* needed_out_count() exactly as the reference computes it
 * (src/transform/falcon_dsp_polyphase_resampler.cc:204-228). */
int fdsp_resampler_needed_out_count(const fdsp_resampler *h, uint32_t n_in, uint32_t *n_out);
/* Current (coeff_phase, xOffset) streaming state. */
int fdsp_resampler_state(const fdsp_resampler *h, uint32_t *coeff_phase, uint64_t *x_offset);
int fdsp_resampler_apply(fdsp_resampler *h, const fdsp_cf32 *d_in, uint64_t n_in, fdsp_cf32 *d_out, uint64_t out_cap,
                         uint64_t *n_out, fdsp_stream_t stream);
int fdsp_resampler_apply_host(fdsp_resampler *h, const fdsp_cf32 *h_in, uint64_t n_in, fdsp_cf32 *h_out,
                              uint64_t out_cap, uint64_t *n_out, fdsp_stream_t stream);
/* complex int16 input (see fdsp_channelizer_apply_ci16), complex64 output */
int fdsp_resampler_apply_ci16(fdsp_resampler *h, const int16_t *d_in, uint64_t n_in, fdsp_cf32 *d_out,
                              uint64_t out_cap, uint64_t *n_out, fdsp_stream_t stream);
/* Arithmetic of later applies (fdsp_precision; no counterpart in the
 * reference): the tensor-core forms run the filter as one persistent
 * tcgen05 launch for any taps per phase, e.g. a long FIR followed by a
 * decimation (up = 1).  1 in *n when the last apply ran on the tensor cores.
 * fdsp_resampler_status: as fdsp_channelizer_status. */
int fdsp_resampler_set_precision(fdsp_resampler *h, int precision);
int fdsp_resampler_tc_groups(const fdsp_resampler *h, uint32_t *n);
int fdsp_resampler_status(fdsp_resampler *h, fdsp_stream_t stream);

/* ------------------------------------------------------------------------
 * One-shot polyphase resampling that allocates nothing.
 * No counterpart in the reference: it is the result of
 * fdsp_resampler_create + fdsp_resampler_apply + fdsp_resampler_destroy on a
 * fresh resampler (same output count, outputs equal within FP32 rounding),
 * for callers that may not allocate once they run: real-time receive loops,
 * where a cudaMalloc/cudaFree would synchronise the device and stall the
 * other streams, and plug-ins whose host owns the device-memory budget.
 *
 *   - The taps go into one fixed device array of
 *     FDSP_RESAMPLE_STATIC_MAX_COEFFS complex values (64 KiB) per device;
 *     num_coeffs above that returns FDSP_ERR_UNSUPPORTED.  As in the
 *     resampler, only the real parts of the taps are used.
 *   - The first call on a device (device current) looks up that array's
 *     address; make it before any stream capture begins.
 *   - coeffs may be a host or a device pointer; it is copied in stream
 *     order, so pinned or device taps must stay unchanged until the stream
 *     reaches the call.  Inside a CUDA graph capture only device or pinned
 *     taps work: a copy from pageable host memory cannot be captured.
 *   - The array's address is looked up once per device and kept for the
 *     life of the process; calls must not span a cudaDeviceReset.
 *   - The array is shared by every call on the device and keeps the last
 *     call's taps: calls that overlap in time (different streams or host
 *     threads without ordering) race on it.  Serialise them.
 *   - d_in and d_out are device buffers; out_cap < the output count returns
 *     FDSP_ERR_CAPACITY.  Enqueues on `stream` and returns.
 * ---------------------------------------------------------------------- */
#define FDSP_RESAMPLE_STATIC_MAX_COEFFS 8192u

int fdsp_resample_static(uint32_t up_rate, uint32_t down_rate, const fdsp_cf32 *coeffs, uint32_t num_coeffs,
                         const fdsp_cf32 *d_in, uint64_t n_in, fdsp_cf32 *d_out, uint64_t out_cap, uint64_t *n_out,
                         fdsp_stream_t stream);

/* ------------------------------------------------------------------------
 * NCO frequency shift, one or many channels over one input.
 * Replaces falcon_dsp_freq_shift_cuda (hdr/transform/falcon_dsp_freq_shift_cuda.h:187-212,
 * src/transform/falcon_dsp_freq_shift_cuda.cu:275-488) and the CPU class
 * (hdr/transform/falcon_dsp_freq_shift.h:84-121).
 * ---------------------------------------------------------------------- */
typedef struct fdsp_freq_shift fdsp_freq_shift;

int fdsp_freq_shift_create(uint32_t input_sample_rate, const int32_t *shifts_hz, uint32_t num_channels,
                           fdsp_freq_shift **out);
int fdsp_freq_shift_destroy(fdsp_freq_shift *h);
int fdsp_freq_shift_reset(fdsp_freq_shift *h);
int fdsp_freq_shift_num_channels(const fdsp_freq_shift *h, uint32_t *n);
/* Rollover-reduced sample counter of channel c (the reference's
 * m_samples_handled / num_samples_handled). */
int fdsp_freq_shift_counter(const fdsp_freq_shift *h, uint32_t c, uint64_t *counter);
/* d_out[c] receives n_in shifted samples for each channel c. */
int fdsp_freq_shift_apply(fdsp_freq_shift *h, const fdsp_cf32 *d_in, uint64_t n_in, fdsp_cf32 *const *d_out,
                          fdsp_stream_t stream);
int fdsp_freq_shift_apply_host(fdsp_freq_shift *h, const fdsp_cf32 *h_in, uint64_t n_in, fdsp_cf32 *const *h_out,
                               fdsp_stream_t stream);
/* int16 overload (src/transform/falcon_dsp_freq_shift.cc:133-162): complex
 * int16 in, converted on load; complex int16 out, truncated toward zero. */
int fdsp_freq_shift_apply_ci16(fdsp_freq_shift *h, const int16_t *d_in, uint64_t n_in, int16_t *const *d_out,
                               fdsp_stream_t stream);
int fdsp_freq_shift_apply_ci16_host(fdsp_freq_shift *h, const int16_t *h_in, uint64_t n_in, int16_t *const *h_out,
                                    fdsp_stream_t stream);

/* ------------------------------------------------------------------------
 * FIR filter with complex taps, output length = input length.
 * Replaces falcon_dsp_fir_filter_cuda (hdr/transform/falcon_dsp_fir_filter_cuda.h:113-138,
 * src/transform/falcon_dsp_fir_filter_cuda.cu:102-373) and the CPU class
 * (hdr/transform/falcon_dsp_fir_filter.h:119-140).
 * ---------------------------------------------------------------------- */
typedef struct fdsp_fir fdsp_fir;

int fdsp_fir_create(const fdsp_cf32 *coeffs, uint32_t num_coeffs, fdsp_fir **out);
int fdsp_fir_destroy(fdsp_fir *h);
int fdsp_fir_reset(fdsp_fir *h);
int fdsp_fir_apply(fdsp_fir *h, const fdsp_cf32 *d_in, uint64_t n_in, fdsp_cf32 *d_out, fdsp_stream_t stream);
int fdsp_fir_apply_host(fdsp_fir *h, const fdsp_cf32 *h_in, uint64_t n_in, fdsp_cf32 *h_out, fdsp_stream_t stream);
/* FDSP_PRECISION_FP32 (default) or the tensor-core split-precision forms
 * FDSP_PRECISION_FP16X3 / FDSP_PRECISION_BF16X3: the FIR as a Toeplitz
 * product on tcgen05 (32 consecutive outputs per row of a tile: 32 output
 * streams whose windows start one sample apart), any number of taps. */
int fdsp_fir_set_precision(fdsp_fir *h, int precision);
/* 1 when the last apply ran on the tensor-core kernel, else 0 */
int fdsp_fir_tc_groups(const fdsp_fir *h, uint32_t *n);
/* as fdsp_channelizer_status */
int fdsp_fir_status(fdsp_fir *h, fdsp_stream_t stream);
/* int16 overload (src/transform/falcon_dsp_fir_filter.cc:151-175): complex
 * int16 in (converted inside the filter kernel), complex int16 out
 * (truncated toward zero). */
int fdsp_fir_apply_ci16(fdsp_fir *h, const int16_t *d_in, uint64_t n_in, int16_t *d_out, fdsp_stream_t stream);
int fdsp_fir_apply_ci16_host(fdsp_fir *h, const int16_t *h_in, uint64_t n_in, int16_t *h_out, fdsp_stream_t stream);

/* ------------------------------------------------------------------------
 * Polar discriminator (FM demodulation core): out[n] = arg(x[n] conj(x[n-1])).
 * Replaces falcon_dsp_polar_discriminator
 * (hdr/transform/falcon_dsp_polar_discriminator.h:97-114,
 *  src/transform/falcon_dsp_polar_discriminator.cc:134-171), which has no
 * CUDA version in the reference.  The first apply after create/reset emits
 * n_in - 1 values, later ones n_in.
 * ---------------------------------------------------------------------- */
typedef struct fdsp_polar fdsp_polar;

int fdsp_polar_create(fdsp_polar **out);
int fdsp_polar_destroy(fdsp_polar *h);
int fdsp_polar_reset(fdsp_polar *h);
int fdsp_polar_out_count(const fdsp_polar *h, uint64_t n_in, uint64_t *n_out);
int fdsp_polar_apply(fdsp_polar *h, const fdsp_cf32 *d_in, uint64_t n_in, float *d_out, uint64_t *n_out,
                     fdsp_stream_t stream);
int fdsp_polar_apply_host(fdsp_polar *h, const fdsp_cf32 *h_in, uint64_t n_in, float *h_out, uint64_t *n_out,
                          fdsp_stream_t stream);

/* ------------------------------------------------------------------------
 * Streaming server: many channelizer streams (jobs) served concurrently on
 * one GPU.  No counterpart in the reference, whose classes run one blocking
 * apply per object.
 *
 *   - fdsp_server_open admits a stream (its channel set, input rate, largest
 *     block length, fdsp_precision) when its device footprint fits the
 *     remaining budget and fewer than max_active streams are open; otherwise
 *     it returns FDSP_ERR_CAPACITY and the caller retries after a close.  The
 *     stream's filter history, resampler phase and NCO counter stay on the
 *     device between its blocks.
 *   - fdsp_server_submit enqueues one block on the stream's own CUDA stream
 *     (host->device copy, channelizer apply, device->host copies into h_out;
 *     a single copy when the h_out regions lie back to back, each at least
 *     ceil(max_block * up / down) + 2 samples as given in out_cap)
 *     and returns a ticket at once; blocks of one stream run in order, blocks
 *     of different streams overlap on the GPU.  Host buffers should be pinned
 *     and must stay valid until the ticket completes.
 *   - fdsp_server_poll reports a ticket once, when done: its output counts and
 *     its latency (submit to completion of the last device->host copy);
 *     fdsp_server_wait_any hands out completed tickets in completion order.
 *   - fdsp_server_stats: p50/p99/p999 block latency (ms), blocks and output
 *     samples completed since the last reset, bytes reserved, open streams.
 * A server is not thread safe: drive it from one host thread.
 * ---------------------------------------------------------------------- */
typedef struct fdsp_server fdsp_server;

int fdsp_server_create(uint64_t budget_bytes, uint32_t max_active, fdsp_server **out);
int fdsp_server_destroy(fdsp_server *s);
int fdsp_server_open(fdsp_server *s, uint32_t input_sample_rate, const fdsp_channel_cfg *channels,
                     uint32_t num_channels, uint64_t max_block, int precision, uint32_t *stream_id);
int fdsp_server_submit(fdsp_server *s, uint32_t stream_id, const fdsp_cf32 *h_in, uint64_t n_in,
                       fdsp_cf32 *const *h_out, const uint64_t *out_cap, uint64_t *ticket);
int fdsp_server_poll(fdsp_server *s, uint64_t ticket, int *done, uint64_t *n_out, double *latency_ms);
/* Next completed ticket in completion order (waits up to timeout_us; *ticket
 * = 0 when none completed); then fdsp_server_poll reports it. */
int fdsp_server_wait_any(fdsp_server *s, uint32_t timeout_us, uint64_t *ticket);
int fdsp_server_close(fdsp_server *s, uint32_t stream_id);
int fdsp_server_stats(fdsp_server *s, double *p50_ms, double *p99_ms, double *p999_ms, uint64_t *blocks,
                      uint64_t *outputs, uint64_t *used_bytes, uint32_t *active);
int fdsp_server_reset_stats(fdsp_server *s);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* FDSP_C_H */
