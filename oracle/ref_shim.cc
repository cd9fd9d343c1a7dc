/*
 * ref_shim.cc -- extern "C" shim over the reference's OWN CPU classes.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
 * the reference's unmodified CPU sources (read in place from the reference
 * checkout, never copied) into oracle/_ref/libfdsp_ref.so.  Tests use it to
 * pin the C restatement in fdsp_oracle.c, and bench.py's reference arm times
 * it as the reference CPU implementation of the path.
 *
 * Wrapped classes (reference paths):
 *   falcon_dsp_freq_shift              hdr/transform/falcon_dsp_freq_shift.h:84-121
 *   falcon_dsp_polyphase_resampler     hdr/transform/falcon_dsp_polyphase_resampler.h:168-195
 *   falcon_dsp_multi_rate_channelizer  hdr/transform/falcon_dsp_multi_rate_channelizer.h:94-134
 *   falcon_dsp_fir_filter              hdr/transform/falcon_dsp_fir_filter.h:119-140
 *   falcon_dsp_polar_discriminator     hdr/transform/falcon_dsp_polar_discriminator.h:97-114
 *   rat_approx                         hdr/utilities/falcon_dsp_utils.h
 */
#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>

#include "signals/falcon_dsp_fm_demod.h"
#include "transform/falcon_dsp_fir_filter.h"
#include "transform/falcon_dsp_iir_filter.h"
#include "transform/falcon_dsp_freq_shift.h"
#include "transform/falcon_dsp_multi_rate_channelizer.h"
#include "transform/falcon_dsp_polar_discriminator.h"
#include "transform/falcon_dsp_polyphase_resampler.h"
#include "utilities/falcon_dsp_utils.h"

using cf = std::complex<float>;

static std::vector<cf> to_vec(const float *p, uint64_t n)
{
    std::vector<cf> v(n);
    if (n) std::memcpy(v.data(), p, n * sizeof(cf));
    return v;
}

extern "C" {

/* ---- frequency shift ---------------------------------------------------- */
void *ref_freq_shift_new(uint32_t fs, int32_t f)
{
    auto *o = new falcon_dsp::falcon_dsp_freq_shift();
    if (!o->initialize(fs, f)) {
        delete o;
        return nullptr;
    }
    return o;
}
void ref_freq_shift_free(void *o) { delete static_cast<falcon_dsp::falcon_dsp_freq_shift *>(o); }
void ref_freq_shift_reset(void *o) { static_cast<falcon_dsp::falcon_dsp_freq_shift *>(o)->reset_state(); }
uint64_t ref_freq_shift_apply(void *o, const float *in, uint64_t n, float *out)
{
    auto vin = to_vec(in, n);
    std::vector<cf> vout;
    static_cast<falcon_dsp::falcon_dsp_freq_shift *>(o)->apply(vin, vout);
    if (!vout.empty()) std::memcpy(out, vout.data(), vout.size() * sizeof(cf));
    return vout.size();
}
void ref_freq_shift_params(uint32_t fs, int32_t f, uint32_t *rollover, double *omega)
{
    auto p = falcon_dsp::falcon_dsp_freq_shift::get_freq_shift_params(fs, f);
    *rollover = p.first;
    *omega = p.second;
}

/* ---- polyphase resampler ------------------------------------------------ */
void *ref_resampler_new(uint32_t up, uint32_t down, const float *coeffs, uint32_t ncoeffs)
{
    auto *o = new falcon_dsp::falcon_dsp_polyphase_resampler();
    if (!o->initialize(up, down, to_vec(coeffs, ncoeffs))) {
        delete o;
        return nullptr;
    }
    return o;
}
void ref_resampler_free(void *o) { delete static_cast<falcon_dsp::falcon_dsp_polyphase_resampler *>(o); }
void ref_resampler_reset(void *o) { static_cast<falcon_dsp::falcon_dsp_polyphase_resampler *>(o)->reset_state(); }
uint32_t ref_resampler_needed_out_count(void *o, uint32_t n)
{
    return static_cast<falcon_dsp::falcon_dsp_polyphase_resampler *>(o)->needed_out_count(n);
}
/* out must hold the loop's output count; returns that count. */
uint64_t ref_resampler_apply(void *o, const float *in, uint64_t n, float *out, uint64_t cap)
{
    auto vin = to_vec(in, n);
    std::vector<cf> vout;
    static_cast<falcon_dsp::falcon_dsp_polyphase_resampler *>(o)->apply(vin, vout);
    uint64_t w = vout.size() < cap ? vout.size() : cap;
    if (w) std::memcpy(out, vout.data(), w * sizeof(cf));
    return vout.size();
}

/* ---- multi-rate channelizer --------------------------------------------- */
void *ref_channelizer_new(uint32_t fs, uint32_t nch, const uint32_t *out_rate, const int64_t *shift,
                          const uint32_t *up, const uint32_t *down, const float *const *coeffs,
                          const uint32_t *ncoeffs)
{
    std::vector<multi_rate_channelizer_channel_s> chans(nch);
    for (uint32_t c = 0; c < nch; ++c) {
        chans[c].output_sample_rate_in_sps = out_rate[c];
        chans[c].freq_shift_in_hz = shift[c];
        chans[c].up_rate = up[c];
        chans[c].down_rate = down[c];
        chans[c].resample_filter_coeffs = to_vec(coeffs[c], ncoeffs[c]);
    }
    auto *o = new falcon_dsp::falcon_dsp_multi_rate_channelizer();
    if (!o->initialize(fs, chans)) {
        delete o;
        return nullptr;
    }
    return o;
}
void ref_channelizer_free(void *o) { delete static_cast<falcon_dsp::falcon_dsp_multi_rate_channelizer *>(o); }
void ref_channelizer_reset(void *o) { static_cast<falcon_dsp::falcon_dsp_multi_rate_channelizer *>(o)->reset_state(); }
/* out[c] must hold cap[c] samples; counts[c] receives the produced count. */
int ref_channelizer_apply(void *o, const float *in, uint64_t n, float *const *out, const uint64_t *cap,
                          uint64_t *counts, uint32_t nch)
{
    auto vin = to_vec(in, n);
    std::vector<std::vector<cf>> vout;
    bool ok = static_cast<falcon_dsp::falcon_dsp_multi_rate_channelizer *>(o)->apply(vin, vout);
    if (vout.size() != nch) return -1;
    for (uint32_t c = 0; c < nch; ++c) {
        counts[c] = vout[c].size();
        uint64_t w = vout[c].size() < cap[c] ? vout[c].size() : cap[c];
        if (w) std::memcpy(out[c], vout[c].data(), w * sizeof(cf));
    }
    return ok ? 0 : 1;
}

/* ---- FIR filter --------------------------------------------------------- */
void *ref_fir_new(const float *coeffs, uint32_t ncoeffs)
{
    auto taps = to_vec(coeffs, ncoeffs);
    return new falcon_dsp::falcon_dsp_fir_filter(taps);
}
void ref_fir_free(void *o) { delete static_cast<falcon_dsp::falcon_dsp_fir_filter *>(o); }
void ref_fir_reset(void *o) { static_cast<falcon_dsp::falcon_dsp_fir_filter *>(o)->reset_state(); }
uint64_t ref_fir_apply(void *o, const float *in, uint64_t n, float *out)
{
    auto vin = to_vec(in, n);
    std::vector<cf> vout;
    static_cast<falcon_dsp::falcon_dsp_fir_filter *>(o)->apply(vin, vout);
    if (!vout.empty()) std::memcpy(out, vout.data(), vout.size() * sizeof(cf));
    return vout.size();
}
/* int16 overload: interleaved int16 in/out (truncating cast back to int16). */
uint64_t ref_fir_apply_i16(void *o, const int16_t *in, uint64_t n, int16_t *out)
{
    std::vector<std::complex<int16_t>> vin(n), vout;
    if (n) std::memcpy(vin.data(), in, n * sizeof(std::complex<int16_t>));
    static_cast<falcon_dsp::falcon_dsp_fir_filter *>(o)->apply(vin, vout);
    if (!vout.empty()) std::memcpy(out, vout.data(), vout.size() * sizeof(std::complex<int16_t>));
    return vout.size();
}

/* ---- polar discriminator ------------------------------------------------ */
void *ref_polar_new(void) { return new falcon_dsp::falcon_dsp_polar_discriminator(); }
void ref_polar_free(void *o) { delete static_cast<falcon_dsp::falcon_dsp_polar_discriminator *>(o); }
void ref_polar_reset(void *o) { static_cast<falcon_dsp::falcon_dsp_polar_discriminator *>(o)->reset_state(); }
uint64_t ref_polar_apply(void *o, const float *in, uint64_t n, float *out)
{
    auto vin = to_vec(in, n);
    std::vector<float> vout;
    static_cast<falcon_dsp::falcon_dsp_polar_discriminator *>(o)->apply(vin, vout);
    if (!vout.empty()) std::memcpy(out, vout.data(), vout.size() * sizeof(float));
    return vout.size();
}

/* ---- IIR filter and FM demodulator ----------------------------------------- */
void *ref_iir_new(const float *b, uint32_t nb, const float *a, uint32_t na)
{
    auto vb = to_vec(b, nb), va = to_vec(a, na);
    auto *o = new falcon_dsp::falcon_dsp_iir_filter();
    if (!o->initialize(vb, va)) { delete o; return nullptr; }
    return o;
}
void ref_iir_free(void *o) { delete static_cast<falcon_dsp::falcon_dsp_iir_filter *>(o); }
void ref_iir_reset(void *o) { static_cast<falcon_dsp::falcon_dsp_iir_filter *>(o)->reset_state(); }
uint64_t ref_iir_apply(void *o, const float *in, uint64_t n, float *out)
{
    auto vin = to_vec(in, n);
    std::vector<cf> vout;
    static_cast<falcon_dsp::falcon_dsp_iir_filter *>(o)->apply(vin, vout);
    if (!vout.empty()) std::memcpy(out, vout.data(), vout.size() * sizeof(cf));
    return vout.size();
}

void *ref_fm_new(uint32_t fs, int32_t offset, float tau)
{
    auto *o = new falcon_dsp::falcon_dsp_fm_demodulator();
    if (!o->initialize(fs, offset, tau)) { delete o; return nullptr; }
    return o;
}
void ref_fm_free(void *o) { delete static_cast<falcon_dsp::falcon_dsp_fm_demodulator *>(o); }
void ref_fm_reset(void *o) { static_cast<falcon_dsp::falcon_dsp_fm_demodulator *>(o)->reset_state(); }
/* demod_mono; returns the int16 count (the reference's bool is count > 0) */
uint64_t ref_fm_demod_mono(void *o, const float *in, uint64_t n, int16_t *out, uint64_t cap)
{
    auto vin = to_vec(in, n);
    std::vector<int16_t> vout;
    static_cast<falcon_dsp::falcon_dsp_fm_demodulator *>(o)->demod_mono(vin, vout);
    if (!vout.empty()) std::memcpy(out, vout.data(), std::min<uint64_t>(vout.size(), cap) * sizeof(int16_t));
    return vout.size();
}

/* ---- utilities ---------------------------------------------------------- */
void ref_rat_approx(double f, int64_t md, int64_t *num, int64_t *den) { falcon_dsp::rat_approx(f, md, *num, *den); }

/* get_resample_fir_params over the reference's own predefined table: returns
 * the coefficient count (0 when the reference returns false); real parts into
 * `re` when cap allows. */
uint32_t ref_get_resample_fir_params(uint32_t in_sps, uint32_t out_sps, int32_t taps, uint32_t source, uint32_t *up,
                                     uint32_t *down, float *re, uint32_t cap)
{
    std::vector<cf> h;
    if (!falcon_dsp::get_resample_fir_params(in_sps, out_sps, static_cast<filter_taps_e>(taps),
                                             static_cast<filter_source_type_e>(source), *up, *down, h))
        return 0;
    for (size_t i = 0; i < h.size() && i < cap; ++i) re[i] = h[i].real();
    return static_cast<uint32_t>(h.size());
}

} /* extern "C" */
