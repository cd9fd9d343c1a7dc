/*
 * Base class of the frequency-shift drop-in, with the reference CPU class's
 * name and virtual interface (hdr/transform/falcon_dsp_freq_shift.h:98-121):
 * get_freq_shift_params(), initialize(fs, shift) once, reset_state(),
 * apply() for complex float and complex int16 blocks.  Callers that hold a
 * falcon_dsp_freq_shift& or * compile unchanged.  There is no CPU
 * implementation behind it: y[n] = x[n] e^{j w (n mod R)} runs on the GPU
 * through the C ABI, with the sample counter carried across applies; the
 * int16 overload converts in and truncates out like
 * src/transform/falcon_dsp_freq_shift.cc:133-162.
 */
#ifndef FALCON_DSP_FREQ_SHIFT_H
#define FALCON_DSP_FREQ_SHIFT_H

#include <complex>
#include <cstdint>
#include <utility>
#include <vector>

#include "falcon_dsp_gb300_detail.h"

namespace falcon_dsp {

class falcon_dsp_freq_shift {
public:
    /* (rollover sample index R, angular frequency) exactly as
     * src/transform/falcon_dsp_freq_shift.cc:194-235 computes them. */
    static std::pair<uint32_t, double> get_freq_shift_params(uint32_t input_sample_rate_in_sps,
                                                             int32_t freq_shift_in_hz) {
        uint32_t r = 0;
        double w = 0.0;
        fdsp_freq_shift_params(input_sample_rate_in_sps, freq_shift_in_hz, &r, &w);
        return std::make_pair(r, w);
    }

    falcon_dsp_freq_shift(void) = default;
    virtual ~falcon_dsp_freq_shift(void) {
        if (m_h) fdsp_freq_shift_destroy(m_h);
    }
    falcon_dsp_freq_shift(const falcon_dsp_freq_shift&) = delete;
    falcon_dsp_freq_shift& operator=(const falcon_dsp_freq_shift&) = delete;

    virtual bool initialize(uint32_t input_sample_rate_in_sps, int32_t freq_shift_in_hz) {
        return create(input_sample_rate_in_sps, std::vector<int32_t>(1, freq_shift_in_hz));
    }

    void reset_state(void) {
        if (m_h) fdsp_freq_shift_reset(m_h);
    }

    virtual bool apply(std::vector<std::complex<int16_t>>& in, std::vector<std::complex<int16_t>>& out) {
        std::vector<std::complex<float>> tin = gb300_detail::to_float(in), tout;
        const bool ok = apply(tin, tout);
        gb300_detail::to_int16(tout, out);
        return ok;
    }

    /* Single channel (the first one when the object shifts several). */
    virtual bool apply(std::vector<std::complex<float>>& in, std::vector<std::complex<float>>& out) {
        std::vector<std::vector<std::complex<float>>> all;
        const bool ok = apply_all(in, all);
        out.clear();
        if (ok) out.swap(all[0]);
        return ok;
    }

protected:
    /* Once only: one GPU object for every channel over the same input. */
    bool create(uint32_t input_sample_rate_in_sps, const std::vector<int32_t>& freq_shift_in_hz) {
        if (m_h || freq_shift_in_hz.empty()) return false;
        if (fdsp_freq_shift_create(input_sample_rate_in_sps, freq_shift_in_hz.data(),
                                   (uint32_t)freq_shift_in_hz.size(), &m_h) != FDSP_OK) {
            m_h = nullptr;
            return false;
        }
        m_nch = freq_shift_in_hz.size();
        return true;
    }

    bool apply_all(std::vector<std::complex<float>>& in, std::vector<std::vector<std::complex<float>>>& out) {
        out.clear();
        if (!m_h || in.empty()) return false;
        out.assign(m_nch, std::vector<std::complex<float>>(in.size()));
        std::vector<fdsp_cf32*> ptr(m_nch);
        for (size_t c = 0; c < m_nch; ++c) ptr[c] = gb300_detail::cf(out[c]);
        if (fdsp_freq_shift_apply_host(m_h, gb300_detail::cf(in), in.size(), ptr.data(), nullptr) != FDSP_OK) {
            out.clear();
            return false;
        }
        return true;
    }

    fdsp_freq_shift* m_h = nullptr;
    size_t m_nch = 0;
};

}  // namespace falcon_dsp

#endif
