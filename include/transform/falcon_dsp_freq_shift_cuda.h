/*
 * Drop-in for libfalcon_dsp's falcon_dsp_freq_shift_cuda
 * (hdr/transform/falcon_dsp_freq_shift_cuda.h:187-212) and the free
 * freq_shift_cuda functions (:142-156): y[n] = x[n] e^{j w (n mod R)} with
 * the sample counter carried across applies, one or many channels over one
 * input.  The int16 overload converts in and truncates out like
 * src/transform/falcon_dsp_freq_shift_cuda.cu:308-329.
 */
#ifndef FALCON_DSP_FREQ_SHIFT_CUDA_H
#define FALCON_DSP_FREQ_SHIFT_CUDA_H

#include <complex>
#include <cstdint>
#include <vector>

#include "falcon_dsp_gb300_detail.h"

namespace falcon_dsp {

class falcon_dsp_freq_shift_cuda {
public:
    falcon_dsp_freq_shift_cuda(void) = default;
    virtual ~falcon_dsp_freq_shift_cuda(void) {
        if (m_h) fdsp_freq_shift_destroy(m_h);
    }
    falcon_dsp_freq_shift_cuda(const falcon_dsp_freq_shift_cuda&) = delete;
    falcon_dsp_freq_shift_cuda& operator=(const falcon_dsp_freq_shift_cuda&) = delete;

    virtual bool initialize(uint32_t input_sample_rate_in_sps, int32_t freq_shift_in_hz) {
        std::vector<int32_t> f(1, freq_shift_in_hz);
        return initialize(input_sample_rate_in_sps, f);
    }
    bool initialize(uint32_t input_sample_rate_in_sps, std::vector<int32_t> freq_shift_in_hz) {
        if (m_h || freq_shift_in_hz.empty()) return false;
        if (fdsp_freq_shift_create(input_sample_rate_in_sps, freq_shift_in_hz.data(), (uint32_t)freq_shift_in_hz.size(),
                                   &m_h) != FDSP_OK) {
            m_h = nullptr;
            return false;
        }
        m_nch = freq_shift_in_hz.size();
        return true;
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

    /* Single channel (the first one when initialized with several). */
    bool apply(std::vector<std::complex<float>>& in, std::vector<std::complex<float>>& out) {
        std::vector<std::vector<std::complex<float>>> all;
        const bool ok = apply(in, all);
        out.clear();
        if (ok) out.swap(all[0]);
        return ok;
    }

    bool apply(std::vector<std::complex<float>>& in, std::vector<std::vector<std::complex<float>>>& out) {
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

private:
    fdsp_freq_shift* m_h = nullptr;
    size_t m_nch = 0;
};

inline bool freq_shift_cuda(uint32_t in_sample_rate_in_sps, std::vector<std::complex<float>>& in,
                            int32_t freq_shift_in_hz, std::vector<std::complex<float>>& out) {
    falcon_dsp_freq_shift_cuda s;
    return s.initialize(in_sample_rate_in_sps, freq_shift_in_hz) && s.apply(in, out);
}

inline bool freq_shift_cuda(uint32_t in_sample_rate_in_sps, std::vector<std::complex<float>>& in,
                            std::vector<int32_t>& freq_shift_in_hz, std::vector<std::vector<std::complex<float>>>& out) {
    falcon_dsp_freq_shift_cuda s;
    return s.initialize(in_sample_rate_in_sps, freq_shift_in_hz) && s.apply(in, out);
}

}  // namespace falcon_dsp

#endif
