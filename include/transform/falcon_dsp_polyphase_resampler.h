/*
 * Base class of the resampler drop-in, with the reference CPU class's name
 * and virtual interface (hdr/transform/falcon_dsp_polyphase_resampler.h:168-195):
 * initialize(up, down, coeffs) once, reset_state(), apply() for real and
 * complex input, needed_out_count(), coeffs_per_phase().  Callers that hold a
 * falcon_dsp_polyphase_resampler& or * (to a falcon_dsp_polyphase_resampler_cuda,
 * or to this class itself) compile unchanged.  There is no CPU implementation
 * behind it: every apply runs on the GPU through the C ABI, with the CPU
 * loop's streaming semantics (carried phase and xOffset, real parts of the
 * taps only, no tail flush).  apply() returns the number of outputs, 0 when
 * not initialized or on failure.
 */
#ifndef FALCON_DSP_POLYPHASE_RESAMPLER_H
#define FALCON_DSP_POLYPHASE_RESAMPLER_H

#include <complex>
#include <cstdint>
#include <vector>

#include "falcon_dsp_gb300_detail.h"

namespace falcon_dsp {

class falcon_dsp_polyphase_resampler {
public:
    falcon_dsp_polyphase_resampler(void) = default;
    virtual ~falcon_dsp_polyphase_resampler(void) {
        if (m_h) fdsp_resampler_destroy(m_h);
    }
    falcon_dsp_polyphase_resampler(const falcon_dsp_polyphase_resampler&) = delete;
    falcon_dsp_polyphase_resampler& operator=(const falcon_dsp_polyphase_resampler&) = delete;

    virtual bool initialize(uint32_t up_rate, uint32_t down_rate,
                            const std::vector<std::complex<float>>& filter_coeffs) {
        if (m_h || filter_coeffs.empty()) return false;
        if (fdsp_resampler_create(up_rate, down_rate, gb300_detail::cf(filter_coeffs), (uint32_t)filter_coeffs.size(),
                                  &m_h) != FDSP_OK) {
            m_h = nullptr;
            return false;
        }
        return true;
    }

    void reset_state(void) {
        if (m_h) fdsp_resampler_reset(m_h);
    }

    /* Real input: taken as complex with zero imaginary part, real part returned
     * (src/transform/falcon_dsp_polyphase_resampler.cc:230-253). */
    virtual int32_t apply(std::vector<float>& in, std::vector<float>& out) {
        out.clear();
        std::vector<std::complex<float>> tin(in.begin(), in.end()), tout;
        const int32_t n = apply(tin, tout);
        out.reserve(tout.size());
        for (const auto& s : tout) out.push_back(s.real());
        return n;
    }

    virtual int32_t apply(std::vector<std::complex<float>>& in, std::vector<std::complex<float>>& out) {
        out.clear();
        if (!m_h) return 0;
        uint64_t cnt = 0, got = 0;
        if (fdsp_resampler_out_count(m_h, in.size(), &cnt) != FDSP_OK) return 0;
        out.resize(cnt);
        if (fdsp_resampler_apply_host(m_h, gb300_detail::cf(in), in.size(), gb300_detail::cf(out), cnt, &got,
                                      nullptr) != FDSP_OK) {
            out.clear();
            return 0;
        }
        out.resize(got);
        return (int32_t)got;
    }

    /* needed_out_count() exactly as the reference computes it
     * (src/transform/falcon_dsp_polyphase_resampler.cc:204-228). */
    uint32_t needed_out_count(uint32_t inCount) {
        uint32_t n = 0;
        return (m_h && fdsp_resampler_needed_out_count(m_h, inCount, &n) == FDSP_OK) ? n : 0;
    }
    uint32_t coeffs_per_phase(void) {
        uint32_t n = 0;
        return (m_h && fdsp_resampler_coeffs_per_phase(m_h, &n) == FDSP_OK) ? n : 0;
    }

protected:
    fdsp_resampler* m_h = nullptr;
};

}  // namespace falcon_dsp

#endif
