/*
 * Base class of the FIR drop-in, with the reference CPU class's name and
 * virtual interface (hdr/transform/falcon_dsp_fir_filter.h:119-140):
 * constructed from the taps, reset_state(), apply() for complex float and
 * complex int16 blocks.  Callers that hold a falcon_dsp_fir_filter& or *
 * compile unchanged.  There is no CPU implementation behind it:
 * y[n] = sum_k h[k] x[n-k] with complex taps runs on the GPU through the C
 * ABI, history carried across applies, output length = input length; the
 * int16 overload converts in and truncates out like
 * src/transform/falcon_dsp_fir_filter.cc:151-175.
 */
#ifndef FALCON_DSP_FIR_FILTER_H
#define FALCON_DSP_FIR_FILTER_H

#include <complex>
#include <cstdint>
#include <vector>

#include "falcon_dsp_gb300_detail.h"

namespace falcon_dsp {

class falcon_dsp_fir_filter {
public:
    /* The reference constructs from the taps; a failed set-up leaves the
     * object unusable and every apply returns false. */
    explicit falcon_dsp_fir_filter(std::vector<std::complex<float>>& coeffs) {
        if (coeffs.empty() ||
            fdsp_fir_create(gb300_detail::cf(coeffs), (uint32_t)coeffs.size(), &m_h) != FDSP_OK)
            m_h = nullptr;
    }
    virtual ~falcon_dsp_fir_filter(void) {
        if (m_h) fdsp_fir_destroy(m_h);
    }
    falcon_dsp_fir_filter(void) = delete;
    falcon_dsp_fir_filter(const falcon_dsp_fir_filter&) = delete;
    falcon_dsp_fir_filter& operator=(const falcon_dsp_fir_filter&) = delete;

    void reset_state(void) {
        if (m_h) fdsp_fir_reset(m_h);
    }

    virtual bool apply(std::vector<std::complex<int16_t>>& in, std::vector<std::complex<int16_t>>& out) {
        std::vector<std::complex<float>> tin = gb300_detail::to_float(in), tout;
        const bool ok = apply(tin, tout);
        gb300_detail::to_int16(tout, out);
        return ok;
    }

    virtual bool apply(std::vector<std::complex<float>>& in, std::vector<std::complex<float>>& out) {
        out.clear();
        if (!m_h || in.empty()) return false;
        out.resize(in.size());
        if (fdsp_fir_apply_host(m_h, gb300_detail::cf(in), in.size(), gb300_detail::cf(out), nullptr) != FDSP_OK) {
            out.clear();
            return false;
        }
        return true;
    }

protected:
    fdsp_fir* m_h = nullptr;
};

}  // namespace falcon_dsp

#endif
