/*
 * Drop-in for libfalcon_dsp's falcon_dsp_fir_filter_cuda
 * (hdr/transform/falcon_dsp_fir_filter_cuda.h:113-138) and the free
 * fir_filter_cuda functions (:87-91).  As in the reference it derives from
 * falcon_dsp_fir_filter (falcon_dsp_fir_filter.h here, GPU-backed too) and
 * overrides both applies, so it can be used through a base-class reference
 * or pointer.
 */
#ifndef FALCON_DSP_FIR_FILTER_CUDA_H
#define FALCON_DSP_FIR_FILTER_CUDA_H

#include <complex>
#include <cstdint>
#include <vector>

#include "falcon_dsp_fir_filter.h"

namespace falcon_dsp {

class falcon_dsp_fir_filter_cuda : public falcon_dsp_fir_filter {
public:
    explicit falcon_dsp_fir_filter_cuda(std::vector<std::complex<float>>& coeffs) : falcon_dsp_fir_filter(coeffs) {}
    ~falcon_dsp_fir_filter_cuda(void) override = default;
    falcon_dsp_fir_filter_cuda(void) = delete;
    falcon_dsp_fir_filter_cuda(const falcon_dsp_fir_filter_cuda&) = delete;
    falcon_dsp_fir_filter_cuda& operator=(const falcon_dsp_fir_filter_cuda&) = delete;

    bool apply(std::vector<std::complex<int16_t>>& in, std::vector<std::complex<int16_t>>& out) override {
        return falcon_dsp_fir_filter::apply(in, out);
    }
    bool apply(std::vector<std::complex<float>>& in, std::vector<std::complex<float>>& out) override {
        return falcon_dsp_fir_filter::apply(in, out);
    }
};

inline bool fir_filter_cuda(std::vector<std::complex<float>>& coeffs, std::vector<std::complex<int16_t>>& in,
                            std::vector<std::complex<int16_t>>& out) {
    falcon_dsp_fir_filter_cuda f(coeffs);
    return f.apply(in, out);
}

inline bool fir_filter_cuda(std::vector<std::complex<float>>& coeffs, std::vector<std::complex<float>>& in,
                            std::vector<std::complex<float>>& out) {
    falcon_dsp_fir_filter_cuda f(coeffs);
    return f.apply(in, out);
}

}  // namespace falcon_dsp

#endif
