/*
 * Drop-in for libfalcon_dsp's falcon_dsp_freq_shift_cuda
 * (hdr/transform/falcon_dsp_freq_shift_cuda.h:187-212) and the free
 * freq_shift_cuda functions (:142-156).  As in the reference it derives from
 * falcon_dsp_freq_shift (falcon_dsp_freq_shift.h here, GPU-backed too) and
 * adds the multi-channel initialize/apply: one or many channels over one
 * input, y[n] = x[n] e^{j w (n mod R)} with the sample counter carried
 * across applies.
 */
#ifndef FALCON_DSP_FREQ_SHIFT_CUDA_H
#define FALCON_DSP_FREQ_SHIFT_CUDA_H

#include <complex>
#include <cstdint>
#include <vector>

#include "falcon_dsp_freq_shift.h"

namespace falcon_dsp {

class falcon_dsp_freq_shift_cuda : public falcon_dsp_freq_shift {
public:
    falcon_dsp_freq_shift_cuda(void) = default;
    ~falcon_dsp_freq_shift_cuda(void) override = default;
    falcon_dsp_freq_shift_cuda(const falcon_dsp_freq_shift_cuda&) = delete;
    falcon_dsp_freq_shift_cuda& operator=(const falcon_dsp_freq_shift_cuda&) = delete;

    bool initialize(uint32_t input_sample_rate_in_sps, int32_t freq_shift_in_hz) override {
        return falcon_dsp_freq_shift::initialize(input_sample_rate_in_sps, freq_shift_in_hz);
    }
    bool initialize(uint32_t input_sample_rate_in_sps, std::vector<int32_t> freq_shift_in_hz) {
        return create(input_sample_rate_in_sps, freq_shift_in_hz);
    }

    bool apply(std::vector<std::complex<int16_t>>& in, std::vector<std::complex<int16_t>>& out) override {
        return falcon_dsp_freq_shift::apply(in, out);
    }
    bool apply(std::vector<std::complex<float>>& in, std::vector<std::complex<float>>& out) override {
        return falcon_dsp_freq_shift::apply(in, out);
    }
    bool apply(std::vector<std::complex<float>>& in, std::vector<std::vector<std::complex<float>>>& out) {
        return apply_all(in, out);
    }
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
