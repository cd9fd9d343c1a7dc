/*
 * Drop-in for libfalcon_dsp's falcon_dsp_polyphase_resampler_cuda
 * (hdr/transform/falcon_dsp_polyphase_resampler_cuda.h:187-226).  As in the
 * reference it derives from falcon_dsp_polyphase_resampler and overrides
 * initialize/apply, so it can be used through a base-class reference or
 * pointer.  Both classes run on the GPU (the base class here has no CPU
 * implementation); see falcon_dsp_polyphase_resampler.h for the semantics.
 */
#ifndef FALCON_DSP_POLYPHASE_RESAMPLER_CUDA_H
#define FALCON_DSP_POLYPHASE_RESAMPLER_CUDA_H

#include <complex>
#include <cstdint>
#include <vector>

#include "falcon_dsp_polyphase_resampler.h"

namespace falcon_dsp {

class falcon_dsp_polyphase_resampler_cuda : public falcon_dsp_polyphase_resampler {
public:
    falcon_dsp_polyphase_resampler_cuda(void) = default;
    ~falcon_dsp_polyphase_resampler_cuda(void) override = default;
    falcon_dsp_polyphase_resampler_cuda(const falcon_dsp_polyphase_resampler_cuda&) = delete;
    falcon_dsp_polyphase_resampler_cuda& operator=(const falcon_dsp_polyphase_resampler_cuda&) = delete;

    bool initialize(uint32_t up_rate, uint32_t down_rate, const std::vector<std::complex<float>>& filter_coeffs) override {
        return falcon_dsp_polyphase_resampler::initialize(up_rate, down_rate, filter_coeffs);
    }
    int32_t apply(std::vector<float>& in, std::vector<float>& out) override {
        return falcon_dsp_polyphase_resampler::apply(in, out);
    }
    int32_t apply(std::vector<std::complex<float>>& in, std::vector<std::complex<float>>& out) override {
        return falcon_dsp_polyphase_resampler::apply(in, out);
    }
};

}  // namespace falcon_dsp

#endif
