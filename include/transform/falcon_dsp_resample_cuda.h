/*
 * Drop-in for libfalcon_dsp's resample_cuda / upfirdn_cuda
 * (hdr/transform/falcon_dsp_resample_cuda.h:85-95,
 * src/transform/falcon_dsp_resample_cuda.cu:124-146): up/down from
 * rat_approx(out_rate / in_rate, 1024), then one resampler apply.
 */
#ifndef FALCON_DSP_RESAMPLE_CUDA_H
#define FALCON_DSP_RESAMPLE_CUDA_H

#include <complex>
#include <cstdint>
#include <vector>

#include "falcon_dsp_polyphase_resampler_cuda.h"

namespace falcon_dsp {

inline bool resample_cuda(uint32_t in_sample_rate_in_sps, std::vector<std::complex<float>>& in,
                          std::vector<std::complex<float>>& filter_coeffs, uint32_t out_sample_rate_in_sps,
                          std::vector<std::complex<float>>& out) {
    int64_t up = 0, down = 0;
    const double ratio = static_cast<double>(out_sample_rate_in_sps) / static_cast<double>(in_sample_rate_in_sps);
    if (fdsp_rat_approx(ratio, 1024, &up, &down) != FDSP_OK) return false;
    falcon_dsp_polyphase_resampler_cuda r;
    return r.initialize((uint32_t)up, (uint32_t)down, filter_coeffs) && r.apply(in, out) > 0;
}

inline bool upfirdn_cuda(uint32_t in_sample_rate_in_sps, std::vector<std::complex<float>>& in,
                         std::vector<std::complex<float>>& filter_coeffs, uint32_t out_sample_rate_in_sps,
                         std::vector<std::complex<float>>& out) {
    return resample_cuda(in_sample_rate_in_sps, in, filter_coeffs, out_sample_rate_in_sps, out);
}

/* Real-tap form declared by the reference header (:93-95). */
inline bool upfirdn_cuda(uint32_t in_sample_rate_in_sps, std::vector<std::complex<float>>& in,
                         std::vector<float>& filter_coeffs, uint32_t out_sample_rate_in_sps,
                         std::vector<std::complex<float>>& out) {
    std::vector<std::complex<float>> c(filter_coeffs.begin(), filter_coeffs.end());
    return resample_cuda(in_sample_rate_in_sps, in, c, out_sample_rate_in_sps, out);
}

}  // namespace falcon_dsp

#endif
