/*
 * Drop-in for libfalcon_dsp's falcon_dsp_fm_demodulator_cuda
 * (hdr/signals/falcon_dsp_fm_demod_cuda.h:83-104).  As in the reference it
 * derives from falcon_dsp_fm_demodulator (falcon_dsp_fm_demod.h here,
 * GPU-backed too) and overrides initialize, reset_state and demod_mono, so
 * it can be used through a base-class reference or pointer.  The constants
 * are those of hdr/signals/falcon_dsp_fm_demod.h:96-100.
 */
#ifndef FALCON_DSP_FM_DEMOD_CUDA_H
#define FALCON_DSP_FM_DEMOD_CUDA_H

#include <complex>
#include <cstdint>
#include <vector>

#include "falcon_dsp_fm_demod.h"

namespace falcon_dsp {

class falcon_dsp_fm_demodulator_cuda : public falcon_dsp_fm_demodulator {
public:
    falcon_dsp_fm_demodulator_cuda(void) = default;
    ~falcon_dsp_fm_demodulator_cuda(void) override = default;
    falcon_dsp_fm_demodulator_cuda(const falcon_dsp_fm_demodulator_cuda&) = delete;
    falcon_dsp_fm_demodulator_cuda& operator=(const falcon_dsp_fm_demodulator_cuda&) = delete;

    bool initialize(uint32_t input_sample_rate_in_sps, int32_t signal_offset_from_dc_in_hz,
                    float deemphasis_time_constant_in_usecs = AMERICAS_FM_DEEMPHASIS_TIME_CONSTANT) override {
        return falcon_dsp_fm_demodulator::initialize(input_sample_rate_in_sps, signal_offset_from_dc_in_hz,
                                                     deemphasis_time_constant_in_usecs);
    }
    void reset_state(void) override { falcon_dsp_fm_demodulator::reset_state(); }
    bool demod_mono(std::vector<std::complex<float>>& in, std::vector<int16_t>& out) override {
        return falcon_dsp_fm_demodulator::demod_mono(in, out);
    }
};

}  // namespace falcon_dsp

#endif
