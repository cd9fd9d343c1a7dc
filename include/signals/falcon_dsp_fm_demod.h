/*
 * Base class of the FM demodulator drop-in, with the reference CPU class's
 * name, constants and virtual interface
 * (hdr/signals/falcon_dsp_fm_demod.h:91-121): initialize(input rate, offset
 * of the station from DC, de-emphasis time constant) once, reset_state(),
 * demod_mono(complex block -> int16 mono audio at 45.6 kS/s).  Callers that
 * hold a falcon_dsp_fm_demodulator& or * compile unchanged.  There is no CPU
 * implementation behind it: every stage (channelizer, discriminator,
 * de-emphasis, mono decimator, rescale) runs on the GPU through the C ABI.
 */
#ifndef FALCON_DSP_FM_DEMOD_H
#define FALCON_DSP_FM_DEMOD_H

#include <complex>
#include <cstdint>
#include <vector>

#include "../transform/falcon_dsp_gb300_detail.h"

namespace falcon_dsp {

class falcon_dsp_fm_demodulator {
public:
    static constexpr float AMERICAS_FM_DEEMPHASIS_TIME_CONSTANT = 75e-6;
    static constexpr float EUROPE_ASIA_FM_DEEMPHASIS_TIME_CONSTANT = 50e-6;
    static const uint32_t FM_RADIO_SAMPLE_RATE_IN_SPS = 228000;
    static const uint32_t FM_RADIO_AUDIO_SAMPLE_RATE_IN_SPS = 45600;

    falcon_dsp_fm_demodulator(void) = default;
    virtual ~falcon_dsp_fm_demodulator(void) {
        if (m_h) fdsp_fm_demod_destroy(m_h);
    }
    falcon_dsp_fm_demodulator(const falcon_dsp_fm_demodulator&) = delete;
    falcon_dsp_fm_demodulator& operator=(const falcon_dsp_fm_demodulator&) = delete;

    /* Once only; false for an unsupported time constant or an input rate
     * without a predefined 228 kS/s filter, as the reference. */
    virtual bool initialize(uint32_t input_sample_rate_in_sps, int32_t signal_offset_from_dc_in_hz,
                            float deemphasis_time_constant_in_usecs = AMERICAS_FM_DEEMPHASIS_TIME_CONSTANT) {
        if (m_h) return false;
        if (fdsp_fm_demod_create(input_sample_rate_in_sps, signal_offset_from_dc_in_hz,
                                 deemphasis_time_constant_in_usecs, &m_h) != FDSP_OK) {
            m_h = nullptr;
            return false;
        }
        return true;
    }

    virtual void reset_state(void) {
        if (m_h) fdsp_fm_demod_reset(m_h);
    }

    virtual bool demod_mono(std::vector<std::complex<float>>& in, std::vector<int16_t>& out) {
        out.clear();
        if (!m_h) return false;
        uint64_t n = 0;
        if (fdsp_fm_demod_out_count(m_h, in.size(), &n) != FDSP_OK) return false;
        out.resize(n);
        uint64_t got = 0;
        if (fdsp_fm_demod_apply_host(m_h, gb300_detail::cf(in), in.size(), out.data(), n, &got, nullptr) !=
            FDSP_OK) {
            out.clear();
            return false;
        }
        out.resize(got);
        return !out.empty();
    }

protected:
    fdsp_fm_demod* m_h = nullptr;
};

}  // namespace falcon_dsp

#endif
