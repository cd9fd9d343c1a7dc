/*
 * Drop-in for libfalcon_dsp's falcon_dsp_multi_rate_channelizer_cuda
 * (hdr/transform/falcon_dsp_multi_rate_channelizer_cuda.h:73-167) on the GB300
 * library: same channel struct, same initialize / apply / reset_state with
 * streaming state carried across applies.  The shift and resampling of all
 * channels run fused on the GPU; apply() copies the input in, computes and
 * copies every channel's output back.
 *
 * Additions (no counterpart in the reference): set_precision() selects the
 * tensor-core split-precision forms, autotune() picks per-group tile heights
 * and forms for a block size, handle() exposes the C ABI handle for
 * device-buffer applies (fdsp_channelizer_apply).
 */
#ifndef FALCON_DSP_MULTI_RATE_CHANNELIZER_CUDA_H
#define FALCON_DSP_MULTI_RATE_CHANNELIZER_CUDA_H

#include <complex>
#include <cstdint>
#include <vector>

#include "falcon_dsp_gb300_detail.h"

#ifndef FALCON_DSP_MULTI_RATE_CHANNELIZER_CHANNEL_S_DEFINED
#define FALCON_DSP_MULTI_RATE_CHANNELIZER_CHANNEL_S_DEFINED
/* Field for field hdr/transform/falcon_dsp_multi_rate_channelizer_cuda.h:73-80. */
struct multi_rate_channelizer_channel_s {
    uint32_t output_sample_rate_in_sps;
    int64_t freq_shift_in_hz;
    uint32_t up_rate;
    uint32_t down_rate;
    std::vector<std::complex<float>> resample_filter_coeffs;
};
#endif

namespace falcon_dsp {

class falcon_dsp_multi_rate_channelizer_cuda {
public:
    falcon_dsp_multi_rate_channelizer_cuda(void) = default;
    ~falcon_dsp_multi_rate_channelizer_cuda(void) {
        if (m_h) fdsp_channelizer_destroy(m_h);
    }
    falcon_dsp_multi_rate_channelizer_cuda(const falcon_dsp_multi_rate_channelizer_cuda&) = delete;
    falcon_dsp_multi_rate_channelizer_cuda& operator=(const falcon_dsp_multi_rate_channelizer_cuda&) = delete;

    /* Works once, like the reference (a second call returns false). */
    bool initialize(uint32_t input_sample_rate, std::vector<multi_rate_channelizer_channel_s> channels) {
        if (m_h || channels.empty()) return false;
        std::vector<fdsp_channel_cfg> cfg(channels.size());
        for (size_t i = 0; i < channels.size(); ++i) {
            cfg[i].output_sample_rate_in_sps = channels[i].output_sample_rate_in_sps;
            cfg[i].freq_shift_in_hz = channels[i].freq_shift_in_hz;
            cfg[i].up_rate = channels[i].up_rate;
            cfg[i].down_rate = channels[i].down_rate;
            cfg[i].resample_filter_coeffs = gb300_detail::cf(channels[i].resample_filter_coeffs);
            cfg[i].num_coeffs = (uint32_t)channels[i].resample_filter_coeffs.size();
        }
        if (fdsp_channelizer_create(input_sample_rate, cfg.data(), (uint32_t)cfg.size(), &m_h) != FDSP_OK) {
            m_h = nullptr;
            return false;
        }
        m_nch = channels.size();
        return true;
    }

    /* out is cleared and receives one vector per channel. */
    bool apply(std::vector<std::complex<float>>& in, std::vector<std::vector<std::complex<float>>>& out) {
        out.clear();
        if (!m_h || in.empty()) return false;
        std::vector<uint64_t> cnt(m_nch), cap(m_nch);
        if (fdsp_channelizer_out_count(m_h, in.size(), cnt.data()) != FDSP_OK) return false;
        out.resize(m_nch);
        std::vector<fdsp_cf32*> ptr(m_nch);
        for (size_t c = 0; c < m_nch; ++c) {
            out[c].resize(cnt[c]);
            cap[c] = cnt[c];
            ptr[c] = gb300_detail::cf(out[c]);
        }
        std::vector<uint64_t> got(m_nch);
        if (fdsp_channelizer_apply_host(m_h, gb300_detail::cf(in), in.size(), ptr.data(), cap.data(), got.data(),
                                        nullptr) != FDSP_OK) {
            out.clear();
            return false;
        }
        for (size_t c = 0; c < m_nch; ++c) out[c].resize(got[c]);
        return true;
    }

    void reset_state(void) {
        if (m_h) fdsp_channelizer_reset(m_h);
    }

    /* FDSP_PRECISION_FP32 (default), FDSP_PRECISION_FP16X3 or FDSP_PRECISION_BF16X3. */
    bool set_precision(int precision) { return m_h && fdsp_channelizer_set_precision(m_h, precision) == FDSP_OK; }
    bool autotune(uint64_t block_len) { return m_h && fdsp_channelizer_autotune(m_h, block_len, nullptr) == FDSP_OK; }
    fdsp_channelizer* handle(void) const { return m_h; }

private:
    fdsp_channelizer* m_h = nullptr;
    size_t m_nch = 0;
};

}  // namespace falcon_dsp

#endif
