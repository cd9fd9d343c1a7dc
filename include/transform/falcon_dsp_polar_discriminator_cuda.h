/*
 * GPU form of libfalcon_dsp's falcon_dsp_polar_discriminator
 * (hdr/transform/falcon_dsp_polar_discriminator.h:97-114), which the
 * reference has only on the CPU: out[n] = arg(x[n] conj(x[n-1])) with x[-1]
 * carried across applies, so the first apply after construction or
 * reset_state() emits N-1 outputs (src/transform/falcon_dsp_polar_discriminator.cc:134-171).
 */
#ifndef FALCON_DSP_POLAR_DISCRIMINATOR_CUDA_H
#define FALCON_DSP_POLAR_DISCRIMINATOR_CUDA_H

#include <complex>
#include <cstdint>
#include <vector>

#include "falcon_dsp_gb300_detail.h"

namespace falcon_dsp {

class falcon_dsp_polar_discriminator_cuda {
public:
    falcon_dsp_polar_discriminator_cuda(void) {
        if (fdsp_polar_create(&m_h) != FDSP_OK) m_h = nullptr;
    }
    virtual ~falcon_dsp_polar_discriminator_cuda(void) {
        if (m_h) fdsp_polar_destroy(m_h);
    }
    falcon_dsp_polar_discriminator_cuda(const falcon_dsp_polar_discriminator_cuda&) = delete;
    falcon_dsp_polar_discriminator_cuda& operator=(const falcon_dsp_polar_discriminator_cuda&) = delete;

    void reset_state(void) {
        if (m_h) fdsp_polar_reset(m_h);
    }

    virtual bool apply(const std::vector<std::complex<int16_t>>& in, std::vector<float>& out) {
        return apply(gb300_detail::to_float(in), out);
    }

    virtual bool apply(const std::vector<std::complex<float>>& in, std::vector<float>& out) {
        out.clear();
        if (!m_h || in.empty()) return false;
        uint64_t cnt = 0, got = 0;
        if (fdsp_polar_out_count(m_h, in.size(), &cnt) != FDSP_OK) return false;
        out.resize(cnt);
        if (fdsp_polar_apply_host(m_h, gb300_detail::cf(in), in.size(), out.data(), &got, nullptr) != FDSP_OK) {
            out.clear();
            return false;
        }
        out.resize(got);
        return true;
    }

private:
    fdsp_polar* m_h = nullptr;
};

inline bool polar_discriminator_cuda(const std::vector<std::complex<float>>& in, std::vector<float>& out) {
    falcon_dsp_polar_discriminator_cuda p;
    return p.apply(in, out);
}

}  // namespace falcon_dsp

#endif
