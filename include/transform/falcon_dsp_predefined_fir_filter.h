/*
 * Drop-in for libfalcon_dsp's resampling filter lookup: the key enums of
 * hdr/transform/falcon_dsp_predefined_fir_filter.h:63-78 (global scope, as
 * there) and falcon_dsp::get_resample_fir_params
 * (hdr/transform/falcon_dsp_fir_filter.h:105, src/transform/
 * falcon_dsp_fir_filter.cc:111-130), over the library's predefined table
 * (the same 51 entries, generated by the same recipe).  Also
 * falcon_dsp::design_resample_firls, the table's FIRLS recipe for any rate
 * pair (no counterpart in the reference).
 */
#ifndef FALCON_DSP_PREDEFINED_FIR_FILTER_H
#define FALCON_DSP_PREDEFINED_FIR_FILTER_H

#include <complex>
#include <cstdint>
#include <vector>

#include "falcon_dsp_gb300_detail.h"

enum class filter_source_type_e : uint32_t { REMEZ = 0, FIRLS };

enum class filter_taps_e : int32_t {
    FILTER_TAPS_OPTIMAL = -1,
    FILTER_TAPS_16 = 16,
    FILTER_TAPS_32 = 32,
    FILTER_TAPS_64 = 64,
    FILTER_TAPS_128 = 128,
    FILTER_TAPS_256 = 256
};

namespace falcon_dsp {

/* True and (up, down, coeffs) when the table has the key; false and empty
 * coeffs otherwise. */
inline bool get_resample_fir_params(uint32_t input_sample_rate, uint32_t output_sample_rate, filter_taps_e taps,
                                    filter_source_type_e source, uint32_t& up_rate, uint32_t& down_rate,
                                    std::vector<std::complex<float>>& coeffs) {
    coeffs.clear();
    uint32_t up = 0, down = 0, n = 0;
    int st = fdsp_get_resample_fir_params(input_sample_rate, output_sample_rate, (int32_t)taps, (uint32_t)source, &up,
                                          &down, nullptr, 0, &n);
    if (st != FDSP_ERR_CAPACITY && st != FDSP_OK) return false;
    coeffs.resize(n);
    st = fdsp_get_resample_fir_params(input_sample_rate, output_sample_rate, (int32_t)taps, (uint32_t)source, &up,
                                      &down, gb300_detail::cf(coeffs), n, &n);
    if (st != FDSP_OK) {
        coeffs.clear();
        return false;
    }
    up_rate = up;
    down_rate = down;
    return true;
}

inline bool design_resample_firls(uint32_t input_sample_rate, uint32_t output_sample_rate, uint32_t num_taps,
                                  double kaiser_beta, uint32_t& up_rate, uint32_t& down_rate,
                                  std::vector<std::complex<float>>& coeffs) {
    coeffs.clear();
    uint32_t n = 0;
    int st = fdsp_design_resample_firls(input_sample_rate, output_sample_rate, num_taps, kaiser_beta, &up_rate,
                                        &down_rate, nullptr, 0, &n);
    if (st != FDSP_ERR_CAPACITY && st != FDSP_OK) return false;
    coeffs.resize(n);
    st = fdsp_design_resample_firls(input_sample_rate, output_sample_rate, num_taps, kaiser_beta, &up_rate,
                                    &down_rate, gb300_detail::cf(coeffs), n, &n);
    if (st != FDSP_OK) coeffs.clear();
    return st == FDSP_OK;
}

}  // namespace falcon_dsp

#endif
