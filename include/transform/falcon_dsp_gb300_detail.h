/*
 * Shared plumbing of the drop-in C++ classes (header only): vector <-> C ABI
 * conversions and the int16 casts of the reference's int16 overloads.
 * The classes in this directory keep the names, signatures and streaming
 * semantics of the _cuda.h classes of libfalcon_dsp's hdr/transform and call the C ABI of
 * include/fdsp_c.h; a failing call returns false (or 0 for the resampler's
 * int32_t count) instead of exiting the process.
 */
#ifndef FALCON_DSP_GB300_DETAIL_H
#define FALCON_DSP_GB300_DETAIL_H

#include <complex>
#include <cstdint>
#include <vector>

#include "../fdsp_c.h"

namespace falcon_dsp {
namespace gb300_detail {

static_assert(sizeof(std::complex<float>) == sizeof(fdsp_cf32), "std::complex<float> must match fdsp_cf32");

inline const fdsp_cf32* cf(const std::vector<std::complex<float>>& v) {
    return reinterpret_cast<const fdsp_cf32*>(v.data());
}
inline fdsp_cf32* cf(std::vector<std::complex<float>>& v) { return reinterpret_cast<fdsp_cf32*>(v.data()); }

// complex<int16_t> -> complex<float>, as the reference's int16 overloads do
// (e.g. src/transform/falcon_dsp_fir_filter.cc:155-160)
inline std::vector<std::complex<float>> to_float(const std::vector<std::complex<int16_t>>& in) {
    std::vector<std::complex<float>> out;
    out.reserve(in.size());
    for (const auto& s : in) out.emplace_back((float)s.real(), (float)s.imag());
    return out;
}

// complex<float> -> complex<int16_t> by C++ conversion (truncation toward
// zero), as src/transform/falcon_dsp_fir_filter.cc:166-170 does
inline void to_int16(const std::vector<std::complex<float>>& in, std::vector<std::complex<int16_t>>& out) {
    out.clear();
    out.reserve(in.size());
    for (const auto& s : in) out.emplace_back((int16_t)s.real(), (int16_t)s.imag());
}

}  // namespace gb300_detail
}  // namespace falcon_dsp

#endif
