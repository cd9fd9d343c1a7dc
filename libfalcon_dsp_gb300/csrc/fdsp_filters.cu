// Resampling filter design, host only.
//
// fdsp_get_resample_fir_params: lookup in the predefined table
//   (src/transform/falcon_dsp_fir_filter.cc:111-130).  The table itself is
//   generated at build time by libfalcon_dsp_gb300/filter_design.py, which
//   restates the reference's generator recipe
//   (test/utilities/generate_predefined_fir_filter_coeffs.ipynb), into
//   _build/gen/fdsp_filter_table.inc.
// fdsp_design_resample_firls: the same FIRLS recipe for any rate pair, in
//   closed form.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "fdsp_c.h"

namespace {

struct PredefinedFilter {
  uint32_t in_sps, out_sps;
  int32_t taps;
  uint32_t source;
  uint32_t up, down, count;
  const float* h;
};

#include "fdsp_filter_table.inc"

// Fraction("%.12f" % ratio).limit_denominator(10**6): the decimal text as an
// exact fraction, then the closest fraction with denominator <= 10^6
// (continued-fraction convergents and the best semiconvergent).
void ratio_fraction(uint32_t in_sps, uint32_t out_sps, uint64_t* num, uint64_t* den) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%.12f", (double)out_sps / (double)in_sps);
  // integer and fractional digits of the text -> N / 10^12
  const char* dot = buf;
  while (*dot && *dot != '.') ++dot;
  uint64_t ip = std::strtoull(buf, nullptr, 10);
  uint64_t fp = *dot ? std::strtoull(dot + 1, nullptr, 10) : 0;
  const uint64_t D0 = 1000000000000ull;
  uint64_t N = ip * D0 + fp, D = D0;
  auto gcd = [](uint64_t a, uint64_t b) {
    while (b) {
      const uint64_t t = a % b;
      a = b;
      b = t;
    }
    return a;
  };
  const uint64_t g = gcd(N, D);
  N /= g;
  D /= g;
  const uint64_t maxd = 1000000ull;
  if (D <= maxd) {
    *num = N;
    *den = D;
    return;
  }
  uint64_t p0 = 0, q0 = 1, p1 = 1, q1 = 0, n = N, d = D;
  for (;;) {
    const uint64_t a = n / d;
    const uint64_t q2 = q0 + a * q1;
    if (q2 > maxd) break;
    const uint64_t p2 = p0 + a * p1;
    p0 = p1;
    q0 = q1;
    p1 = p2;
    q1 = q2;
    const uint64_t r = n - a * d;
    n = d;
    d = r;
  }
  const uint64_t k = (maxd - q0) / q1;
  const uint64_t bn = p0 + k * p1, bd = q0 + k * q1;
  // |p1/q1 - N/D| <= |bn/bd - N/D| picks the convergent (ties to it)
  const __int128 e2 = (__int128)p1 * D - (__int128)N * q1;
  const __int128 e1 = (__int128)bn * D - (__int128)N * bd;
  const __int128 a2 = (e2 < 0 ? -e2 : e2) * (__int128)bd;
  const __int128 a1 = (e1 < 0 ? -e1 : e1) * (__int128)q1;
  if (a2 <= a1) {
    *num = p1;
    *den = q1;
  } else {
    *num = bn;
    *den = bd;
  }
}

// modified Bessel function I0 by its power series (terms (x/2)^2k / (k!)^2)
double bessel_i0(double x) {
  const double y = 0.25 * x * x;
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 500; ++k) {
    term *= y / ((double)k * (double)k);
    sum += term;
    if (term < sum * 1e-17) break;
  }
  return sum;
}

}  // namespace

extern "C" {

int fdsp_get_resample_fir_params(uint32_t in_sps, uint32_t out_sps, int32_t taps, uint32_t source, uint32_t* up_rate,
                                 uint32_t* down_rate, fdsp_cf32* coeffs, uint32_t cap, uint32_t* n_coeffs) {
  if (n_coeffs) *n_coeffs = 0;
  for (const PredefinedFilter& f : kPredefined) {
    if (f.in_sps != in_sps || f.out_sps != out_sps || f.taps != taps || f.source != source) continue;
    if (up_rate) *up_rate = f.up;
    if (down_rate) *down_rate = f.down;
    if (n_coeffs) *n_coeffs = f.count;
    if (coeffs == nullptr || cap < f.count) return FDSP_ERR_CAPACITY;
    for (uint32_t i = 0; i < f.count; ++i) coeffs[i] = fdsp_cf32{f.h[i], 0.0f};
    return FDSP_OK;
  }
  return FDSP_ERR_NOT_FOUND;
}

int fdsp_design_resample_firls(uint32_t in_sps, uint32_t out_sps, uint32_t num_taps, double kaiser_beta,
                               uint32_t* up_rate, uint32_t* down_rate, fdsp_cf32* coeffs, uint32_t cap,
                               uint32_t* n_coeffs) {
  if (n_coeffs) *n_coeffs = 0;
  if (in_sps == 0 || out_sps == 0 || num_taps == 0 || num_taps > (1u << 24) || !(kaiser_beta >= 0.0))
    return FDSP_ERR_INVALID_ARG;
  uint64_t p = 0, q = 0;
  ratio_fraction(in_sps, out_sps, &p, &q);
  if (p == 0 || q == 0 || p > 0xffffffffull || q > 0xffffffffull) return FDSP_ERR_INVALID_ARG;
  const uint32_t n = (num_taps % 2 == 0) ? num_taps + 1 : num_taps;
  if (up_rate) *up_rate = (uint32_t)p;
  if (down_rate) *down_rate = (uint32_t)q;
  if (n_coeffs) *n_coeffs = n;
  if (coeffs == nullptr || cap < n) return FDSP_ERR_CAPACITY;
  // Least squares over [0, e] (gain 1) and [e, 1] (gain 0), e = 1/m of
  // Nyquist, m = max(up, down): with the two bands covering [0, 1] the
  // normal equations are diagonal and the solution is the truncated ideal
  // lowpass h[k] = e sinc(e (k - M)), M = (n - 1)/2.
  const double m = (double)(p > q ? p : q);
  const double e = 1.0 / m;
  const double M = 0.5 * (double)(n - 1);
  const double i0b = bessel_i0(kaiser_beta);
  const double kPi = 3.14159265358979323846;
  for (uint32_t k = 0; k < n; ++k) {
    const double t = ((double)k - M) * e;
    const double sinc = t == 0.0 ? 1.0 : std::sin(kPi * t) / (kPi * t);
    const double x = n > 1 ? 2.0 * (double)k / (double)(n - 1) - 1.0 : 0.0;
    const double w = bessel_i0(kaiser_beta * std::sqrt(std::fmax(0.0, 1.0 - x * x))) / i0b;
    coeffs[k] = fdsp_cf32{(float)((double)p * e * sinc * w), 0.0f};
  }
  return FDSP_OK;
}

}  // extern "C"
