// Drives the drop-in C++ classes of include/transform the way a libfalcon_dsp
// caller would, on deterministic inputs, and writes every input and output as
// raw little-endian arrays into the directory given as argv[1]; the Python
// test compares them with the oracle.  The *_cuda objects are driven through
// references and pointers to their base classes (falcon_dsp_polyphase_resampler,
// falcon_dsp_freq_shift, falcon_dsp_fir_filter, falcon_dsp_fm_demodulator),
// as callers written against the reference's class hierarchy hold them.
// Exit status 0 when every call succeeded.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "signals/falcon_dsp_fm_demod_cuda.h"
#include "transform/falcon_dsp_fir_filter_cuda.h"
#include "transform/falcon_dsp_freq_shift_cuda.h"
#include "transform/falcon_dsp_multi_rate_channelizer_cuda.h"
#include "transform/falcon_dsp_polar_discriminator_cuda.h"
#include "transform/falcon_dsp_polyphase_resampler_cuda.h"
#include "transform/falcon_dsp_predefined_fir_filter.h"
#include "transform/falcon_dsp_resample_cuda.h"

using cvec = std::vector<std::complex<float>>;

static std::string g_dir;
static int g_fail = 0;

static void check(bool ok, const char* what) {
    if (!ok) {
        std::fprintf(stderr, "FAILED: %s\n", what);
        g_fail = 1;
    }
}

template <class T>
static void dump(const std::string& name, const std::vector<T>& v) {
    FILE* f = std::fopen((g_dir + "/" + name).c_str(), "wb");
    if (!f) {
        g_fail = 1;
        return;
    }
    if (!v.empty()) std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
}

// xorshift noise in [-1, 1)
static uint64_t g_s = 0x9E3779B97F4A7C15ull;
static float rnd() {
    g_s ^= g_s << 13;
    g_s ^= g_s >> 7;
    g_s ^= g_s << 17;
    return (float)((g_s >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
}
static cvec noise(size_t n) {
    cvec v(n);
    for (auto& s : v) s = {rnd(), rnd()};
    return v;
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    g_dir = argv[1];
    using namespace falcon_dsp;

    // channelizer: 3 channels, two streaming applies
    {
        std::vector<multi_rate_channelizer_channel_s> ch(3);
        const uint32_t up[3] = {1, 3, 2}, down[3] = {8, 25, 5};
        const int64_t shift[3] = {125000, -770000, 0};
        for (int c = 0; c < 3; ++c) {
            ch[c].output_sample_rate_in_sps = 0;
            ch[c].freq_shift_in_hz = shift[c];
            ch[c].up_rate = up[c];
            ch[c].down_rate = down[c];
            ch[c].resample_filter_coeffs = noise(24 * up[c] + c);
            dump("chan_taps" + std::to_string(c) + ".bin", ch[c].resample_filter_coeffs);
        }
        falcon_dsp_multi_rate_channelizer_cuda m;
        check(m.initialize(10000000, ch), "channelizer initialize");
        check(!m.initialize(10000000, ch), "channelizer second initialize refused");
        for (int b = 0; b < 2; ++b) {
            cvec in = noise(5000 + 333 * b);
            std::vector<cvec> out;
            check(m.apply(in, out) && out.size() == 3, "channelizer apply");
            dump("chan_in" + std::to_string(b) + ".bin", in);
            for (int c = 0; c < 3; ++c) dump("chan_out" + std::to_string(b) + "_" + std::to_string(c) + ".bin", out[c]);
        }
    }
    // resampler 147/160, two applies, complex and real overloads
    {
        cvec taps = noise(3528);
        for (auto& t : taps) t = {t.real(), 0.f};
        dump("rs_taps.bin", taps);
        falcon_dsp_polyphase_resampler_cuda r_obj;
        falcon_dsp_polyphase_resampler& r = r_obj;  // virtual dispatch through the base class
        check(r.initialize(147, 160, taps), "resampler initialize");
        check(r.coeffs_per_phase() == 24, "coeffs_per_phase");
        for (int b = 0; b < 2; ++b) {
            cvec in = noise(4096 + 77 * b), out;
            const int32_t n = r.apply(in, out);
            check(n == (int32_t)out.size() && n > 0, "resampler apply");
            dump("rs_in" + std::to_string(b) + ".bin", in);
            dump("rs_out" + std::to_string(b) + ".bin", out);
        }
        std::unique_ptr<falcon_dsp_polyphase_resampler> rr(new falcon_dsp_polyphase_resampler_cuda());
        check(rr->initialize(2, 3, taps), "real resampler initialize");
        std::vector<float> rin(1000), rout;
        for (auto& s : rin) s = rnd();
        check(rr->apply(rin, rout) > 0, "real resampler apply");
        dump("rsr_in.bin", rin);
        dump("rsr_out.bin", rout);
    }
    // frequency shift: 2 channels over one input, then a single-channel int16 shifter
    {
        falcon_dsp_freq_shift_cuda s;
        std::vector<int32_t> f = {1000, -250000};
        check(s.initialize(1000000, f), "freq shift initialize");
        cvec in = noise(3000);
        std::vector<cvec> out;
        check(s.apply(in, out) && out.size() == 2, "freq shift apply");
        dump("fs_in.bin", in);
        dump("fs_out0.bin", out[0]);
        dump("fs_out1.bin", out[1]);
        falcon_dsp_freq_shift_cuda s16_obj;
        falcon_dsp_freq_shift& s16 = s16_obj;
        check(s16.initialize(1000000, 123456), "int16 freq shift initialize");
        std::vector<std::complex<int16_t>> i16(500), o16;
        for (auto& v : i16) v = {(int16_t)(rnd() * 3000), (int16_t)(rnd() * 3000)};
        check(s16.apply(i16, o16) && o16.size() == i16.size(), "int16 freq shift apply");
        dump("fs16_in.bin", i16);
        dump("fs16_out.bin", o16);
    }
    // FIR: complex taps, two applies, and the int16 overload
    {
        cvec taps = noise(129);
        dump("fir_taps.bin", taps);
        falcon_dsp_fir_filter_cuda f_obj(taps);
        falcon_dsp_fir_filter& f = f_obj;
        for (int b = 0; b < 2; ++b) {
            cvec in = noise(2000 + 50 * b), out;
            check(f.apply(in, out) && out.size() == in.size(), "fir apply");
            dump("fir_in" + std::to_string(b) + ".bin", in);
            dump("fir_out" + std::to_string(b) + ".bin", out);
        }
        cvec t3 = {{0.5f, 0.f}, {2.f, 0.f}, {4.f, 0.f}};
        std::unique_ptr<falcon_dsp_fir_filter> f16p(new falcon_dsp_fir_filter_cuda(t3));
        falcon_dsp_fir_filter& f16 = *f16p;
        std::vector<std::complex<int16_t>> i16(64), o16;
        for (size_t k = 0; k < i16.size(); ++k) i16[k] = {(int16_t)(k * 7 % 101 - 50), (int16_t)(k * 3 % 53 - 26)};
        check(f16.apply(i16, o16) && o16.size() == i16.size(), "int16 fir apply");
        dump("fir16_in.bin", i16);
        dump("fir16_out.bin", o16);
    }
    // polar discriminator: two applies (first emits N-1)
    {
        falcon_dsp_polar_discriminator_cuda p;
        for (int b = 0; b < 2; ++b) {
            cvec in = noise(1500);
            std::vector<float> out;
            check(p.apply(in, out), "polar apply");
            check(out.size() == (b == 0 ? in.size() - 1 : in.size()), "polar count");
            dump("pd_in" + std::to_string(b) + ".bin", in);
            dump("pd_out" + std::to_string(b) + ".bin", out);
        }
    }
    // resample_cuda: 48 kHz -> 44.1 kHz
    {
        cvec taps = noise(3528), in = noise(9000), out;
        for (auto& t : taps) t = {t.real(), 0.f};
        check(resample_cuda(48000, in, taps, 44100, out), "resample_cuda");
        dump("rsc_taps.bin", taps);
        dump("rsc_in.bin", in);
        dump("rsc_out.bin", out);
    }
    // predefined filter lookup (host only)
    {
        uint32_t up = 0, down = 0;
        cvec h;
        check(get_resample_fir_params(228000, 45600, filter_taps_e::FILTER_TAPS_64, filter_source_type_e::REMEZ, up,
                                      down, h),
              "get_resample_fir_params");
        check(up == 1 && down == 5 && h.size() == 64, "predefined 228k -> 45.6k");
        dump("pf_taps.bin", h);
        check(!get_resample_fir_params(48000, 44100, filter_taps_e::FILTER_TAPS_64, filter_source_type_e::REMEZ, up,
                                       down, h) && h.empty(),
              "missing key");
    }
    // FM demodulator: station at -150 kHz in a 1.14 MS/s capture
    {
        falcon_dsp_fm_demodulator_cuda fm_obj;
        falcon_dsp_fm_demodulator& fm = fm_obj;
        check(!fm.initialize(1140000, 150000, 60e-6f), "fm bad time constant");
        check(fm.initialize(1140000, 150000), "fm initialize");
        check(!fm.initialize(1140000, 150000), "fm initialize once");
        for (int b = 0; b < 2; ++b) {
            cvec in(114000 + 7 * b);
            for (size_t i = 0; i < in.size(); ++i) {
                const double t = (double)(i + b * 114000) / 1140000.0;
                const double ph = -2 * M_PI * 150000.0 * t + 5.0 * std::sin(2 * M_PI * 1000.0 * t);
                in[i] = {(float)std::cos(ph), (float)std::sin(ph)};
            }
            std::vector<int16_t> out;
            check(fm.demod_mono(in, out), "fm demod_mono");
            dump("fm_in" + std::to_string(b) + ".bin", in);
            dump("fm_out" + std::to_string(b) + ".bin", out);
        }
    }
    std::printf(g_fail ? "dropin_check: FAILED\n" : "dropin_check: ok\n");
    return g_fail;
}
