"""int16 front end: complex int16 input converted inside the first kernel
that reads it (channelizer FP32 and tensor-core paths, resampler, FIR,
frequency shift), against converting first.

The reference's int16 overloads (src/transform/falcon_dsp_freq_shift.cc:
133-162, src/transform/falcon_dsp_fir_filter.cc:151-175) convert
complex<int16_t> to complex<float> and run the float path, truncating
toward zero on the way out.  So: int16 input must give BIT-EXACTLY the
outputs of the float path on the converted input (the conversion is exact);
int16 outputs equal the truncated float outputs; streaming state carries
across int16 and float calls alike.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ci16(n, seed, amp=3000):
    rng = np.random.default_rng(seed)
    return rng.integers(-amp, amp, size=(n, 2)).astype(np.int16)


def _as_c64(x16):
    return (x16[:, 0].astype(np.float32) + 1j * x16[:, 1].astype(np.float32)).astype(np.complex64)


@pytest.mark.parametrize("precision", ["fp32", "fp16x3"])
def test_channelizer_int16_equals_converted(precision):
    import torch

    import libfalcon_dsp_gb300 as F
    from libfalcon_dsp_gb300.workloads import channelizer_256_plan, tone_signal
    fs = 61440000
    _, freqs = tone_signal(1 << 12, float(fs), 32, seed=5)
    chans = channelizer_256_plan(float(fs), freqs, nch=24, seed=6)
    a, b = F.MultiRateChannelizerCuda(fs, chans), F.MultiRateChannelizerCuda(fs, chans)
    a.set_precision(precision)
    b.set_precision(precision)
    for i, n in enumerate([70001, 3, 131072]):
        x16 = _ci16(n, 10 + i)
        if i == 1:  # host entry point
            ya, yb = a.apply(x16), b.apply(_as_c64(x16))
        else:
            ya = [y.cpu().numpy() for y in a.apply(torch.from_numpy(x16).cuda())]
            yb = [y.cpu().numpy() for y in b.apply(torch.from_numpy(_as_c64(x16)).cuda())]
        for u, v in zip(ya, yb):
            assert u.size == v.size and np.array_equal(u, v)


def test_resampler_fir_shift_int16():
    import torch

    import libfalcon_dsp_gb300 as F
    rng = np.random.default_rng(2)
    taps = (rng.standard_normal(96) * 0.1).astype(np.complex64)
    ra, rb = F.PolyphaseResamplerCuda(3, 7, taps), F.PolyphaseResamplerCuda(3, 7, taps)
    fa, fb = F.FirFilterCuda(taps[:40] * (1 + 0.5j)), F.FirFilterCuda(taps[:40] * (1 + 0.5j))
    sa, sb = F.FreqShiftCuda(1000000, [12345, -250000]), F.FreqShiftCuda(1000000, [12345, -250000])
    for i, n in enumerate([5000, 17, 40000]):
        x16 = _ci16(n, 30 + i)
        xc = _as_c64(x16)
        xd16, xdc = torch.from_numpy(x16).cuda(), torch.from_numpy(xc).cuda()
        # resampler: complex64 out
        assert np.array_equal(ra.apply(xd16).cpu().numpy(), rb.apply(xdc).cpu().numpy())
        # FIR: int16 out = truncated float out
        got = fa.apply(xd16).cpu().numpy() if i != 1 else fa.apply(x16)
        y = fb.apply(xdc).cpu().numpy()
        want = np.stack([np.trunc(y.real), np.trunc(y.imag)], axis=1).astype(np.int16)
        assert np.array_equal(got, want)
        # frequency shift, two channels
        got = [g.cpu().numpy() for g in sa.apply(xd16)] if i != 1 else sa.apply(x16)
        ys = [g.cpu().numpy() for g in sb.apply(xdc)]
        for g, y in zip(got, ys):
            want = np.stack([np.trunc(y.real), np.trunc(y.imag)], axis=1).astype(np.int16)
            assert np.array_equal(g, want)
