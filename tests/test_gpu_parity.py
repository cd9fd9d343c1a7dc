"""GPU parity tests: every call goes through the C ABI of
libfalcon_dsp_gb300.so (via the Python mirror of the reference classes) and is
checked against the oracle (oracle/fdsp_oracle.c, pinned to the reference's
CPU code and golden vectors by tests/test_oracle.py).

Tolerances:
  * output counts and streaming state (coeff_phase, xOffset, NCO counter):
    bit-exact;
  * FP32 samples: relative RMS error <= 1e-5 against the oracle's FP32 path
    (the same bound is also checked against the FP64 oracle);
  * golden vectors: the reference tests' own per-component rules.
"""
import numpy as np
import pytest

import libfalcon_dsp_gb300 as F
from oracle import oracle as O
from tests.golden_io import manifest, near_per_component, read_c16, read_taps, rel_rms

pytestmark = pytest.mark.gpu
MAN = manifest()
RMS = 1e-5


def _rand(n, seed, scale=1000.0):
    r = np.random.default_rng(seed)
    return ((r.standard_normal(n) + 1j * r.standard_normal(n)) * scale).astype(np.complex64)


def _blocks(n, seed, sizes=(1, 2, 7, 33, 500, 4096, 20000)):
    r = np.random.default_rng(seed)
    cuts, i = [], 0
    while i < n:
        k = int(r.choice(sizes))
        cuts.append((i, min(n, i + k)))
        i += k
    return cuts


# ------------------------------------------------------------------ resampler
def test_resampler_kats():
    # falcon_dsp_polyphase_resample_cuda_unit_tests.cu:165-301
    y = F.PolyphaseResamplerCuda(1, 2, [0.5, 1.0, 2.0]).apply(np.ones(7, np.complex64))
    np.testing.assert_allclose(y, [0.5, 3.5, 3.5, 3.5], atol=1e-6)
    y = F.PolyphaseResamplerCuda(1, 2, [0.5, 1.0, 2.0]).apply(np.ones(1000, np.complex64))
    assert y.size == 500 and abs(y[0] - 0.5) < 1e-6 and np.all(np.abs(y[1:] - 3.5) < 1e-6)
    h = [0.5, 0.5, 1.0, 0.3, 0.07, 0.1, 0.4]
    y = F.PolyphaseResamplerCuda(1, 2, h).apply(np.ones(1000, np.complex64))
    np.testing.assert_allclose(y[:3].real, [0.5, 2.0, 2.37], atol=1e-5)
    assert np.all(np.abs(y[3:] - 2.87) < 1e-5)
    y = F.PolyphaseResamplerCuda(4, 5, [0.5, 1.0, 2.0]).apply(np.ones(10, np.complex64))
    np.testing.assert_allclose(y.real, [0.5, 1, 2, 0, 0.5, 1, 2, 0], atol=1e-6)
    # apply(vector<float>) overload returns floats
    y = F.PolyphaseResamplerCuda(1, 2, [0.5, 1.0, 2.0]).apply(np.ones(7, np.float32))
    assert y.dtype == np.float32 and np.allclose(y, [0.5, 3.5, 3.5, 3.5])


@pytest.mark.parametrize("up,down,ntaps", [(1, 2, 3), (4, 5, 3), (147, 160, 3528), (3, 125, 300), (2, 1, 41),
                                           (1, 1, 17), (7, 3, 64), (11, 250, 5001), (1, 10, 4095)])
def test_resampler_streaming_vs_oracle(up, down, ntaps):
    x = _rand(60000, 1)
    h = _rand(ntaps, 2, 0.05)
    g, o = F.PolyphaseResamplerCuda(up, down, h), O.Resampler(up, down, h)
    ys_g, ys_o = [], []
    for i, j in _blocks(x.size, 3):
        assert g.out_count(j - i) == o.loop_out_count(j - i)
        assert g.needed_out_count(j - i) == o.needed_out_count(j - i)
        ys_g.append(g.apply(x[i:j]))
        ys_o.append(o.apply(x[i:j]))
        assert ys_g[-1].size == ys_o[-1].size
        assert g.state() == (o.phase, o.xoffset)
    yg, yo = np.concatenate(ys_g), np.concatenate(ys_o)
    assert rel_rms(yg, yo) <= RMS
    assert g.coeffs_per_phase() == o.coeffs_per_phase


@pytest.mark.parametrize("name", ["004", "005", "006", "007", "008", "009"])
def test_resampler_golden(name):
    m = MAN[name]
    x = read_c16(f"test_{name}_x.bin")
    h = read_taps(f"test_{name}.filter_coeffs.txt")
    y = F.resample_cuda(m["fs_in"], x, h, m["fs_out"])
    y_o = O.Resampler(m["up"], m["down"], h).apply(x)
    assert y.size == y_o.size and rel_rms(y, y_o) <= RMS
    d = h.size // min(m["up"], m["down"]) // 2
    ok, bad = near_per_component(y[d:], read_c16(f"test_{name}_y.bin")[d:], 0.01, 10.0)
    assert ok, bad


def test_resampler_reset_and_device_path():
    torch = pytest.importorskip("torch")
    x = _rand(10000, 5)
    h = _rand(96, 6, 0.1)
    g = F.PolyphaseResamplerCuda(3, 8, h)
    y1 = g.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    g.reset_state()
    assert g.state() == (0, 0)
    y2 = g.apply(x)
    np.testing.assert_array_equal(y1, y2)
    assert rel_rms(y1, O.Resampler(3, 8, h).apply(x)) <= RMS


# ------------------------------------------------------------------ channelizer
def _chan_cfg(name):
    m = MAN[name]
    chans = [dict(output_sample_rate_in_sps=c["rate"], freq_shift_in_hz=c["shift"], up_rate=c["up"],
                  down_rate=c["down"], coeffs=read_taps(f"test_{name}_resamp_coeffs_{c['shift']}_hz.txt"))
             for c in m["channels"]]
    return m, chans


@pytest.mark.parametrize("name", ["015", "016", "017", "018"])
def test_channelizer_golden(name):
    # cuda_multi_rate_chan_015..018: NUM_ITERATIONS=2 with reset_state between
    m, chans = _chan_cfg(name)
    x = read_c16(f"test_{name}_x.bin")
    g = F.MultiRateChannelizerCuda(m["fs_in"], chans)
    ref = O.Channelizer(m["fs_in"], chans).apply(x)
    for it in range(2):
        ys = g.apply(x)
        for c, y, yo in zip(m["channels"], ys, ref):
            assert y.size == yo.size
            assert rel_rms(y, yo) <= RMS, (c["shift"], rel_rms(y, yo))
            ok, bad = near_per_component(y, read_c16(f"test_{name}_y_shift_{c['shift']}_hz.bin"), 0.05, 40.96)
            assert ok, (c["shift"], bad)
        g.reset_state()


@pytest.mark.parametrize("name,seg", [("015", 700), ("017", 2048), ("018", 1000)])
def test_channelizer_golden_segments(name, seg):
    # cuda_multi_rate_chan_segment_*: blocks carried through the streaming state
    m, chans = _chan_cfg(name)
    x = read_c16(f"test_{name}_x.bin")
    g = F.MultiRateChannelizerCuda(m["fs_in"], chans)
    parts = [g.apply(x[i:i + seg]) for i in range(0, x.size, seg)]
    ref = O.Channelizer(m["fs_in"], chans).apply(x)
    for ci, c in enumerate(m["channels"]):
        y = np.concatenate([p[ci] for p in parts])
        assert y.size == ref[ci].size and rel_rms(y, ref[ci]) <= RMS


def _random_plan(seed, nch, fs):
    r = np.random.default_rng(seed)
    chans = []
    for c in range(nch):
        u = int(r.choice([1, 1, 2, 3, 5]))
        d = int(r.choice([2, 3, 8, 13, 25, 64, 125, 320]))
        t = int(r.integers(3, 70))
        # shifts with small rollover (R = 1e5 .. 1e6) so windows straddle rollovers often
        f = int(r.choice([100000, -100000, 250000, 12345, -77777, 0, 3, -1]))
        chans.append(dict(freq_shift_in_hz=f, up_rate=u, down_rate=d, coeffs=_rand(u * t - int(r.integers(0, u)), 10 + c, 0.05)))
    return chans


@pytest.mark.parametrize("seed,nch", [(1, 1), (2, 5), (3, 17), (4, 40)])
def test_channelizer_streaming_vs_oracle(seed, nch):
    fs = 1000000
    chans = _random_plan(seed, nch, fs)
    x = _rand(400000, seed + 100)
    g = F.MultiRateChannelizerCuda(fs, chans)
    o = O.Channelizer(fs, chans)
    o64 = O.Channelizer(fs, chans, precision="f64")
    got = [[] for _ in chans]
    exp = [[] for _ in chans]
    exp64 = [[] for _ in chans]
    for i, j in _blocks(x.size, seed, sizes=(1, 5, 999, 4096, 65536, 150000)):
        assert g.out_count(j - i) == [r.loop_out_count(j - i) for r in o.rs]
        yg, yo, y6 = g.apply(x[i:j]), o.apply(x[i:j]), o64.apply(x[i:j])
        for c in range(nch):
            got[c].append(yg[c])
            exp[c].append(yo[c])
            exp64[c].append(y6[c])
    for c in range(nch):
        a, b, b64 = np.concatenate(got[c]), np.concatenate(exp[c]), np.concatenate(exp64[c])
        assert a.size == b.size
        assert rel_rms(a, b) <= RMS, (c, chans[c]["freq_shift_in_hz"], rel_rms(a, b))
        assert rel_rms(a, b64) <= RMS


def test_channelizer_device_path_and_capacity():
    torch = pytest.importorskip("torch")
    fs = 2000000
    chans = _random_plan(9, 6, fs)
    x = _rand(50000, 9)
    g = F.MultiRateChannelizerCuda(fs, chans)
    xd = torch.from_numpy(x).cuda()
    ys = g.apply(xd)
    torch.cuda.synchronize()
    ref = O.Channelizer(fs, chans).apply(x)
    for a, b in zip(ys, ref):
        assert rel_rms(a.cpu().numpy(), b) <= RMS
    # output buffers that are too small are rejected before anything runs
    small = [torch.empty(1, dtype=torch.complex64, device="cuda") for _ in chans]
    with pytest.raises(F.FdspError) as ei:
        g.apply(xd, out=small)
    assert ei.value.status == -5


def test_channelizer_edge_cases():
    fs = 1000000
    chans = [dict(freq_shift_in_hz=100000, up_rate=1, down_rate=320, coeffs=_rand(640, 1, 0.01)),
             dict(freq_shift_in_hz=-3, up_rate=3, down_rate=2, coeffs=_rand(7, 2, 0.1))]
    g = F.MultiRateChannelizerCuda(fs, chans)
    o = O.Channelizer(fs, chans)
    # empty block: no outputs, no state change
    ys = g.apply(np.zeros(0, np.complex64))
    assert [y.size for y in ys] == [0, 0]
    # tiny blocks shorter than the filter history and than the decimation
    x = _rand(3000, 3)
    for i in range(0, 3000, 3):
        yg, yo = g.apply(x[i:i + 3]), o.apply(x[i:i + 3])
        for a, b in zip(yg, yo):
            assert a.size == b.size
            if b.size:
                assert rel_rms(a, b) <= RMS
    # initialize twice is refused, as in the reference
    assert g.initialize(fs, chans) is False
    with pytest.raises(F.FdspError):
        F.MultiRateChannelizerCuda(fs, [dict(freq_shift_in_hz=0, up_rate=0, down_rate=1, coeffs=[1.0])])


# ------------------------------------------------------------------ freq shift
@pytest.mark.parametrize("name", ["001", "003"])
def test_freq_shift_golden(name):
    m = MAN[name]
    x = read_c16(f"test_{name}_x.bin")
    y = F.freq_shift_cuda(m["fs_in"], x, m["freq_shift"])
    assert rel_rms(y, O.NCO(m["fs_in"], m["freq_shift"]).apply(x)) <= RMS
    ok, bad = near_per_component(np.trunc(y.real) + 1j * np.trunc(y.imag), read_c16(f"test_{name}_y.bin"), 0.0, 51.2)
    assert ok, bad


@pytest.mark.parametrize("name", ["012", "013", "014"])
def test_freq_shift_multichan_golden_and_segments(name):
    m = MAN[name]
    x = read_c16(f"test_{name}_x.bin")
    g = F.FreqShiftCuda(m["fs_in"], m["shifts"])
    ys = g.apply(x)
    for f, y in zip(m["shifts"], ys):
        ok, bad = near_per_component(y, read_c16(f"test_{name}_y_shift_{f}_hz.bin"), 0.0, 51.2)
        assert ok, (f, bad)
    # cuda_multi_chan_freq_shift_by_segment_014: same result in segments
    g.reset_state()
    parts = [g.apply(x[i:i + 1250]) for i in range(0, x.size, 1250)]
    for c, y in enumerate(ys):
        np.testing.assert_allclose(np.concatenate([p[c] for p in parts]), y, rtol=0, atol=1e-3)


def test_freq_shift_streaming_vs_oracle_rollover():
    fs = 1000000
    shifts = [100000, -100000, 12345, 0, -5000, 499999]
    x = _rand(1300000, 4)
    g = F.FreqShiftCuda(fs, shifts)
    os_ = [O.NCO(fs, f) for f in shifts]
    for i, j in _blocks(x.size, 4, sizes=(1, 3, 4096, 100000, 333333)):
        ys = g.apply(x[i:j])
        for c, (y, o) in enumerate(zip(ys, os_)):
            assert rel_rms(y, o.apply(x[i:j])) <= RMS
            if shifts[c] != 0:
                # For 0 Hz the reference's rollover is (uint32_t)round(fs / 0.0), an
                # undefined conversion (0 on x86-64, UINT32_MAX on aarch64); the
                # counter then multiplies an angular frequency of 0 and never
                # affects a sample, so only shifted channels compare counters.
                assert g.counter(c) == o.counter


# ------------------------------------------------------------------ FIR
def test_fir_kats():
    h = [0.5, 2.0, 4.0]
    np.testing.assert_array_equal(F.fir_filter_cuda(h, np.ones(3, np.complex64)).real, [0.5, 2.5, 6.5])
    f = F.FirFilterCuda(h)
    y = np.concatenate([f.apply(np.ones(1, np.complex64)) for _ in range(8)])
    np.testing.assert_array_equal(y.real, [0.5, 2.5] + [6.5] * 6)
    x = np.array([1, 1, 1, 2, 2, 2, 5, 5, 5, 1, 1], np.complex64)
    np.testing.assert_array_equal(F.FirFilterCuda(h).apply(x).real,
                                  [0.5, 2.5, 6.5, 7.0, 9.0, 13.0, 14.5, 20.5, 32.5, 30.5, 22.5])
    # int16 overload truncates back to int16 (fir_filter_cpp_unit_tests.cc:147-174)
    y16 = F.FirFilterCuda([0.5, 2.0, 4.0]).apply(np.array([[1, 0]] * 3, np.int16))
    np.testing.assert_array_equal(y16[:, 0], [0, 2, 6])


@pytest.mark.parametrize("name", ["010", "011"])
def test_fir_golden(name):
    x = read_c16(f"test_{name}_x.bin")
    h = read_taps(f"test_{name}.filter_coeffs.txt")
    y = F.fir_filter_cuda(h, x)
    assert rel_rms(y, O.FIR(h).apply(x)) <= RMS
    ok, bad = near_per_component(y, read_c16(f"test_{name}_y.bin"), 0.01, 10.0)
    assert ok, bad


@pytest.mark.parametrize("ntaps", [1, 3, 129, 4095])
def test_fir_streaming_complex_taps(ntaps):
    x = _rand(50000, 12)
    h = _rand(ntaps, 13, 0.05)
    g, o = F.FirFilterCuda(h), O.FIR(h)
    ys_g, ys_o = [], []
    for i, j in _blocks(x.size, 14):
        ys_g.append(g.apply(x[i:j]))
        ys_o.append(o.apply(x[i:j]))
    assert rel_rms(np.concatenate(ys_g), np.concatenate(ys_o)) <= RMS


# ------------------------------------------------------------------ polar discriminator
def test_polar_kat_and_streaming():
    x = np.array([88 - 85j, 22 + 97j, 54 + 91j, 6 - 13j, -29 + 58j], np.complex64)
    y = F.polar_discriminator_cuda(x)
    np.testing.assert_allclose(y, [2.11582422, -0.31252633, -2.17362758, -3.11035282], atol=1e-4)
    xs = _rand(100000, 15)
    g, o = F.PolarDiscriminatorCuda(), O.Polar()
    for i, j in _blocks(xs.size, 16):
        a, b = g.apply(xs[i:j]), o.apply(xs[i:j])
        assert a.size == b.size
        # compare angles modulo 2 pi: a product whose imaginary part rounds
        # to the other side of zero flips atan2 between +pi and -pi
        np.testing.assert_allclose(np.angle(np.exp(1j * (a.astype(np.float64) - b))), 0, atol=2e-6)
    g.reset_state()
    assert g.apply(xs[:10]).size == 9
