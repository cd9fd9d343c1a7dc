"""CPU tests of the parity oracle (no GPU).

1. The reference's own known-answer tests, run on the C restatement
   (test/tests/transform/*_unit_tests.*, test/tests/utilities/falcon_dsp_utils_unit_tests.cc).
2. The golden vectors (tests/golden, regenerated from the reference's
   notebooks) with the reference tests' tolerances.
3. The C restatement against the reference's OWN CPU classes compiled from its
   sources (oracle/_ref), on seeded random inputs streamed in uneven blocks:
   identical output counts and streaming state, identical samples.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.golden_io import manifest, near_per_component, read_c16, read_taps

MAN = manifest()


# ---------------------------------------------------------------- 1. KATs
def test_kat_resample_001():
    # falcon_dsp_polyphase_resample_cpp_unit_tests.cc:167-200 (upfirdn([.5,1,2], ones(7), 1, 2))
    y = O.Resampler(1, 2, [0.5, 1.0, 2.0]).apply(np.ones(7))
    assert y.size == 4  # streaming apply emits no tail flush
    np.testing.assert_allclose(y.real, [0.5, 3.5, 3.5, 3.5], atol=0.1)


def test_kat_resample_cuda_002_003_004():
    # falcon_dsp_polyphase_resample_cuda_unit_tests.cu:198-301
    y = O.Resampler(1, 2, [0.5, 1.0, 2.0]).apply(np.ones(1000))
    assert abs(y[0] - 0.5) < 0.1 and np.all(np.abs(y[1:] - 3.5) < 0.1)
    h = [0.5, 0.5, 1.0, 0.3, 0.07, 0.1, 0.4]
    y = O.Resampler(1, 2, h).apply(np.ones(1000))
    np.testing.assert_allclose(y[:3].real, [0.5, 2.0, 2.37], atol=0.1)
    assert np.all(np.abs(y[3:] - 2.87) < 0.1)
    y = O.Resampler(4, 5, [0.5, 1.0, 2.0]).apply(np.ones(10))
    np.testing.assert_allclose(y.real, [0.5, 1, 2, 0, 0.5, 1, 2, 0], atol=0.1)


def test_kat_fir():
    # falcon_dsp_fir_filter_cpp_unit_tests.cc:147-306
    h = [0.5, 2.0, 4.0]
    np.testing.assert_array_equal(O.FIR(h).apply(np.ones(3)).real, [0.5, 2.5, 6.5])
    np.testing.assert_array_equal(O.FIR(h).apply(np.ones(8)).real, [0.5, 2.5] + [6.5] * 6)
    f = O.FIR(h)
    y = np.concatenate([f.apply(np.ones(1)) for _ in range(8)])  # sample by sample
    np.testing.assert_array_equal(y.real, [0.5, 2.5] + [6.5] * 6)
    x = np.array([1, 1, 1, 2, 2, 2, 5, 5, 5, 1, 1], dtype=np.float32)
    np.testing.assert_array_equal(O.FIR(h).apply(x).real,
                                  [0.5, 2.5, 6.5, 7.0, 9.0, 13.0, 14.5, 20.5, 32.5, 30.5, 22.5])


def test_kat_polar():
    # falcon_dsp_polar_discriminator_cpp_unit_tests.cc:78-107
    x = np.array([88 - 85j, 22 + 97j, 54 + 91j, 6 - 13j, -29 + 58j])
    y = O.Polar().apply(x)
    np.testing.assert_allclose(y, [2.11582422, -0.31252633, -2.17362758, -3.11035282], atol=1e-4)


def test_kat_rat_approx():
    # falcon_dsp_utils_unit_tests.cc:175-218
    cases = [(1.0, 1, 1, 1), (0.5, 1, 0, 1), (0.5, 10, 1, 2), (0.33333, 100, 1, 3), (0.28571, 100, 2, 7),
             (0.625, 100, 5, 8), (0.768, 100, 53, 69), (1.30208, 100, 125, 96)]
    for f, md, n, d in cases:
        assert O.rat_approx(f, md) == (n, d)


def test_freq_shift_params():
    # rollover scaled by 10 until >= 1e5 (freq_shift.cc:216-229)
    assert O.freq_shift_params(1000000, 100000)[0] == 100000
    assert O.freq_shift_params(1000000, -5000)[0] == 200000
    r, w = O.freq_shift_params(30720000, 1000)
    assert r == 307200 and abs(w - 2 * np.pi * 1000 / 30720000) < 1e-15


# ---------------------------------------------------------------- 2. golden
def _delay(ntaps, up, down):
    return ntaps // min(up, down) // 2  # calculate_filter_delay_from_up_down_rates


@pytest.mark.parametrize("name", ["004", "005", "006", "007", "008", "009"])
def test_golden_resample(name):
    # falcon_dsp_polyphase_resample_cpp_unit_tests.cc:98-165: resample() then
    # max(1% |expected|, 10) per component after the filter delay
    m = MAN[name]
    x = read_c16(f"test_{name}_x.bin")
    h = read_taps(f"test_{name}.filter_coeffs.txt")
    y_exp = read_c16(f"test_{name}_y.bin")
    up, down = O.rat_approx(m["fs_out"] / m["fs_in"], 1024)
    assert (up, down) == (m["up"], m["down"])
    y = O.Resampler(up, down, h).apply(x)
    assert y.size <= y_exp.size + 1
    d = _delay(h.size, up, down)
    ok, bad = near_per_component(y[d:], y_exp[d:], 0.01, 10.0)
    assert ok, f"first mismatch at {bad + d}"


@pytest.mark.parametrize("name", ["001", "003"])
def test_golden_freq_shift(name):
    # falcon_dsp_freq_shift_cpp_unit_tests.cc:76-130 (int16 in/out, +-40.96)
    m = MAN[name]
    x = read_c16(f"test_{name}_x.bin")
    y = O.NCO(m["fs_in"], m["freq_shift"]).apply(x)
    y16 = np.trunc(y.real) + 1j * np.trunc(y.imag)
    y_exp = read_c16(f"test_{name}_y.bin")
    ok, bad = near_per_component(y16, y_exp, 0.0, 2048 * 0.02)
    assert ok, bad


@pytest.mark.parametrize("name", ["012", "013", "014"])
def test_golden_multichan_shift(name):
    m = MAN[name]
    x = read_c16(f"test_{name}_x.bin")
    for f in m["shifts"]:
        y = O.NCO(m["fs_in"], f).apply(x)
        ok, bad = near_per_component(y, read_c16(f"test_{name}_y_shift_{f}_hz.bin"), 0.0, 2048 * 0.02)
        assert ok, (f, bad)


@pytest.mark.parametrize("name", ["010", "011"])
def test_golden_fir(name):
    # falcon_dsp_fir_filter_cpp_unit_tests.cc:96-145: max(1%, 10)
    x = read_c16(f"test_{name}_x.bin")
    h = read_taps(f"test_{name}.filter_coeffs.txt")
    y = O.FIR(h).apply(x)
    ok, bad = near_per_component(y, read_c16(f"test_{name}_y.bin"), 0.01, 10.0)
    assert ok, bad


def _chan_cfg(name):
    m = MAN[name]
    chans = []
    for c in m["channels"]:
        chans.append(dict(output_sample_rate_in_sps=c["rate"], freq_shift_in_hz=c["shift"], up_rate=c["up"],
                          down_rate=c["down"], coeffs=read_taps(f"test_{name}_resamp_coeffs_{c['shift']}_hz.txt")))
    return m, chans


@pytest.mark.parametrize("name", ["015", "016", "017", "018"])
def test_golden_channelizer(name):
    # falcon_dsp_multi_rate_channelizer_cpp_unit_tests.cc:76-190: max(5%, 40.96)
    m, chans = _chan_cfg(name)
    x = read_c16(f"test_{name}_x.bin")
    ys = O.Channelizer(m["fs_in"], chans).apply(x)
    for c, y in zip(m["channels"], ys):
        y_exp = read_c16(f"test_{name}_y_shift_{c['shift']}_hz.bin")
        ok, bad = near_per_component(y, y_exp, 0.05, 2048 * 0.02)
        assert ok, (c["shift"], bad)


def test_golden_channelizer_segments_018():
    # cpp_multi_rate_chan_segment_018 (:429-452): same vectors, streamed in segments
    m, chans = _chan_cfg("018")
    x = read_c16("test_018_x.bin")
    ch = O.Channelizer(m["fs_in"], chans)
    parts = [ch.apply(x[i:i + 1000]) for i in range(0, x.size, 1000)]
    for ci, c in enumerate(m["channels"]):
        y = np.concatenate([p[ci] for p in parts])
        ok, bad = near_per_component(y, read_c16(f"test_018_y_shift_{c['shift']}_hz.bin"), 0.05, 2048 * 0.02)
        assert ok, (c["shift"], bad)


# ---------------------------------------------------------------- 3. vs reference CPU
needs_ref = pytest.mark.skipif(not O.have_reference(), reason="reference sources not built here (oracle/_ref)")


def _rand(n, seed, scale=1000.0):
    r = np.random.default_rng(seed)
    return ((r.standard_normal(n) + 1j * r.standard_normal(n)) * scale).astype(np.complex64)


def _blocks(n, seed):
    r = np.random.default_rng(seed)
    cuts, i = [], 0
    while i < n:
        k = int(r.choice([1, 2, 7, 33, 500, 4096]))
        cuts.append((i, min(n, i + k)))
        i += k
    return cuts


@needs_ref
@pytest.mark.parametrize("up,down,ntaps", [(1, 2, 3), (4, 5, 3), (147, 160, 3528), (3, 125, 300), (2, 1, 41),
                                           (1, 1, 17), (7, 3, 64)])
def test_port_matches_reference_resampler(up, down, ntaps):
    x = _rand(20000, 1)
    h = _rand(ntaps, 2, 1.0)
    a, b = O.Resampler(up, down, h), O.RefResampler(up, down, h)
    for i, j in _blocks(x.size, 3):
        assert a.needed_out_count(j - i) == b.needed_out_count(j - i)
        ya, yb = a.apply(x[i:j]), b.apply(x[i:j])
        assert ya.size == yb.size
        np.testing.assert_array_equal(ya, yb)


@needs_ref
def test_port_matches_reference_channelizer():
    x = _rand(30000, 4)
    chans = [dict(freq_shift_in_hz=f, up_rate=u, down_rate=d, coeffs=_rand(t, 5 + i, 1.0))
             for i, (f, u, d, t) in enumerate([(-350000, 1, 10, 201), (60000, 1, 4, 81), (27000, 77, 200, 400),
                                               (0, 3, 20, 61)])]
    a, b = O.Channelizer(1000000, chans), O.RefChannelizer(1000000, chans)
    for rep in range(2):
        for i, j in _blocks(x.size, 6 + rep):
            ya, yb = a.apply(x[i:j]), b.apply(x[i:j])
            for u, v in zip(ya, yb):
                assert u.size == v.size
                np.testing.assert_array_equal(u, v)
        a.reset_state()
        b.reset_state()


@needs_ref
def test_port_matches_reference_fir_polar():
    x = _rand(5000, 7)
    h = _rand(129, 8, 0.1)
    a, b = O.FIR(h), O.ref_lib()
    hr = O.as_c64(h)
    hb = b.ref_fir_new(O._f32p(hr.view(np.float32)), hr.size)
    for i, j in _blocks(x.size, 9):
        ya = a.apply(x[i:j])
        xb = O.as_c64(x[i:j])
        yb = np.empty_like(xb)
        b.ref_fir_apply(hb, O._f32p(xb.view(np.float32)), xb.size, O._f32p(yb.view(np.float32)))
        np.testing.assert_allclose(ya, yb, rtol=1e-5, atol=1e-2)
    b.ref_fir_free(hb)
    pa, pb = O.Polar(), b.ref_polar_new()
    for i, j in _blocks(x.size, 10):
        ya = pa.apply(x[i:j])
        xb = O.as_c64(x[i:j])
        yb = np.empty(xb.size, np.float32)
        n = b.ref_polar_apply(pb, O._f32p(xb.view(np.float32)), xb.size, O._f32p(yb))
        assert n == ya.size
        np.testing.assert_allclose(ya, yb[:n], atol=1e-6)
    b.ref_polar_free(pb)


@needs_ref
def test_port_matches_reference_rat_approx_and_params():
    r = np.random.default_rng(11)
    lib = O.ref_lib()
    import ctypes as C
    for _ in range(300):
        f = float(r.uniform(0.001, 4.0))
        md = int(r.choice([10, 100, 1024, 5000]))
        n, d = C.c_int64(), C.c_int64()
        lib.ref_rat_approx(f, md, C.byref(n), C.byref(d))
        assert O.rat_approx(f, md) == (n.value, d.value)
    for _ in range(300):
        fs = int(r.integers(1000, 100_000_000))
        f = int(r.integers(-fs // 2, fs // 2))
        if f == 0:
            continue
        rr, w = C.c_uint32(), C.c_double()
        lib.ref_freq_shift_params(fs, f, C.byref(rr), C.byref(w))
        assert O.freq_shift_params(fs, f) == (rr.value, w.value)
