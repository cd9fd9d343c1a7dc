"""The oracle's C restatement against outputs of the reference's own CPU
classes, stored as fixtures (tests/golden/ref_fixtures.npz, made by
tests/golden/gen_ref_fixtures.py from the reference compiled in place).

These run everywhere, with or without a reference checkout, so the oracle
that every GPU parity test trusts is pinned to the reference on every run:
resampler counts and samples bit-exact over ragged streaming blocks, the
channelizer bit-exact over two passes with a reset, FIR and polar within
FP32 summation-order tolerance, rat_approx and get_freq_shift_params exact,
the IIR filter bit-exact, the FM demodulator within one int16 count, and
every predefined filter-table entry by SHA-256 of its coefficients.
"""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, HERE)
import gen_ref_fixtures as G  # noqa: E402

FX = np.load(os.path.join(HERE, "ref_fixtures.npz"))


@pytest.mark.parametrize("up,down,ntaps", G.RESAMPLER_CASES)
def test_resampler_matches_reference_fixture(up, down, ntaps):
    x = G.rand_c64(3000, 1)
    r = O.Resampler(up, down, G.rand_c64(ntaps, 2, 1.0))
    ys = [r.apply(x[i:j]) for i, j in G.block_cuts(x.size, 3)]
    np.testing.assert_array_equal(np.array([y.size for y in ys]), FX[f"resamp_{up}_{down}_{ntaps}_counts"])
    np.testing.assert_array_equal(np.concatenate(ys), FX[f"resamp_{up}_{down}_{ntaps}"])


def test_channelizer_matches_reference_fixture():
    x = G.rand_c64(8000, 4)
    chans = [dict(freq_shift_in_hz=f, up_rate=u, down_rate=d, coeffs=G.rand_c64(t, 5 + i, 1.0))
             for i, (f, u, d, t) in enumerate(G.CHANNELIZER_CASE)]
    ch = O.Channelizer(1000000, chans)
    for rep in range(2):
        outs = [[] for _ in chans]
        for i, j in G.block_cuts(x.size, 6 + rep):
            for c, y in enumerate(ch.apply(x[i:j])):
                outs[c].append(y)
        for c in range(len(chans)):
            np.testing.assert_array_equal(np.concatenate(outs[c]), FX[f"chan_rep{rep}_ch{c}"])
        ch.reset_state()


def test_fir_and_polar_match_reference_fixture():
    x = G.rand_c64(5000, 7)
    f = O.FIR(G.rand_c64(129, 8, 0.1))
    y = np.concatenate([f.apply(x[i:j]) for i, j in G.block_cuts(x.size, 9)])
    np.testing.assert_allclose(y, FX["fir_129"], rtol=1e-5, atol=1e-2)
    p = O.Polar()
    y = np.concatenate([p.apply(x[i:j]) for i, j in G.block_cuts(x.size, 10)])
    np.testing.assert_allclose(y, FX["polar"], atol=1e-6)


def test_rat_approx_and_shift_params_match_reference_fixture():
    for (f, md), (n, d) in zip(FX["rat_approx_in"], FX["rat_approx_out"]):
        assert O.rat_approx(float(f), int(md)) == (int(n), int(d))
    for (fs, f), R, w in zip(FX["shift_params_in"], FX["shift_params_R"], FX["shift_params_w"]):
        assert O.freq_shift_params(int(fs), int(f)) == (int(R), float(w))


@pytest.mark.parametrize("ci", [0, 1])
def test_iir_matches_reference_fixture(ci):
    f = O.IIR(FX[f"iir{ci}_b"], FX[f"iir{ci}_a"])
    x, want = FX[f"iir{ci}_x"], FX[f"iir{ci}_y"]
    got, i = [], 0
    for n in (1, 3, 700, 2, 1500):
        got.append(f.apply(x[i:i + n]))
        i += n
    assert np.array_equal(np.concatenate(got), want)


def test_fm_demod_matches_reference_fixture():
    from libfalcon_dsp_gb300 import filter_design as FD
    from libfalcon_dsp_gb300.workloads import FM_RADIO_FS, fm_station
    t = FD.design_table()
    d = O.FmDemod(FM_RADIO_FS, G.FM_OFFSET, t[(FM_RADIO_FS, 228000, 64, FD.REMEZ)],
                  t[(228000, 45600, 64, FD.REMEZ)])
    xs, _ = fm_station(3 * 57000 + 123)
    outs = [d.demod_mono(b) for b in (xs[:57000], xs[57000:114123], xs[114123:])]
    np.testing.assert_array_equal([o.size for o in outs], FX["fm_counts"])
    a, b = np.concatenate(outs).astype(np.int32), FX["fm_audio"].astype(np.int32)
    assert np.max(np.abs(a - b)) <= 1
    assert np.mean(a == b) >= 0.999


def test_filter_table_matches_reference_digests():
    import libfalcon_dsp_gb300 as F
    found = 0
    for row, dig in zip(FX["table_rows"], FX["table_digests"]):
        key = tuple(int(v) for v in row[:4])
        got = F.get_resample_fir_params(*key)
        if row[4] < 0:
            assert got is None, key
            continue
        found += 1
        assert got is not None and got[:2] == (int(row[4]), int(row[5])), key
        assert G.entry_digest(got[2].real) == str(dig), key
    assert found == 51
