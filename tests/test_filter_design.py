"""Resampling filter design: the predefined table behind
fdsp_get_resample_fir_params (src/transform/falcon_dsp_fir_filter.cc:111-130)
and the native FIRLS designer.

Host-only functions of the library, so these run without a GPU:

* every key of the reference's table (51 entries: 6 rate pairs x tap counts
  x REMEZ/FIRLS) returns the reference's up/down and coefficients
  BIT-EXACTLY (checked against the reference's own compiled table where the
  reference build is present, else against the generator);
* keys the reference lacks (REMEZ above 200 taps, unknown rates) return
  FDSP_ERR_NOT_FOUND, the reference's `false`;
* the native FIRLS designer equals the table's FIRLS entries to within the
  table's 8-decimal rounding, and the float64 closed form.
"""
import ctypes as C

import numpy as np
import pytest

import libfalcon_dsp_gb300 as F
from libfalcon_dsp_gb300 import _capi
from libfalcon_dsp_gb300 import filter_design as FD
from oracle import oracle as O

TAPS = [16, 32, 64, 128, 256, -1]


def _all_keys():
    return [(fi, fo, t, s) for fi, fo in FD.RATE_PAIRS for t in TAPS for s in (F.REMEZ, F.FIRLS)]


@pytest.fixture(scope="module")
def table():
    return FD.design_table()


def test_table_has_the_reference_key_set(table):
    assert len(table) == 51
    # REMEZ exists only up to 200 taps; OPTIMAL orders are 20 max(up, down) + 1
    for (fi, fo, t, s), (p, q, h) in table.items():
        m = max(p, q)
        n = {-1: 20 * m + 1}.get(t, t)
        if s == F.FIRLS:
            assert h.size == (n + 1 if n % 2 == 0 else n)
        else:
            assert h.size == n and n <= 200


def test_library_table_matches_generator(table):
    for key in _all_keys():
        got = F.get_resample_fir_params(*key)
        want = table.get(key)
        if want is None:
            assert got is None, key
            continue
        up, down, h = got
        assert (up, down) == want[:2], key
        assert np.array_equal(h.real, want[2]) and not np.any(h.imag), key


@pytest.mark.skipif(not O.have_reference(), reason="reference build (oracle/_ref) not present")
def test_library_table_matches_reference_bit_exactly():
    found = 0
    for key in _all_keys():
        ref = O.ref_get_resample_fir_params(*key)
        got = F.get_resample_fir_params(*key)
        if ref is None:
            assert got is None, key
            continue
        found += 1
        assert got is not None, key
        assert got[:2] == ref[:2], key
        assert got[2].size == ref[2].size and np.array_equal(got[2].real, ref[2]), key
    assert found == 51


def test_missing_keys_and_sizing():
    assert F.get_resample_fir_params(1140000, 200000, -1, F.REMEZ) is None  # 1141 taps: no REMEZ design
    assert F.get_resample_fir_params(48000, 44100, 64, F.FIRLS) is None
    up, down, n = C.c_uint32(), C.c_uint32(), C.c_uint32()
    lib = _capi.lib()
    st = lib.fdsp_get_resample_fir_params(228000, 45600, 64, 0, C.byref(up), C.byref(down), None, 0, C.byref(n))
    assert st == _capi.FDSP_ERR_CAPACITY and n.value == 64 and (up.value, down.value) == (1, 5)
    st = lib.fdsp_get_resample_fir_params(228000, 45600, 64, 7, C.byref(up), C.byref(down), None, 0, C.byref(n))
    assert st == _capi.FDSP_ERR_NOT_FOUND and n.value == 0


def test_native_firls_designer_matches_table(table):
    for (fi, fo, t, s), (p, q, h) in table.items():
        if s != F.FIRLS:
            continue
        up, down, g = F.design_resample_firls(fi, fo, h.size)
        assert (up, down) == (p, q)
        assert g.size == h.size
        # the table rounds to 8 decimals before the float conversion
        assert np.max(np.abs(g.real.astype(np.float64) - h)) <= 5e-9 + 1e-7 * np.max(np.abs(h))
        ref64 = FD.kaiser_firls_lowpass(h.size, p, q)
        assert np.max(np.abs(g.real - ref64)) <= 1e-7 * np.max(np.abs(ref64))


def test_native_designer_any_rate():
    up, down, g = F.design_resample_firls(48000, 44100, 300, beta=8.6)
    assert (up, down) == (147, 160) and g.size == 301
    ref64 = FD.kaiser_firls_lowpass(301, 147, 160, beta=8.6)
    assert np.max(np.abs(g.real - ref64)) <= 1e-6 * np.max(np.abs(ref64))
    assert FD.up_down(48000, 44100) == (147, 160)


def test_iq_files_round_trip(tmp_path):
    from libfalcon_dsp_gb300 import iq_files as IQ
    rng = np.random.default_rng(9)
    x16 = rng.integers(-32768, 32768, size=(1001, 2)).astype(np.int16)
    xc = (rng.standard_normal(77) + 1j * rng.standard_normal(77)).astype(np.complex64)
    for t in (IQ.BINARY, IQ.ASCII):
        p = str(tmp_path / f"a{t}")
        assert IQ.write_complex_data_to_file(p, t, x16)
        assert np.array_equal(IQ.read_complex_data_from_file(p, t), x16)
        p = str(tmp_path / f"b{t}")
        assert IQ.write_complex_data_to_file(p, t, xc)
        assert np.array_equal(IQ.read_complex_data_from_file(p, t, dtype=np.float32), xc)
    # BINARY int16 is little-endian "<2h" pairs
    raw = np.fromfile(str(tmp_path / "a0"), dtype="<i2").reshape(-1, 2)
    assert np.array_equal(raw, x16)
    assert IQ.read_complex_data_from_file(str(tmp_path / "missing"), IQ.BINARY) is None
