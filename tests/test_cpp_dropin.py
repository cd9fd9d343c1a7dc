"""The drop-in C++ classes (include/transform/*.h) used the way a
libfalcon_dsp caller uses them.

tests/cpp/dropin_check.cc drives every class (channelizer, resampler with
its real overload, multi-channel and int16 frequency shift, FIR with its
int16 overload, polar discriminator, resample_cuda) over two streaming
applies and writes inputs and outputs; here they are compared with the
oracle on the same inputs: FP32 results within 1e-5 relative RMS, output
counts exact, int16 outputs within one count (a truncated value may sit on
an integer boundary that FP32 rounding crosses).

The CPU test compiles and links the program against the library; the GPU
test runs it.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from libfalcon_dsp_gb300 import filter_design as FD
from oracle import oracle as O
from tests.golden_io import rel_rms

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "libfalcon_dsp_gb300", "_lib")
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_check.cc")


def _compile(tmp_path) -> str:
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "dropin_check")
    cmd = [cxx, "-std=c++14", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", LIBDIR, "-lfalcon_dsp_gb300", f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_dropin_headers_compile_and_link(tmp_path):
    exe = _compile(tmp_path)
    assert os.path.exists(exe)


def _c64(d, name):
    return np.fromfile(os.path.join(d, name), dtype=np.complex64)


def _i16(d, name):
    a = np.fromfile(os.path.join(d, name), dtype=np.int16).reshape(-1, 2)
    return a


def _near_i16(got, want_c64):
    want = np.stack([np.trunc(want_c64.real), np.trunc(want_c64.imag)], axis=1)
    assert got.shape == want.shape
    assert np.max(np.abs(got.astype(np.int64) - want.astype(np.int64))) <= 1


@pytest.mark.gpu
def test_dropin_classes_match_oracle(tmp_path):
    exe = _compile(tmp_path)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([exe, str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    d = str(out)

    # channelizer, two streaming applies
    ups, downs, shifts = [1, 3, 2], [8, 25, 5], [125000, -770000, 0]
    chans = [dict(freq_shift_in_hz=shifts[c], up_rate=ups[c], down_rate=downs[c],
                  coeffs=_c64(d, f"chan_taps{c}.bin")) for c in range(3)]
    oc = O.Channelizer(10000000, chans)
    for b in range(2):
        ref = oc.apply(_c64(d, f"chan_in{b}.bin"))
        for c in range(3):
            got = _c64(d, f"chan_out{b}_{c}.bin")
            assert got.size == ref[c].size
            assert rel_rms(got, ref[c]) <= 1e-5

    # resampler 147/160, streaming; real overload at 2/3
    orr = O.Resampler(147, 160, _c64(d, "rs_taps.bin"))
    for b in range(2):
        ref = orr.apply(_c64(d, f"rs_in{b}.bin"))
        got = _c64(d, f"rs_out{b}.bin")
        assert got.size == ref.size and rel_rms(got, ref) <= 1e-5
    rin = np.fromfile(os.path.join(d, "rsr_in.bin"), dtype=np.float32)
    ref = O.Resampler(2, 3, _c64(d, "rs_taps.bin")).apply(rin.astype(np.complex64)).real
    got = np.fromfile(os.path.join(d, "rsr_out.bin"), dtype=np.float32)
    assert got.size == ref.size and rel_rms(got, ref) <= 1e-5

    # frequency shift: two channels, then int16 in/out
    x = _c64(d, "fs_in.bin")
    for c, f in enumerate([1000, -250000]):
        ref = O.NCO(1000000, f).apply(x)
        assert rel_rms(_c64(d, f"fs_out{c}.bin"), ref) <= 1e-5
    i16 = _i16(d, "fs16_in.bin")
    ref = O.NCO(1000000, 123456).apply((i16[:, 0] + 1j * i16[:, 1]).astype(np.complex64))
    _near_i16(_i16(d, "fs16_out.bin"), ref)

    # FIR: complex taps, streaming; int16 overload with the reference's [.5, 2, 4]
    of = O.FIR(_c64(d, "fir_taps.bin"))
    for b in range(2):
        ref = of.apply(_c64(d, f"fir_in{b}.bin"))
        assert rel_rms(_c64(d, f"fir_out{b}.bin"), ref) <= 1e-5
    i16 = _i16(d, "fir16_in.bin")
    ref = O.FIR(np.array([0.5, 2, 4], np.complex64)).apply((i16[:, 0] + 1j * i16[:, 1]).astype(np.complex64))
    _near_i16(_i16(d, "fir16_out.bin"), ref)

    # polar discriminator: the first apply emits N-1
    op = O.Polar()
    for b in range(2):
        ref = op.apply(_c64(d, f"pd_in{b}.bin"))
        got = np.fromfile(os.path.join(d, f"pd_out{b}.bin"), dtype=np.float32)
        assert got.size == ref.size
        assert np.max(np.abs(got - ref)) <= 1e-5

    # resample_cuda 48 kHz -> 44.1 kHz (rat_approx -> 147/160)
    ref = O.Resampler(147, 160, _c64(d, "rsc_taps.bin")).apply(_c64(d, "rsc_in.bin"))
    got = _c64(d, "rsc_out.bin")
    assert got.size == ref.size and rel_rms(got, ref) <= 1e-5

    # predefined filter lookup: the generator's REMEZ-64 228 kS/s -> 45.6 kS/s entry
    table = FD.design_table()
    want = table[(228000, 45600, 64, FD.REMEZ)]
    assert np.array_equal(_c64(d, "pf_taps.bin").real, want[2])

    # FM demodulator, two streaming calls, against the oracle's demod_mono
    om = O.FmDemod(1140000, 150000, table[(1140000, 228000, 64, FD.REMEZ)], want)
    for b in range(2):
        ref = om.demod_mono(_c64(d, f"fm_in{b}.bin"))
        got = np.fromfile(os.path.join(d, f"fm_out{b}.bin"), dtype=np.int16)
        assert got.size == ref.size and got.size > 0
        assert np.max(np.abs(got.astype(np.int32) - ref.astype(np.int32))) <= 1
