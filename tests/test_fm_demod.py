"""FM mono demodulator (falcon_dsp_fm_demodulator_cuda,
src/signals/falcon_dsp_fm_demod_cuda.cu) and its de-emphasis IIR
(src/transform/falcon_dsp_iir_filter.cc).

CPU tests pin the oracle against the reference's own compiled classes
(oracle/_ref, present where the reference checkout is): the IIR bit-exactly,
the whole demodulator's int16 audio exactly.  The GPU test runs the library's
demodulator (every stage on the device) over three streaming calls, then a
reset, against the oracle: counts exact, int16 audio within one count (a
truncated value can sit on an integer boundary that FP32 rounding crosses:
the GPU's filters sum their taps in another order than the reference's
loop, which moves a scaled sample by ~1e-3 of a count) and equal on
>= 99.5 % of samples.
"""
import ctypes as C

import numpy as np
import pytest

from libfalcon_dsp_gb300 import _capi
from libfalcon_dsp_gb300 import filter_design as FD
from libfalcon_dsp_gb300.workloads import FM_RADIO_FS, audio_snr_db, fm_station
from oracle import oracle as O

OFFSET = 150000


def _oracle_demod(tau=75e-6):
    t = FD.design_table()
    iso = t[(FM_RADIO_FS, 228000, 64, FD.REMEZ)]
    mono = t[(228000, 45600, 64, FD.REMEZ)]
    return O.FmDemod(FM_RADIO_FS, OFFSET, iso, mono, tau)


@pytest.mark.skipif(not O.have_reference(), reason="reference build (oracle/_ref) not present")
def test_oracle_iir_matches_reference_bit_exactly():
    rng = np.random.default_rng(3)
    cases = [(np.array([0.064493014968382223], np.complex64), np.array([1.0, -0.93550698503161778], np.complex64)),
             ((rng.standard_normal(4) + 1j * rng.standard_normal(4)).astype(np.complex64),
              np.array([1.0, 0.2 - 0.1j, -0.05 + 0.02j], np.complex64))]
    for b, a in cases:
        o, r = O.IIR(b, a), O.RefIIR(b, a)
        for n in (1, 3, 700, 2, 1500):
            x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
            assert np.array_equal(o.apply(x), r.apply(x))
        o.reset_state()
        r.reset_state()
        x = rng.standard_normal(50).astype(np.complex64)
        assert np.array_equal(o.apply(x), r.apply(x))


@pytest.mark.skipif(not O.have_reference(), reason="reference build (oracle/_ref) not present")
def test_oracle_fm_demod_matches_reference():
    x, _ = fm_station(3 * 57000 + 123)
    o, r = _oracle_demod(), O.RefFmDemod(FM_RADIO_FS, OFFSET)
    for blk in (x[:57000], x[57000:114123], x[114123:]):
        a, b = o.demod_mono(blk), r.demod_mono(blk)
        assert a.size == b.size and a.size > 0
        assert np.max(np.abs(a.astype(np.int32) - b.astype(np.int32))) <= 1
        assert np.mean(a == b) >= 0.999
    assert O.RefFmDemod(FM_RADIO_FS, OFFSET, 60e-6)._h is None  # unsupported time constant


def test_create_rejects_what_the_reference_rejects():
    h = C.c_void_p()
    lib = _capi.lib()
    assert lib.fdsp_fm_demod_create(FM_RADIO_FS, OFFSET, C.c_float(60e-6), C.byref(h)) == -1
    assert lib.fdsp_fm_demod_create(2400000, OFFSET, C.c_float(75e-6), C.byref(h)) == _capi.FDSP_ERR_NOT_FOUND
    assert not h.value


@pytest.mark.gpu
@pytest.mark.parametrize("tau", [75e-6, 50e-6])
def test_gpu_fm_demod_matches_oracle(tau):
    import torch

    import libfalcon_dsp_gb300 as F
    x, tones = fm_station(1 << 19, seed=41)
    dem = F.FmDemodulatorCuda(FM_RADIO_FS, OFFSET, tau)
    o = _oracle_demod(tau)
    cuts = [0, 100003, 100004, 300000, x.size]
    audio = []
    for i in range(4):
        blk = x[cuts[i]:cuts[i + 1]]
        want = o.demod_mono(blk)
        if i % 2 == 0:
            got = dem.demod_mono(blk)
        else:
            got = dem.demod_mono(torch.from_numpy(blk).cuda()).cpu().numpy()
        assert got.size == want.size, (i, got.size, want.size)
        if want.size:
            d = np.abs(got.astype(np.int32) - want.astype(np.int32))
            assert d.max() <= 1 and np.mean(d == 0) >= 0.995, (i, d.max(), np.mean(d == 0))
        audio.append(got)
    # the demodulated audio carries the station's tones
    a = np.concatenate([audio[0], audio[2], audio[3]]).astype(np.float64)
    assert audio_snr_db(audio[3].astype(np.float64), 45600.0, tones, skip=256) > 30.0
    # reset_state: a fresh stream again
    dem.reset_state()
    o.reset_state()
    got, want = dem.demod_mono(x[:50000]), o.demod_mono(x[:50000])
    assert got.size == want.size
    assert np.max(np.abs(got.astype(np.int32) - want.astype(np.int32))) <= 1
    assert a.size > 0
