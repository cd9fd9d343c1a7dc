"""Edge cases of the entry points added beside the channelizer: empty and
tiny blocks, capacity errors, a one-tap tensor-core FIR, int16 inputs of
zero length.  Each follows the reference's behaviour for the same input
(empty in -> empty out, the discriminator's first call emitting N - 1)."""
import ctypes as C

import numpy as np
import pytest

import libfalcon_dsp_gb300 as F
from libfalcon_dsp_gb300 import _capi
from libfalcon_dsp_gb300 import filter_design as FD
from libfalcon_dsp_gb300.workloads import FM_RADIO_FS, fm_station
from oracle import oracle as O
from tests.golden_io import rel_rms

pytestmark = pytest.mark.gpu


def test_fm_demod_tiny_and_empty_blocks():
    t = FD.design_table()
    dem = F.FmDemodulatorCuda(FM_RADIO_FS, 150000)
    o = O.FmDemod(FM_RADIO_FS, 150000, t[(FM_RADIO_FS, 228000, 64, FD.REMEZ)], t[(228000, 45600, 64, FD.REMEZ)])
    x, _ = fm_station(40000, seed=3)
    assert dem.demod_mono(x[:0]).size == 0
    for a, b in ((0, 3), (3, 11), (11, 5000), (5000, 40000)):  # blocks too short to emit, then normal ones
        got, want = dem.demod_mono(x[a:b]), o.demod_mono(x[a:b])
        assert got.size == want.size, (a, b)
        if want.size:
            assert np.max(np.abs(got.astype(np.int32) - want.astype(np.int32))) <= 1
    # an output buffer below the count is refused
    n = dem.out_count(10000)
    buf = np.empty(max(n - 1, 1), np.int16)
    got = C.c_uint64()
    st = _capi.lib().fdsp_fm_demod_apply_host(dem._h, x.ctypes.data, 10000, buf.ctypes.data, n - 1, C.byref(got), None)
    assert st == _capi.FDSP_ERR_CAPACITY


def test_int16_zero_length_and_one_sample():
    import torch
    rng = np.random.default_rng(5)
    h = ((rng.standard_normal(16) + 1j * rng.standard_normal(16)) * 0.1).astype(np.complex64)
    f, fo = F.FirFilterCuda(h), O.FIR(h)
    s = F.FreqShiftCuda(1000000, [2500])
    for n in (0, 1, 7):
        x16 = rng.integers(-100, 100, size=(n, 2)).astype(np.int16)
        xc = (x16[:, 0] + 1j * x16[:, 1]).astype(np.complex64)
        y = f.apply(torch.from_numpy(x16).cuda()).cpu().numpy() if n else f.apply(x16)
        assert y.shape == (n, 2)
        if n:
            ref = fo.apply(xc)
            want = np.stack([np.trunc(ref.real), np.trunc(ref.imag)], axis=1)
            assert np.max(np.abs(y.astype(np.int32) - want.astype(np.int32))) <= 1
        else:
            fo.apply(xc)
        z = s.apply(x16)[0]
        assert z.shape == (n, 2)


def test_one_tap_tensor_core_fir():
    import torch
    h = np.array([0.75 - 0.25j], np.complex64)
    f = F.FirFilterCuda(h)
    f.set_precision("fp16x3")
    x = ((np.random.default_rng(6).standard_normal(300000) + 1j) * 0.5).astype(np.complex64)
    y = f.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    ref = (x.astype(np.complex128) * h[0]).astype(np.complex128)
    err = np.sum(np.abs(y - ref) ** 2) / np.sum(np.abs(ref) ** 2)
    assert 10 * np.log10(1 / err) >= 60.0


def test_channelizer_int16_empty_then_block():
    import torch
    rng = np.random.default_rng(7)
    taps = (rng.standard_normal(3 * 40) * 0.05).astype(np.complex64)
    chans = [dict(freq_shift_in_hz=12345, up_rate=3, down_rate=40, coeffs=taps)]
    ch, co = F.MultiRateChannelizerCuda(4000000, chans), O.Channelizer(4000000, chans)
    e = ch.apply(torch.zeros((0, 2), dtype=torch.int16, device="cuda"))
    assert e[0].numel() == 0
    x16 = rng.integers(-3000, 3000, size=(50000, 2)).astype(np.int16)
    y = ch.apply(torch.from_numpy(x16).cuda())[0].cpu().numpy()
    ref = co.apply((x16[:, 0] + 1j * x16[:, 1]).astype(np.complex64))[0]
    assert y.size == ref.size and rel_rms(y, ref) <= 1e-5
