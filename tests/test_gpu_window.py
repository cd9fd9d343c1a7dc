"""The FP32 kernel's sliding-window form (single-channel work sets, long
filters, blocks large enough to fill the GPU with its tiles): real taps
(resampler semantics, 2 FMAs a tap), complex taps (FIR), and a shifted
channel (complex modulated taps and the NCO rotation epilogue), each against
the FP32 oracle within 1e-5 relative RMS over two streaming applies, output
counts exact.  Block sizes are chosen so the launch takes the sliding-window
form (rows >= its tile rows x the SM count)."""
import numpy as np
import pytest

import libfalcon_dsp_gb300 as F
from oracle import oracle as O
from tests.golden_io import rel_rms

pytestmark = pytest.mark.gpu


def _x(n, seed):
    rng = np.random.default_rng(seed)
    return ((rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 0.5).astype(np.complex64)


def test_window_resampler_real_taps():
    import torch
    rng = np.random.default_rng(1)
    h = (rng.standard_normal(4095) * 0.02).astype(np.complex64)  # resampler: real parts only
    rs = F.PolyphaseResamplerCuda(1, 10, h)
    ro = O.Resampler(1, 10, h)
    for b, n in enumerate((1 << 22, (1 << 22) + 37)):
        x = _x(n, 10 + b)
        y = rs.apply(torch.from_numpy(x).cuda()).cpu().numpy()
        ref = ro.apply(x)
        assert y.size == ref.size
        assert rel_rms(y, ref) <= 1e-5


def test_window_fir_complex_taps():
    import torch
    rng = np.random.default_rng(2)
    h = ((rng.standard_normal(64) + 1j * rng.standard_normal(64)) * 0.1).astype(np.complex64)
    f = F.FirFilterCuda(h)
    fo = O.FIR(h)
    for b, n in enumerate((1 << 22, 999_983)):
        x = _x(n, 20 + b)
        y = f.apply(torch.from_numpy(x).cuda()).cpu().numpy()
        assert rel_rms(y, fo.apply(x)) <= 1e-5


def test_window_shifted_channel():
    import torch
    fs = 10_000_000
    rng = np.random.default_rng(3)
    h = (rng.standard_normal(8 * 160) * 0.05).astype(np.complex64)  # 160 taps a phase, up 1 down 8
    chans = [dict(freq_shift_in_hz=-1234567, up_rate=1, down_rate=8, coeffs=h)]
    ch = F.MultiRateChannelizerCuda(fs, chans)
    co = O.Channelizer(fs, chans)
    for b, n in enumerate((1 << 23, (1 << 22) + 5)):
        x = _x(n, 30 + b)
        y = ch.apply(torch.from_numpy(x).cuda())[0].cpu().numpy()
        ref = co.apply(x)[0]
        assert y.size == ref.size
        assert rel_rms(y, ref) <= 1e-5
