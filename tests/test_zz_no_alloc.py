"""fdsp_resample_static, the entry point that allocates nothing, against the
resampler handle (fdsp_resampler_create + fdsp_resampler_apply on a fresh
state): same output count, outputs equal within FP32 rounding.

Two calls in a row with different configurations share the fixed tap array;
the second has fewer taps than the first, so stale taps left in the array by
the first call would show up in its outputs.  One case has more phases than
taps (up > num_coeffs), so most phases read only the zero padding.  After a
warm-up call, further calls leave the device's free memory unchanged: the
entry point allocates nothing.  The file name sorts last so the test also
runs after every other GPU test of the suite.
"""
import numpy as np
import pytest

import libfalcon_dsp_gb300 as F
from tests.golden_io import rel_rms

pytestmark = pytest.mark.gpu

CASES = [
    # (up, down, taps, n_in, seed)
    (3, 2, 401, 50_000, 1),
    (2, 5, 23, 40_001, 2),
    (1, 8, 2048, 65_536, 3),
    (7, 3, 5, 30_000, 4),  # up > num_coeffs: phases 5 and 6 hold only padding
]


def _taps(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)


def _signal(n, seed, torch):
    rng = np.random.default_rng(seed + 100)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    return torch.from_numpy(x).cuda()


def test_static_matches_resampler_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    for up, down, nt, n_in, seed in CASES:
        h = _taps(nt, seed)
        x = _signal(n_in, seed, torch)
        ref = F.PolyphaseResamplerCuda(up, down, h).apply(x)
        out = torch.full((ref.numel() + 3,), complex(7.0, -7.0), dtype=torch.complex64, device="cuda")
        got = F.resample_static(up, down, h, x, out)
        torch.cuda.synchronize()
        assert got.numel() == ref.numel()
        assert rel_rms(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-5, (up, down, nt)
        # nothing past the output count is written
        assert torch.all(out[ref.numel():] == complex(7.0, -7.0))


def test_static_rejects_oversized_taps_and_small_output():
    torch = pytest.importorskip("torch")
    x = _signal(1000, 5, torch)
    out = torch.empty(4000, dtype=torch.complex64, device="cuda")
    with pytest.raises(ValueError):
        F.resample_static(2, 1, _taps(F.RESAMPLE_STATIC_MAX_COEFFS + 1, 5), x, out)
    with pytest.raises(F.FdspError):
        F.resample_static(4, 1, _taps(16, 5), x, torch.empty(10, dtype=torch.complex64, device="cuda"))
    # the array still serves a valid call afterwards
    h = _taps(64, 6)
    ref = F.PolyphaseResamplerCuda(2, 1, h).apply(x)
    got = F.resample_static(2, 1, h, x, out)
    torch.cuda.synchronize()
    assert rel_rms(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-5


def test_static_allocates_nothing_after_warmup():
    torch = pytest.importorskip("torch")
    x = _signal(200_000, 7, torch)
    out = torch.empty(800_000, dtype=torch.complex64, device="cuda")
    h = _taps(1024, 7)
    F.resample_static(3, 1, h, x, out)  # warm-up: first-call set-up of the device
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for up, down, nt in ((3, 1, 1024), (2, 7, 8000), (5, 4, 3)):
        F.resample_static(up, down, _taps(nt, up), x, out)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_static_up_rate_near_2_32_keeps_one_tap_per_phase():
    # taps per phase = ceil(16 / (2^32 - 1)) = 1: computed without wrapping,
    # so y[m] = Re(h[0]) x[m] for up = down
    torch = pytest.importorskip("torch")
    x = _signal(4096, 8, torch)
    out = torch.empty(4096, dtype=torch.complex64, device="cuda")
    h = _taps(16, 8)
    big = (1 << 32) - 1
    got = F.resample_static(big, big, h, x, out)
    torch.cuda.synchronize()
    assert got.numel() == 4096
    want = x.cpu().numpy() * np.float32(h[0].real)
    assert rel_rms(got.cpu().numpy(), want) <= 1e-6
