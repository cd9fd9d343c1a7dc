"""Tensor-core FIR (fdsp_fir_set_precision): the full-rate complex-tap FIR of
falcon_dsp_fir_filter_cuda (src/transform/falcon_dsp_fir_filter_cuda.cu:
102-373) as a Toeplitz product on tcgen05, split precision (hi+lo)(hi+lo)
with FP32 accumulation.

Bounds: >= 60 dB SNR against an FP64 evaluation of the same filter on every
block of a streaming run (ragged block sizes, state carried); output counts
equal the input counts; the tensor-core kernel really ran; the FP32 form
still meets 1e-5 relative RMS against the oracle after switching back and a
reset.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.golden_io import rel_rms

pytestmark = pytest.mark.gpu


def _snr_db(got, ref):
    ref = ref.astype(np.complex128)
    return 10 * np.log10(np.sum(np.abs(ref) ** 2) / max(np.sum(np.abs(got - ref) ** 2), 1e-300))


@pytest.mark.parametrize("mode", ["fp16x3", "bf16x3"])
@pytest.mark.parametrize("ntaps", [7, 48, 64])
def test_tc_fir_streaming_snr(mode, ntaps):
    import torch

    import libfalcon_dsp_gb300 as F
    rng = np.random.default_rng(ntaps)
    h = ((rng.standard_normal(ntaps) + 1j * rng.standard_normal(ntaps)) * 0.2).astype(np.complex64)
    x = ((rng.standard_normal(400000) + 1j * rng.standard_normal(400000)) * 0.5).astype(np.complex64)
    f = F.FirFilterCuda(h)
    f.set_precision(mode)
    ref = np.convolve(x.astype(np.complex128), h.astype(np.complex128))[: x.size]
    cuts = [0, 100003, 100010, 362144, 400000]
    for i in range(4):
        blk = x[cuts[i]:cuts[i + 1]]
        y = f.apply(torch.from_numpy(blk).cuda()).cpu().numpy() if i != 1 else f.apply(blk)
        assert y.size == blk.size
        r = ref[cuts[i]:cuts[i + 1]]
        assert _snr_db(y, r) >= 60.0, (i, _snr_db(y, r))
        if blk.size > 100000:
            assert f.tc_groups() == 1
    # back to FP32 (the streaming state carries over): a fresh stream after a
    # reset within the FIR bound
    f.set_precision("fp32")
    f.reset_state()
    y = f.apply(x[:50000])
    assert rel_rms(y, O.FIR(h).apply(x[:50000])) <= 1e-5


def test_tc_fir_int16_and_long_filter_fallback():
    import torch

    import libfalcon_dsp_gb300 as F
    rng = np.random.default_rng(5)
    h = ((rng.standard_normal(40) + 1j * rng.standard_normal(40)) * 0.1).astype(np.complex64)
    x16 = rng.integers(-2000, 2000, size=(70000, 2)).astype(np.int16)
    xc = (x16[:, 0] + 1j * x16[:, 1]).astype(np.complex64)
    a, b = F.FirFilterCuda(h), F.FirFilterCuda(h)
    a.set_precision("fp16x3")
    b.set_precision("fp16x3")
    got = a.apply(torch.from_numpy(x16).cuda()).cpu().numpy()
    y = b.apply(torch.from_numpy(xc).cuda()).cpu().numpy()
    assert np.array_equal(got, np.stack([np.trunc(y.real), np.trunc(y.imag)], axis=1).astype(np.int16))
    # a long filter (200 taps) on the tensor cores too (K chunked)
    g = ((rng.standard_normal(200) + 1j * rng.standard_normal(200)) * 0.1).astype(np.complex64)
    c = F.FirFilterCuda(g)
    c.set_precision("fp16x3")
    y = c.apply(xc)
    assert c.tc_groups() == 1
    assert _snr_db(y, np.convolve(xc.astype(np.complex128), g.astype(np.complex128))[: xc.size]) >= 100.0
