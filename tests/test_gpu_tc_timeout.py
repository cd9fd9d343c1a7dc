"""Bounded waits of the tensor-core kernel report to the caller.

A test hook withholds every operand copy of the next launches and the wait
limit is cut to a few polls, so each role's first wait runs out before any
copy or MMA is issued: the kernel records the failure in the engine's error
flag and exits with nothing in flight.  The caller sees FDSP_ERR_TIMEOUT
from fdsp_channelizer_status (device applies) and from the host-buffer apply
itself, the record clears once read, and the next normal apply on the same
handle (after a reset) matches the FP64 oracle.  No GPU fault is involved.
"""
import numpy as np
import pytest

import libfalcon_dsp_gb300 as F
from libfalcon_dsp_gb300 import _capi
from oracle import oracle as O
from tests.golden_io import snr_db

pytestmark = pytest.mark.gpu


def _chans():
    r = np.random.default_rng(3)
    return [dict(freq_shift_in_hz=f, up_rate=u, down_rate=d,
                 coeffs=(r.standard_normal(u * t) * 0.05).astype(np.complex64))
            for f, u, d, t in [(100000, 1, 8, 40), (-25000, 2, 25, 33), (0, 3, 16, 57)]]


def test_tc_timeout_reaches_caller_and_handle_recovers():
    torch = pytest.importorskip("torch")
    fs = 1000000
    rng = np.random.default_rng(4)
    x = ((rng.standard_normal(60000) + 1j * rng.standard_normal(60000)) * 100).astype(np.complex64)
    g = F.MultiRateChannelizerCuda(fs, _chans())
    g.set_precision("fp16x3")
    g.set_tc_wait(64, withhold_copies=True)
    g.apply(torch.from_numpy(x).cuda())
    with pytest.raises(F.FdspError) as e:
        g.status()
    assert e.value.status == _capi.FDSP_ERR_TIMEOUT
    g.status()  # the record was cleared by the read
    with pytest.raises(F.FdspError) as e:
        g.apply(x)  # host buffers: the apply itself reports it
    assert e.value.status == _capi.FDSP_ERR_TIMEOUT
    # normal waits again: a fresh stream matches the oracle
    g.set_tc_wait(1 << 20, withhold_copies=False)
    g.reset_state()
    ys = [y.cpu().numpy() for y in g.apply(torch.from_numpy(x).cuda())]
    g.status()
    ref = O.Channelizer(fs, _chans(), precision="f64").apply(x)
    for y, r in zip(ys, ref):
        assert y.size == r.size
        assert snr_db(y, r) >= 100.0
