"""Eight-channel streaming channelizer over QPSK carriers (16 carriers with
root-raised-cosine pulses, roll-off 0.35, 25-250 kBd, AWGN 20 dB below each
carrier, 10 MSps), streamed in 2^16-sample blocks through the C ABI's
device-buffer call fdsp_channelizer_apply with the streaming state carried
across blocks -- the reference's channelizer test shape
(test/tests/transform/falcon_dsp_multi_rate_channelizer_cuda_unit_tests.cu:
351-514) on this workload.

Bounds: per block and channel the output count equals the oracle's
(bit-exact) and the samples stay within 1e-5 relative RMS of the oracle's
FP32 restatement; the whole stream equals one-shot processing within the
same bound."""
import ctypes as C

import numpy as np
import pytest

from libfalcon_dsp_gb300.workloads import channelizer_8ch
from oracle import oracle as O
from tests.golden_io import rel_rms

pytestmark = pytest.mark.gpu


def test_qpsk_channelizer_streamed_through_c_abi():
    torch = pytest.importorskip("torch")
    import libfalcon_dsp_gb300 as F
    from libfalcon_dsp_gb300 import _capi
    n, blk = 1 << 20, 1 << 16
    x, fs, chans = channelizer_8ch(n, seed=2025)
    assert len(chans) == 8
    g = F.MultiRateChannelizerCuda(fs, chans)
    ref = O.Channelizer(fs, chans)
    lib = _capi.lib()
    nch = len(chans)
    caps = [c + 2 for c in g.out_count(blk)]
    outs = [torch.empty(c, dtype=torch.complex64, device="cuda") for c in caps]
    optr = (C.c_void_p * nch)(*[o.data_ptr() for o in outs])
    cap_arr = (C.c_uint64 * nch)(*caps)
    n_out = (C.c_uint64 * nch)()
    xd = torch.from_numpy(x).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    got = [[] for _ in range(nch)]
    for b in range(n // blk):
        xb = xd[b * blk:(b + 1) * blk]
        st = lib.fdsp_channelizer_apply(g._h, C.c_void_p(xb.data_ptr()), blk, optr, cap_arr, n_out,
                                        C.c_void_p(stream))
        assert st == 0, st
        torch.cuda.synchronize()
        exp = ref.apply(x[b * blk:(b + 1) * blk])
        for c in range(nch):
            assert n_out[c] == exp[c].size, (b, c)
            y = outs[c][: n_out[c]].cpu().numpy()
            if exp[c].size:
                assert rel_rms(y, exp[c]) <= 1e-5, (b, c, rel_rms(y, exp[c]))
            got[c].append(y)
    # the streamed result equals one shot over the whole signal
    one = O.Channelizer(fs, chans).apply(x)
    for c in range(nch):
        s = np.concatenate(got[c])
        assert s.size == one[c].size
        assert rel_rms(s, one[c]) <= 1e-5

