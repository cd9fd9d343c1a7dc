"""Host-buffer applies (fdsp_channelizer_apply_host) copy every group's
outputs back on a second stream as soon as the launches that write them are
enqueued, while later groups compute.  With pinned host buffers those copies
really overlap the kernels; the outputs must equal the device-buffer apply's
bit for bit, in every form, over a streaming sequence (state carried)."""
import ctypes as C

import numpy as np
import pytest

from libfalcon_dsp_gb300.workloads import channelizer_256_plan, tone_signal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["fp32", "fp16x3"])
def test_apply_host_pinned_equals_device_apply(mode):
    torch = pytest.importorskip("torch")
    import libfalcon_dsp_gb300 as F
    from libfalcon_dsp_gb300 import _capi
    fs = 61440000
    chans = channelizer_256_plan(float(fs), None, 256, 9)
    x, _ = tone_signal(1 << 20, float(fs), 512, seed=21)
    dev = F.MultiRateChannelizerCuda(fs, chans)
    host = F.MultiRateChannelizerCuda(fs, chans)
    for g in (dev, host):
        g.set_precision(mode)
        g.set_graph(True)
    nch = len(chans)
    lib = _capi.lib()
    cuts = [0, 1000, 300001, 1 << 20]
    for i, j in zip(cuts[:-1], cuts[1:]):
        n = j - i
        xd = torch.from_numpy(x[i:j]).cuda()
        ys = [y.cpu().numpy() for y in dev.apply(xd)]
        hin = torch.from_numpy(x[i:j]).pin_memory()
        caps = [c + 2 for c in host.out_count(n)]
        houts = [torch.empty(c, dtype=torch.complex64).pin_memory() for c in caps]
        optr = (C.c_void_p * nch)(*[h.data_ptr() for h in houts])
        cap_arr = (C.c_uint64 * nch)(*caps)
        n_out = (C.c_uint64 * nch)()
        stream = torch.cuda.current_stream().cuda_stream
        st = lib.fdsp_channelizer_apply_host(host._h, C.c_void_p(hin.data_ptr()), n, optr, cap_arr, n_out,
                                             C.c_void_p(stream))
        assert st == 0, st
        for c in range(nch):
            assert n_out[c] == ys[c].size
            assert np.array_equal(houts[c][: n_out[c]].numpy(), ys[c]), (mode, c)
    if mode != "fp32":
        assert host.tc_groups() >= 1
