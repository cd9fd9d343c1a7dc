"""GPU tests of the tensor-core (tcgen05) split-precision channelizer.

The FP16/BF16 hi+lo forms are validated against the FP64 oracle (the same
indexing and rollover rule evaluated in double) and against the plain FP32
path.  Bound (stated in the test): every channel >= 60 dB SNR against FP64,
output counts identical to the reference loop.
"""
import numpy as np
import pytest

import libfalcon_dsp_gb300 as F
from libfalcon_dsp_gb300.workloads import channelizer_256_plan, tone_signal
from oracle import oracle as O
from tests.golden_io import snr_db

pytestmark = pytest.mark.gpu
SNR_MIN_DB = 60.0


def _rand(n, seed, scale=1000.0):
    r = np.random.default_rng(seed)
    return ((r.standard_normal(n) + 1j * r.standard_normal(n)) * scale).astype(np.complex64)


@pytest.mark.parametrize("mode", ["fp16x3", "bf16x3"])
def test_tc_single_channel_no_shift(mode):
    x = _rand(20000, 1)
    h = _rand(32, 2, 0.1).real.astype(np.complex64)
    chans = [dict(freq_shift_in_hz=0, up_rate=1, down_rate=4, coeffs=h)]
    g = F.MultiRateChannelizerCuda(1000000, chans)
    g.set_precision(mode)
    y = g.apply(x)[0]
    ref = O.Channelizer(1000000, chans, precision="f64").apply(x)[0]
    assert y.size == ref.size
    assert snr_db(y, ref) >= SNR_MIN_DB, snr_db(y, ref)


@pytest.mark.parametrize("mode", ["fp16x3", "bf16x3"])
def test_tc_workload_slice_vs_fp64(mode):
    fs = 61440000
    x, freqs = tone_signal(1 << 17, float(fs), 512, seed=5)
    chans = channelizer_256_plan(float(fs), freqs, nch=48, seed=6)
    g = F.MultiRateChannelizerCuda(fs, chans)
    g.set_precision(mode)
    got = [[] for _ in chans]
    o64 = O.Channelizer(fs, chans, precision="f64")
    exp = [[] for _ in chans]
    for i in range(0, x.size, 40000):
        for c, (a, b) in enumerate(zip(g.apply(x[i:i + 40000]), o64.apply(x[i:i + 40000]))):
            assert a.size == b.size
            got[c].append(a)
            exp[c].append(b)
    worst = min(snr_db(np.concatenate(a), np.concatenate(b)) for a, b in zip(got, exp))
    assert worst >= SNR_MIN_DB, worst


def test_tc_rollover_straddles_and_matches_fp32_path():
    fs = 1000000
    r = np.random.default_rng(7)
    chans = [dict(freq_shift_in_hz=f, up_rate=u, down_rate=d, coeffs=_rand(u * t, 10 + i, 0.05).real.astype(np.complex64))
             for i, (f, u, d, t) in enumerate([(100000, 1, 4, 64), (-100000, 3, 8, 40), (12345, 2, 25, 33),
                                               (250000, 1, 8, 12), (-1, 3, 16, 57), (0, 1, 4, 20)])]
    x = _rand(500000, 8)
    g32 = F.MultiRateChannelizerCuda(fs, chans)
    gtc = F.MultiRateChannelizerCuda(fs, chans)
    gtc.set_precision("fp16x3")
    o64 = O.Channelizer(fs, chans, precision="f64")
    for i, j in [(0, 1), (1, 99999), (99999, 250000), (250000, 500000)]:
        a, b, c = g32.apply(x[i:j]), gtc.apply(x[i:j]), o64.apply(x[i:j])
        for ya, yb, yc in zip(a, b, c):
            assert ya.size == yb.size == yc.size
            if yc.size > 8:
                assert snr_db(yb, yc) >= SNR_MIN_DB, snr_db(yb, yc)
                assert snr_db(ya, yc) >= 100.0


def test_tc_exact_pass_for_every_output():
    """The exact rotation pass (tc_fix_kernel) over every output of a slot --
    the path of slots whose row stride spans more than the NCO rollover (31
    rows of D' samples >= R), forced here by the test hook on an ordinary
    plan -- and over the straddling windows alone, within the tensor-core
    bound of the FP64 oracle and equal to each other within FP32 rounding."""
    fs = 1000000
    chans = [dict(freq_shift_in_hz=f, up_rate=u, down_rate=d, coeffs=_rand(u * t, 50 + i, 0.05).real.astype(np.complex64))
             for i, (f, u, d, t) in enumerate([(100000, 1, 4, 64), (-100000, 3, 8, 40), (12345, 2, 25, 33),
                                               (0, 1, 4, 20)])]
    x = _rand(300000, 51)
    a = F.MultiRateChannelizerCuda(fs, chans)
    b = F.MultiRateChannelizerCuda(fs, chans)
    for g in (a, b):
        g.set_precision("fp16x3")
    b.set_tc_exact_all(True)
    o64 = O.Channelizer(fs, chans, precision="f64")
    for i, j in [(0, 4001), (4001, 150000), (150000, 300000)]:
        for ya, yb, yc in zip(a.apply(x[i:j]), b.apply(x[i:j]), o64.apply(x[i:j])):
            assert ya.size == yb.size == yc.size
            if yc.size > 8:
                assert snr_db(yb, yc) >= SNR_MIN_DB, snr_db(yb, yc)
                assert snr_db(yb, ya) >= 110.0, snr_db(yb, ya)
    assert b.tc_groups() == a.tc_groups() >= 1


@pytest.mark.parametrize("split", [1, 2, 4])
def test_tc_row_split_matches_fp64(split):
    """Row split (rows j = S i + b of a group run as S output streams whose
    rows are S D apart): within the tensor-core bound of the FP64 oracle over
    a streaming sequence whose windows straddle NCO rollovers, with the split
    each group used reported by group_info (odd down rates always split)."""
    fs = 1000000
    chans = [dict(freq_shift_in_hz=f, up_rate=u, down_rate=d, coeffs=_rand(u * t, 30 + i, 0.05).real.astype(np.complex64))
             for i, (f, u, d, t) in enumerate([(100000, 1, 4, 64), (-100000, 3, 8, 40), (12345, 2, 25, 33),
                                               (250000, 1, 8, 12), (-1, 3, 16, 57), (0, 1, 4, 20)])]
    x = _rand(300000, 31)
    g = F.MultiRateChannelizerCuda(fs, chans)
    g.set_precision("fp16x3")
    g.set_tc_split(split)
    o64 = O.Channelizer(fs, chans, precision="f64")
    for i, j in [(0, 777), (777, 100001), (100001, 300000)]:
        for yb, yc in zip(g.apply(x[i:j]), o64.apply(x[i:j])):
            assert yb.size == yc.size
            if yc.size > 8:
                assert snr_db(yb, yc) >= SNR_MIN_DB, snr_db(yb, yc)
    info = g.group_info()
    for gi in info:
        lim = max(split, 2) if gi["down_rate"] % 2 else split
        assert 1 <= gi["tc_split"] <= lim, info
        if gi["down_rate"] % 2:
            assert gi["tc_split"] % 2 == 0, info
    assert max(gi["tc_split"] for gi in info) >= split, info
    assert g.tc_groups() == len(info)


@pytest.mark.parametrize("mode", ["fp32", "fp16x3"])
def test_graph_recaptures_when_the_launch_sequence_changes(mode):
    """The graph is captured once and later applies only rewrite its kernel
    nodes; block sizes that change the launch sequence (tile counts, tiny
    blocks where some groups emit nothing, a precision switch) make it
    capture afresh.  Every apply equals direct launches bit for bit."""
    torch = pytest.importorskip("torch")
    fs = 61440000
    chans = channelizer_256_plan(float(fs), [1.5e6, -4.0e6, 8.5e6], 24, 13)
    sizes = [50000, 50000, 3, 50000, 700, 131072, 131072, 1, 50000]
    x, _ = tone_signal(sum(sizes), float(fs), 48, seed=14)
    xd = torch.from_numpy(x).cuda()
    outs = {}
    for graph in (False, True):
        g = F.MultiRateChannelizerCuda(fs, chans)
        g.set_precision(mode)
        g.set_graph(graph)
        s = torch.cuda.Stream()
        ys, n0 = [], 0
        with torch.cuda.stream(s):
            for i, n in enumerate(sizes):
                if i == 6:  # switch the form mid-stream and back
                    g.set_precision("fp32" if mode != "fp32" else "fp16x3")
                if i == 7:
                    g.set_precision(mode)
                ys.append([y.clone() for y in g.apply(xd[n0:n0 + n])])
                n0 += n
        s.synchronize()
        outs[graph] = [[y.cpu().numpy() for y in blk] for blk in ys]
        if graph:
            assert g.graph_replays() == len(sizes)
    for a, b in zip(outs[False], outs[True]):
        for ya, yb in zip(a, b):
            assert np.array_equal(ya, yb)


def test_autotune_keeps_results_and_streaming():
    """The autotuner only picks tile heights and forms: outputs after it stay
    within the tensor-core bound of the FP64 oracle, from a reset state, and
    the groups it gives the tensor-core form run on the tensor-core kernel."""
    torch = pytest.importorskip("torch")
    fs = 61440000
    chans = channelizer_256_plan(float(fs), [1.0e6, -3.0e6, 7.5e6, -12.0e6], 24, 5)
    x, _ = tone_signal(1 << 16, float(fs), 64, seed=3)
    g = F.MultiRateChannelizerCuda(fs, chans)
    g.set_precision("fp16x3")
    info = g.autotune(1 << 16)
    assert len(info) == len({c["down_rate"] for c in chans})
    assert all(i["tile_rows"] % 32 == 0 and i["tile_rows"] >= 32 for i in info)
    ys = [y.cpu().numpy() for y in g.apply(torch.from_numpy(x).cuda())]
    ref = O.Channelizer(fs, chans, precision="f64").apply(x)
    for y, r in zip(ys, ref):
        assert y.size == r.size
        assert snr_db(y, r) >= SNR_MIN_DB
    assert g.tc_groups() == sum(i["tensor_core"] for i in info)


@pytest.mark.parametrize("mode", ["fp32", "fp16x3"])
def test_graph_replay_matches_direct_launches(mode):
    """Applies replayed as CUDA graphs give bit-identical outputs to direct
    launches over a streaming sequence (the graph is updated as the
    streaming state moves the window offsets)."""
    torch = pytest.importorskip("torch")
    fs = 61440000
    chans = channelizer_256_plan(float(fs), [2.0e6, -9.0e6, 5.5e6], 32, 9)
    x, _ = tone_signal(3 * 20000 + 77, float(fs), 48, seed=4)
    xd = torch.from_numpy(x).cuda()
    outs = {}
    for graph in (False, True):
        g = F.MultiRateChannelizerCuda(fs, chans)
        g.set_precision(mode)
        g.set_graph(graph)
        s = torch.cuda.Stream()
        ys = []
        with torch.cuda.stream(s):
            for b in range(3):
                n0, n1 = b * 20000, (b + 1) * 20000 + (77 if b == 2 else 0)
                ys.append([y.clone() for y in g.apply(xd[n0:n1])])
        s.synchronize()
        outs[graph] = [[y.cpu().numpy() for y in blk] for blk in ys]
        if graph:
            assert g.graph_replays() == 3
    for a, b in zip(outs[False], outs[True]):
        for ya, yb in zip(a, b):
            assert np.array_equal(ya, yb)


@pytest.mark.parametrize("mode", ["fp16x3", "bf16x3"])
def test_concurrent_launch_packs_match_serial_packs(mode):
    """The 256-channel plan needs several launch packs; they run at the same
    time on side streams (each with its own launch record and B images),
    directly or replayed as a graph.  With kernel timing on they run one
    after another on the caller's stream.  Every form gives bit-identical
    outputs over a streaming sequence (state carried)."""
    torch = pytest.importorskip("torch")
    fs = 61440000
    chans = channelizer_256_plan(float(fs), None, 256, 9)
    x, _ = tone_signal(3 * 150000 + 31, float(fs), 256, seed=12)
    xd = torch.from_numpy(x).cuda()
    outs = {}
    for form in ("serial", "direct", "graph"):
        g = F.MultiRateChannelizerCuda(fs, chans)
        g.set_precision(mode)
        g.set_graph(form == "graph")
        if form == "serial":
            g.set_profile(True)
        s = torch.cuda.Stream()
        ys = []
        with torch.cuda.stream(s):
            for b in range(3):
                n0, n1 = b * 150000, (b + 1) * 150000 + (31 if b == 2 else 0)
                ys.append([y.clone() for y in g.apply(xd[n0:n1])])
                if b == 0:
                    # tensor-core form, more than one pack (3 launches a pack + history update)
                    assert g.tc_groups() >= 2
                    assert g.kernel_launches() >= 7
        s.synchronize()
        outs[form] = [[y.cpu().numpy() for y in blk] for blk in ys]
        if form == "serial":
            ms, n = g.read_profile()
            assert n >= 2 * 3 and ms > 0.0
        if form == "graph":
            assert g.graph_replays() == 3
    for form in ("direct", "graph"):
        for a, b in zip(outs["serial"], outs[form]):
            for ya, yb in zip(a, b):
                assert np.array_equal(ya, yb), form
