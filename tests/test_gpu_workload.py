"""GPU tests at the benchmark's scale (256 channels, 2^26 samples).

At full size the CPU oracle is too slow to replay everything, so these tests
combine an oracle check on a prefix with size-independent properties:
  * output counts equal the reference loop's counts (closed form, bit-exact);
  * streaming the block in 2^16-sample pieces equals one-shot processing;
  * scaling the input by 2 scales every output by exactly 2 (bit-exact);
  * the tensor-core forms stay above a per-form SNR floor (TC_FLOOR_DB) from
    the plain FP32 form;
  * on a prefix, every channel matches the oracle (FP32 <= 1e-5 relative RMS,
    tensor cores above a per-form SNR floor against the FP64 oracle).
"""
import numpy as np
import pytest

import libfalcon_dsp_gb300 as F
from libfalcon_dsp_gb300.workloads import channelizer_256, channelizer_256_plan, tone_freqs, tone_signal
from oracle import oracle as O
from tests.golden_io import rel_rms, snr_db

pytestmark = pytest.mark.gpu
FS = 61440000

# Per-form SNR floors (dB) of the tensor-core forms on this workload: the
# lowest channel measured on a GB300 (fp16x3 116.3-117.4 dB, bf16x3
# 106.2-106.5 dB, against the FP64 oracle and against the FP32 form) minus
# a 3 dB margin.
TC_FLOOR_DB = {"fp16x3": 113.0, "bf16x3": 103.0}


def test_plan_prefix_vs_oracle_all_channels():
    torch = pytest.importorskip("torch")
    chans = channelizer_256_plan(float(FS), tone_freqs(1 << 26, float(FS), 512, 2026), 256, 2027)
    x, _ = tone_signal(1 << 17, float(FS), 512, seed=11)
    o32 = O.Channelizer(FS, chans).apply(x)
    o64 = O.Channelizer(FS, chans, precision="f64").apply(x)
    xd = torch.from_numpy(x).cuda()
    res = {}
    for mode in ["fp32", "fp16x3", "bf16x3"]:
        g = F.MultiRateChannelizerCuda(FS, chans)
        g.set_precision(mode)
        ys = [y.cpu().numpy() for y in g.apply(xd)]
        torch.cuda.synchronize()
        if mode != "fp32":
            # the tensor-core kernel really computed groups of the plan
            assert g.tc_groups() >= 1, mode
        snrs = []
        for y, a, b in zip(ys, o32, o64):
            assert y.size == a.size
            if mode == "fp32":
                assert rel_rms(y, a) <= 1e-5
            snrs.append(snr_db(y, b))
        res[mode] = (min(snrs), float(np.median(snrs)))
        assert min(snrs) >= TC_FLOOR_DB.get(mode, 60.0), (mode, min(snrs))
    print("SNR vs FP64 oracle over 256 channels (min, median dB):", res)


@pytest.fixture(scope="module")
def full():
    torch = pytest.importorskip("torch")
    x, fs, chans = channelizer_256(1 << 26, 2026, device=torch.device("cuda"))
    return torch, x, fs, chans


def _run(F_, torch, x, fs, chans, mode, blocks=1):
    g = F_.MultiRateChannelizerCuda(fs, chans)
    g.set_precision(mode)
    if blocks == 1:
        ys = g.apply(x)
    else:
        n = x.numel() // blocks
        parts = [g.apply(x[i * n:(i + 1) * n]) for i in range(blocks)]
        ys = [torch.cat([p[c] for p in parts]) for c in range(len(chans))]
    torch.cuda.synchronize()
    return ys


def test_full_size_counts_streaming_and_linearity(full):
    torch, x, fs, chans = full
    y1 = _run(F, torch, x, fs, chans, "fp32")
    # counts: closed form of the reference loop from a fresh state
    for ch, y in zip(chans, y1):
        assert y.numel() == O.Resampler(ch["up_rate"], ch["down_rate"], np.ones(1, np.complex64)).loop_out_count(x.numel())
    # streaming in 2^16-sample blocks (1024 applies) == one shot
    ys = _run(F, torch, x, fs, chans, "fp32", blocks=1024)
    worst = 0.0
    for a, b in zip(y1, ys):
        assert a.numel() == b.numel()
        d = torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(a)
        worst = max(worst, float(d))
    assert worst <= 1e-5, worst
    del ys
    # exact linearity in scale: y(2x) == 2 y(x)
    y2 = _run(F, torch, x * 2, fs, chans, "fp32")
    for a, b in zip(y1, y2):
        assert torch.equal(b, a * 2)


@pytest.mark.parametrize("mode", ["fp16x3", "bf16x3"])
def test_full_size_tensor_core_vs_fp32(full, mode):
    torch, x, fs, chans = full
    y32 = _run(F, torch, x, fs, chans, "fp32")
    ytc = _run(F, torch, x, fs, chans, mode)
    worst = 1e9
    for a, b in zip(y32, ytc):
        assert a.numel() == b.numel()
        err = torch.linalg.vector_norm(a - b) ** 2
        sig = torch.linalg.vector_norm(a) ** 2
        worst = min(worst, float(10 * torch.log10(sig / err)))
    print(f"{mode}: worst channel SNR vs plain FP32 over 2^26 samples: {worst:.1f} dB")
    assert worst >= TC_FLOOR_DB[mode], (mode, worst)
    # linearity in scale: exact for BF16 (its exponent range keeps every lo
    # part normal); FP16 lo parts of tiny samples are subnormal, so scaling
    # moves their rounding -- there the bound is 100 dB
    y2 = _run(F, torch, x * 2, fs, chans, mode)
    for a, b in zip(ytc, y2):
        if mode == "bf16x3":
            assert torch.equal(b, a * 2)
        else:
            err = torch.linalg.vector_norm(b - a * 2) ** 2
            assert float(10 * torch.log10(torch.linalg.vector_norm(b) ** 2 / err)) >= 100.0




@pytest.mark.parametrize("mode", ["fp16x3", "bf16x3"])
def test_full_size_prefix_matches_oracle(full, mode):
    """Every one of the 256 channels of the full-size tensor-core run, on the
    outputs of the first 2^16 input samples, against the FP64 oracle."""
    torch, x, fs, chans = full
    ys = _run(F, torch, x, fs, chans, mode)
    n = 1 << 16
    xp = x[:n].cpu().numpy()
    o64 = O.Channelizer(fs, chans, precision="f64").apply(xp)
    snrs = []
    for y, b in zip(ys, o64):
        # outputs of the prefix depend only on the prefix (no lookahead)
        a = y[: b.size].cpu().numpy()
        snrs.append(snr_db(a, b))
    print(f"{mode}: SNR vs FP64 over 256 channels: min {min(snrs):.1f} median {np.median(snrs):.1f} dB")
    assert min(snrs) >= TC_FLOOR_DB[mode], (mode, min(snrs))
