#!/usr/bin/env python3
"""Channelizer throughput benchmark (output Msamples/s).

Workload (the 256-channel configuration of the benchmark spec): one 2^26-sample
complex<float> stream at 61.44 MSps (512 seeded tones + noise), 256 output
channels with decimation D in {8,16,25,40,64,125,160,320}, up-factor U in
{1,2,3}, 12-64 taps per phase; every channel shifts one tone to DC and
resamples by U/D.  One step = one streaming apply of the whole 2^26-sample
block through all 256 channels (NCO shift + polyphase resampling, fused).

Reported (one JSON line, rank 0):
  value      Sum of channel output samples / s with the input already resident
             in HBM (CUDA events on the launch stream, max over ranks).
  e2e        The same metric through the C ABI's host-buffer call
             (fdsp_channelizer_apply_host): pinned host input -> H2D -> kernels
             -> D2H of every output sample, per step.
  roofline   Dominant kernel (tc_filter_kernel, the tensor-core filter bank;
             tc_prep_kernel splits the input beside it) against the measured
             HBM copy bandwidth: algorithmic bytes of a step (8 B per input
             sample + 8 B per output sample) / the summed duration of the
             step's tc_filter_kernel launches, timed live with CUDA events on
             the launch stream; traffic from the committed ncu summary
             (profiles/*_dram.txt, written by libfalcon_dsp_gb300.ncu_summary
             from ncu's CSV output).
  cpu_baseline  The reference CPU channelizer path (oracle/_ref when built from
             the reference sources, else the oracle's C restatement) on a
             bounded sample of the same workload (the same sample length as
             the reference arm), channels spread over all host threads, and
             on one thread.
Multi-GPU: replicas only -- every rank runs the same workload on its own GPU,
with no collective on the data path; value sums ranks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = ("channelizer_256: 2^26 complex64 @ 61.44 MSps, 512 tones + noise, 256 channels, "
            "D in {8,16,25,40,64,125,160,320}, U in {1,2,3}, 12-64 taps/phase, Kaiser sinc")
SEED = 2026


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1 << 26, help="input samples per step (profiling uses smaller)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=1 << 20, help="input samples of the CPU baseline sample")
    ap.add_argument("--precision", default="fp16x3", choices=["fp32", "fp16x3", "bf16x3"],
                    help="filter-bank arithmetic of the headline number (tensor-core split forms or plain FP32)")
    ap.add_argument("--no-fp32-compare", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-other-configs", action="store_true")
    ap.add_argument("--no-kernel-timing", action="store_true", help="skip the per-kernel CUDA-event pass")
    ap.add_argument("--serve-seconds", type=float, default=3.0)
    ap.add_argument("--serve-streams", type=int, default=16, help="concurrent streams the server admits")
    return ap.parse_args()


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons while the
    timed region runs."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.rows = []
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        if gpu_id:
            cmd += ["-i", gpu_id]
        try:
            self.p = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        self.t = threading.Thread(target=self._read, daemon=True)
        if self.p:
            self.t.start()

    def _read(self):
        for line in self.p.stdout:
            parts = [s.strip() for s in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def stop(self) -> dict:
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.t.join(timeout=2)
        sm = [float(r[0]) for r in self.rows if re.match(r"^[0-9.]+$", r[0])]
        mx = [float(r[1]) for r in self.rows if re.match(r"^[0-9.]+$", r[1])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# --------------------------------------------------------------------------- helpers
def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def ncu_traffic(summary: str, kernel: str, n_in: int):
    """DRAM bytes of one step's launches of `kernel`, from the committed ncu
    summary (profiles/<summary>.txt, written by libfalcon_dsp_gb300.ncu_summary
    from ncu's CSV) scaled to n_in input samples; with the whole step's bytes
    per input sample.  None when no capture was summarised."""
    from libfalcon_dsp_gb300 import ncu_summary
    p = os.path.join(ROOT, "profiles", f"{summary}.txt")
    if not os.path.exists(p):
        return None
    d = ncu_summary.read(p)
    k = d.get(f"{kernel}.dram_bytes_per_input_sample")
    if k is None:
        return None
    return {"bytes_per_step": round(k * n_in), "bytes_per_input_sample": round(k, 2),
            "step_bytes_per_input_sample": round(d.get("step.dram_bytes_per_input_sample", 0.0), 2),
            "captured_n_in": int(d.get("n_in", 0)), "source": f"profiles/{summary}.txt"}


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith("model name"):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_channelizer_rate(fs, chans, x, threads, use_reference: bool) -> tuple[float, str, int]:
    """Output Msamples/s of the reference CPU channelizer path on sample x,
    channels split over `threads` host threads (ctypes releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    threads = max(1, min(threads, len(chans)))
    groups = [list(range(i, len(chans), threads)) for i in range(threads)]
    if use_reference:
        objs = [O.RefChannelizer(fs, [chans[i] for i in g]) for g in groups]
        kind = "reference"
    else:
        objs = [O.Channelizer(fs, [chans[i] for i in g]) for g in groups]
        kind = "port"

    def work(o):
        return sum(y.size for y in o.apply(x))

    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        tot = sum(ex.map(work, objs))
    dt = time.perf_counter() - t0
    return tot / dt / 1e6, kind, threads


def cpu_baseline(fs, chans, x, use_reference: bool, single_thread: bool = True) -> dict:
    """The CPU leg on sample x: channel-parallel over every host thread, and
    (single_thread) the same sample on one thread."""
    rate, kind, used = cpu_channelizer_rate(fs, chans, x, cpu_threads(), use_reference)
    out = {"value": round(rate, 3), "unit": "Msamples/s", "cores": used, "kind": kind, "cpu_model": cpu_model(),
           "sample": f"{x.size} input samples of the workload x {len(chans)} channels, channels over {used} threads"}
    if single_thread:
        r1, _, _ = cpu_channelizer_rate(fs, chans, x, 1, use_reference)
        out["single_thread"] = {"value": round(r1, 3), "unit": "Msamples/s", "cores": 1}
    return out


def _time_device(fn, reps: int = 5, warm: int = 3):
    """Median ms of fn() over reps runs, CUDA events on the current stream."""
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts)), out


def fp64_fm_chain(x, h, down: int):
    """FP64 arm of the long-FIR chain, for comparison only (library FFT
    convolution in complex128 on the GPU, then the polar discriminator in
    FP64): y[m] = sum_k h[k] x[m D - k] from a zero history, as the
    resampler's first apply computes it."""
    import torch
    n, t = x.numel(), h.size
    nf = 1 << (n + t - 1 - 1).bit_length()
    X = torch.fft.fft(x.to(torch.complex128), nf)
    H = torch.fft.fft(torch.from_numpy(h.astype(np.complex128)).to(x.device), nf)
    y = torch.fft.ifft(X * H)[:n:down]
    del X, H
    return y, torch.angle(y[1:] * torch.conj(y[:-1]))


def other_configs(dev, lib) -> dict:
    import torch

    import libfalcon_dsp_gb300 as F
    from libfalcon_dsp_gb300.workloads import audio_snr_db, channelizer_8ch, fm_chain, resampler_1ch
    res = {}
    pk = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    # single-channel resampler 48 kHz -> 44.1 kHz, 2^20 samples, 3528 taps
    x, up, down, h = resampler_1ch(1 << 20, 2024, device=dev)
    rs = F.PolyphaseResamplerCuda(up, down, h)
    out = torch.empty(rs.out_count(x.numel()) + 2, dtype=torch.complex64, device=dev)

    def c1():
        rs.reset_state()
        return rs.apply(x, out=out).numel()
    ms, n_out = _time_device(c1)
    res["resampler_147_160"] = {"n_in": x.numel(), "n_out": n_out, "ms": round(ms, 4),
                                "value": round(n_out / ms / 1e3, 1), "unit": "Msamples/s"}
    # 8-channel channelizer over 16 QPSK carriers, 2^24 samples streamed in
    # 2^16-sample blocks through the C ABI's device-buffer call
    x, fs, chans = channelizer_8ch(1 << 24, 2025, device=dev)
    ch = F.MultiRateChannelizerCuda(fs, chans)
    blk = 1 << 16
    nch = len(chans)
    caps = [c + 2 for c in ch.out_count(blk)]
    outs = [torch.empty(c, dtype=torch.complex64, device=dev) for c in caps]
    optr = (C.c_void_p * nch)(*[o.data_ptr() for o in outs])
    cap_arr = (C.c_uint64 * nch)(*caps)
    n_out_arr = (C.c_uint64 * nch)()
    s = torch.cuda.Stream(device=dev)
    sh = C.c_void_p(s.cuda_stream)
    ch.set_graph(True)
    xptrs = [C.c_void_p(x[b * blk:].data_ptr()) for b in range(x.numel() // blk)]

    def c2():
        ch.reset_state()
        tot = 0
        s.wait_stream(torch.cuda.current_stream())
        for xp in xptrs:
            st = lib.fdsp_channelizer_apply(ch._h, xp, blk, optr, cap_arr, n_out_arr, sh)
            if st != 0:
                raise F.FdspError("fdsp_channelizer_apply", st, lib.fdsp_last_cuda_error())
            tot += sum(n_out_arr)
        torch.cuda.current_stream().wait_stream(s)
        return tot
    ms, n_out = _time_device(c2, reps=3, warm=1)
    res["channelizer_8ch_qpsk_blocks_2p16"] = {
        "n_in": x.numel(), "blocks": x.numel() // blk, "n_out": n_out, "ms": round(ms, 3),
        "value": round(n_out / ms / 1e3, 1), "unit": "Msamples/s", "cuda_graph": True,
        "call": "fdsp_channelizer_apply (device buffers), one call per 2^16-sample block"}
    del x, outs
    # FIR 4095 taps / decimate 10 / polar discriminator, 2^26 samples: the
    # tensor-core forms, plain FP32 and an FP64 comparison arm
    x, fs, h, tones = fm_chain(1 << 26, 2027, device=dev)
    rs = F.PolyphaseResamplerCuda(1, 10, h)
    pd = F.PolarDiscriminatorCuda()
    y = torch.empty(rs.out_count(x.numel()) + 2, dtype=torch.complex64, device=dev)
    a = torch.empty(y.numel() + 2, dtype=torch.float32, device=dev)
    fm = {"n_in": x.numel(), "taps": int(h.size), "down": 10}
    for mode in ("fp16x3", "bf16x3", "fp32"):
        rs.set_precision(mode)

        def c5():
            rs.reset_state()
            pd.reset_state()
            yy = rs.apply(x, out=y)
            return pd.apply(yy, out=a).numel()
        ms, n_aud = _time_device(c5, reps=3, warm=1)
        snr = audio_snr_db(a[:n_aud].cpu().numpy(), fs / 10, tones)
        useful = 8.0 * h.size * (n_aud + 1)  # complex tap x complex sample: 8 flops
        arm = {"ms": round(ms, 3), "value": round(x.numel() / ms / 1e3, 1), "unit": "input Msamples/s",
               "audio_snr_db": round(snr, 2), "fir_tflops": round(useful / ms / 1e9, 2)}
        if mode != "fp32":
            arm["tensor_core"] = bool(rs.tc_groups())
            if pk.get("bf16_tflops_sustained"):
                arm["fir_tflops_frac_of_bf16_sustained"] = round(useful / ms / 1e9 / pk["bf16_tflops_sustained"], 4)
        fm[mode] = arm
    rs.set_precision("fp32")

    def c64():
        return fp64_fm_chain(x, h, 10)[1].numel()
    ms, _ = _time_device(c64, reps=1, warm=1)
    _, a64 = fp64_fm_chain(x, h, 10)
    fm["fp64"] = {"ms": round(ms, 3), "value": round(x.numel() / ms / 1e3, 1), "unit": "input Msamples/s",
                  "audio_snr_db": round(audio_snr_db(a64.cpu().numpy(), fs / 10, tones), 2),
                  "how": "torch complex128 FFT convolution + FP64 discriminator on the GPU (comparison arm)"}
    del a64
    res["fir4095_dec10_fm"] = fm
    del x
    # standalone complex FIR, 64 complex taps at full rate, 2^26 samples: the
    # FP32 kernel and the tensor-core Toeplitz form (fp16 hi+lo)
    g = torch.Generator(device="cpu").manual_seed(2030)
    hf = (torch.randn(64, dtype=torch.complex64, generator=g) * 0.1).numpy()
    x = torch.randn(1 << 26, dtype=torch.complex64, device=dev) * 0.5
    y = torch.empty_like(x)
    fir = {"n_in": x.numel(), "taps": 64}
    for mode in ("fp32", "fp16x3"):
        f = F.FirFilterCuda(hf)
        f.set_precision(mode)

        def c6(f=f):
            f.reset_state()
            f.apply(x, out=y)
            return x.numel()
        ms, n = _time_device(c6, reps=3, warm=2)
        fir[mode] = {"ms": round(ms, 3), "value": round(n / ms / 1e3, 1), "unit": "output Msamples/s",
                     "tflops": round(8 * 64 * n / ms / 1e9, 2)}
        if mode != "fp32":
            fir[mode]["tensor_core"] = bool(f.tc_groups())
    res["fir64_complex_2p26"] = fir
    return res


def replica_aggregate(t, units, world: int, dev):
    """Whole-job numbers of N independent replicas (no data exchange on the
    path): the slowest rank's time and the units all ranks processed."""
    if world <= 1:
        return float(t), float(units)
    import torch
    import torch.distributed as dist
    tt = torch.tensor([float(t)], device=dev, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    uu = torch.tensor([float(units)], device=dev, dtype=torch.float64)
    dist.all_reduce(uu)
    return float(tt.item()), float(uu.item())


# --------------------------------------------------------------------------- reference arm
def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from libfalcon_dsp_gb300.workloads import channelizer_256_cpu_sample
    from oracle import oracle as O
    O.build()
    n = args.cpu_sample
    x, fs, chans = channelizer_256_cpu_sample(n, args.n, SEED)
    use_ref = O.have_reference()
    threads = cpu_threads()
    for _ in range(max(args.warmup, 0)):
        cpu_channelizer_rate(fs, chans, x, threads, use_ref)
    rates = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r, kind, used = cpu_channelizer_rate(fs, chans, x, threads, use_ref)
        rates.append(r)
    wall = time.perf_counter() - t0
    value = float(np.median(rates))
    r1, _, _ = cpu_channelizer_rate(fs, chans, x, 1, use_ref)
    line = {
        "impl": "reference", "metric": "channelizer output Msamples/s", "value": value, "unit": "Msamples/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": f"{n} input samples per step x 256 channels", "seed": SEED},
        "cpu_baseline": {"value": value, "unit": "Msamples/s", "cores": used, "kind": kind,
                         "cpu_model": cpu_model(), "sample": f"{n} input samples x 256 channels per step",
                         "single_thread": {"value": round(r1, 3), "unit": "Msamples/s", "cores": 1}},
        "e2e": {"value": value, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- our arm
def run_ours(args) -> None:
    import torch
    import torch.distributed as dist

    import libfalcon_dsp_gb300 as F
    from libfalcon_dsp_gb300 import _capi
    from libfalcon_dsp_gb300.workloads import algorithmic_bytes, channelizer_256

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    x, fs, chans = channelizer_256(args.n, SEED, device=dev)
    ch = F.MultiRateChannelizerCuda(fs, chans)
    ch.set_precision(args.precision)
    # per decimation group: FP32 tile height and tensor-core vs FP32 form,
    # timed on this workload's block size (resets the streaming state)
    tune = ch.autotune(x.numel()) if not args.no_autotune else ch.group_info()
    # each step's launches replayed as one CUDA graph (updated in place)
    ch.set_graph(not args.no_graph)
    nch = len(chans)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream
    # outputs sized for the largest per-step count (counts vary by <= 1 between steps)
    caps = [c + 2 for c in ch.out_count(x.numel())]
    outs = [torch.empty(c, dtype=torch.complex64, device=dev) for c in caps]
    optr = (C.c_void_p * nch)(*[o.data_ptr() for o in outs])
    cap_arr = (C.c_uint64 * nch)(*caps)
    n_out = (C.c_uint64 * nch)()
    lib = _capi.lib()
    xp = C.c_void_p(x.data_ptr())
    torch.cuda.synchronize()

    def step():
        st = lib.fdsp_channelizer_apply(ch._h, xp, x.numel(), optr, cap_arr, n_out, C.c_void_p(sh))
        if st != 0:
            raise F.FdspError("fdsp_channelizer_apply", st, lib.fdsp_last_cuda_error())
        return sum(n_out)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    nl = C.c_uint32()
    lib.fdsp_channelizer_kernel_launches(ch._h, C.byref(nl))
    launches_per_step = nl.value

    gpu_id = None
    try:
        gpu_id = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    clocks = ClockSampler(gpu_id)
    time.sleep(0.3)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")
    e0.record(stream)
    outputs = 0
    for _ in range(args.steps):
        outputs += step()
    e1.record(stream)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()

    # the plain FP32 form of the same step, timed the same way, for comparison
    plain = None
    if args.precision != "fp32" and not args.no_fp32_compare:
        ch.set_precision("fp32")
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        fo = 0
        for _ in range(args.steps):
            fo += step()
        f1.record(stream)
        torch.cuda.synchronize()
        fms = f0.elapsed_time(f1)
        plain = {"value": round(fo / (fms / 1e3) / 1e6, 1), "unit": "Msamples/s", "ms_per_step": round(fms / args.steps, 4)}
        ch.set_precision(args.precision)
    ms, outputs_all = replica_aggregate(ms, outputs, world, dev)
    ms_per_step = ms / args.steps
    value = outputs_all / (ms / 1e3) / 1e6

    # roofline of the dominant kernel: its launches of a step timed live with
    # CUDA events on the launch stream (direct launches while timing)
    bytes_per_step = algorithmic_bytes(x.numel(), outputs // args.steps)
    kname = "tc_filter_kernel" if args.precision != "fp32" else "poly_fp32_kernel"
    roof = None
    if not args.no_kernel_timing:
        ch.set_profile(True)
        for _ in range(args.steps):
            step()
        kms, kl = ch.read_profile()
        ch.set_profile(False)
        if world > 1:
            kms, _ = replica_aggregate(kms, 0, world, dev)
        kms_step = kms / args.steps
        achieved_gbs = bytes_per_step / (kms_step / 1e3) / 1e9
        pk = peaks()
        traffic = ncu_traffic(f"{kname}_channelizer_256_dram", kname, x.numel())
        roof = {"bound": "hbm", "achieved": round(achieved_gbs, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": round(achieved_gbs / pk["hbm_gbs"], 4),
                "traffic": traffic["bytes_per_step"] if traffic else None, "traffic_detail": traffic,
                "kernel": kname, "peak_source": pk["source"] + " (burst copy)",
                "kernel_ms_per_step": round(kms_step, 4), "kernel_launches_per_step": kl // max(args.steps, 1),
                "kernel_share_of_step": round(kms_step / ms_per_step, 3),
                "algorithmic_bytes_per_step": bytes_per_step,
                "note": "achieved = algorithmic bytes of a step (input read once + every output written once) / "
                        "summed duration of the step's launches of the kernel; traffic = DRAM bytes of those "
                        "launches (ncu, scaled by input samples)"}

    # end to end through the host-buffer C ABI call (pinned host memory)
    e2e = None
    if not args.no_e2e:
        hin = torch.empty(x.numel(), dtype=torch.complex64, pin_memory=True)
        hin.copy_(x.cpu())
        houts = [torch.empty(c, dtype=torch.complex64, pin_memory=True) for c in caps]
        hptr = (C.c_void_p * nch)(*[h.data_ptr() for h in houts])
        ch.reset_state()

        def step_host():
            st = lib.fdsp_channelizer_apply_host(ch._h, C.c_void_p(hin.data_ptr()), hin.numel(), hptr, cap_arr,
                                                 n_out, C.c_void_p(sh))
            if st != 0:
                raise F.FdspError("fdsp_channelizer_apply_host", st, lib.fdsp_last_cuda_error())
            return sum(n_out)

        step_host()  # warm-up: allocates the library's device staging buffers
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eo = 0
        for _ in range(args.e2e_steps):
            eo += step_host()
        dt = time.perf_counter() - t0
        dt, eo = replica_aggregate(dt, eo, world, dev)
        e2e = {"value": eo / dt / 1e6, "unit": "Msamples/s", "h2d_bytes_per_step": 8 * hin.numel(),
               "d2h_bytes_per_step": 8 * (eo // args.e2e_steps if world == 1 else int(eo / world) // args.e2e_steps),
               "steps": args.e2e_steps, "ms_per_step": 1000 * dt / args.e2e_steps}

    # the other workloads of the path, each timed on the device (inputs
    # resident, CUDA events, after warm-up): single-channel 147/160 resampler,
    # 8-channel streaming channelizer in 2^16-sample blocks, and the 4095-tap
    # FIR / decimate-by-10 / FM discriminator chain
    others = None
    if not args.no_other_configs:
        others = other_configs(dev, lib)

    # streaming serving loop: Poisson job arrivals at 2000/s, 1-64 channels,
    # blocks of 4096-1M samples, host buffers in and out, FP32 form
    serving = None
    if not args.no_serving:
        from libfalcon_dsp_gb300.serving import run_serving
        st = run_serving(duration_s=args.serve_seconds, rate_hz=2000.0, seed=SEED, budget_bytes=120 << 30,
                         max_active=args.serve_streams, precision=0)
        serving = {"p50_ms": round(st["p50_ms"], 4), "p99_ms": round(st["p99_ms"], 4),
                   "p999_ms": round(st["p999_ms"], 4), "blocks": st["blocks"],
                   "value": round(st["out_msps"], 1), "unit": "Msamples/s",
                   "streams": args.serve_streams, "jobs_admitted": st["admitted"], "jobs_arrived": st["arrived"],
                   "served_fraction": round(st["served_fraction"], 4),
                   "admit_wait_p50_ms": round(st["admit_wait_p50_ms"], 3),
                   "admit_wait_p99_ms": round(st["admit_wait_p99_ms"], 3),
                   "seconds": round(st["wall_s"], 3),
                   "note": "latency = submit to output back in pinned host memory; jobs arrive faster than one GPU "
                           "serves them (served_fraction of the arrivals are admitted within the window), admission "
                           "is by the memory budget (one device pool, no allocation per stream) and the stream "
                           "limit; admit_wait = arrival to admission"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build(with_reference=None)
        n_s = min(args.cpu_sample, x.numel())
        cpu = cpu_baseline(fs, chans, x[:n_s].cpu().numpy(), O.have_reference())

    if rank == 0:
        line = {
            "metric": "channelizer output Msamples/s", "value": round(value, 1), "unit": "Msamples/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32" if args.precision == "fp32" else args.precision + "(fp32 accumulate)",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "n_in": x.numel(), "channels": nch, "seed": SEED,
                       "path": {"fp32": "plain FP32 SIMT",
                                "fp16x3": "tensor cores (tcgen05), FP16 (hi+lo)(hi+lo), FP32 accumulate",
                                "bf16x3": "tensor cores (tcgen05), BF16 (hi+lo)(hi+lo), FP32 accumulate"}[args.precision],
                       "autotune": [{"down": t["down_rate"], "tile_rows": t["tile_rows"], "tc": t["tensor_core"],
                                     "tc_split": t["tc_split"]}
                                    for t in tune],
                       "cuda_graph": not args.no_graph, "graph_replays": ch.graph_replays(),
                       "l2": "no flush: each step reads 512 MiB and writes ~9.6 GB, far above the 129 MB L2",
                       "parallelism": f"replicas x{world}"},
            "gpu_launches": launches_per_step * args.steps,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "serving": serving,
            "other_configs": others,
            "plain_fp32": plain,
            "tc_speedup_vs_plain_fp32": round(ms_per_step / plain["ms_per_step"], 3) ** -1 if plain else None,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
