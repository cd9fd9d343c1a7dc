"""Streaming serving loop over the native channelizer server (fdsp_server_*).

``ChannelizerServer`` wraps the C ABI.  ``run_serving`` drives it with the
streaming-serving workload: jobs arrive as a Poisson process, each a stream
with 1-64 channels (log-uniform), a block size uniform in 4096-1,048,576
complex64 samples, 10-200 blocks, at an input rate in 10-61.44 MS/s; each
channel has its own NCO offset, decimation from {8, 16, 25, 40, 64, 125, 160,
320}, up factor {1, 2, 3} and 12-64 taps per phase.  A job is admitted when
the server's device-memory budget and active-stream limit allow (continuous
batching: admission happens as soon as earlier streams close), then submits
its blocks one after another, each as soon as the previous one completed;
blocks of different jobs overlap on the GPU.  Reported: p50/p99/p999 block
latency and aggregate output Msamples/s.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from collections import deque

import numpy as np

from . import _capi
from ._capi import FdspError, channel_cfg
from .workloads import kaiser_lowpass

DECIM = [8, 16, 25, 40, 64, 125, 160, 320]
UPS = [1, 2, 3]


class ChannelizerServer:
    def __init__(self, budget_bytes: int, max_active: int):
        self._h = C.c_void_p(0)
        _capi.call("fdsp_server_create", int(budget_bytes), int(max_active), C.byref(self._h))
        self._keep = {}
        self._ticket = C.c_uint64()
        self._ticket_ref = C.byref(self._ticket)
        self._done, self._lat = C.c_int(), C.c_double()

    def __del__(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            try:
                _capi.lib().fdsp_server_destroy(self._h)
            except Exception:
                pass
            self._h = C.c_void_p(0)

    def open(self, fs: int, channels: list[dict], max_block: int, precision: int = 0) -> int | None:
        """Stream id, or None when the budget or the stream limit is full."""
        arr = (channel_cfg * len(channels))()
        keep = []
        for i, ch in enumerate(channels):
            taps = np.ascontiguousarray(ch["coeffs"], dtype=np.complex64)
            keep.append(taps)
            arr[i].output_sample_rate_in_sps = 0
            arr[i].freq_shift_in_hz = int(ch["freq_shift_in_hz"])
            arr[i].up_rate = int(ch["up_rate"])
            arr[i].down_rate = int(ch["down_rate"])
            arr[i].resample_filter_coeffs = taps.ctypes.data
            arr[i].num_coeffs = taps.size
        sid = C.c_uint32()
        st = _capi.lib().fdsp_server_open(self._h, int(fs), arr, len(channels), int(max_block), int(precision),
                                          C.byref(sid))
        if st == _capi.FDSP_ERR_CAPACITY:
            return None
        _capi.check("fdsp_server_open", st)
        return sid.value

    @staticmethod
    def out_args(out_ptrs, out_caps):
        """ctypes arrays of output pointers and capacities, built once per job."""
        n = len(out_ptrs)
        return (C.c_void_p * n)(*out_ptrs), (C.c_uint64 * n)(*out_caps)

    def submit(self, sid: int, in_ptr: int, n_in: int, out_ptrs, out_caps) -> int:
        if not isinstance(out_ptrs, C.Array):
            out_ptrs, out_caps = self.out_args(out_ptrs, out_caps)
        t = self._ticket
        st = _capi.lib().fdsp_server_submit(self._h, sid, in_ptr, n_in, out_ptrs, out_caps, self._ticket_ref)
        if st:
            _capi.check("fdsp_server_submit", st)
        return t.value

    def poll(self, ticket: int, nch: int, n_out=None):
        """(done, output counts, latency ms); a done ticket is reported once.
        `n_out` may be a reused (c_uint64 * nch) array."""
        if n_out is None:
            n_out = (C.c_uint64 * nch)()
        st = _capi.lib().fdsp_server_poll(self._h, ticket, C.byref(self._done), n_out, C.byref(self._lat))
        if st:
            _capi.check("fdsp_server_poll", st)
        return bool(self._done.value), n_out, self._lat.value

    def wait_any(self, timeout_us: int = 1000) -> int:
        """Next completed ticket (0 when none completed within the timeout)."""
        t = C.c_uint64()
        _capi.call("fdsp_server_wait_any", self._h, int(timeout_us), C.byref(t))
        return t.value

    def close(self, sid: int) -> None:
        _capi.call("fdsp_server_close", self._h, int(sid))

    def stats(self) -> dict:
        p50, p99, p999 = C.c_double(), C.c_double(), C.c_double()
        blocks, outs, used = C.c_uint64(), C.c_uint64(), C.c_uint64()
        act = C.c_uint32()
        _capi.call("fdsp_server_stats", self._h, C.byref(p50), C.byref(p99), C.byref(p999), C.byref(blocks),
                   C.byref(outs), C.byref(used), C.byref(act))
        return {"p50_ms": p50.value, "p99_ms": p99.value, "p999_ms": p999.value, "blocks": blocks.value,
                "outputs": outs.value, "used_bytes": used.value, "active": act.value}

    def reset_stats(self) -> None:
        _capi.call("fdsp_server_reset_stats", self._h)


_TAPS: dict = {}


def _taps(u: int, d: int, tpp: int) -> np.ndarray:
    key = (u, d, tpp)
    if key not in _TAPS:
        _TAPS[key] = kaiser_lowpass(u, d, tpp).astype(np.complex64)
    return _TAPS[key]


def random_job(rng: np.random.Generator, max_channels: int = 64, block_range=(4096, 1 << 20),
               blocks_range=(10, 200)) -> dict:
    """One streaming job of the serving workload (parameters as documented above)."""
    nch = int(round(math.exp(rng.uniform(0.0, math.log(max_channels)))))
    nch = max(1, min(max_channels, nch))
    fs = int(rng.uniform(10e6, 61.44e6))
    chans = []
    for _ in range(nch):
        d = int(rng.choice(DECIM))
        u = int(rng.choice(UPS))
        g = math.gcd(u, d)
        u, d = u // g, d // g
        tpp = int(rng.integers(12, 65))
        chans.append({"freq_shift_in_hz": int(rng.uniform(-0.45, 0.45) * fs), "up_rate": u, "down_rate": d,
                      "coeffs": _taps(u, d, tpp)})
    return {"fs": fs, "channels": chans, "block": int(rng.integers(block_range[0], block_range[1] + 1)),
            "blocks": int(rng.integers(blocks_range[0], blocks_range[1] + 1))}


def _out_caps(job: dict) -> list[int]:
    b = job["block"]
    return [(b * c["up_rate"] + c["down_rate"] - 1) // c["down_rate"] + 2 for c in job["channels"]]


def run_serving(duration_s: float = 5.0, rate_hz: float = 2000.0, seed: int = 4, budget_bytes: int = 120 << 30,
                max_active: int = 16, precision: int = 0, max_blocks_per_job: int | None = None,
                block_range=(4096, 1 << 20)) -> dict:
    """Drive the server for `duration_s` of arrivals, then drain the admitted
    jobs; returns the server statistics plus throughput and queue figures."""
    import torch

    rng = np.random.default_rng(seed)
    srv = ChannelizerServer(budget_bytes, max_active)
    # one pinned input pool (jobs read a slice of it) and one pinned output
    # arena per active slot, sized for the largest job
    pool_n = block_range[1] + 4096
    x = (rng.standard_normal(pool_n) + 1j * rng.standard_normal(pool_n)).astype(np.complex64) * 0.1
    pin_in = torch.from_numpy(x.view(np.float32)).pin_memory()
    in_base = pin_in.data_ptr()
    arena_bytes = 8 * (64 * ((block_range[1] * 3) // 8 + 2) + 1024)
    free_arenas = deque(torch.empty(arena_bytes, dtype=torch.uint8, pin_memory=True) for _ in range(max_active))
    pending: deque = deque()
    active = {}
    t0 = time.perf_counter()
    next_arrival = t0 + rng.exponential(1.0 / rate_hz)
    arrived = admitted = completed_jobs = 0
    wait_admit = []
    head = None
    by_ticket = {}
    while True:
        now = time.perf_counter()
        while next_arrival <= now and next_arrival - t0 < duration_s:
            pending.append(next_arrival)  # the job itself is drawn when it is admitted
            arrived += 1
            next_arrival += rng.exponential(1.0 / rate_hz)
        # admission: as many waiting jobs as memory and slots allow
        while pending and free_arenas:
            if head is None:
                head = random_job(rng, block_range=block_range)
                if max_blocks_per_job:
                    head["blocks"] = min(head["blocks"], max_blocks_per_job)
                head["t_arrive"] = pending[0]
            job = head
            sid = srv.open(job["fs"], job["channels"], job["block"], precision)
            if sid is None:
                break
            pending.popleft()
            head = None
            arena = free_arenas.popleft()
            caps = _out_caps(job)
            ptrs, off = [], 0
            for c in caps:
                ptrs.append(arena.data_ptr() + off)
                off += 8 * c
            optr, ocap = ChannelizerServer.out_args(ptrs, caps)
            job.update(sid=sid, arena=arena, caps=ocap, ptrs=optr, left=job["blocks"],
                       n_out=(C.c_uint64 * len(caps))(),
                       src=in_base + 8 * int(rng.integers(0, pool_n - job["block"])))
            wait_admit.append(time.perf_counter() - job["t_arrive"])
            t = srv.submit(sid, job["src"], job["block"], optr, ocap)
            by_ticket[t] = sid
            job["left"] -= 1
            active[sid] = job
            admitted += 1
        # progress: the next block of each job whose previous block completed
        # (completed tickets come from the server's completion queue)
        t = srv.wait_any(200 if active else 0)
        while t:
            sid = by_ticket.pop(t)
            job = active[sid]
            srv.poll(t, len(job["channels"]), job["n_out"])
            if job["left"] > 0:
                t2 = srv.submit(sid, job["src"], job["block"], job["ptrs"], job["caps"])
                by_ticket[t2] = sid
                job["left"] -= 1
            else:
                srv.close(sid)
                free_arenas.append(job["arena"])
                del active[sid]
                completed_jobs += 1
            t = srv.wait_any(0)
        if now - t0 >= duration_s and not active:
            break
        if now - t0 >= duration_s and pending:
            pending.clear()  # arrivals after the window are not served
    wall = time.perf_counter() - t0
    st = srv.stats()
    st.update(wall_s=wall, arrived=arrived, admitted=admitted, completed_jobs=completed_jobs,
              out_msps=st["outputs"] / wall / 1e6,
              admit_wait_p50_ms=1e3 * float(np.percentile(wait_admit, 50)) if wait_admit else 0.0,
              admit_wait_p99_ms=1e3 * float(np.percentile(wait_admit, 99)) if wait_admit else 0.0,
              served_fraction=admitted / arrived if arrived else 0.0)
    return st
