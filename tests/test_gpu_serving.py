"""The streaming server (fdsp_server_*): admission by device-memory budget,
per-stream state resident across blocks, and continuous batching -- every
job's outputs are the same alone and in the mix (bit-exact: the same kernels
run on the same per-stream state whatever else shares the GPU)."""
import numpy as np
import pytest

from libfalcon_dsp_gb300.serving import ChannelizerServer, random_job, run_serving

pytestmark = pytest.mark.gpu


def _jobs(n, seed):
    rng = np.random.default_rng(seed)
    jobs = []
    for _ in range(n):
        j = random_job(rng, max_channels=12, block_range=(4096, 40000), blocks_range=(3, 5))
        j["x"] = [((rng.standard_normal(j["block"]) + 1j * rng.standard_normal(j["block"])) * 0.2)
                  .astype(np.complex64) for _ in range(j["blocks"])]
        jobs.append(j)
    return jobs


def _caps(j):
    return [(j["block"] * c["up_rate"] + c["down_rate"] - 1) // c["down_rate"] + 2 for c in j["channels"]]


def _run(jobs, max_active, precision, contiguous=False):
    """Process every job's blocks in order; jobs run concurrently up to
    max_active (round-robin submission as each job's previous block ends)."""
    srv = ChannelizerServer(64 << 30, max_active)
    res = {i: [] for i in range(len(jobs))}
    queue = list(range(len(jobs)))
    active = {}
    while queue or active:
        while queue and len(active) < max_active:
            i = queue.pop(0)
            j = jobs[i]
            sid = srv.open(j["fs"], j["channels"], j["block"], precision)
            assert sid is not None
            active[i] = {"sid": sid, "k": 0, "ticket": None, "bufs": None}
        for i in list(active):
            a, j = active[i], jobs[i]
            if a["ticket"] is not None:
                done, n_out, _ = srv.poll(a["ticket"], len(j["channels"]))
                if not done:
                    continue
                res[i].append([b[:n].copy() for b, n in zip(a["bufs"], n_out)])
                a["ticket"] = None
            if a["k"] == j["blocks"]:
                srv.close(a["sid"])
                del active[i]
                continue
            caps = _caps(j)
            if contiguous:  # one host arena, channel regions back to back: the single-copy path
                arena = np.empty(sum(caps), np.complex64)
                offs = np.concatenate([[0], np.cumsum(caps)[:-1]])
                a["bufs"] = [arena[o:o + c] for o, c in zip(offs, caps)]
            else:
                a["bufs"] = [np.empty(c, np.complex64) for c in caps]
            a["ticket"] = srv.submit(a["sid"], j["x"][a["k"]].ctypes.data, j["block"],
                                     [b.ctypes.data for b in a["bufs"]], caps)
            a["in"] = j["x"][a["k"]]
            a["k"] += 1
    st = srv.stats()
    assert st["active"] == 0 and st["used_bytes"] == 0
    return res


def test_single_copy_outputs_equal_per_channel_copies():
    jobs = _jobs(4, 21)
    sep = _run(jobs, 4, 0)
    one = _run(jobs, 4, 0, contiguous=True)
    for i in range(len(jobs)):
        for a, b in zip(sep[i], one[i]):
            for u, v in zip(a, b):
                assert np.array_equal(u, v)


@pytest.mark.parametrize("precision", [0, 1])
def test_results_same_alone_and_in_the_mix(precision):
    jobs = _jobs(6, 7 + precision)
    alone = _run(jobs, 1, precision)
    mix = _run(jobs, 6, precision)
    for i in range(len(jobs)):
        assert len(alone[i]) == len(mix[i]) == jobs[i]["blocks"]
        for a, m in zip(alone[i], mix[i]):
            for ya, ym in zip(a, m):
                assert ya.size == ym.size
                assert np.array_equal(ya, ym)


def test_admission_by_budget():
    rng = np.random.default_rng(3)
    j = random_job(rng, max_channels=4, block_range=(1 << 20, 1 << 20), blocks_range=(1, 1))
    srv = ChannelizerServer(4 << 20, 4)          # 4 MiB: too small for a 1M-sample block
    assert srv.open(j["fs"], j["channels"], j["block"]) is None
    srv2 = ChannelizerServer(1 << 30, 1)         # room for one stream only
    a = srv2.open(j["fs"], j["channels"], j["block"])
    assert a is not None
    assert srv2.open(j["fs"], j["channels"], j["block"]) is None
    srv2.close(a)
    b = srv2.open(j["fs"], j["channels"], j["block"])
    assert b is not None
    srv2.close(b)


def test_serving_loop_reports_latency_and_throughput():
    st = run_serving(duration_s=1.0, rate_hz=200.0, seed=5, max_active=8, max_blocks_per_job=5,
                     block_range=(4096, 1 << 18))
    assert st["blocks"] > 0 and st["outputs"] > 0
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["p999_ms"]
    assert st["active"] == 0
    print("serving:", st)
