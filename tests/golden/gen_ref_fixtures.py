"""Fixtures made by the reference's own CPU classes (oracle/_ref, compiled in
place from a libfalcon_dsp checkout by oracle/Makefile): seeded inputs, the
reference's outputs, stored in tests/golden/ref_fixtures.npz.

    FDSP_REF_ROOT=<libfalcon_dsp checkout> python tests/golden/gen_ref_fixtures.py

tests/test_ref_fixtures.py compares the oracle's C restatement with these
outputs on every run, so the restatement stays pinned to the reference where
no reference checkout exists (the GPU machine, a fresh clone).  The predefined
filter table is pinned by a SHA-256 of each entry's coefficients, not by the
coefficients themselves.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "ref_fixtures.npz")

RESAMPLER_CASES = [(1, 2, 3), (4, 5, 3), (147, 160, 3528), (3, 125, 300), (2, 1, 41), (1, 1, 17), (7, 3, 64)]
CHANNELIZER_CASE = [(-350000, 1, 10, 201), (60000, 1, 4, 81), (27000, 77, 200, 400), (0, 3, 20, 61)]
FM_OFFSET = -150000


def rand_c64(n, seed, scale=1000.0):
    r = np.random.default_rng(seed)
    return ((r.standard_normal(n) + 1j * r.standard_normal(n)) * scale).astype(np.complex64)


def block_cuts(n, seed):
    r = np.random.default_rng(seed)
    cuts, i = [], 0
    while i < n:
        k = int(r.choice([1, 2, 7, 33, 500, 1500]))
        cuts.append((i, min(n, i + k)))
        i += k
    return cuts


TABLE_TAPS = [16, 32, 64, 128, 256, -1]


def table_keys():
    import libfalcon_dsp_gb300 as F
    from libfalcon_dsp_gb300 import filter_design as FD
    return [(fi, fo, t, s) for fi, fo in FD.RATE_PAIRS for t in TABLE_TAPS for s in (F.REMEZ, F.FIRLS)]


def entry_digest(h) -> str:
    """SHA-256 of the coefficients as float32 (+0.0 added, so -0.0 and 0.0,
    equal values, hash alike)."""
    v = np.ascontiguousarray(np.asarray(h, np.float32) + np.float32(0.0))
    return hashlib.sha256(v.tobytes()).hexdigest()


def main() -> None:
    from oracle import oracle as O
    if not O.have_reference():
        O.build(with_reference=True)
    fx = {}
    # resampler: streamed in ragged blocks, counts and samples
    x = rand_c64(3000, 1)
    for (up, down, ntaps) in RESAMPLER_CASES:
        h = rand_c64(ntaps, 2, 1.0)
        r = O.RefResampler(up, down, h)
        ys = [r.apply(x[i:j]) for i, j in block_cuts(x.size, 3)]
        fx[f"resamp_{up}_{down}_{ntaps}"] = np.concatenate(ys).astype(np.complex64)
        fx[f"resamp_{up}_{down}_{ntaps}_counts"] = np.array([y.size for y in ys], np.int64)
    # channelizer: two passes with a reset between
    x = rand_c64(8000, 4)
    chans = [dict(freq_shift_in_hz=f, up_rate=u, down_rate=d, coeffs=rand_c64(t, 5 + i, 1.0))
             for i, (f, u, d, t) in enumerate(CHANNELIZER_CASE)]
    ref = O.RefChannelizer(1000000, chans)
    for rep in range(2):
        outs = [[] for _ in chans]
        for i, j in block_cuts(x.size, 6 + rep):
            for c, y in enumerate(ref.apply(x[i:j])):
                outs[c].append(y)
        for c in range(len(chans)):
            fx[f"chan_rep{rep}_ch{c}"] = np.concatenate(outs[c]).astype(np.complex64)
        ref.reset_state()
    # FIR (complex taps) and polar discriminator, streamed
    lib = O.ref_lib()
    x = rand_c64(5000, 7)
    h = O.as_c64(rand_c64(129, 8, 0.1))
    hb = lib.ref_fir_new(O._f32p(h.view(np.float32)), h.size)
    ys = []
    for i, j in block_cuts(x.size, 9):
        xb = O.as_c64(x[i:j])
        yb = np.empty_like(xb)
        lib.ref_fir_apply(hb, O._f32p(xb.view(np.float32)), xb.size, O._f32p(yb.view(np.float32)))
        ys.append(yb)
    lib.ref_fir_free(hb)
    fx["fir_129"] = np.concatenate(ys)
    pb = lib.ref_polar_new()
    ys = []
    for i, j in block_cuts(x.size, 10):
        xb = O.as_c64(x[i:j])
        yb = np.empty(xb.size, np.float32)
        n = lib.ref_polar_apply(pb, O._f32p(xb.view(np.float32)), xb.size, O._f32p(yb))
        ys.append(yb[:n])
    lib.ref_polar_free(pb)
    fx["polar"] = np.concatenate(ys)
    # rat_approx and get_freq_shift_params
    r = np.random.default_rng(11)
    ra = []
    for _ in range(300):
        f = float(r.uniform(0.001, 4.0))
        md = int(r.choice([10, 100, 1024, 5000]))
        n, d = C.c_int64(), C.c_int64()
        lib.ref_rat_approx(f, md, C.byref(n), C.byref(d))
        ra.append((f, md, n.value, d.value))
    fx["rat_approx_in"] = np.array([(a, b) for a, b, _, _ in ra], np.float64)
    fx["rat_approx_out"] = np.array([(c, d) for _, _, c, d in ra], np.int64)
    ps = []
    for _ in range(300):
        fs = int(r.integers(1000, 100_000_000))
        f = int(r.integers(-fs // 2, fs // 2))
        if f == 0:
            continue
        rr, w = C.c_uint32(), C.c_double()
        lib.ref_freq_shift_params(fs, f, C.byref(rr), C.byref(w))
        ps.append((fs, f, rr.value, w.value))
    fx["shift_params_in"] = np.array([(a, b) for a, b, _, _ in ps], np.int64)
    fx["shift_params_R"] = np.array([c for _, _, c, _ in ps], np.int64)
    fx["shift_params_w"] = np.array([d for _, _, _, d in ps], np.float64)
    # IIR (de-emphasis taps and a general complex filter)
    rng = np.random.default_rng(3)
    iir_cases = [(np.array([0.064493014968382223], np.complex64), np.array([1.0, -0.93550698503161778], np.complex64)),
                 ((rng.standard_normal(4) + 1j * rng.standard_normal(4)).astype(np.complex64),
                  np.array([1.0, 0.2 - 0.1j, -0.05 + 0.02j], np.complex64))]
    for ci, (b, a) in enumerate(iir_cases):
        rf = O.RefIIR(b, a)
        xs, ys = [], []
        for n in (1, 3, 700, 2, 1500):
            xx = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
            xs.append(xx)
            ys.append(rf.apply(xx))
        fx[f"iir{ci}_b"], fx[f"iir{ci}_a"] = b, a
        fx[f"iir{ci}_x"] = np.concatenate(xs)
        fx[f"iir{ci}_y"] = np.concatenate(ys)
    # FM mono demodulator on a synthetic station, three blocks
    from libfalcon_dsp_gb300.workloads import FM_RADIO_FS, fm_station
    xs, _ = fm_station(3 * 57000 + 123)
    rf = O.RefFmDemod(FM_RADIO_FS, FM_OFFSET)
    outs = [rf.demod_mono(b) for b in (xs[:57000], xs[57000:114123], xs[114123:])]
    fx["fm_audio"] = np.concatenate(outs).astype(np.int16)
    fx["fm_counts"] = np.array([o.size for o in outs], np.int64)
    # predefined filter table: (key, up, down, digest) per entry that exists
    rows, digests = [], []
    for key in table_keys():
        got = O.ref_get_resample_fir_params(*key)
        if got is None:
            rows.append(list(key) + [-1, -1])
            digests.append("")
        else:
            rows.append(list(key) + [got[0], got[1]])
            digests.append(entry_digest(np.asarray(got[2]).real))
    fx["table_rows"] = np.array(rows, np.int64)
    fx["table_digests"] = np.array(digests)
    np.savez_compressed(OUT, **fx)
    print(f"wrote {OUT}: {len(fx)} arrays, {os.path.getsize(OUT)} bytes")


if __name__ == "__main__":
    main()
