"""Readers for the golden fixtures in tests/golden, in the reference's file
formats (src/utilities/falcon_dsp_utils.cc): complex int16 little-endian
pairs for data, "re im" text lines for taps."""
from __future__ import annotations

import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def manifest() -> dict:
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def read_c16(name: str) -> np.ndarray:
    raw = np.fromfile(os.path.join(GOLDEN, name), dtype="<i2").reshape(-1, 2)
    return (raw[:, 0].astype(np.float32) + 1j * raw[:, 1].astype(np.float32)).astype(np.complex64)


def read_taps(name: str) -> np.ndarray:
    v = np.loadtxt(os.path.join(GOLDEN, name), dtype=np.float64).reshape(-1, 2)
    return (v[:, 0] + 1j * v[:, 1]).astype(np.complex64)


def near_per_component(got: np.ndarray, exp: np.ndarray, rel: float, floor: float) -> tuple[bool, int]:
    """The reference tests' EXPECT_NEAR rule: per real/imag component,
    |got - exp| <= max(rel * |exp|, floor).  Returns (ok, first_bad_index)."""
    n = min(got.size, exp.size)
    g, e = got[:n], exp[:n]
    tol_r = np.maximum(np.abs(e.real) * rel, floor)
    tol_i = np.maximum(np.abs(e.imag) * rel, floor)
    bad = (np.abs(g.real - e.real) > tol_r) | (np.abs(g.imag - e.imag) > tol_i)
    idx = np.flatnonzero(bad)
    return (idx.size == 0, int(idx[0]) if idx.size else -1)


def rel_rms(got: np.ndarray, exp: np.ndarray) -> float:
    got = np.asarray(got, dtype=np.complex128)
    exp = np.asarray(exp, dtype=np.complex128)
    den = np.sqrt(np.mean(np.abs(exp) ** 2))
    if den == 0:
        return float(np.sqrt(np.mean(np.abs(got) ** 2)))
    return float(np.sqrt(np.mean(np.abs(got - exp) ** 2)) / den)


def snr_db(got: np.ndarray, exp: np.ndarray) -> float:
    got = np.asarray(got, dtype=np.complex128)
    exp = np.asarray(exp, dtype=np.complex128)
    err = np.sum(np.abs(got - exp) ** 2)
    sig = np.sum(np.abs(exp) ** 2)
    return float("inf") if err == 0 else float(10 * np.log10(sig / err))
