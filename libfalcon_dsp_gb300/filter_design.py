"""Resampling anti-alias filters: the predefined table and its generator.

libfalcon_dsp ships a table of resampling lowpass filters keyed by
(input rate, output rate, tap count, algorithm) and looked up by
``get_resample_fir_params`` (src/transform/falcon_dsp_fir_filter.cc:111-130;
key and enums in hdr/transform/falcon_dsp_predefined_fir_filter.h:63-141).
The table is generated offline by a published recipe
(test/utilities/generate_predefined_fir_filter_coeffs.ipynb), restated here:

* rate pairs 1.14 M -> 228 k, 1.14 M -> 200 k, 1 M -> 200 k, 228 k -> 45.6 k,
  200 k -> 45 k, 200 k -> 44 k;
* up/down from the output/input ratio printed to 12 decimals and reduced to
  the closest fraction (``Fraction.limit_denominator``);
* tap counts 32, 64, 128, 256 plus the "optimal" 20 max(up, down) + 1;
* FIRLS: ``up * firls(n, [0, 1/m, 1/m, 1], [1, 1, 0, 0]) * kaiser(n, 5)``
  with n made odd and m = max(up, down);
* REMEZ (n <= 200 taps): ``remez(n, [0, out, out + (in/2 - out)/4, in/2],
  [1, 0], fs=in, maxiter=100)``;
* every coefficient printed with 8 decimals (then read back as float).

``write_table_inc`` writes the table as a C++ include for the library's
``fdsp_get_resample_fir_params``; the library build calls it, so the table
is generated where the library is built (scipy is a build-time tool only).
"""
from __future__ import annotations

import math
import os
import warnings
from fractions import Fraction

import numpy as np

RATE_PAIRS = [(1140000, 228000), (1140000, 200000), (1000000, 200000), (228000, 45600), (200000, 45000),
              (200000, 44000)]
FILTER_ORDERS = [32, 64, 128, 256]
NAMED_TAPS = (16, 32, 64, 128, 256)  # filter_taps_e values; anything else is FILTER_TAPS_OPTIMAL (-1)
TAPS_OPTIMAL = -1
REMEZ, FIRLS = 0, 1  # filter_source_type_e


def up_down(in_sps: int, out_sps: int) -> tuple[int, int]:
    fr = Fraction("%.12f" % (out_sps / in_sps)).limit_denominator()
    return fr.numerator, fr.denominator


def _round8(h: np.ndarray) -> np.ndarray:
    # the table stores "%+.8f" text; the compiler reads it back as float
    return np.array([float("%+.8f" % v) for v in h], dtype=np.float64).astype(np.float32)


def design_table() -> dict:
    """{(in_sps, out_sps, taps_enum, source): (up, down, float32 coeffs)}."""
    from scipy import signal
    from scipy.signal import windows

    table = {}
    for in_sps, out_sps in RATE_PAIRS:
        p, q = up_down(in_sps, out_sps)
        m = max(p, q)
        cutoff = 1.0 / 2.0 / m
        orders = sorted(set(FILTER_ORDERS + [2 * 10 * m + 1]))
        for order in orders:
            key_taps = order if order in NAMED_TAPS else TAPS_OPTIMAL
            n = order + 1 if order % 2 == 0 else order
            h = float(p) * signal.firls(n, [0, 2.0 * cutoff, 2.0 * cutoff, 1.0], [1.0, 1.0, 0.0, 0.0])
            h = h * windows.kaiser(n, beta=5)
            table[(in_sps, out_sps, key_taps, FIRLS)] = (p, q, _round8(h))
            if order <= 200:
                try:
                    with warnings.catch_warnings():
                        warnings.simplefilter("ignore")
                        h = signal.remez(order, [0, out_sps, out_sps + (in_sps / 2 - out_sps) / 4, in_sps / 2],
                                         [1, 0], fs=in_sps, maxiter=100)
                except Exception:  # the recipe leaves out designs that do not converge
                    continue
                table[(in_sps, out_sps, key_taps, REMEZ)] = (p, q, _round8(h))
    return table


def write_table_inc(path: str) -> None:
    """The table as C++ initialisers: one float array per entry, then
    ``{in, out, taps, source, up, down, count, array}`` rows."""
    table = design_table()
    lines = ["// generated by libfalcon_dsp_gb300/filter_design.py: do not edit", ""]
    rows = []
    for i, ((fi, fo, taps, src), (p, q, h)) in enumerate(sorted(table.items())):
        vals = ", ".join("%.9ef" % v for v in h)
        lines.append(f"static const float kFilt{i}[{h.size}] = {{{vals}}};")
        rows.append(f"  {{{fi}u, {fo}u, {taps}, {src}u, {p}u, {q}u, {h.size}u, kFilt{i}}},")
    lines.append("")
    lines.append("static const PredefinedFilter kPredefined[] = {")
    lines += rows
    lines.append("};")
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        f.write("\n".join(lines) + "\n")
    os.replace(tmp, path)


def kaiser_firls_lowpass(num_taps: int, up: int, down: int, beta: float = 5.0) -> np.ndarray:
    """The FIRLS recipe for any up/down (float64): the least-squares lowpass
    over the two contiguous bands is the truncated ideal lowpass with edge
    1/max(up, down) of Nyquist, then scaled by `up` and Kaiser windowed.
    The library's native designer (fdsp_design_resample_firls) computes the
    same closed form."""
    n = num_taps + 1 if num_taps % 2 == 0 else num_taps
    m = max(up, down)
    k = np.arange(n) - (n - 1) / 2
    h = np.sinc(k / m) / m
    x = 2.0 * np.arange(n) / (n - 1) - 1.0
    w = np.i0(beta * np.sqrt(np.clip(1.0 - x * x, 0.0, None))) / np.i0(beta)
    return up * h * w


__all__ = ["RATE_PAIRS", "FILTER_ORDERS", "TAPS_OPTIMAL", "REMEZ", "FIRLS", "up_down", "design_table",
           "write_table_inc", "kaiser_firls_lowpass"]

if __name__ == "__main__":  # pragma: no cover
    t = design_table()
    print(len(t), "entries")
    _ = math
