"""Regenerate the golden vectors of libfalcon_dsp's unit tests.

The reference defines its test vectors in test/generate_test_vectors.sh
(environment settings per vector) and four Jupyter notebooks under
test/utilities/ (the generators), but ships test/vectors/ empty.  This script
restates those notebook cells as plain numpy/scipy so the vectors can be
rebuilt without Jupyter:

  polyphase / single-channel shift  generate_polyphase_test_vectors.ipynb        (vectors 001-009)
  FIR                               generate_fir_filter_test_vectors.ipynb       (vectors 010-011)
  multi-channel shift               generate_multi_chan_freq_shift_test_vectors.ipynb (012-014)
  multi-rate channelizer            generate_multi_rate_channelizer_test_vectors.ipynb (015-018)

Deviations, all forced by the environment and none affecting the algorithm:
  * scipy.signal.kaiser is gone from scipy 1.18; scipy.signal.windows.kaiser
    is the same window.
  * Python loops the notebooks use for max-abs normalisation and int16
    packing are vectorised (same values: int() truncates toward zero, as
    np.trunc does).
  * Vectors 010/011 draw their tones from an unseeded generator in the
    notebook; here they are seeded (4010 / 4011) so the fixture is stable.
  * To keep the committed fixtures small, each vector is generated at the
    notebook's full length (so seeds, normalisation and noise are exactly the
    notebook's) and then only a prefix is written: the first NKEEP input
    samples and the outputs that depend on them alone.  Filtered outputs are
    computed on the prefix, which gives the same leading outputs as filtering
    the full vector.

Files use the reference's formats (src/utilities/falcon_dsp_utils.cc):
complex int16 little-endian pairs ``<2h`` for data, ``"%0.12f %0.12f\\n"`` text
for taps.  A manifest (golden.json) records every vector's parameters.

Run:  python tests/golden/gen_golden.py  (writes next to this file)
"""
from __future__ import annotations

import json
import os
from fractions import Fraction

import numpy as np
from scipy import signal

HERE = os.path.dirname(os.path.abspath(__file__))
NKEEP = 8192


def _trunc_i16_pairs(y: np.ndarray) -> np.ndarray:
    out = np.empty((y.size, 2), dtype="<i2")
    out[:, 0] = np.trunc(y.real).astype(np.int64)
    out[:, 1] = np.trunc(y.imag).astype(np.int64)
    return out


def write_c16(path: str, y: np.ndarray) -> None:
    _trunc_i16_pairs(np.asarray(y)).tofile(path)


def write_taps(path: str, taps: np.ndarray) -> None:
    with open(path, "w") as f:
        for c in np.asarray(taps, dtype=np.complex128):
            f.write("%0.12f %0.12f\n" % (c.real, c.imag))


def resample_taps(p: int, q: int, cutoff: float | None = None) -> np.ndarray:
    """p * firls(2*10*max(p,q)+1, [0, 2fc, 2fc, 1], [1,1,0,0]) * kaiser(beta=5)."""
    pqmax = max(p, q)
    if cutoff is None:
        cutoff = 1 / 2 / pqmax
    order = 2 * 10 * pqmax + 1
    h = float(p) * signal.firls(order, [0, 2.0 * cutoff, 2.0 * cutoff, 1.0], [1.0, 1.0, 0.0, 0.0])
    return h * signal.windows.kaiser(order, beta=5)


def rollover_index(fs: float, shift: float) -> float:
    r = fs / abs(shift)
    while r < 1e5:
        r = r * 10.0
    return float(np.round(r))


# ---------------------------------------------------------------------------
def polyphase_vector(name, freq_shift, fs_in, fs_out, num_out, manifest):
    """generate_polyphase_test_vectors.ipynb (deterministic: a single tone)."""
    ratio = Fraction("%.12f" % (fs_out / fs_in)).limit_denominator()
    p, q = ratio.numerator, ratio.denominator
    if p != 1 or q != 1:
        taps = resample_taps(p, q)
    else:
        taps = resample_taps(p, q, cutoff=0.25)
    us_tone = (fs_in * 0.3) / 2
    ds_tone = (fs_out * 0.4) / 2
    tone = float(us_tone) if us_tone < ds_tone else float(ds_tone)
    if p == 1 and q == 1:
        tone = float(fs_in * 0.1)
    n_in_full = int(num_out * q / p)
    n_in = min(n_in_full, NKEEP)
    t = np.arange(0, n_in, dtype=np.float64)
    if abs(freq_shift) > 1:
        t = np.mod(t, rollover_index(fs_in, freq_shift))
    x = (1024 * np.exp(1j * 2 * np.pi * t * float(tone / fs_in))).astype(np.complex64)
    if p == 1 and q == 1:
        w = 2.0 * np.pi * (freq_shift / fs_in)
        y = x * (np.cos(w * t) + 1j * np.sin(w * t))
    else:
        y = signal.upfirdn(taps, x, p, q)
        n_valid = (n_in * p) // q  # outputs that depend on the kept prefix only
        y = y[:n_valid]
    write_c16(os.path.join(HERE, f"test_{name}_x.bin"), x)
    write_c16(os.path.join(HERE, f"test_{name}_y.bin"), y)
    write_taps(os.path.join(HERE, f"test_{name}.filter_coeffs.txt"), taps)
    manifest[name] = dict(kind="polyphase", freq_shift=freq_shift, fs_in=fs_in, fs_out=fs_out,
                          up=p, down=q, n_in=n_in, n_out=int(y.size), ntaps=int(taps.size))


def fir_vector(name, order, num_tones, fs, num_out, seed, manifest):
    """generate_fir_filter_test_vectors.ipynb (seeded here)."""
    rng = np.random.RandomState(seed)
    order = order + 1
    cutoff_ratio = 0.2
    cutoff = cutoff_ratio * fs
    taps = signal.firls(order, [0, cutoff_ratio, cutoff_ratio * 1.1, 1.0], [1.0, 1.0, 0.0, 0.0])
    taps = taps * signal.windows.kaiser(order, beta=5)
    n_in_full = num_out + order
    t = np.arange(0, n_in_full, dtype=np.float64)
    x = 2048 * np.exp(1j * 2 * np.pi * t * float(cutoff * 0.1 / fs))
    n_neg = rng.randint(0, num_tones)
    n_pos = num_tones - n_neg
    for _ in range(n_neg):
        f = rng.randint(-int(fs / 2), int(-cutoff * 1.1))
        x += (2048 * np.exp(1j * 2 * np.pi * t * float(f / fs))).astype(np.complex64)
    for _ in range(n_pos):
        f = rng.randint(int(cutoff * 1.1), int(fs / 2))
        x += (2048 * np.exp(1j * 2 * np.pi * t * float(f / fs))).astype(np.complex64)
    x += rng.normal(scale=np.sqrt(0.001 * fs / 2), size=t.shape)
    x = x[:NKEEP]
    y = signal.lfilter(taps, 1.0, x)
    write_c16(os.path.join(HERE, f"test_{name}_x.bin"), x)
    write_c16(os.path.join(HERE, f"test_{name}_y.bin"), y)
    write_taps(os.path.join(HERE, f"test_{name}.filter_coeffs.txt"), taps)
    manifest[name] = dict(kind="fir", fs_in=fs, n_in=int(x.size), ntaps=int(taps.size), seed=seed)


def _tone_mix(fs, n, seed, tone_draw):
    """Shared front half of the multi-channel notebooks: seeded tones,
    normalisation to +-2048, additive noise, int16 truncation."""
    np.random.seed(seed)
    t = np.arange(0, n, dtype=np.float64)
    x = 2048.0 * np.exp(1j * 2 * np.pi * t * float(fs / fs))
    tones = tone_draw()
    for f in tones:
        x += (2048.0 * np.exp(1j * 2 * np.pi * t * float(f / fs))).astype(np.complex64)
    m = max(np.abs(x.real).max(), np.abs(x.imag).max())
    x = x * (2048.0 / m)
    x += np.random.normal(scale=np.sqrt(0.001 * fs / 2), size=t.shape)
    x = x.astype(np.complex64)
    xi = np.trunc(x.real) + 1j * np.trunc(x.imag)
    return xi.astype(np.complex64), tones


def shift_block(x, fs, shift):
    r = rollover_index(fs, shift)
    t = np.mod(np.arange(0, x.size, dtype=np.float64), r).astype(np.float32)
    w = 2.0 * np.pi * (shift / fs)
    return x * (np.cos(w * t.astype(np.float64)) + 1j * np.sin(w * t.astype(np.float64)))


def multichan_shift_vector(name, num_tones, fs, num_out, seed, manifest):
    """generate_multi_chan_freq_shift_test_vectors.ipynb."""
    def draw():
        n_neg = np.random.randint(0, num_tones)
        n_pos = num_tones - n_neg
        out = []
        for _ in range(n_neg):
            out.append(int(np.random.randint(-int((fs / 2) / 100), 0) * 100))
        for _ in range(n_pos):
            out.append(int(np.random.randint(0, int((fs / 2) / 100)) * 100))
        return out

    x, tones = _tone_mix(fs, num_out, seed, draw)
    x = x[:NKEEP]
    write_c16(os.path.join(HERE, f"test_{name}_x.bin"), x)
    for f in tones:
        write_c16(os.path.join(HERE, f"test_{name}_y_shift_{f}_hz.bin"), shift_block(x, fs, f))
    manifest[name] = dict(kind="multichan_shift", fs_in=fs, n_in=int(x.size), shifts=tones, seed=seed)


def channelizer_vector(name, fs, rates, shifts, n_in_full, seed, manifest):
    """generate_multi_rate_channelizer_test_vectors.ipynb."""
    def draw():
        out = []
        for _ in range(10):
            out.append(int(np.random.randint(-int(fs / 2), 0)))
        for _ in range(10):
            out.append(int(np.random.randint(0, int(fs / 2))))
        return out

    x, _ = _tone_mix(fs, n_in_full, seed, draw)
    x = x[:NKEEP]
    write_c16(os.path.join(HERE, f"test_{name}_x.bin"), x)
    chans = []
    for rate, f in zip(rates, shifts):
        ratio = Fraction("%.12f" % (rate / fs)).limit_denominator()
        p, q = ratio.numerator, ratio.denominator
        taps = resample_taps(p, q)
        y = signal.upfirdn(taps, shift_block(x, fs, f), p, q)
        y = y[: (x.size * p) // q]
        write_taps(os.path.join(HERE, f"test_{name}_resamp_coeffs_{f}_hz.txt"), taps)
        write_c16(os.path.join(HERE, f"test_{name}_y_shift_{f}_hz.bin"), y)
        chans.append(dict(rate=rate, shift=f, up=p, down=q, ntaps=int(taps.size), n_out=int(y.size)))
    manifest[name] = dict(kind="channelizer", fs_in=fs, n_in=int(x.size), channels=chans, seed=seed)


def main():
    manifest = {}
    # generate_test_vectors.sh:17-114
    polyphase_vector("001", 100000, 1000000, 1000000, 1000000, manifest)
    polyphase_vector("003", -5000, 1000000, 1000000, 10000, manifest)
    polyphase_vector("004", 0, 1000000, 500000, 100000, manifest)
    polyphase_vector("005", 0, 1000000, 600000, 1000000, manifest)
    polyphase_vector("006", 0, 1000000, 2000000, 10000, manifest)
    polyphase_vector("007", 0, 1000000, 800000, 10000, manifest)
    polyphase_vector("008", 0, 1000000, 450000, 10000, manifest)
    polyphase_vector("009", 0, 1000000, 44000, 100000, manifest)
    # generate_test_vectors.sh:116-134
    fir_vector("010", 128, 4, 1000000, 100000, 4010, manifest)
    fir_vector("011", 128, 5, 1000000, 1000000, 4011, manifest)
    # generate_test_vectors.sh:136-164
    multichan_shift_vector("012", 2, 1000000, 1000000, 3758, manifest)
    multichan_shift_vector("013", 5, 1000000, 1000000, 6277, manifest)
    multichan_shift_vector("014", 10, 1000000, 1000000, 3999, manifest)
    # generate_test_vectors.sh:166-207
    channelizer_vector("015", 1000000, [100000, 250000], [-350000, 60000], 2000000, 2020, manifest)
    channelizer_vector("016", 2000000, [300000, 125000, 45000, 770000, 25000],
                       [-400000, -50000, 10000, 27000, 334000], 1000000, 2021, manifest)
    sh = [-5000000, -4000000, -3000000, -2000000, -1000000, 1000, 1000000, 2000000, 3000000, 4000000, 5000000]
    channelizer_vector("017", 30720000, [1920000] * 11, sh, 3072000, 2022, manifest)
    channelizer_vector("018", 30720000, [3686400] * 11, sh, 3072000, 2023, manifest)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
