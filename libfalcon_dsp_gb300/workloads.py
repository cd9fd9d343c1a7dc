"""Seeded synthetic workloads of the channelizer benchmarks.

No public dataset is involved: every input is generated from a seed with the
shapes, rates and value distributions of the benchmark configurations.

* ``channelizer_256``  2^26 complex<float> samples at 61.44 MSps (512 random
  tones, amplitudes U[0.1, 1], random phases, plus CN(0, 0.01^2) noise); 256
  output channels with decimation D in {8,16,25,40,64,125,160,320}, up-factor
  U in {1,2,3} and 12-64 taps per phase (Kaiser-windowed sinc, beta 8.6); each
  channel's NCO brings one tone to DC.
* ``resampler_1ch``    2^20 samples at 48 kHz (3 tones + noise), 147/160,
  Kaiser sinc beta 8.6 with 3528 taps (24 per phase).
* ``channelizer_8ch``  2^24 samples at 10 MSps: 16 QPSK carriers (random
  centre frequencies in +-4.5 MHz, symbol rates 25-250 kBd drawn as whole
  samples per symbol, root-raised-cosine pulses with roll-off 0.35, unit power
  each) plus AWGN 20 dB below each carrier's power; 8 channels with ratios
  1/40, 3/125, 1/80, 2/625, 1/50, 1/20, 3/200, 1/100, each shifting one
  carrier to DC, 16-48 taps per phase, streamed in 2^16-sample blocks.

Tones sit on the frequency grid of the signal length so a whole signal is one
inverse FFT of a sparse spectrum (fast at 2^26 samples).
"""
from __future__ import annotations

import math

import numpy as np
from scipy import signal as _sig

C3_DECIM = [8, 16, 25, 40, 64, 125, 160, 320]
C3_UP = [1, 2, 3]


def kaiser_lowpass(up: int, down: int, taps_per_phase: int, beta: float = 8.6) -> np.ndarray:
    """Anti-alias lowpass for an up/down resampler: U*T taps at the upsampled
    rate, cutoff at the narrower of the two Nyquist bands, passband gain U."""
    n = up * taps_per_phase
    h = _sig.firwin(n, 1.0 / max(up, down), window=("kaiser", beta))
    return (up * h).astype(np.complex64)


def _tones(rng, n, fs, tones, max_freq):
    lim = fs / 2 if max_freq is None else max_freq
    bins = rng.integers(-int(lim / fs * n), int(lim / fs * n), size=tones)
    amp = rng.uniform(0.1, 1.0, size=tones)
    ph = rng.uniform(0, 2 * np.pi, size=tones)
    return bins, amp, ph, bins * fs / n


def tone_freqs(n: int, fs: float, tones: int, seed: int, max_freq: float | None = None) -> np.ndarray:
    """Tone frequencies tone_signal(n, fs, tones, seed) would use, without
    synthesising the signal."""
    return _tones(np.random.default_rng(seed), n, fs, tones, max_freq)[3]


def tone_signal(n: int, fs: float, tones: int, seed: int, noise_sigma: float = 0.01, max_freq: float | None = None,
                device=None):
    """Sum of `tones` complex tones + complex Gaussian noise.  Returns
    (samples complex64, tone frequencies in Hz).  With `device` (a torch CUDA
    device) the signal is synthesised on the GPU and returned as a tensor."""
    rng = np.random.default_rng(seed)
    bins, amp, ph, freqs = _tones(rng, n, fs, tones, max_freq)
    if device is None:
        spec = np.zeros(n, np.complex128)
        np.add.at(spec, bins % n, amp * np.exp(1j * ph))
        x = np.fft.ifft(spec) * n
        x += (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * (noise_sigma / math.sqrt(2))
        return x.astype(np.complex64), freqs
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    spec = torch.zeros(n, dtype=torch.complex64, device=device)
    vals = torch.tensor(amp * np.exp(1j * ph), dtype=torch.complex64, device=device)
    spec.index_add_(0, torch.tensor(bins % n, device=device), vals)
    x = torch.fft.ifft(spec) * n
    noise = torch.randn(n, dtype=torch.complex64, device=device, generator=g) * noise_sigma
    return (x + noise).contiguous(), freqs


def channelizer_256_plan(fs: float = 61.44e6, tone_freqs=None, nch: int = 256, seed: int = 3) -> list[dict]:
    rng = np.random.default_rng(seed)
    chans = []
    for c in range(nch):
        d = int(rng.choice(C3_DECIM))
        u = int(rng.choice(C3_UP))
        g = math.gcd(u, d)
        u, d = u // g, d // g
        t = int(rng.integers(12, 65))
        if tone_freqs is not None and len(tone_freqs):
            f = -int(round(float(tone_freqs[int(rng.integers(0, len(tone_freqs)))])))
        else:
            f = int(rng.integers(-int(fs / 2), int(fs / 2)))
        chans.append(dict(output_sample_rate_in_sps=int(fs * u / d), freq_shift_in_hz=f, up_rate=u, down_rate=d,
                          coeffs=kaiser_lowpass(u, d, t)))
    return chans


def channelizer_256(n: int = 1 << 26, seed: int = 2026, device=None):
    fs = 61.44e6
    x, freqs = tone_signal(n, fs, 512, seed, device=device)
    return x, int(fs), channelizer_256_plan(fs, freqs, 256, seed + 1)


def channelizer_256_cpu_sample(n_sample: int, n: int = 1 << 26, seed: int = 2026):
    """A bounded CPU sample of channelizer_256: the same 256-channel plan (NCOs
    from the full-length signal's tones) over an n_sample-sample signal drawn
    from the same distribution."""
    fs = 61.44e6
    chans = channelizer_256_plan(fs, tone_freqs(n, fs, 512, seed), 256, seed + 1)
    x, _ = tone_signal(n_sample, fs, 512, seed)
    return x, int(fs), chans


def resampler_1ch(n: int = 1 << 20, seed: int = 2024, device=None):
    fs = 48000.0
    x, _ = tone_signal(n, fs, 3, seed, max_freq=20000.0, device=device)
    return x, 147, 160, kaiser_lowpass(147, 160, 24)


C2_RATIOS = [(1, 40), (3, 125), (1, 80), (2, 625), (1, 50), (1, 20), (3, 200), (1, 100)]


def rrc_spectrum(f: np.ndarray, symbol_rate: float, alpha: float = 0.35) -> np.ndarray:
    """Root-raised-cosine frequency response (1 in the passband) at
    frequencies f (Hz) for the given symbol rate and roll-off."""
    af = np.abs(f) / symbol_rate
    lo, hi = (1 - alpha) / 2, (1 + alpha) / 2
    h = np.zeros(f.shape)
    h[af <= lo] = 1.0
    mid = (af > lo) & (af < hi)
    h[mid] = np.sqrt(0.5 * (1 + np.cos(np.pi / alpha * (af[mid] - lo))))
    return h


def qpsk_carriers(n: int, fs: float, carriers: int, seed: int, max_freq: float, min_baud: float = 25e3,
                  max_baud: float = 250e3, alpha: float = 0.35, snr_db: float = 20.0):
    """Sum of `carriers` QPSK carriers with root-raised-cosine pulses plus
    AWGN, synthesised as one circular band-limited signal of n samples.

    A carrier carries nsym symbols over the n samples (symbol rate fs nsym / n,
    drawn in [min_baud, max_baud]); a band-limited pulse train with period n
    has at bin k the nsym-point DFT of the symbols at k mod nsym times the
    pulse's response at k fs / n, so each carrier is filled in over its own
    band only, scaled to unit power (Parseval) and moved to a centre frequency
    on the fs/n grid.  Noise power is 10^(-snr_db/10) relative to one carrier.
    Returns (x complex64, centre frequencies in Hz)."""
    from scipy import fft as sfft
    rng = np.random.default_rng(seed)
    spec = np.zeros(n, np.complex128)
    freqs = np.empty(carriers)
    const = np.exp(1j * np.pi * (np.arange(4) / 2 + 0.25))
    for c in range(carriers):
        nsym = int(rng.integers(int(np.ceil(min_baud * n / fs)), int(max_baud * n / fs) + 1))
        A = sfft.fft(const[rng.integers(0, 4, nsym)])
        kb = int((1 + alpha) / 2 * nsym)
        k = np.arange(-kb, kb + 1)
        S = A[k % nsym] * rrc_spectrum(k * (fs / n), fs * nsym / n, alpha)
        S *= np.sqrt(n * n / max(np.sum(np.abs(S) ** 2), 1e-300))  # unit mean power
        kc = int(rng.integers(-int(max_freq / fs * n) + kb, int(max_freq / fs * n) - kb + 1))
        freqs[c] = kc * fs / n
        np.add.at(spec, (k + kc) % n, S)
    x = sfft.ifft(spec, workers=-1)
    sigma = np.sqrt(10 ** (-snr_db / 10) / 2)
    x += sigma * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    return (0.25 * x).astype(np.complex64), freqs


def channelizer_8ch(n: int = 1 << 24, seed: int = 2025, device=None):
    fs = 10e6
    x, freqs = qpsk_carriers(n, fs, 16, seed, 4.5e6)
    if device is not None:
        import torch
        x = torch.from_numpy(x).to(device)
    rng = np.random.default_rng(seed + 1)
    chans = []
    for c, (u, d) in enumerate(C2_RATIOS):
        t = int(rng.integers(16, 49))
        chans.append(dict(output_sample_rate_in_sps=int(fs * u / d), freq_shift_in_hz=-int(round(freqs[c])),
                          up_rate=u, down_rate=d, coeffs=kaiser_lowpass(u, d, t)))
    return x, int(fs), chans


def algorithmic_bytes(n_in: int, n_out_total: int) -> int:
    """HBM bytes one apply must move: the complex64 input read once plus every
    complex64 output written once (taps, history and NCO state excluded)."""
    return 8 * n_in + 8 * n_out_total


def algorithmic_flops(chans: list[dict], n_out: list[int]) -> int:
    """4 flops per real tap x complex sample, T taps per phase per output."""
    tot = 0
    for ch, m in zip(chans, n_out):
        t = -(-len(ch["coeffs"]) // ch["up_rate"])
        tot += 4 * t * m
    return tot


FM_FS = 2.4e6


def fm_chain(n: int = 1 << 26, seed: int = 2027, device=None):
    """Long FIR + FM demodulation workload: a wideband FM signal at 2.4 MS/s
    whose message is 5 tones in 50 Hz - 15 kHz (peak deviation 75 kHz), AWGN at
    15 dB SNR; a 4095-tap Kaiser (beta 10) lowpass with a 100 kHz cutoff,
    used as a 1/10 polyphase resampler (FIR then decimate by 10), then the
    polar discriminator.  Returns (x, fs, taps, tone_freqs)."""
    rng = np.random.default_rng(seed)
    tones = np.sort(rng.uniform(50.0, 15000.0, 5))
    amps = rng.uniform(0.3, 1.0, 5)
    amps /= amps.sum()                       # peak |message| <= 1
    ph = rng.uniform(0, 2 * np.pi, 5)
    t = np.arange(n, dtype=np.float64) / FM_FS
    # phase = 2 pi * 75 kHz * integral(message)
    integ = np.zeros(n)
    for f, a, p in zip(tones, amps, ph):
        integ += a * (np.sin(2 * np.pi * f * t + p) - np.sin(p)) / (2 * np.pi * f)
    phase = 2 * np.pi * 75e3 * integ
    x = np.exp(1j * phase)
    sigma = np.sqrt(10 ** (-15 / 10) / 2)
    x = x + sigma * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    m = np.arange(4095) - 2047
    h = 2 * 100e3 / FM_FS * np.sinc(2 * 100e3 / FM_FS * m) * np.kaiser(4095, 10.0)
    x = x.astype(np.complex64)
    if device is not None:
        import torch
        x = torch.from_numpy(x).to(device)
    return x, int(FM_FS), h.astype(np.complex64), tones


FM_RADIO_FS = 1140000  # the input rate of the FM receiver's predefined filters


def fm_station(n: int, station_hz: int = -150000, seed: int = 2031, fs: int = FM_RADIO_FS, snr_db: float = 25.0):
    """A broadcast FM station at `station_hz` in a complex baseband capture at
    `fs` (a receiver tuned to it shifts by -station_hz): message of 3 tones in
    300 Hz - 12 kHz, 75 kHz peak deviation, plus a weaker station 550 kHz
    away and AWGN.  Returns (x complex64, tone_freqs)."""
    rng = np.random.default_rng(seed)
    tones = np.sort(rng.uniform(300.0, 12000.0, 3))
    amps = rng.uniform(0.3, 1.0, 3)
    amps /= amps.sum()
    ph = rng.uniform(0, 2 * np.pi, 3)
    t = np.arange(n, dtype=np.float64) / fs
    integ = np.zeros(n)
    for f, a, p in zip(tones, amps, ph):
        integ += a * (np.sin(2 * np.pi * f * t + p) - np.sin(p)) / (2 * np.pi * f)
    x = np.exp(1j * (2 * np.pi * 75e3 * integ + 2 * np.pi * station_hz * t))
    other = station_hz + 550000
    x += 0.3 * np.exp(1j * (2 * np.pi * 20e3 * np.sin(2 * np.pi * 700.0 * t) / 700.0 + 2 * np.pi * other * t))
    sigma = np.sqrt(10 ** (-snr_db / 10) / 2)
    x = x + sigma * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    return x.astype(np.complex64), tones


def audio_snr_db(audio: np.ndarray, fs_audio: float, tones, skip: int = 1024) -> float:
    """Recovered-audio SNR: least-squares fit of the known message tones (and
    a constant) to the demodulated audio, fit power over residual power."""
    y = np.asarray(audio, dtype=np.float64)[skip:]
    t = (np.arange(y.size) + skip) / fs_audio
    cols = [np.ones_like(t)]
    for f in tones:
        cols += [np.cos(2 * np.pi * f * t), np.sin(2 * np.pi * f * t)]
    A = np.stack(cols, axis=1)
    coef, *_ = np.linalg.lstsq(A, y, rcond=None)
    fit = A @ coef
    sig = np.sum((fit - coef[0]) ** 2)
    err = np.sum((y - fit) ** 2)
    return float(10 * np.log10(sig / err))
