"""Seeded synthetic workloads (CPU): the generators' stated properties."""
import numpy as np

from libfalcon_dsp_gb300.workloads import channelizer_8ch, qpsk_carriers, rrc_spectrum


def test_qpsk_workload_properties():
    """Unit-power carriers plus noise 20 dB down, centre frequencies inside
    +-4.5 MHz, and the 8 channels' NCOs on 8 of the carriers."""
    x, freqs = qpsk_carriers(1 << 16, 10e6, 16, 7, 4.5e6)
    p = np.mean(np.abs(x.astype(np.complex128) / 0.25) ** 2)
    assert abs(p - 16.01) < 0.05, p
    assert np.all(np.abs(freqs) <= 4.5e6)
    x8, fs, chans = channelizer_8ch(1 << 16, seed=2025)
    _, f16 = qpsk_carriers(1 << 16, 10e6, 16, 2025, 4.5e6)
    assert fs == 10_000_000 and len(chans) == 8
    for c in chans:
        assert -c["freq_shift_in_hz"] in set(int(round(f)) for f in f16)


def test_rrc_spectrum_squares_to_raised_cosine():
    """|H|^2 of the root-raised-cosine response is the raised-cosine
    response: Nyquist (folded copies at the symbol rate sum to 1)."""
    rs = 100e3
    f = np.linspace(0, rs, 1001)
    h2 = rrc_spectrum(f, rs) ** 2 + rrc_spectrum(f - rs, rs) ** 2
    assert np.allclose(h2, 1.0, atol=1e-12)
