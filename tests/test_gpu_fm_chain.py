"""Long FIR + FM demodulation chain: 4095-tap lowpass as a 1/10 polyphase
resampler, then the polar discriminator, streamed in blocks.  The GPU chain
matches the oracle (resampler output <= 1e-5 relative RMS, discriminator
within 1e-4 rad absolute, counts exact) and recovers the FM message: the
audio keeps >= 20 dB SNR against a fit of the five message tones."""
import numpy as np
import pytest

import libfalcon_dsp_gb300 as F
from libfalcon_dsp_gb300.workloads import audio_snr_db, fm_chain
from oracle import oracle as O
from tests.golden_io import rel_rms

pytestmark = pytest.mark.gpu


def test_fm_chain_matches_oracle_and_recovers_audio():
    torch = pytest.importorskip("torch")
    n, blk = 1 << 18, 1 << 16
    x, fs, h, tones = fm_chain(n, seed=11)
    rs = F.PolyphaseResamplerCuda(1, 10, h)
    pd = F.PolarDiscriminatorCuda()
    ors, opd = O.Resampler(1, 10, h), O.Polar()
    xd = torch.from_numpy(x).cuda()
    audio, ref_audio = [], []
    for b in range(n // blk):
        y = rs.apply(xd[b * blk:(b + 1) * blk])
        a = pd.apply(y)
        torch.cuda.synchronize()
        yo = ors.apply(x[b * blk:(b + 1) * blk])
        ao = opd.apply(yo)
        assert y.numel() == yo.size and a.numel() == ao.size
        assert rel_rms(y.cpu().numpy(), yo) <= 1e-5
        assert np.max(np.abs(a.cpu().numpy() - ao)) <= 1e-4
        audio.append(a.cpu().numpy())
        ref_audio.append(ao)
    snr = audio_snr_db(np.concatenate(audio), fs / 10, tones)
    print(f"recovered audio SNR {snr:.1f} dB")
    assert snr >= 20.0
