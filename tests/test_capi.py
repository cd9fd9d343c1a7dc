"""CPU tests of the C ABI boundary (no GPU needed, no kernel launched).

* the in-tree library loads and exports every function include/fdsp_c.h declares;
* the host-only helpers (rat_approx, get_freq_shift_params, the closed-form
  output-count / state recurrence) agree with the oracle;
* handle-taking entry points reject NULL handles with a status code instead of
  crashing or exiting.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

from libfalcon_dsp_gb300 import _capi
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(fdsp_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = _capi.lib()
    names = _declared_functions()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding table covers the whole header
    assert set(names) <= set(_capi.SIGNATURES), set(names) - set(_capi.SIGNATURES)


def test_status_strings_and_version():
    lib = _capi.lib()
    assert lib.fdsp_status_string(0) == b"ok"
    assert lib.fdsp_status_string(-5) == b"output buffer too small"
    assert lib.fdsp_version() >= 100


def test_rat_approx_matches_oracle():
    r = np.random.default_rng(0)
    lib = _capi.lib()
    for _ in range(500):
        f = float(r.uniform(0.0005, 8.0))
        md = int(r.choice([2, 10, 100, 1024, 9999]))
        n, d = C.c_int64(), C.c_int64()
        assert lib.fdsp_rat_approx(f, md, C.byref(n), C.byref(d)) == 0
        assert (n.value, d.value) == O.rat_approx(f, md)
    assert lib.fdsp_rat_approx(0.5, 10, None, None) == -1


def test_freq_shift_params_match_oracle():
    r = np.random.default_rng(1)
    lib = _capi.lib()
    for _ in range(500):
        fs = int(r.integers(1000, 200_000_000))
        f = int(r.integers(-fs // 2, fs // 2)) or 1
        rr, w = C.c_uint32(), C.c_double()
        assert lib.fdsp_freq_shift_params(fs, f, C.byref(rr), C.byref(w)) == 0
        assert (rr.value, w.value) == O.freq_shift_params(fs, f)


def test_closed_form_index_recurrence_matches_loop():
    """fdsp_polyphase_advance (closed form) == the reference loop, state and
    count, over random rates, phases, offsets and block sizes."""
    r = np.random.default_rng(2)
    lib = _capi.lib()
    for _ in range(300):
        up = int(r.integers(1, 200))
        down = int(r.integers(1, 400))
        res = O.Resampler(up, down, np.ones(1, np.complex64))
        for n in r.integers(0, 3000, size=8):
            n = int(n)
            cnt, ph, xo = C.c_uint64(), C.c_uint32(), C.c_uint64()
            st = lib.fdsp_polyphase_advance(up, down, res.phase, res.xoffset, n, C.byref(cnt), C.byref(ph),
                                            C.byref(xo))
            assert st == 0
            assert cnt.value == res.loop_out_count(n)
            res.apply(np.zeros(n, np.complex64))
            assert (ph.value, xo.value) == (res.phase, res.xoffset)


def test_null_handles_are_rejected_not_fatal():
    lib = _capi.lib()
    n = C.c_uint64()
    assert lib.fdsp_channelizer_apply(None, None, 0, None, None, None, None) == -2
    assert lib.fdsp_channelizer_out_count(None, 5, C.byref(n)) == -2
    assert lib.fdsp_resampler_apply(None, None, 0, None, 0, None, None) == -2
    assert lib.fdsp_fir_apply(None, None, 0, None, None) == -2
    assert lib.fdsp_polar_apply(None, None, 0, None, None, None) == -2
    assert lib.fdsp_freq_shift_apply(None, None, 0, None, None) == -2
    assert lib.fdsp_channelizer_destroy(None) == -2
    # creation arguments are validated before any CUDA call
    h = C.c_void_p()
    assert lib.fdsp_channelizer_create(0, None, 0, C.byref(h)) == -1
    assert lib.fdsp_resampler_create(0, 1, None, 0, C.byref(h)) == -1
    assert lib.fdsp_polyphase_advance(0, 1, 0, 0, 10, None, None, None) == -1


def test_python_mirror_has_reference_class_names():
    import libfalcon_dsp_gb300 as F
    for name in ["falcon_dsp_multi_rate_channelizer_cuda", "falcon_dsp_polyphase_resampler_cuda",
                 "falcon_dsp_freq_shift_cuda", "falcon_dsp_fir_filter_cuda", "falcon_dsp_polar_discriminator_cuda"]:
        cls = getattr(F, name)
        for meth in ["apply", "reset_state"]:
            assert hasattr(cls, meth)
    assert hasattr(F.PolyphaseResamplerCuda, "needed_out_count")
    assert hasattr(F.PolyphaseResamplerCuda, "coeffs_per_phase")
