"""ctypes bindings for the parity oracle (test infrastructure only).

Two CPU implementations of libfalcon_dsp's channelizer path are exposed with
the same Python surface:

* ``port``      -- oracle/fdsp_oracle.c, a C restatement of the reference's
                   CPU algorithms (FP32 flavour mirrors the reference data
                   path; FP64 flavour is the precision oracle).
* ``reference`` -- oracle/_ref/libfdsp_ref.so, the reference's own CPU classes
                   compiled in place with oracle/ref_shim.cc.  Only present
                   where the reference checkout was available at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs import this module, and only as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libfdsp_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfdsp_ref.so")

_vp = C.c_void_p
_u32, _i32, _u64, _i64, _dbl = C.c_uint32, C.c_int32, C.c_uint64, C.c_int64, C.c_double
_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)


def build(with_reference: bool | None = None) -> None:
    """Compile the C restatement and, when FDSP_REF_ROOT names a reference
    checkout, the reference's own CPU sources (oracle/_ref).  Without
    FDSP_REF_ROOT the reference build is skipped; the committed fixtures
    under tests/golden/ (made from that build) still pin the restatement."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref_root = os.environ.get("FDSP_REF_ROOT")
    if with_reference is None:
        with_reference = bool(ref_root)
    if with_reference:
        if not ref_root or not os.path.isdir(os.path.join(ref_root, "src", "transform")):
            raise RuntimeError("FDSP_REF_ROOT must name a libfalcon_dsp checkout (with src/transform) "
                               "to build the reference's CPU sources")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={ref_root}"], check=True)


def _f32p(a: np.ndarray):
    return a.ctypes.data_as(_fp)


def _f64p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def as_c64(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.complex64))


def as_c128(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.complex128))


# --------------------------------------------------------------------------
# C restatement
# --------------------------------------------------------------------------
_port = None


def port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build(with_reference=False)
        lib = C.CDLL(PORT_SO)
        sig = {
            "orc_freq_shift_params": (None, [_u32, _i32, C.POINTER(_u32), C.POINTER(_dbl)]),
            "orc_nco_new": (_vp, [_u32, _i32]),
            "orc_nco_free": (None, [_vp]),
            "orc_nco_reset": (None, [_vp]),
            "orc_nco_rollover": (_u32, [_vp]),
            "orc_nco_omega": (_dbl, [_vp]),
            "orc_nco_counter": (_u64, [_vp]),
            "orc_nco_apply_f32": (None, [_vp, _fp, _u64, _fp]),
            "orc_nco_apply_f64": (None, [_vp, _dp, _u64, _dp]),
            "orc_resampler_new": (_vp, [_u32, _u32, _fp, _u32]),
            "orc_resampler_free": (None, [_vp]),
            "orc_resampler_reset": (None, [_vp]),
            "orc_resampler_cpp": (_u32, [_vp]),
            "orc_resampler_phase": (_u32, [_vp]),
            "orc_resampler_xoffset": (_u32, [_vp]),
            "orc_resampler_needed_out_count": (_u32, [_vp, _u32]),
            "orc_resampler_loop_out_count": (_u64, [_vp, _u64]),
            "orc_resampler_apply_f32": (_u64, [_vp, _fp, _u64, _fp, _u64]),
            "orc_resampler_apply_f64": (_u64, [_vp, _dp, _u64, _dp, _u64]),
            "orc_fir_new": (_vp, [_fp, _u32]),
            "orc_fir_free": (None, [_vp]),
            "orc_fir_reset": (None, [_vp]),
            "orc_fir_apply_f32": (_u64, [_vp, _fp, _u64, _fp]),
            "orc_polar_new": (_vp, []),
            "orc_polar_free": (None, [_vp]),
            "orc_polar_reset": (None, [_vp]),
            "orc_polar_apply_f32": (_u64, [_vp, _fp, _u64, _fp]),
            "orc_rat_approx": (None, [_dbl, _i64, C.POINTER(_i64), C.POINTER(_i64)]),
            "orc_iir_new": (_vp, [_fp, _u32, _fp, _u32]),
            "orc_iir_free": (None, [_vp]),
            "orc_iir_reset": (None, [_vp]),
            "orc_iir_apply_f32": (_u64, [_vp, _fp, _u64, _fp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _port = lib
    return _port


def freq_shift_params(fs: int, f: int) -> tuple[int, float]:
    r, w = _u32(), _dbl()
    port_lib().orc_freq_shift_params(fs, f, C.byref(r), C.byref(w))
    return r.value, w.value


def rat_approx(f: float, md: int) -> tuple[int, int]:
    n, d = _i64(), _i64()
    port_lib().orc_rat_approx(f, md, C.byref(n), C.byref(d))
    return n.value, d.value


class NCO:
    """falcon_dsp_freq_shift (CPU) restated; f32 and f64 flavours."""

    def __init__(self, fs: int, f: int):
        self._lib = port_lib()
        self._h = self._lib.orc_nco_new(fs, int(np.int32(f)))

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_nco_free(self._h)
            self._h = None

    @property
    def rollover(self) -> int:
        return self._lib.orc_nco_rollover(self._h)

    @property
    def omega(self) -> float:
        return self._lib.orc_nco_omega(self._h)

    @property
    def counter(self) -> int:
        return self._lib.orc_nco_counter(self._h)

    def reset_state(self):
        self._lib.orc_nco_reset(self._h)

    def apply(self, x) -> np.ndarray:
        x = as_c64(x)
        y = np.empty_like(x)
        self._lib.orc_nco_apply_f32(self._h, _f32p(x.view(np.float32)), x.size, _f32p(y.view(np.float32)))
        return y

    def apply64(self, x) -> np.ndarray:
        x = as_c128(x)
        y = np.empty_like(x)
        self._lib.orc_nco_apply_f64(self._h, _f64p(x.view(np.float64)), x.size, _f64p(y.view(np.float64)))
        return y


class Resampler:
    """falcon_dsp_polyphase_resampler (CPU) restated; f32 and f64 flavours
    (keep one object per flavour: each carries its own streaming state)."""

    def __init__(self, up: int, down: int, coeffs):
        self._lib = port_lib()
        c = as_c64(coeffs)
        self._keep = c
        self._h = self._lib.orc_resampler_new(up, down, _f32p(c.view(np.float32)), c.size)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_resampler_free(self._h)
            self._h = None

    @property
    def coeffs_per_phase(self) -> int:
        return self._lib.orc_resampler_cpp(self._h)

    @property
    def phase(self) -> int:
        return self._lib.orc_resampler_phase(self._h)

    @property
    def xoffset(self) -> int:
        return self._lib.orc_resampler_xoffset(self._h)

    def reset_state(self):
        self._lib.orc_resampler_reset(self._h)

    def needed_out_count(self, n: int) -> int:
        return self._lib.orc_resampler_needed_out_count(self._h, n)

    def loop_out_count(self, n: int) -> int:
        return self._lib.orc_resampler_loop_out_count(self._h, n)

    def apply(self, x) -> np.ndarray:
        x = as_c64(x)
        n = self.loop_out_count(x.size)
        y = np.empty(max(n, 1), dtype=np.complex64)
        got = self._lib.orc_resampler_apply_f32(self._h, _f32p(x.view(np.float32)), x.size,
                                                _f32p(y.view(np.float32)), n)
        assert got == n
        return y[:n]

    def apply64(self, x) -> np.ndarray:
        x = as_c128(x)
        n = self.loop_out_count(x.size)
        y = np.empty(max(n, 1), dtype=np.complex128)
        got = self._lib.orc_resampler_apply_f64(self._h, _f64p(x.view(np.float64)), x.size,
                                                _f64p(y.view(np.float64)), n)
        assert got == n
        return y[:n]


class Channelizer:
    """falcon_dsp_multi_rate_channelizer (CPU) restated: per channel an NCO
    then a polyphase resampler (multi_rate_channelizer.cc:146-164)."""

    def __init__(self, fs: int, channels, precision: str = "f32"):
        self.precision = precision
        self.nco = []
        self.rs = []
        for ch in channels:
            self.nco.append(NCO(fs, int(np.int32(ch["freq_shift_in_hz"]))))
            self.rs.append(Resampler(ch["up_rate"], ch["down_rate"], ch["coeffs"]))

    def reset_state(self):
        for n, r in zip(self.nco, self.rs):
            n.reset_state()
            r.reset_state()

    def apply(self, x) -> list[np.ndarray]:
        out = []
        for n, r in zip(self.nco, self.rs):
            if self.precision == "f64":
                out.append(r.apply64(n.apply64(x)))
            else:
                out.append(r.apply(n.apply(x)))
        return out


class FIR:
    """falcon_dsp_fir_filter (CPU) restated (complex taps)."""

    def __init__(self, coeffs):
        self._lib = port_lib()
        c = as_c64(coeffs)
        self._h = self._lib.orc_fir_new(_f32p(c.view(np.float32)), c.size)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_fir_free(self._h)
            self._h = None

    def reset_state(self):
        self._lib.orc_fir_reset(self._h)

    def apply(self, x) -> np.ndarray:
        x = as_c64(x)
        y = np.empty_like(x)
        self._lib.orc_fir_apply_f32(self._h, _f32p(x.view(np.float32)), x.size, _f32p(y.view(np.float32)))
        return y


class Polar:
    """falcon_dsp_polar_discriminator (CPU) restated."""

    def __init__(self):
        self._lib = port_lib()
        self._h = self._lib.orc_polar_new()

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_polar_free(self._h)
            self._h = None

    def reset_state(self):
        self._lib.orc_polar_reset(self._h)

    def apply(self, x) -> np.ndarray:
        x = as_c64(x)
        y = np.empty(max(x.size, 1), dtype=np.float32)
        n = self._lib.orc_polar_apply_f32(self._h, _f32p(x.view(np.float32)), x.size, _f32p(y))
        return y[:n]


class IIR:
    """falcon_dsp_iir_filter (src/transform/falcon_dsp_iir_filter.cc) restated:
    complex<float> direct form, b/a normalised by a[0]."""

    def __init__(self, b, a):
        self._lib = port_lib()
        b, a = as_c64(b), as_c64(a)
        self._h = self._lib.orc_iir_new(_f32p(b.view(np.float32)), b.size, _f32p(a.view(np.float32)), a.size)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_iir_free(self._h)
            self._h = None

    def reset_state(self):
        self._lib.orc_iir_reset(self._h)

    def apply(self, x) -> np.ndarray:
        x = as_c64(x)
        y = np.empty(max(x.size, 1), dtype=np.complex64)
        n = self._lib.orc_iir_apply_f32(self._h, _f32p(x.view(np.float32)), x.size, _f32p(y.view(np.float32)))
        return y[:n]


# de-emphasis taps (b0, a1) of src/signals/falcon_dsp_fm_demod.cc:119-133
DEEMPHASIS = {75e-6: (0.064493014968382223, -0.93550698503161778),
              50e-6: (0.095162581964040482, -0.90483741803595952)}


class FmDemod:
    """falcon_dsp_fm_demodulator::demod_mono (src/signals/falcon_dsp_fm_demod.cc)
    restated from the oracle's own stages: NCO + isolation resampler, polar
    discriminator, de-emphasis IIR, mono resampler, then x * (10000 / max |x|)
    truncated to int16.  The two resampling filters are given (the predefined
    REMEZ-64 entries of the reference's table)."""

    def __init__(self, fs: int, offset_hz: int, iso, mono, tau: float = 75e-6):
        up, down, h = iso
        mup, mdown, mh = mono
        self.chan = Channelizer(fs, [dict(freq_shift_in_hz=int(offset_hz), up_rate=up, down_rate=down, coeffs=h)])
        self.polar = Polar()
        b0, a1 = DEEMPHASIS[tau]
        self.iir = IIR(np.array([b0], np.complex64), np.array([1.0, a1], np.complex64))
        self.mono = Resampler(mup, mdown, mh)

    def reset_state(self):
        self.chan.reset_state()
        self.polar.reset_state()
        self.iir.reset_state()
        self.mono.reset_state()

    def demod_mono(self, x) -> np.ndarray:
        iso = self.chan.apply(x)[0]
        pol = self.polar.apply(iso)
        emph = self.iir.apply(pol.astype(np.complex64)).real.astype(np.float32) if pol.size else pol
        m = self.mono.apply(emph.astype(np.complex64)).real.astype(np.float32) if emph.size else emph
        if m.size == 0:
            return np.zeros(0, np.int16)
        amax = np.float32(np.max(np.abs(m)))
        scale = np.float32(10000.0 / float(amax))
        return np.trunc(m * scale).astype(np.int16)


# --------------------------------------------------------------------------
# The reference's own CPU classes (oracle/_ref), when built
# --------------------------------------------------------------------------
_ref = None


def have_reference() -> bool:
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        lib = C.CDLL(REF_SO)
        sig = {
            "ref_freq_shift_new": (_vp, [_u32, _i32]),
            "ref_freq_shift_free": (None, [_vp]),
            "ref_freq_shift_reset": (None, [_vp]),
            "ref_freq_shift_apply": (_u64, [_vp, _fp, _u64, _fp]),
            "ref_freq_shift_params": (None, [_u32, _i32, C.POINTER(_u32), C.POINTER(_dbl)]),
            "ref_resampler_new": (_vp, [_u32, _u32, _fp, _u32]),
            "ref_resampler_free": (None, [_vp]),
            "ref_resampler_reset": (None, [_vp]),
            "ref_resampler_needed_out_count": (_u32, [_vp, _u32]),
            "ref_resampler_apply": (_u64, [_vp, _fp, _u64, _fp, _u64]),
            "ref_channelizer_new": (_vp, [_u32, _u32, C.POINTER(_u32), C.POINTER(_i64), C.POINTER(_u32),
                                          C.POINTER(_u32), C.POINTER(_fp), C.POINTER(_u32)]),
            "ref_channelizer_free": (None, [_vp]),
            "ref_channelizer_reset": (None, [_vp]),
            "ref_channelizer_apply": (C.c_int, [_vp, _fp, _u64, C.POINTER(_fp), C.POINTER(_u64),
                                                C.POINTER(_u64), _u32]),
            "ref_fir_new": (_vp, [_fp, _u32]),
            "ref_fir_free": (None, [_vp]),
            "ref_fir_reset": (None, [_vp]),
            "ref_fir_apply": (_u64, [_vp, _fp, _u64, _fp]),
            "ref_fir_apply_i16": (_u64, [_vp, C.POINTER(C.c_int16), _u64, C.POINTER(C.c_int16)]),
            "ref_polar_new": (_vp, []),
            "ref_polar_free": (None, [_vp]),
            "ref_polar_reset": (None, [_vp]),
            "ref_polar_apply": (_u64, [_vp, _fp, _u64, _fp]),
            "ref_rat_approx": (None, [_dbl, _i64, C.POINTER(_i64), C.POINTER(_i64)]),
            "ref_get_resample_fir_params": (_u32, [_u32, _u32, C.c_int32, _u32, C.POINTER(_u32), C.POINTER(_u32),
                                                   _fp, _u32]),
            "ref_iir_new": (_vp, [_fp, _u32, _fp, _u32]),
            "ref_iir_free": (None, [_vp]),
            "ref_iir_reset": (None, [_vp]),
            "ref_iir_apply": (_u64, [_vp, _fp, _u64, _fp]),
            "ref_fm_new": (_vp, [_u32, _i32, C.c_float]),
            "ref_fm_free": (None, [_vp]),
            "ref_fm_reset": (None, [_vp]),
            "ref_fm_demod_mono": (_u64, [_vp, _fp, _u64, C.POINTER(C.c_int16), _u64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _ref = lib
    return _ref


def ref_get_resample_fir_params(in_sps: int, out_sps: int, taps: int, source: int):
    """(up, down, float32 taps) from the reference's own table, or None."""
    up, down = _u32(), _u32()
    buf = np.zeros(4096, np.float32)
    n = ref_lib().ref_get_resample_fir_params(in_sps, out_sps, taps, source, C.byref(up), C.byref(down),
                                              _f32p(buf), buf.size)
    if n == 0:
        return None
    return up.value, down.value, buf[:n].copy()


class RefIIR:
    def __init__(self, b, a):
        b, a = as_c64(b), as_c64(a)
        self._h = ref_lib().ref_iir_new(_f32p(b.view(np.float32)), b.size, _f32p(a.view(np.float32)), a.size)

    def __del__(self):
        if getattr(self, "_h", None):
            ref_lib().ref_iir_free(self._h)
            self._h = None

    def reset_state(self):
        ref_lib().ref_iir_reset(self._h)

    def apply(self, x):
        x = as_c64(x)
        y = np.empty(max(x.size, 1), np.complex64)
        n = ref_lib().ref_iir_apply(self._h, _f32p(x.view(np.float32)), x.size, _f32p(y.view(np.float32)))
        return y[:n]


class RefFmDemod:
    """The reference's own CPU falcon_dsp_fm_demodulator (None handle when
    its initialize() fails)."""

    def __init__(self, fs, offset_hz, tau=75e-6):
        self._h = ref_lib().ref_fm_new(int(fs), int(offset_hz), float(tau))

    def __del__(self):
        if getattr(self, "_h", None):
            ref_lib().ref_fm_free(self._h)
            self._h = None

    def reset_state(self):
        ref_lib().ref_fm_reset(self._h)

    def demod_mono(self, x):
        x = as_c64(x)
        y = np.empty(x.size + 16, np.int16)
        n = ref_lib().ref_fm_demod_mono(self._h, _f32p(x.view(np.float32)), x.size,
                                        y.ctypes.data_as(C.POINTER(C.c_int16)), y.size)
        return y[:n].copy()


class RefResampler:
    def __init__(self, up, down, coeffs):
        self._lib = ref_lib()
        c = as_c64(coeffs)
        self._h = self._lib.ref_resampler_new(up, down, _f32p(c.view(np.float32)), c.size)
        self._port = Resampler(up, down, c)  # index bookkeeping for the output size

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.ref_resampler_free(self._h)
            self._h = None

    def reset_state(self):
        self._lib.ref_resampler_reset(self._h)
        self._port.reset_state()

    def needed_out_count(self, n):
        return self._lib.ref_resampler_needed_out_count(self._h, n)

    def apply(self, x):
        x = as_c64(x)
        cap = self._port.loop_out_count(x.size)
        y = np.empty(max(cap, 1), dtype=np.complex64)
        n = self._lib.ref_resampler_apply(self._h, _f32p(x.view(np.float32)), x.size,
                                          _f32p(y.view(np.float32)), cap)
        # keep the port's (phase, xoffset) in step for the next size query
        self._port.apply(x)
        assert n == cap, (n, cap)
        return y[:n]


class RefChannelizer:
    """The reference's falcon_dsp_multi_rate_channelizer (CPU)."""

    def __init__(self, fs, channels):
        self._lib = ref_lib()
        n = len(channels)
        self.n = n
        self._coeffs = [as_c64(ch["coeffs"]) for ch in channels]
        rate = (_u32 * n)(*[int(ch.get("output_sample_rate_in_sps", 0)) for ch in channels])
        shift = (_i64 * n)(*[int(ch["freq_shift_in_hz"]) for ch in channels])
        up = (_u32 * n)(*[int(ch["up_rate"]) for ch in channels])
        dn = (_u32 * n)(*[int(ch["down_rate"]) for ch in channels])
        cp = (_fp * n)(*[_f32p(c.view(np.float32)) for c in self._coeffs])
        nc = (_u32 * n)(*[c.size for c in self._coeffs])
        self._h = self._lib.ref_channelizer_new(fs, n, rate, shift, up, dn, cp, nc)
        # (phase, xoffset) bookkeeping to size the outputs
        self._count = [Resampler(ch["up_rate"], ch["down_rate"], np.ones(1, np.complex64)) for ch in channels]

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.ref_channelizer_free(self._h)
            self._h = None

    def reset_state(self):
        self._lib.ref_channelizer_reset(self._h)
        for r in self._count:
            r.reset_state()

    def apply(self, x):
        x = as_c64(x)
        caps = [r.loop_out_count(x.size) for r in self._count]
        outs = [np.empty(max(c, 1), np.complex64) for c in caps]
        op = (_fp * self.n)(*[_f32p(o.view(np.float32)) for o in outs])
        cap = (_u64 * self.n)(*caps)
        cnt = (_u64 * self.n)()
        self._lib.ref_channelizer_apply(self._h, _f32p(x.view(np.float32)), x.size, op, cap, cnt, self.n)
        for r in self._count:
            r.apply(np.zeros(x.size, np.complex64))
        return [o[: cnt[i]] for i, o in enumerate(outs)]
