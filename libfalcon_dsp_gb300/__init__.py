"""libfalcon_dsp_gb300 -- GB300-native implementation of libfalcon_dsp's
multi-rate channelizer path (NCO shift -> polyphase resampling -> FIR / FM
demodulation), exposed with the reference's class interface.

Each class mirrors one reference class (same name in the reference's
``falcon_dsp`` namespace, same ``initialize / apply / reset_state`` streaming
semantics) and calls the C ABI of ``_lib/libfalcon_dsp_gb300.so``:

==============================  ==================================================
Python class                    reference class (hdr/...)
==============================  ==================================================
``FreqShiftCuda``               transform/falcon_dsp_freq_shift_cuda.h:187-212
``PolyphaseResamplerCuda``      transform/falcon_dsp_polyphase_resampler_cuda.h:187-226
``MultiRateChannelizerCuda``    transform/falcon_dsp_multi_rate_channelizer_cuda.h:94-167
``FirFilterCuda``               transform/falcon_dsp_fir_filter_cuda.h:113-138
``PolarDiscriminatorCuda``      transform/falcon_dsp_polar_discriminator.h:97-114 (CPU-only there)
==============================  ==================================================

``apply`` accepts numpy arrays (host buffers; copied in and out like the
reference's std::vector apply) or CUDA ``torch.Tensor`` of complex64 (device
buffers; enqueued on the current torch stream, results returned as tensors).
A failing call raises ``FdspError``; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import FdspError, cf32, channel_cfg

__all__ = [
    "FdspError", "FreqShiftCuda", "PolyphaseResamplerCuda", "MultiRateChannelizerCuda", "FirFilterCuda",
    "PolarDiscriminatorCuda", "freq_shift_params", "rat_approx", "freq_shift_cuda", "resample_cuda",
    "upfirdn_cuda", "fir_filter_cuda", "polar_discriminator_cuda", "channel", "resample_static",
    "get_resample_fir_params", "design_resample_firls", "FILTER_TAPS_OPTIMAL", "REMEZ", "FIRLS",
    "FmDemodulatorCuda",
]

# filter_taps_e / filter_source_type_e (hdr/transform/falcon_dsp_predefined_fir_filter.h:63-78)
FILTER_TAPS_OPTIMAL = -1
REMEZ, FIRLS = 0, 1


def _is_tensor(x) -> bool:
    return type(x).__module__.startswith("torch") and hasattr(x, "is_cuda")


def _torch():
    import torch
    return torch


def _stream_handle() -> int:
    torch = _torch()
    return torch.cuda.current_stream().cuda_stream


def _c64(x) -> np.ndarray:
    a = np.asarray(x)
    if a.dtype == np.int16 and a.ndim == 2 and a.shape[-1] == 2:  # interleaved int16 pairs
        a = a[:, 0].astype(np.float32) + 1j * a[:, 1].astype(np.float32)
    return np.ascontiguousarray(a, dtype=np.complex64).reshape(-1)


def _ci16_host(x) -> np.ndarray | None:
    """Interleaved complex int16 (N x 2 int16 numpy array) as a contiguous
    array, else None."""
    if isinstance(x, np.ndarray) and x.dtype == np.int16 and x.ndim == 2 and x.shape[-1] == 2:
        return np.ascontiguousarray(x)
    return None


def _ci16_dev(x):
    """A CUDA int16 tensor of shape (N, 2) (interleaved I, Q), else None."""
    torch = _torch()
    if x.dtype == torch.int16 and x.dim() == 2 and x.shape[-1] == 2:
        return x.contiguous()
    return None


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data) if a.size else C.c_void_p(0)


def _tptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def _dev_c64(t):
    torch = _torch()
    if t.dtype != torch.complex64:
        raise TypeError("device input must be a complex64 CUDA tensor")
    return t.contiguous().reshape(-1)


def freq_shift_params(fs: int, f: int) -> tuple[int, float]:
    """get_freq_shift_params (src/transform/falcon_dsp_freq_shift.cc:194-235)."""
    r, w = C.c_uint32(), C.c_double()
    _capi.call("fdsp_freq_shift_params", fs, int(np.int32(f)), C.byref(r), C.byref(w))
    return r.value, w.value


def rat_approx(f: float, max_denom: int) -> tuple[int, int]:
    """rat_approx (src/utilities/falcon_dsp_utils.cc:231-294)."""
    n, d = C.c_int64(), C.c_int64()
    _capi.call("fdsp_rat_approx", float(f), int(max_denom), C.byref(n), C.byref(d))
    return n.value, d.value


def _filter_call(fn: str, *args):
    up, down, n = C.c_uint32(), C.c_uint32(), C.c_uint32()
    st = getattr(_capi.lib(), fn)(*args, C.byref(up), C.byref(down), None, 0, C.byref(n))
    if st == _capi.FDSP_ERR_NOT_FOUND:
        return None
    if st not in (_capi.FDSP_OK, _capi.FDSP_ERR_CAPACITY):
        _capi.check(fn, st)
    h = np.empty(n.value, np.complex64)
    _capi.call(fn, *args, C.byref(up), C.byref(down), h.ctypes.data, h.size, C.byref(n))
    return up.value, down.value, h


def get_resample_fir_params(input_sample_rate: int, output_sample_rate: int, taps: int = 64, source: int = REMEZ):
    """get_resample_fir_params (src/transform/falcon_dsp_fir_filter.cc:111-130):
    (up_rate, down_rate, complex64 coeffs) of the predefined anti-alias
    filter, or None where the reference returns false (no such entry).
    taps: 16/32/64/128/256 or FILTER_TAPS_OPTIMAL; source: REMEZ or FIRLS."""
    return _filter_call("fdsp_get_resample_fir_params", int(input_sample_rate), int(output_sample_rate), int(taps),
                        int(source))


def design_resample_firls(input_sample_rate: int, output_sample_rate: int, num_taps: int, beta: float = 5.0):
    """The FIRLS recipe of the predefined table for any rate pair (native
    designer): (up_rate, down_rate, complex64 coeffs)."""
    return _filter_call("fdsp_design_resample_firls", int(input_sample_rate), int(output_sample_rate),
                        int(num_taps), float(beta))


def channel(output_sample_rate_in_sps: int, freq_shift_in_hz: int, up_rate: int, down_rate: int,
            resample_filter_coeffs) -> dict:
    """multi_rate_channelizer_channel_s
    (hdr/transform/falcon_dsp_multi_rate_channelizer.h:70-77) as a dict."""
    return dict(output_sample_rate_in_sps=int(output_sample_rate_in_sps), freq_shift_in_hz=int(freq_shift_in_hz),
                up_rate=int(up_rate), down_rate=int(down_rate), coeffs=_c64(resample_filter_coeffs))


class _Handle:
    _destroy = ""

    def __init__(self):
        self._h = C.c_void_p(0)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                getattr(_capi.lib(), self._destroy)(h)
            except Exception:
                pass
            self._h = C.c_void_p(0)


class MultiRateChannelizerCuda(_Handle):
    """falcon_dsp_multi_rate_channelizer_cuda: per channel NCO shift, then
    polyphase up/down resampling, all channels fused in one launch."""
    _destroy = "fdsp_channelizer_destroy"

    def __init__(self, input_sample_rate: int | None = None, channels=None):
        super().__init__()
        self.initialized = False
        if input_sample_rate is not None and channels is not None:
            if not self.initialize(input_sample_rate, channels):
                raise FdspError("fdsp_channelizer_create", -1)

    def initialize(self, input_sample_rate: int, channels) -> bool:
        if self.initialized or input_sample_rate == 0 or len(channels) == 0:
            return False
        self._keep = []
        arr = (channel_cfg * len(channels))()
        for i, ch in enumerate(channels):
            taps = _c64(ch["coeffs"] if "coeffs" in ch else ch["resample_filter_coeffs"])
            self._keep.append(taps)
            arr[i].output_sample_rate_in_sps = int(ch.get("output_sample_rate_in_sps", 0))
            arr[i].freq_shift_in_hz = int(ch["freq_shift_in_hz"])
            arr[i].up_rate = int(ch["up_rate"])
            arr[i].down_rate = int(ch["down_rate"])
            arr[i].resample_filter_coeffs = taps.ctypes.data
            arr[i].num_coeffs = taps.size
        _capi.call("fdsp_channelizer_create", int(input_sample_rate), arr, len(channels), C.byref(self._h))
        self.num_channels = len(channels)
        self.initialized = True
        return True

    def out_count(self, n_in: int) -> list[int]:
        out = (C.c_uint64 * self.num_channels)()
        _capi.call("fdsp_channelizer_out_count", self._h, int(n_in), out)
        return list(out)

    PRECISION = {"fp32": 0, "fp16x3": 1, "bf16x3": 2}

    def set_precision(self, mode: str = "fp32") -> None:
        """'fp32' (SIMT FP32, default), or the tensor-core split-precision forms
        'fp16x3' / 'bf16x3' (hi+lo operands, full (hi+lo)(hi+lo) product,
        FP32 accumulation)."""
        _capi.call("fdsp_channelizer_set_precision", self._h, self.PRECISION[mode])

    def set_tc_split(self, max_split: int) -> None:
        """Largest row split (1..32, default 32) of the tensor-core form: a
        group's rows j = S i + b run as S output streams whose rows are
        S x down_rate apart, so one tile of input rows feeds S times the
        channel columns."""
        _capi.call("fdsp_channelizer_set_tc_split", self._h, int(max_split))

    def status(self, stream: int | None = None) -> None:
        """Synchronise `stream` and raise FdspError (FDSP_ERR_TIMEOUT) when a
        tensor-core kernel's bounded wait gave up since the last check."""
        s = _stream_handle() if stream is None else stream
        _capi.call("fdsp_channelizer_status", self._h, C.c_void_p(s))

    def set_tc_wait(self, max_polls: int = 1 << 20, withhold_copies: bool = False) -> None:
        """Polls before a tensor-core wait gives up; withhold_copies is a test
        hook that makes every wait run out."""
        _capi.call("fdsp_channelizer_set_tc_wait", self._h, int(max_polls), 1 if withhold_copies else 0)

    def set_tc_exact_all(self, on: bool = True) -> None:
        """Test hook: every output takes the tensor-core kernel's exact
        rotation pass (as slots whose row stride spans the NCO rollover do)."""
        _capi.call("fdsp_channelizer_set_tc_exact_all", self._h, 1 if on else 0)

    def kernel_launches(self) -> int:
        v = C.c_uint32()
        _capi.call("fdsp_channelizer_kernel_launches", self._h, C.byref(v))
        return v.value

    def set_profile(self, enable: bool = True) -> None:
        """Time every filter-bank launch of later applies with CUDA events on
        the apply's stream (applies launch directly, no graph); enabling
        restarts the record."""
        _capi.call("fdsp_channelizer_profile", self._h, 1 if enable else 0)

    def read_profile(self) -> tuple[float, int]:
        """(summed milliseconds, launches) of the timed filter-bank launches."""
        ms, n = C.c_double(), C.c_uint32()
        _capi.call("fdsp_channelizer_profile_read", self._h, C.byref(ms), C.byref(n))
        return ms.value, n.value

    def autotune(self, n_in: int, stream: int | None = None) -> list[dict]:
        """Time each decimation group on an n_in-sample block and keep the
        fastest FP32 tile height per group; resets the streaming state.
        Returns group_info()."""
        s = _stream_handle() if stream is None else stream
        _capi.call("fdsp_channelizer_autotune", self._h, int(n_in), C.c_void_p(s))
        return self.group_info()

    def set_graph(self, enable: bool = True) -> None:
        """Replay every later apply's launches as one CUDA graph (applies on
        the legacy default stream launch directly)."""
        _capi.call("fdsp_channelizer_set_graph", self._h, 1 if enable else 0)

    def graph_replays(self) -> int:
        v = C.c_uint32()
        _capi.call("fdsp_channelizer_graph_replays", self._h, C.byref(v))
        return v.value

    def group_info(self) -> list[dict]:
        n = C.c_uint32()
        _capi.call("fdsp_channelizer_num_groups", self._h, C.byref(n))
        out = []
        for g in range(n.value):
            d, q, tcf, sp = C.c_uint32(), C.c_uint32(), C.c_int(), C.c_uint32()
            _capi.call("fdsp_channelizer_group_info", self._h, g, C.byref(d), C.byref(q), C.byref(tcf))
            _capi.call("fdsp_channelizer_group_tc_split", self._h, g, C.byref(sp))
            out.append({"down_rate": d.value, "tile_rows": q.value, "tensor_core": bool(tcf.value),
                        "tc_split": sp.value})
        return out

    def tc_groups(self) -> int:
        """Decimation groups the last apply computed on the tensor-core kernel."""
        v = C.c_uint32()
        _capi.call("fdsp_channelizer_tc_groups", self._h, C.byref(v))
        return v.value

    def reset_state(self) -> None:
        _capi.call("fdsp_channelizer_reset", self._h)

    def apply(self, x, out=None, stream: int | None = None):
        """Complex64 input, or complex int16 (N x 2 int16, converted on the
        GPU inside the first kernel); one complex64 output per channel."""
        if _is_tensor(x):
            x16 = _ci16_dev(x)
            if x16 is not None:
                return self._apply_ci16_device(x16, out, stream)
            return self._apply_device(x, out, stream)
        x16 = _ci16_host(x)
        if x16 is not None:
            cnt = self.out_count(x16.shape[0])
            outs = [np.empty(max(c, 1), np.complex64) for c in cnt]
            optr = (C.c_void_p * self.num_channels)(*[o.ctypes.data for o in outs])
            n_out = (C.c_uint64 * self.num_channels)()
            _capi.call("fdsp_channelizer_apply_ci16_host", self._h, _ptr(x16), x16.shape[0], optr, None, n_out,
                       C.c_void_p(stream or 0))
            return [o[: n_out[i]] for i, o in enumerate(outs)]
        x = _c64(x)
        cnt = self.out_count(x.size)
        outs = [np.empty(max(c, 1), np.complex64) for c in cnt]
        optr = (C.c_void_p * self.num_channels)(*[o.ctypes.data for o in outs])
        n_out = (C.c_uint64 * self.num_channels)()
        _capi.call("fdsp_channelizer_apply_host", self._h, _ptr(x), x.size, optr, None, n_out,
                   C.c_void_p(stream or 0))
        return [o[: n_out[i]] for i, o in enumerate(outs)]

    def _apply_ci16_device(self, x16, out, stream):
        torch = _torch()
        n = x16.shape[0]
        if out is None:
            out = [torch.empty(max(c, 1), dtype=torch.complex64, device=x16.device) for c in self.out_count(n)]
        optr = (C.c_void_p * self.num_channels)(*[o.data_ptr() for o in out])
        cap = (C.c_uint64 * self.num_channels)(*[o.numel() for o in out])
        n_out = (C.c_uint64 * self.num_channels)()
        s = _stream_handle() if stream is None else stream
        _capi.call("fdsp_channelizer_apply_ci16", self._h, _tptr(x16), n, optr, cap, n_out, C.c_void_p(s))
        return [o[: n_out[i]] for i, o in enumerate(out)]

    def _apply_device(self, x, out, stream):
        torch = _torch()
        x = _dev_c64(x)
        if out is None:
            cnt = self.out_count(x.numel())
            out = [torch.empty(max(c, 1), dtype=torch.complex64, device=x.device) for c in cnt]
        # the ctypes pointer / capacity arrays are rebuilt only when the
        # caller's output buffers change (streaming loops reuse them)
        ptrs = tuple(o.data_ptr() for o in out)
        oc = getattr(self, "_out_cache", None)
        if oc is None or oc[0] != ptrs:
            n = self.num_channels
            oc = (ptrs, (C.c_void_p * n)(*ptrs), (C.c_uint64 * n)(*[o.numel() for o in out]), (C.c_uint64 * n)())
            self._out_cache = oc
        _, optr, cap, n_out = oc
        s = _stream_handle() if stream is None else stream
        st = _capi.lib().fdsp_channelizer_apply(self._h, x.data_ptr(), x.numel(), optr, cap, n_out, s)
        if st:
            _capi.check("fdsp_channelizer_apply", st)
        # views of the output buffers, reused while the counts repeat
        counts = tuple(n_out)
        vc = getattr(self, "_view_cache", None)
        if vc is None or vc[0] != ptrs or vc[1] != counts:
            vc = (ptrs, counts, [o[:k] for o, k in zip(out, counts)])
            self._view_cache = vc
        return list(vc[2])


class PolyphaseResamplerCuda(_Handle):
    """falcon_dsp_polyphase_resampler_cuda with the CPU class's streaming
    semantics (carried phase and xOffset; only the taps' real parts used)."""
    _destroy = "fdsp_resampler_destroy"

    def __init__(self, up_rate: int | None = None, down_rate: int | None = None, coeffs=None):
        super().__init__()
        self.initialized = False
        if up_rate is not None:
            if not self.initialize(up_rate, down_rate, coeffs):
                raise FdspError("fdsp_resampler_create", -1)

    def initialize(self, up_rate: int, down_rate: int, coeffs) -> bool:
        if self.initialized:
            return False
        taps = _c64(coeffs)
        _capi.call("fdsp_resampler_create", int(up_rate), int(down_rate), _ptr(taps), taps.size, C.byref(self._h))
        self.initialized = True
        return True

    def reset_state(self) -> None:
        _capi.call("fdsp_resampler_reset", self._h)

    def coeffs_per_phase(self) -> int:
        v = C.c_uint32()
        _capi.call("fdsp_resampler_coeffs_per_phase", self._h, C.byref(v))
        return v.value

    def needed_out_count(self, n_in: int) -> int:
        v = C.c_uint32()
        _capi.call("fdsp_resampler_needed_out_count", self._h, int(n_in), C.byref(v))
        return v.value

    def out_count(self, n_in: int) -> int:
        v = C.c_uint64()
        _capi.call("fdsp_resampler_out_count", self._h, int(n_in), C.byref(v))
        return v.value

    def state(self) -> tuple[int, int]:
        ph, xo = C.c_uint32(), C.c_uint64()
        _capi.call("fdsp_resampler_state", self._h, C.byref(ph), C.byref(xo))
        return ph.value, xo.value

    def set_precision(self, mode: str = "fp32") -> None:
        """'fp32' (default), or the tensor-core forms 'fp16x3' / 'bf16x3'."""
        _capi.call("fdsp_resampler_set_precision", self._h, MultiRateChannelizerCuda.PRECISION[mode])

    def tc_groups(self) -> int:
        """1 when the last apply ran on the tensor-core kernel."""
        v = C.c_uint32()
        _capi.call("fdsp_resampler_tc_groups", self._h, C.byref(v))
        return v.value

    def status(self, stream: int | None = None) -> None:
        s = _stream_handle() if stream is None else stream
        _capi.call("fdsp_resampler_status", self._h, C.c_void_p(s))

    def apply(self, x, out=None, stream: int | None = None):
        if _is_tensor(x):
            torch = _torch()
            x16 = _ci16_dev(x)
            fn = "fdsp_resampler_apply_ci16" if x16 is not None else "fdsp_resampler_apply"
            x = x16 if x16 is not None else _dev_c64(x)
            n_in = x.shape[0] if x16 is not None else x.numel()
            n = self.out_count(n_in)
            if out is None:
                out = torch.empty(max(n, 1), dtype=torch.complex64, device=x.device)
            got = C.c_uint64()
            s = _stream_handle() if stream is None else stream
            _capi.call(fn, self._h, _tptr(x), n_in, _tptr(out), out.numel(), C.byref(got), C.c_void_p(s))
            return out[: got.value]
        real_in = np.isrealobj(x) and np.asarray(x).dtype != np.int16
        xa = _c64(x)
        n = self.out_count(xa.size)
        y = np.empty(max(n, 1), np.complex64)
        got = C.c_uint64()
        _capi.call("fdsp_resampler_apply_host", self._h, _ptr(xa), xa.size, _ptr(y), y.size, C.byref(got),
                   C.c_void_p(stream or 0))
        y = y[: got.value]
        return y.real.copy() if real_in else y  # apply(vector<float>) overload


class FreqShiftCuda(_Handle):
    """falcon_dsp_freq_shift_cuda: one or many NCO shifts of one input."""
    _destroy = "fdsp_freq_shift_destroy"

    def __init__(self, input_sample_rate: int | None = None, shifts=None):
        super().__init__()
        self.initialized = False
        if input_sample_rate is not None:
            if not self.initialize(input_sample_rate, shifts):
                raise FdspError("fdsp_freq_shift_create", -1)

    def initialize(self, input_sample_rate: int, shifts) -> bool:
        if self.initialized:
            return False
        self.single = np.isscalar(shifts)
        sh = np.atleast_1d(np.asarray(shifts, dtype=np.int64)).astype(np.int32)
        arr = (C.c_int32 * sh.size)(*[int(v) for v in sh])
        _capi.call("fdsp_freq_shift_create", int(input_sample_rate), arr, sh.size, C.byref(self._h))
        self.num_channels = int(sh.size)
        self.initialized = True
        return True

    def reset_state(self) -> None:
        _capi.call("fdsp_freq_shift_reset", self._h)

    def counter(self, c: int = 0) -> int:
        v = C.c_uint64()
        _capi.call("fdsp_freq_shift_counter", self._h, c, C.byref(v))
        return v.value

    def apply(self, x, out=None, stream: int | None = None):
        """Complex64 in and out, or (the int16 overload) complex int16 (N x 2
        int16) in and out, converted on load and truncated on store."""
        if _is_tensor(x) and _ci16_dev(x) is not None:
            torch = _torch()
            x16 = _ci16_dev(x)
            n = x16.shape[0]
            if out is None:
                out = [torch.empty((max(n, 1), 2), dtype=torch.int16, device=x16.device)
                       for _ in range(self.num_channels)]
            optr = (C.c_void_p * self.num_channels)(*[o.data_ptr() for o in out])
            s = _stream_handle() if stream is None else stream
            _capi.call("fdsp_freq_shift_apply_ci16", self._h, _tptr(x16), n, optr, C.c_void_p(s))
            res = [o[:n] for o in out]
            return res[0] if self.single else res
        if not _is_tensor(x) and _ci16_host(x) is not None:
            x16 = _ci16_host(x)
            n = x16.shape[0]
            res = [np.empty((max(n, 1), 2), np.int16) for _ in range(self.num_channels)]
            optr = (C.c_void_p * self.num_channels)(*[o.ctypes.data for o in res])
            _capi.call("fdsp_freq_shift_apply_ci16_host", self._h, _ptr(x16), n, optr, C.c_void_p(stream or 0))
            res = [o[:n] for o in res]
            return res[0] if self.single else res
        if _is_tensor(x):
            torch = _torch()
            x = _dev_c64(x)
            if out is None:
                out = [torch.empty(max(x.numel(), 1), dtype=torch.complex64, device=x.device)
                       for _ in range(self.num_channels)]
            optr = (C.c_void_p * self.num_channels)(*[o.data_ptr() for o in out])
            s = _stream_handle() if stream is None else stream
            _capi.call("fdsp_freq_shift_apply", self._h, _tptr(x), x.numel(), optr, C.c_void_p(s))
            res = [o[: x.numel()] for o in out]
        else:
            xa = _c64(x)
            res = [np.empty(max(xa.size, 1), np.complex64) for _ in range(self.num_channels)]
            optr = (C.c_void_p * self.num_channels)(*[o.ctypes.data for o in res])
            _capi.call("fdsp_freq_shift_apply_host", self._h, _ptr(xa), xa.size, optr, C.c_void_p(stream or 0))
            res = [o[: xa.size] for o in res]
        return res[0] if self.single else res


class FirFilterCuda(_Handle):
    """falcon_dsp_fir_filter_cuda: complex-tap FIR, output length = input
    length, history carried across apply calls."""
    _destroy = "fdsp_fir_destroy"

    def __init__(self, coeffs):
        super().__init__()
        taps = _c64(coeffs)
        _capi.call("fdsp_fir_create", _ptr(taps), taps.size, C.byref(self._h))

    def reset_state(self) -> None:
        _capi.call("fdsp_fir_reset", self._h)

    def set_precision(self, mode: str = "fp32") -> None:
        """'fp32' (default) or the tensor-core forms 'fp16x3' / 'bf16x3'
        (Toeplitz product, (hi+lo)(hi+lo), FP32 accumulation; any number of
        taps).  The streaming state carries over."""
        _capi.call("fdsp_fir_set_precision", self._h, MultiRateChannelizerCuda.PRECISION[mode])

    def status(self, stream: int | None = None) -> None:
        s = _stream_handle() if stream is None else stream
        _capi.call("fdsp_fir_status", self._h, C.c_void_p(s))

    def tc_groups(self) -> int:
        v = C.c_uint32()
        _capi.call("fdsp_fir_tc_groups", self._h, C.byref(v))
        return v.value

    def apply(self, x, out=None, stream: int | None = None):
        """Complex64 in and out, or (the int16 overload, fir_filter.cc:151-175)
        complex int16 (N x 2 int16) in and out: converted inside the filter
        kernel, truncated toward zero on the way out."""
        if _is_tensor(x):
            torch = _torch()
            x16 = _ci16_dev(x)
            s = _stream_handle() if stream is None else stream
            if x16 is not None:
                n = x16.shape[0]
                if out is None:
                    out = torch.empty((max(n, 1), 2), dtype=torch.int16, device=x16.device)
                _capi.call("fdsp_fir_apply_ci16", self._h, _tptr(x16), n, _tptr(out), C.c_void_p(s))
                return out[:n]
            x = _dev_c64(x)
            if out is None:
                out = torch.empty(max(x.numel(), 1), dtype=torch.complex64, device=x.device)
            _capi.call("fdsp_fir_apply", self._h, _tptr(x), x.numel(), _tptr(out), C.c_void_p(s))
            return out[: x.numel()]
        x16 = _ci16_host(x)
        if x16 is not None:
            n = x16.shape[0]
            out16 = np.empty((max(n, 1), 2), np.int16)
            _capi.call("fdsp_fir_apply_ci16_host", self._h, _ptr(x16), n, _ptr(out16), C.c_void_p(stream or 0))
            return out16[:n]
        xa = _c64(x)
        y = np.empty(max(xa.size, 1), np.complex64)
        _capi.call("fdsp_fir_apply_host", self._h, _ptr(xa), xa.size, _ptr(y), C.c_void_p(stream or 0))
        return y[: xa.size]


class PolarDiscriminatorCuda(_Handle):
    """falcon_dsp_polar_discriminator on the GPU (the reference has only the
    CPU class): out[n] = arg(x[n] * conj(x[n-1]))."""
    _destroy = "fdsp_polar_destroy"

    def __init__(self):
        super().__init__()
        _capi.call("fdsp_polar_create", C.byref(self._h))

    def reset_state(self) -> None:
        _capi.call("fdsp_polar_reset", self._h)

    def apply(self, x, out=None, stream: int | None = None):
        if _is_tensor(x):
            torch = _torch()
            x = _dev_c64(x)
            if out is None:
                out = torch.empty(max(x.numel(), 1), dtype=torch.float32, device=x.device)
            got = C.c_uint64()
            s = _stream_handle() if stream is None else stream
            _capi.call("fdsp_polar_apply", self._h, _tptr(x), x.numel(), _tptr(out), C.byref(got), C.c_void_p(s))
            return out[: got.value]
        xa = _c64(x)
        y = np.empty(max(xa.size, 1), np.float32)
        got = C.c_uint64()
        _capi.call("fdsp_polar_apply_host", self._h, _ptr(xa), xa.size, _ptr(y), C.byref(got),
                   C.c_void_p(stream or 0))
        return y[: got.value]


class FmDemodulatorCuda(_Handle):
    """falcon_dsp_fm_demodulator_cuda (hdr/signals/falcon_dsp_fm_demod_cuda.h:
    83-104) with every stage on the GPU: channelizer to 228 kS/s (predefined
    REMEZ-64 filter), polar discriminator, de-emphasis, mono decimator to
    45.6 kS/s, rescale to int16 (x * 10000 / max |x| of the call)."""
    _destroy = "fdsp_fm_demod_destroy"
    AMERICAS_FM_DEEMPHASIS_TIME_CONSTANT = 75e-6
    EUROPE_ASIA_FM_DEEMPHASIS_TIME_CONSTANT = 50e-6
    FM_RADIO_SAMPLE_RATE_IN_SPS = 228000
    FM_RADIO_AUDIO_SAMPLE_RATE_IN_SPS = 45600

    def __init__(self, input_sample_rate: int | None = None, signal_offset_from_dc_in_hz: int = 0,
                 deemphasis_time_constant: float = 75e-6):
        super().__init__()
        self.initialized = False
        if input_sample_rate is not None:
            if not self.initialize(input_sample_rate, signal_offset_from_dc_in_hz, deemphasis_time_constant):
                raise FdspError("fdsp_fm_demod_create", _capi.FDSP_ERR_NOT_FOUND)

    def initialize(self, input_sample_rate: int, signal_offset_from_dc_in_hz: int,
                   deemphasis_time_constant: float = 75e-6) -> bool:
        """False where the reference's initialize() fails: a second call, an
        unsupported time constant, or no predefined filter for the rate."""
        if self.initialized:
            return False
        st = _capi.lib().fdsp_fm_demod_create(int(input_sample_rate), int(np.int32(signal_offset_from_dc_in_hz)),
                                              float(np.float32(deemphasis_time_constant)), C.byref(self._h))
        if st in (_capi.FDSP_ERR_NOT_FOUND, -1):
            return False
        _capi.check("fdsp_fm_demod_create", st)
        self.initialized = True
        return True

    def reset_state(self) -> None:
        _capi.call("fdsp_fm_demod_reset", self._h)

    def out_count(self, n_in: int) -> int:
        v = C.c_uint64()
        _capi.call("fdsp_fm_demod_out_count", self._h, int(n_in), C.byref(v))
        return v.value

    def demod_mono(self, x, out=None, stream: int | None = None):
        """int16 mono audio of one block (numpy in -> numpy out, or CUDA
        complex64 tensor in -> CUDA int16 tensor out)."""
        n = self.out_count(x.numel() if _is_tensor(x) else np.asarray(x).shape[0])
        got = C.c_uint64()
        if _is_tensor(x):
            torch = _torch()
            x = _dev_c64(x)
            if out is None:
                out = torch.empty(max(n, 1), dtype=torch.int16, device=x.device)
            s = _stream_handle() if stream is None else stream
            _capi.call("fdsp_fm_demod_apply", self._h, _tptr(x), x.numel(), _tptr(out), out.numel(), C.byref(got),
                       C.c_void_p(s))
            return out[: got.value]
        xa = _c64(x)
        y = np.empty(max(n, 1), np.int16)
        _capi.call("fdsp_fm_demod_apply_host", self._h, _ptr(xa), xa.size, _ptr(y), y.size, C.byref(got),
                   C.c_void_p(stream or 0))
        return y[: got.value]


# ---- free functions (one-shot), as in the reference headers ---------------
def freq_shift_cuda(input_sample_rate: int, x, shift):
    """freq_shift_cuda (src/transform/falcon_dsp_freq_shift_cuda.cu:90-119)."""
    return FreqShiftCuda(input_sample_rate, shift).apply(x)


RESAMPLE_STATIC_MAX_COEFFS = 8192


def resample_static(up_rate: int, down_rate: int, coeffs, x, out):
    """One-shot resampling of a CUDA complex64 tensor through
    fdsp_resample_static, the entry point that allocates nothing: the taps go
    into a fixed 64 KiB device array (at most RESAMPLE_STATIC_MAX_COEFFS
    taps) and ``out`` must be a preallocated CUDA complex64 tensor.  Equal to
    a fresh PolyphaseResamplerCuda(up_rate, down_rate, coeffs).apply(x).
    Calls that overlap in time share that array and race on it."""
    if not (_is_tensor(x) and _is_tensor(out)):
        raise TypeError("resample_static takes CUDA tensors for x and out")
    taps = _c64(coeffs)
    if taps.size > RESAMPLE_STATIC_MAX_COEFFS:
        raise ValueError(f"resample_static: {taps.size} taps exceed the fixed array of "
                         f"{RESAMPLE_STATIC_MAX_COEFFS}")
    x = _dev_c64(x)
    got = C.c_uint64()
    _capi.call("fdsp_resample_static", int(up_rate), int(down_rate), _ptr(taps), taps.size, _tptr(x), x.numel(),
               _tptr(out), out.numel(), C.byref(got), C.c_void_p(_stream_handle()))
    return out[: got.value]


def resample_cuda(input_sample_rate: int, x, coeffs, output_sample_rate: int):
    """resample_cuda (src/transform/falcon_dsp_resample_cuda.cu:124-135):
    up/down from rat_approx(fs_out/fs_in, 1024), then one apply."""
    up, down = rat_approx(float(output_sample_rate) / float(input_sample_rate), 1024)
    return PolyphaseResamplerCuda(up, down, coeffs).apply(x)


upfirdn_cuda = resample_cuda


def fir_filter_cuda(coeffs, x):
    """fir_filter_cuda (src/transform/falcon_dsp_fir_filter_cuda.cu:86-97)."""
    return FirFilterCuda(coeffs).apply(x)


def polar_discriminator_cuda(x):
    return PolarDiscriminatorCuda().apply(x)


# Reference spellings of the class names.
falcon_dsp_multi_rate_channelizer_cuda = MultiRateChannelizerCuda
falcon_dsp_polyphase_resampler_cuda = PolyphaseResamplerCuda
falcon_dsp_freq_shift_cuda = FreqShiftCuda
falcon_dsp_fir_filter_cuda = FirFilterCuda
falcon_dsp_polar_discriminator_cuda = PolarDiscriminatorCuda
