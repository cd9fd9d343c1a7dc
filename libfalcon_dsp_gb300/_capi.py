"""ctypes bindings of the C ABI declared in include/fdsp_c.h.

The shared library is built in-tree (libfalcon_dsp_gb300/_lib).  If it is
missing this module raises at import of `lib()`: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libfalcon_dsp_gb300.so")

FDSP_OK = 0
FDSP_ERR_CAPACITY = -5
STATUS = {
    0: "FDSP_OK",
    -1: "FDSP_ERR_INVALID_ARG",
    -2: "FDSP_ERR_NOT_INITIALIZED",
    -3: "FDSP_ERR_ALLOC",
    -4: "FDSP_ERR_CUDA",
    -5: "FDSP_ERR_CAPACITY",
    -6: "FDSP_ERR_UNSUPPORTED",
    -7: "FDSP_ERR_NO_DEVICE",
    -8: "FDSP_ERR_NOT_FOUND",
    -9: "FDSP_ERR_TIMEOUT",
}
FDSP_ERR_NOT_FOUND = -8
FDSP_ERR_TIMEOUT = -9


class cf32(C.Structure):
    _fields_ = [("re", C.c_float), ("im", C.c_float)]


class channel_cfg(C.Structure):
    """fdsp_channel_cfg == multi_rate_channelizer_channel_s (+ tap pointer/count)."""
    _fields_ = [
        ("output_sample_rate_in_sps", C.c_uint32),
        ("freq_shift_in_hz", C.c_int64),
        ("up_rate", C.c_uint32),
        ("down_rate", C.c_uint32),
        ("resample_filter_coeffs", C.c_void_p),
        ("num_coeffs", C.c_uint32),
    ]


class FdspError(RuntimeError):
    def __init__(self, fn: str, status: int, cuda_err: int = 0):
        msg = f"{fn} failed: {STATUS.get(status, status)}"
        if status == -4:
            msg += f" (cudaError {cuda_err})"
        super().__init__(msg)
        self.status = status


_vp = C.c_void_p
_pp = C.POINTER(C.c_void_p)
_u32, _i32, _u64, _i64, _dbl = C.c_uint32, C.c_int32, C.c_uint64, C.c_int64, C.c_double
_pu32, _pu64, _pi64, _pdbl = C.POINTER(_u32), C.POINTER(_u64), C.POINTER(_i64), C.POINTER(_dbl)

# name -> argtypes (all return int status unless listed in _RES)
SIGNATURES = {
    "fdsp_status_string": [C.c_int],
    "fdsp_last_cuda_error": [],
    "fdsp_version": [],
    "fdsp_freq_shift_params": [_u32, _i32, _pu32, _pdbl],
    "fdsp_rat_approx": [_dbl, _i64, _pi64, _pi64],
    "fdsp_get_resample_fir_params": [_u32, _u32, _i32, _u32, _pu32, _pu32, _vp, _u32, _pu32],
    "fdsp_design_resample_firls": [_u32, _u32, _u32, _dbl, _pu32, _pu32, _vp, _u32, _pu32],
    "fdsp_polyphase_advance": [_u32, _u32, _u32, _u64, _u64, _pu64, _pu32, _pu64],
    "fdsp_channelizer_create": [_u32, C.POINTER(channel_cfg), _u32, _pp],
    "fdsp_channelizer_destroy": [_vp],
    "fdsp_channelizer_reset": [_vp],
    "fdsp_channelizer_num_channels": [_vp, _pu32],
    "fdsp_channelizer_out_count": [_vp, _u64, _pu64],
    "fdsp_channelizer_apply": [_vp, _vp, _u64, _pp, _pu64, _pu64, _vp],
    "fdsp_channelizer_apply_host": [_vp, _vp, _u64, _pp, _pu64, _pu64, _vp],
    "fdsp_channelizer_kernel_launches": [_vp, _pu32],
    "fdsp_channelizer_apply_ci16": [_vp, _vp, _u64, _pp, _pu64, _pu64, _vp],
    "fdsp_channelizer_apply_ci16_host": [_vp, _vp, _u64, _pp, _pu64, _pu64, _vp],
    "fdsp_resampler_apply_ci16": [_vp, _vp, _u64, _vp, _u64, _pu64, _vp],
    "fdsp_freq_shift_apply_ci16": [_vp, _vp, _u64, _pp, _vp],
    "fdsp_freq_shift_apply_ci16_host": [_vp, _vp, _u64, _pp, _vp],
    "fdsp_fir_apply_ci16": [_vp, _vp, _u64, _vp, _vp],
    "fdsp_fir_set_precision": [_vp, C.c_int],
    "fdsp_fir_tc_groups": [_vp, _pu32],
    "fdsp_fir_apply_ci16_host": [_vp, _vp, _u64, _vp, _vp],
    "fdsp_channelizer_tc_groups": [_vp, _pu32],
    "fdsp_channelizer_status": [_vp, _vp],
    "fdsp_channelizer_set_tc_wait": [_vp, _u32, C.c_int],
    "fdsp_channelizer_set_tc_exact_all": [_vp, C.c_int],
    "fdsp_channelizer_profile": [_vp, C.c_int],
    "fdsp_channelizer_profile_read": [_vp, _pdbl, _pu32],
    "fdsp_resampler_set_precision": [_vp, C.c_int],
    "fdsp_resampler_tc_groups": [_vp, _pu32],
    "fdsp_resampler_status": [_vp, _vp],
    "fdsp_fir_status": [_vp, _vp],
    "fdsp_server_create": [_u64, _u32, _pp],
    "fdsp_server_destroy": [_vp],
    "fdsp_server_open": [_vp, _u32, _vp, _u32, _u64, C.c_int, _pu32],
    "fdsp_server_submit": [_vp, _u32, _vp, _u64, _vp, _vp, _pu64],
    "fdsp_server_poll": [_vp, _u64, C.POINTER(C.c_int), _pu64, _pdbl],
    "fdsp_server_close": [_vp, _u32],
    "fdsp_server_wait_any": [_vp, _u32, _pu64],
    "fdsp_server_stats": [_vp, _pdbl, _pdbl, _pdbl, _pu64, _pu64, _pu64, _pu32],
    "fdsp_server_reset_stats": [_vp],
    "fdsp_channelizer_autotune": [_vp, _u64, _vp],
    "fdsp_channelizer_num_groups": [_vp, _pu32],
    "fdsp_channelizer_set_graph": [_vp, C.c_int],
    "fdsp_channelizer_graph_replays": [_vp, _pu32],
    "fdsp_channelizer_group_info": [_vp, _u32, _pu32, _pu32, C.POINTER(C.c_int)],
    "fdsp_channelizer_group_tc_split": [_vp, _u32, _pu32],
    "fdsp_channelizer_set_tc_split": [_vp, _u32],
    "fdsp_channelizer_set_precision": [_vp, C.c_int],
    "fdsp_resampler_create": [_u32, _u32, _vp, _u32, _pp],
    "fdsp_resampler_destroy": [_vp],
    "fdsp_resampler_reset": [_vp],
    "fdsp_resampler_coeffs_per_phase": [_vp, _pu32],
    "fdsp_resampler_out_count": [_vp, _u64, _pu64],
    "fdsp_resampler_needed_out_count": [_vp, _u32, _pu32],
    "fdsp_resampler_state": [_vp, _pu32, _pu64],
    "fdsp_resampler_apply": [_vp, _vp, _u64, _vp, _u64, _pu64, _vp],
    "fdsp_resampler_apply_host": [_vp, _vp, _u64, _vp, _u64, _pu64, _vp],
    "fdsp_resample_static": [_u32, _u32, _vp, _u32, _vp, _u64, _vp, _u64, _pu64, _vp],
    "fdsp_freq_shift_create": [_u32, C.POINTER(_i32), _u32, _pp],
    "fdsp_freq_shift_destroy": [_vp],
    "fdsp_freq_shift_reset": [_vp],
    "fdsp_freq_shift_num_channels": [_vp, _pu32],
    "fdsp_freq_shift_counter": [_vp, _u32, _pu64],
    "fdsp_freq_shift_apply": [_vp, _vp, _u64, _pp, _vp],
    "fdsp_freq_shift_apply_host": [_vp, _vp, _u64, _pp, _vp],
    "fdsp_fir_create": [_vp, _u32, _pp],
    "fdsp_fir_destroy": [_vp],
    "fdsp_fir_reset": [_vp],
    "fdsp_fir_apply": [_vp, _vp, _u64, _vp, _vp],
    "fdsp_fir_apply_host": [_vp, _vp, _u64, _vp, _vp],
    "fdsp_fm_demod_create": [_u32, _i32, C.c_float, _pp],
    "fdsp_fm_demod_destroy": [_vp],
    "fdsp_fm_demod_reset": [_vp],
    "fdsp_fm_demod_out_count": [_vp, _u64, _pu64],
    "fdsp_fm_demod_apply": [_vp, _vp, _u64, _vp, _u64, _pu64, _vp],
    "fdsp_fm_demod_apply_host": [_vp, _vp, _u64, _vp, _u64, _pu64, _vp],
    "fdsp_polar_create": [_pp],
    "fdsp_polar_destroy": [_vp],
    "fdsp_polar_reset": [_vp],
    "fdsp_polar_out_count": [_vp, _u64, _pu64],
    "fdsp_polar_apply": [_vp, _vp, _u64, _vp, _pu64, _vp],
    "fdsp_polar_apply_host": [_vp, _vp, _u64, _vp, _pu64, _vp],
}
_RES = {"fdsp_status_string": C.c_char_p}

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m libfalcon_dsp_gb300.build` "
                "(nvcc for sm_103a); there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RES.get(name, C.c_int)
        _lib = L
    return _lib


def check(fn_name: str, status: int) -> None:
    if status != FDSP_OK:
        raise FdspError(fn_name, status, lib().fdsp_last_cuda_error())


def call(fn_name: str, *args) -> None:
    check(fn_name, getattr(lib(), fn_name)(*args))
