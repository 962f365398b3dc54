"""ctypes binding of ``libfastxc_gb300.so`` (the C ABI in ``include/fastxc_gb300.h``).

The binding is thin on purpose: every call goes straight to the CUDA library,
and a missing library raises ``FxcLibraryMissing`` — there is no Python or
CPU fallback for any compute entry point.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "lib" / "libfastxc_gb300.so"

FXC_OK = 0
FXC_ERR_INVALID = -1
FXC_ERR_CUDA = -2
FXC_ERR_UNSUPPORTED = -3
FXC_ERR_NOMEM = -4
FXC_ERR_IO = -5
FXC_ERR_NODEVICE = -6
FXC_ERR_TIMEOUT = -7
FXC_ERR_NOTFOUND = -8

FXC_XC_PLAIN = 0
FXC_XC_TENSOR = 1
FXC_XC_LAYOUT_AUTO, FXC_XC_LAYOUT_WHOLE_BIN, FXC_XC_LAYOUT_TILED = 0, 1, 2


class FxcError(RuntimeError):
    def __init__(self, status: int, message: str, func: str):
        super().__init__(f"{func} failed with status {status}: {message}")
        self.status = status
        self.message = message
        self.func = func


class FxcLibraryMissing(ImportError):
    pass


class XcShape(C.Structure):
    _fields_ = [
        ("nspec", C.c_int32),
        ("nstep", C.c_int32),
        ("nfft", C.c_int32),
        ("half_cc", C.c_int32),
        ("cc_size", C.c_int32),
        ("dt", C.c_float),
    ]


_vp = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64
_int = C.c_int
_f32 = C.c_float

# name -> (restype, argtypes); every int-returning function is status-checked.
_SIGNATURES: dict[str, tuple] = {
    "fxc_last_error": (C.c_char_p, []),
    "fxc_version": (_int, []),
    "fxc_launch_count": (_i64, []),
    "fxc_launch_count_reset": (None, []),
    "fxc_ctx_kernel_timing": (_int, [_vp, _int]),
    "fxc_ctx_kernel_time": (_int, [_vp, C.c_char_p, C.POINTER(C.c_double), C.POINTER(_i64)]),
    "fxc_ctx_host_phases": (_int, [_vp, C.POINTER(C.c_double), _i32]),
    "fxc_ctx_create": (_int, [_int, _vp, C.POINTER(_vp)]),
    "fxc_ctx_destroy": (_int, [_vp]),
    "fxc_ctx_set_stream": (_int, [_vp, _vp]),
    "fxc_ctx_synchronize": (_int, [_vp]),
    "fxc_graph_begin": (_int, [_vp]),
    "fxc_graph_end": (_int, [_vp, C.POINTER(_vp)]),
    "fxc_graph_launch": (_int, [_vp, _vp]),
    "fxc_graph_destroy": (_int, [_vp]),
    "fxc_device_alloc": (_int, [_vp, C.c_size_t, C.POINTER(_vp)]),
    "fxc_device_free": (_int, [_vp, _vp]),
    "fxc_host_alloc": (_int, [C.c_size_t, C.POINTER(_vp)]),
    "fxc_host_free": (_int, [_vp]),
    "fxc_memcpy": (_int, [_vp, _vp, _vp, C.c_size_t, C.c_int]),
    "fxc_fft_c2c": (_int, [_vp, _vp, _vp, _int, _int, _i64, _i64, _int]),
    "fxc_fft_r2c": (_int, [_vp, _vp, _vp, _int, _int, _i64, _i64]),
    "fxc_fft_c2r": (_int, [_vp, _vp, _vp, _int, _int, _i64, _i64]),
    "fxc_fft_supported": (_int, [_int, _int]),
    "fxc_xc_shape_init": (_int, [_i32, _i32, _f32, _f32, C.POINTER(XcShape)]),
    "fxc_pairplan_create": (_int, [_vp, _vp, _vp, _i64, _i32, C.POINTER(_vp)]),
    "fxc_pairplan_destroy": (_int, [_vp]),
    "fxc_pairplan_npairs": (_i64, [_vp]),
    "fxc_pairplan_ntiles": (_i64, [_vp]),
    "fxc_xc_stack": (_int, [_vp, _vp, _vp, _i64, _i32, _i32, _i64, _vp, _f32, _vp, _i64, _int]),
    "fxc_xc_packed_bytes": (_int, [_i32, _i64, _i32, C.POINTER(_i64)]),
    "fxc_xc_pack": (_int, [_vp, _vp, _i64, _i32, _i32, _i64, _vp, _vp]),
    "fxc_xc_stack_packed": (_int, [_vp, _vp, _vp, _i64, _i32, _f32, _vp, _i64]),
    "fxc_xc_finalize": (_int, [_vp, _vp, _i64, _i64, C.POINTER(XcShape), _vp]),
    "fxc_xc_stack_finalize_packed": (_int, [_vp, _vp, _vp, _i64, _i32, _f32, C.POINTER(XcShape), _vp]),
    "fxc_xc_run": (_int, [_vp, _vp, _vp, _i64, _i32, _i64, _vp, _f32, C.POINTER(XcShape), _vp, _int]),
    "fxc_xc_run_host": (_int, [_vp, _vp, _vp, _i64, _i32, _i64, _vp, _f32, C.POINTER(XcShape), _vp, _int]),
    "fxc_xc_rows_accumulate": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _i64, _vp, _i64, _i64, _i32, _i32]),
    "fxc_rotate_matrix": (_int, [C.c_double, C.c_double, _vp]),
    "fxc_rotate_enz_rtz": (_int, [_vp, _vp, _i64, _i32, _i64, _vp, _vp]),
    "fxc_xc_run_noalloc": (_int, [_vp, _vp, _vp, _i64, _vp, _i64, _i32, _i64, _vp, _f32, C.POINTER(XcShape), _vp]),
}

# Functions whose int return value is a count/flag, not a status.
_NOT_STATUS = {"fxc_version", "fxc_fft_supported", "fxc_launch_count", "fxc_pairplan_npairs", "fxc_pairplan_ntiles"}


def declared_symbols() -> list[str]:
    return list(_SIGNATURES)


class _Lib:
    def __init__(self, path: Path):
        if not path.exists():
            raise FxcLibraryMissing(
                f"{path} not found: build it with `python -m fastxc_gb300.build` "
                "(the GPU path has no fallback)"
            )
        self.path = path
        self.cdll = C.CDLL(str(path), mode=C.RTLD_GLOBAL)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(self.cdll, name)
            fn.restype = res
            fn.argtypes = args
            setattr(self, "_raw_" + name, fn)

    def last_error(self) -> str:
        msg = self._raw_fxc_last_error()
        return msg.decode("utf-8", "replace") if msg else ""

    def __getattr__(self, name: str):
        raw = self.__dict__.get("_raw_" + name)
        if raw is None:
            raise AttributeError(name)
        if raw.restype is not _int or name in _NOT_STATUS:
            return raw

        def checked(*args):
            st = raw(*args)
            if st != FXC_OK:
                raise FxcError(st, self.last_error(), name)
            return st

        checked.__name__ = name
        return checked


_LIB: _Lib | None = None


def lib() -> _Lib:
    global _LIB
    if _LIB is None:
        _LIB = _Lib(Path(os.environ.get("FXC_LIB", LIB_PATH)))
    return _LIB


class S2sPlan(C.Structure):
    """fxc_s2s_plan (include/fastxc_gb300.h)."""

    _fields_ = [
        ("delta", C.c_float),
        ("npts", C.c_int32),
        ("segment_pts", C.c_int32),
        ("shift_pts", C.c_int32),
        ("nstep", C.c_int32),
        ("output_nfft", C.c_int32),
        ("nspec", C.c_int32),
        ("filter_padding", C.c_int32),
        ("filter_nfft", C.c_int32),
        ("freq_low", C.c_float),
        ("freq_high", C.c_float),
        ("f_idx1", C.c_int32),
        ("f_idx2", C.c_int32),
        ("f_idx3", C.c_int32),
        ("f_idx4", C.c_int32),
        ("taper_pts", C.c_int32),
        ("runabs_win", C.c_int32),
        ("whiten_win", C.c_int32),
        ("whiten", C.c_int32),
        ("normalize", C.c_int32),
        ("phase_only", C.c_int32),
        ("nfilters", C.c_int32),
        ("band_freq_low", C.c_float * 100),
    ]


_SIGNATURES.update({
    "fxc_s2s_plan_init": (_int, [_f32, _f32, _f32, _f32, _f32, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32,
                                 C.POINTER(S2sPlan)]),
    "fxc_s2s_filter_response": (_int, [C.POINTER(S2sPlan), _vp, _vp, _i32, _vp]),
    "fxc_s2s_run": (_int, [_vp, C.POINTER(S2sPlan), _vp, _i64, _i64, _i32, _i32, _vp, _i32, _vp, _vp, _i64]),
})

_SIGNATURES.update({
    "fxc_linear_stack": (_int, [_vp, _vp, _vp, _vp, _i32, _i32, _vp]),
    "fxc_stack_prestack": (_int, [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp]),
    "fxc_pws_stream_add": (_int, [_vp, _vp, _i64, _i32, _i32, _f32, _vp, _vp]),
    "fxc_pws_stream_finish": (_int, [_vp, _vp, _vp, _i32, _i32, _f32, _vp]),
    "fxc_pws_run": (_int, [_vp, _vp, _vp, _vp, _vp, _i32, _vp, _i32, _f32, _vp]),
    "fxc_tfpws_run": (_int, [_vp, _vp, _vp, _vp, _vp, _i32, _vp, _i32, _f32, _i32, _f32, _f32, _f32, _f32, _vp]),
})


class ServerConfig(C.Structure):
    """fxc_server_config (include/fastxc_gb300.h)."""

    _fields_ = [("device", C.c_int32), ("slots", C.c_int32), ("cache_gib", C.c_double), ("work_gib", C.c_double),
                ("chunk_gib", C.c_double), ("synthetic", C.c_int32), ("seed", C.c_uint64), ("win_len", C.c_float),
                ("lag_max", C.c_float), ("max_wait_s", C.c_double), ("keep_results", C.c_int32)]


class Job(C.Structure):
    """fxc_job."""

    _fields_ = [("stations", C.POINTER(C.c_int32)), ("nsta", C.c_int32), ("day0", C.c_int32), ("ndays", C.c_int32),
                ("delta", C.c_float), ("lag", C.c_float), ("method", C.c_int32), ("pws", C.c_int32),
                ("pws_power", C.c_float)]


class JobInfo(C.Structure):
    """fxc_job_info."""

    _fields_ = [("npairs", C.c_int64), ("cc_size", C.c_int64), ("nspec", C.c_int64), ("pair_windows", C.c_int64),
                ("submit_s", C.c_double), ("start_s", C.c_double), ("end_s", C.c_double), ("status", C.c_int32)]


class ServerStats(C.Structure):
    """fxc_server_stats_t."""

    _fields_ = [("jobs_done", C.c_int64), ("pair_windows", C.c_int64), ("queued", C.c_int64),
                ("cache_entries", C.c_int64), ("cache_used_bytes", C.c_int64), ("work_used_bytes", C.c_int64)]


_SIGNATURES.update({
    "fxc_xc_autotune": (_int, [_vp, _vp, _vp, _i64, _i32, _i32, _i64, C.POINTER(_i32), C.POINTER(_f32),
                                C.POINTER(_f32)]),
    "fxc_xc_autotune_layout": (_int, [_vp, _vp, _vp, _i64, _i32, _i32, _i64, C.POINTER(_i32), C.POINTER(_i32),
                                       C.POINTER(_f32)]),
    "fxc_pairplan_set_layout": (_int, [_vp, _i32]),
    "fxc_pairplan_layouts": (_int, [_vp, _i64, C.POINTER(_i32), C.POINTER(_i32)]),
    "fxc_server_create": (_int, [C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "fxc_server_destroy": (_int, [_vp]),
    "fxc_server_geometry": (_int, [_vp, _f32, C.POINTER(_i32), C.POINTER(_i32)]),
    "fxc_server_put_spectra": (_int, [_vp, _i32, _i32, _f32, _vp]),
    "fxc_server_submit": (_int, [_vp, C.POINTER(Job), C.POINTER(_i64)]),
    "fxc_server_wait": (_int, [_vp, _i64, C.c_double, C.POINTER(JobInfo)]),
    "fxc_server_fetch": (_int, [_vp, _i64, _vp, _vp]),
    "fxc_server_release": (_int, [_vp, _i64]),
    "fxc_server_stats": (_int, [_vp, C.POINTER(ServerStats)]),
})


class SourcePackTotals(C.Structure):
    """fxc_sourcepack_totals."""

    _fields_ = [("timestamps", C.c_int64), ("records", C.c_int64), ("sources", C.c_int64),
                ("bytes_indexed", C.c_int64)]


_SIGNATURES.update({
    "fxc_sourcepack_build": (_int, [C.c_char_p, C.c_char_p, C.c_char_p, _int, C.c_char_p,
                                    C.POINTER(SourcePackTotals), C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t]),
    "fxc_sourcepack_async_start": (_int, [C.c_char_p, C.c_char_p, _int, C.c_char_p, C.c_double, C.POINTER(_vp)]),
    "fxc_sourcepack_async_finish": (_int, [_vp, _int, C.c_char_p, C.POINTER(SourcePackTotals)]),
})

_SIGNATURES.update({
    "fxc_xc_host_bytes": (_int, [_i64, _i64, _i32, _i64, C.POINTER(XcShape), _int, _int, C.POINTER(_i64)]),
    "fxc_plan_xc_pairs": (_int, [_i64, _i64, _i32, _i64, C.POINTER(XcShape), _int, _int, _i64, C.POINTER(_i64),
                                 C.POINTER(_i64)]),
    "fxc_stack_batch_bytes": (_int, [_int, _i64, _i32, _i64, _i64, _i32, C.POINTER(_i64)]),
    "fxc_plan_stack_traces": (_int, [_int, _i32, _i32, _i32, _i64, C.POINTER(_i64), C.POINTER(_i64)]),
})
