"""Host-side mirror of the sac2spec stage (planning, filter responses, the
per-batch compute call). The compute runs in libfastxc_gb300.so."""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import S2sPlan, lib
from .core import Context, _ptr

WHITEN_NONE, WHITEN_BEFORE, WHITEN_AFTER, WHITEN_BOTH = 0, 1, 2, 3
NORM_NONE, NORM_RUNABS_MF, NORM_ONEBIT, NORM_RUNABS = 0, 1, 2, 3


@dataclass
class Filters:
    """filter.txt contents: the broad band first, then every band."""

    freq_low: np.ndarray  # float32 [n]
    freq_high: np.ndarray  # float32 [n]
    b: np.ndarray  # float64 [n][5]
    a: np.ndarray  # float64 [n][5]

    @property
    def n(self) -> int:
        return int(self.b.shape[0])


def read_filter_file(path) -> Filters:
    """readButterworthFilters (native/sac2spec/core/filter_response.c:129-184)."""
    lo, hi, bs, as_ = [], [], [], []
    state = 0
    cur = None
    for line in open(path, encoding="ascii"):
        if line.startswith("#"):
            try:
                l, h = line[1:].strip().split("/")
                cur = (float(np.float32(float(l))), float(np.float32(float(h))))
                state = 1
            except ValueError:
                pass
            continue
        vals = line.split()
        if state == 1 and len(vals) >= 5:
            bcur = [float(v) for v in vals[:5]]
            state = 2
        elif state == 2:
            if len(vals) >= 5:
                lo.append(cur[0]); hi.append(cur[1]); bs.append(bcur); as_.append([float(v) for v in vals[:5]])
            state = 0
    return Filters(np.array(lo, np.float32), np.array(hi, np.float32), np.array(bs, np.float64), np.array(as_, np.float64))


def plan(sac_len: float, win_len: float, shift_len: float, xcorr_lag: float, delta: float, filters: Filters,
         whiten: int = WHITEN_AFTER, normalize: int = NORM_RUNABS, phase_only: bool = False) -> S2sPlan:
    """Segment / FFT / band planning (native/sac2spec/cuda.main.cu:203-296)."""
    p = S2sPlan()
    b = np.ascontiguousarray(filters.b, np.float64)
    a = np.ascontiguousarray(filters.a, np.float64)
    lo = np.ascontiguousarray(filters.freq_low, np.float32)
    hi = np.ascontiguousarray(filters.freq_high, np.float32)
    lib().fxc_s2s_plan_init(sac_len, win_len, shift_len, xcorr_lag, delta, _ptr(b), _ptr(a), _ptr(lo), _ptr(hi),
                            filters.n, whiten, normalize, 1 if phase_only else 0, C.byref(p))
    return p


def filter_response(p: S2sPlan, filters: Filters) -> np.ndarray:
    """[nfilters][filter_nfft/2+1] float32 power responses."""
    out = np.zeros((filters.n, p.filter_nfft // 2 + 1), np.float32)
    b = np.ascontiguousarray(filters.b, np.float64)
    a = np.ascontiguousarray(filters.a, np.float64)
    lib().fxc_s2s_filter_response(C.byref(p), _ptr(b), _ptr(a), filters.n, _ptr(out))
    return out


def run(ctx: Context, p: S2sPlan, d_series, series_pitch: int, series_len: int, nrows: int, num_ch: int,
        steps, d_responses, d_out, out_pitch: int) -> None:
    """ComputeWorkerBatch for the given window steps (device buffers)."""
    st = np.ascontiguousarray(steps, np.int32)
    lib().fxc_s2s_run(ctx.handle, C.byref(p), _ptr(d_series), series_pitch, series_len, nrows, num_ch,
                      _ptr(st), st.size, _ptr(d_responses), _ptr(d_out), out_pitch)
