"""Host-side mirror of the stacking stages (ncf_pws, ncf_tfpws and the
cross-timestamp linear stack). Each pair's NCF traces are rows of one device
array; a pair owns the rows [offset, offset + count)."""

from __future__ import annotations

import numpy as np

from ._lib import lib
from .core import Context, _ptr

MODE_PWS = 0    # group means (native/pws/io/sourcepack_io.cu:385-478)
MODE_TFPWS = 1  # group sums  (native/tfpws/io/sourcepack_io.cu:440-490)


def linear_stack(ctx: Context, d_traces, offsets, counts, nsamples: int, d_out) -> None:
    off = np.ascontiguousarray(offsets, np.int64)
    cnt = np.ascontiguousarray(counts, np.int32)
    lib().fxc_linear_stack(ctx.handle, _ptr(d_traces), _ptr(off), _ptr(cnt), off.size, nsamples, _ptr(d_out))


def prestack(ctx: Context, torch, d_traces, offsets, counts, nsamples: int, substack: int, mode: int):
    """Returns (d_groups, d_weights, d_linear, group_offsets, group_counts)."""
    off = np.ascontiguousarray(offsets, np.int64)
    cnt = np.ascontiguousarray(counts, np.int32)
    b = substack if substack >= 2 else 1
    ngroups = int(sum((c + b - 1) // b for c in cnt))
    dev = d_traces.device
    d_groups = torch.empty((max(ngroups, 1), nsamples), dtype=torch.float32, device=dev)
    d_weights = torch.empty((max(ngroups, 1),), dtype=torch.float32, device=dev)
    d_linear = torch.empty((max(off.size, 1), nsamples), dtype=torch.float32, device=dev)
    goff = np.zeros(off.size, np.int64)
    gcnt = np.zeros(off.size, np.int32)
    lib().fxc_stack_prestack(ctx.handle, _ptr(d_traces), _ptr(off), _ptr(cnt), off.size, nsamples, substack, mode,
                             _ptr(d_groups), _ptr(d_weights), _ptr(d_linear), _ptr(goff), _ptr(gcnt))
    return d_groups, d_weights, d_linear, goff, gcnt


def pws(ctx: Context, d_groups, d_weights, goff, gcnt, d_linear, nsamples: int, d_out, power: float = 1.0) -> None:
    goff = np.ascontiguousarray(goff, np.int64)
    gcnt = np.ascontiguousarray(gcnt, np.int32)
    lib().fxc_pws_run(ctx.handle, _ptr(d_groups), _ptr(d_weights), _ptr(goff), _ptr(gcnt), goff.size,
                      _ptr(d_linear), nsamples, float(power), _ptr(d_out))


def pws_stream_add(ctx: Context, d_rows, rows_pitch: int, npairs: int, nsamples: int, weight: float, d_acc,
                   d_lin) -> None:
    """Adds one group per pair (row p of d_rows) to the streaming PWS sums."""
    lib().fxc_pws_stream_add(ctx.handle, _ptr(d_rows), rows_pitch, npairs, nsamples, float(weight), _ptr(d_acc),
                             _ptr(d_lin))


def pws_stream_finish(ctx: Context, d_acc, d_lin, npairs: int, nsamples: int, power: float, d_out) -> None:
    lib().fxc_pws_stream_finish(ctx.handle, _ptr(d_acc), _ptr(d_lin), npairs, nsamples, float(power), _ptr(d_out))


def tfpws(ctx: Context, d_groups, d_weights, goff, gcnt, d_linear, nsamples: int, d_out, delta: float,
          band=None, taper_hz: float = -1.0, power: float = 1.0) -> None:
    goff = np.ascontiguousarray(goff, np.int64)
    gcnt = np.ascontiguousarray(gcnt, np.int32)
    lim = 1 if band is not None else 0
    fmin, fmax = (band if band is not None else (0.0, 0.0))
    lib().fxc_tfpws_run(ctx.handle, _ptr(d_groups), _ptr(d_weights), _ptr(goff), _ptr(gcnt), goff.size,
                        _ptr(d_linear), nsamples, float(delta), lim, float(fmin), float(fmax), float(taper_hz),
                        float(power), _ptr(d_out))
