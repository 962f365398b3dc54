"""Python handles over the C ABI: contexts, pair plans and the xc entry points.

Device buffers are passed as raw pointers (``int``), e.g. ``tensor.data_ptr()``
of a CUDA torch tensor; host buffers as numpy arrays. The compute always runs
in ``libfastxc_gb300.so``.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import FXC_XC_PLAIN, FXC_XC_TENSOR, XcShape, lib

__all__ = [
    "Context",
    "PairPlan",
    "xc_shape",
    "FXC_XC_PLAIN",
    "FXC_XC_TENSOR",
]


def _ptr(x) -> int | None:
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError(f"cannot take a pointer of {type(x)!r}")


class Context:
    """One library context (device + stream + scratch)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._h = C.c_void_p()
        lib().fxc_ctx_create(device, stream, C.byref(self._h))
        self.device = device

    @property
    def handle(self) -> C.c_void_p:
        if not self._h:
            raise RuntimeError("context closed")
        return self._h

    def set_stream(self, stream: int | None) -> None:
        lib().fxc_ctx_set_stream(self.handle, stream)

    def synchronize(self) -> None:
        lib().fxc_ctx_synchronize(self.handle)

    def kernel_timing(self, enable: bool) -> None:
        """Bracket the dominant kernels' launches with CUDA events (or stop)."""
        lib().fxc_ctx_kernel_timing(self.handle, int(bool(enable)))

    def kernel_time(self, kernel: str) -> tuple[float, int]:
        """(summed ms, launches) of `kernel` since the last query."""
        ms = C.c_double()
        n = C.c_int64()
        lib().fxc_ctx_kernel_time(self.handle, kernel.encode(), C.byref(ms), C.byref(n))
        return ms.value, n.value

    def graph_begin(self) -> None:
        """Start recording this context's calls into a CUDA graph."""
        lib().fxc_graph_begin(self.handle)

    def graph_end(self) -> "Graph":
        h = C.c_void_p()
        lib().fxc_graph_end(self.handle, C.byref(h))
        return Graph(self, h)

    def host_phases(self) -> dict:
        """Phases (ms) of the last xc_run_host made while kernel timing was on."""
        out = (C.c_double * 6)()
        lib().fxc_ctx_host_phases(self.handle, out, 6)
        keys = ("total", "copy_busy", "last_copy_end", "compute_busy", "tail_after_last_copy", "finalize_and_d2h")
        return {k: (v if v >= 0 else None) for k, v in zip(keys, out)}

    def close(self) -> None:
        if self._h:
            lib().fxc_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- FFT ----------------------------------------------------------------
    def fft_c2c(self, d_in, d_out, n, batch, in_pitch=None, out_pitch=None, inverse=False):
        lib().fxc_fft_c2c(self.handle, _ptr(d_in), _ptr(d_out), n, batch,
                          in_pitch or n, out_pitch or n, 1 if inverse else 0)

    def fft_r2c(self, d_in, d_out, n, batch, in_pitch=None, out_pitch=None):
        lib().fxc_fft_r2c(self.handle, _ptr(d_in), _ptr(d_out), n, batch,
                          in_pitch or n, out_pitch or (n // 2 + 1))

    def fft_c2r(self, d_in, d_out, n, batch, in_pitch=None, out_pitch=None):
        lib().fxc_fft_c2r(self.handle, _ptr(d_in), _ptr(d_out), n, batch,
                          in_pitch or (n // 2 + 1), out_pitch or n)

    # ---- xc -----------------------------------------------------------------
    def xc_stack(self, plan: "PairPlan", d_spec, nwin, nchan, nspec, spec_pitch, d_mask, scale,
                 d_stack, stack_pitch, method=FXC_XC_PLAIN):
        lib().fxc_xc_stack(self.handle, plan.handle, _ptr(d_spec), nwin, nchan, nspec, spec_pitch,
                           _ptr(d_mask), float(scale), _ptr(d_stack), stack_pitch, method)

    def xc_autotune(self, plan: "PairPlan", d_spec, nwin, nchan, nspec, spec_pitch):
        """(method, plain sample ms, tensor sample ms) from fxc_xc_autotune."""
        m, a, b = C.c_int32(), C.c_float(), C.c_float()
        lib().fxc_xc_autotune(self.handle, plan.handle, _ptr(d_spec), nwin, nchan, nspec, spec_pitch, C.byref(m),
                              C.byref(a), C.byref(b))
        return int(m.value), float(a.value), float(b.value)

    def xc_autotune_layout(self, plan: "PairPlan", d_spec, nwin, nchan, nspec, spec_pitch):
        """(method, tensor layout, {"plain", "whole_bin", "tiled"} sample ms)
        from fxc_xc_autotune_layout; the plan takes the faster layout."""
        m, lay, ms = C.c_int32(), C.c_int32(), (C.c_float * 3)()
        lib().fxc_xc_autotune_layout(self.handle, plan.handle, _ptr(d_spec), nwin, nchan, nspec, spec_pitch,
                                     C.byref(m), C.byref(lay), ms)
        return int(m.value), int(lay.value), dict(zip(("plain", "whole_bin", "tiled"), (float(v) for v in ms)))

    @staticmethod
    def xc_packed_bytes(nchan, nwin, nspec) -> int:
        out = C.c_int64()
        lib().fxc_xc_packed_bytes(nchan, nwin, nspec, C.byref(out))
        return int(out.value)

    def xc_pack(self, d_spec, nwin, nchan, nspec, spec_pitch, d_mask, d_packed):
        lib().fxc_xc_pack(self.handle, _ptr(d_spec), nwin, nchan, nspec, spec_pitch, _ptr(d_mask),
                          _ptr(d_packed))

    def xc_stack_packed(self, plan: "PairPlan", d_packed, nwin, nspec, scale, d_stack, stack_pitch):
        lib().fxc_xc_stack_packed(self.handle, plan.handle, _ptr(d_packed), nwin, nspec, float(scale),
                                  _ptr(d_stack), stack_pitch)

    def xc_stack_finalize_packed(self, plan: "PairPlan", d_packed, nwin, nspec, scale, shape: XcShape, d_ncf):
        lib().fxc_xc_stack_finalize_packed(self.handle, plan.handle, _ptr(d_packed), nwin, nspec, float(scale),
                                           C.byref(shape), _ptr(d_ncf))

    def xc_finalize(self, d_stack, npairs, stack_pitch, shape: XcShape, d_ncf):
        lib().fxc_xc_finalize(self.handle, _ptr(d_stack), npairs, stack_pitch, C.byref(shape),
                              _ptr(d_ncf))

    def xc_run(self, plan: "PairPlan", d_spec, nwin, nchan, spec_pitch, d_mask, scale,
               shape: XcShape, d_ncf, method=FXC_XC_PLAIN):
        lib().fxc_xc_run(self.handle, plan.handle, _ptr(d_spec), nwin, nchan, spec_pitch,
                         _ptr(d_mask), float(scale), C.byref(shape), _ptr(d_ncf), method)

    def xc_run_host(self, plan: "PairPlan", h_spec: np.ndarray, nwin, nchan, spec_pitch,
                    h_mask, scale, shape: XcShape, h_ncf: np.ndarray, method=FXC_XC_PLAIN):
        if h_spec.dtype != np.complex64 or not h_spec.flags.c_contiguous:
            raise ValueError("h_spec must be C-contiguous complex64")
        if h_ncf.dtype != np.float32 or not h_ncf.flags.c_contiguous:
            raise ValueError("h_ncf must be C-contiguous float32")
        lib().fxc_xc_run_host(self.handle, plan.handle, _ptr(h_spec), nwin, nchan, spec_pitch,
                              _ptr(h_mask), float(scale), C.byref(shape), _ptr(h_ncf), method)


class PairPlan:
    """Correlation plan for an ordered pair list (see fxc_pairplan_create)."""

    def __init__(self, ctx: Context, src, rec, nchan: int):
        src = np.ascontiguousarray(src, dtype=np.int32)
        rec = np.ascontiguousarray(rec, dtype=np.int32)
        if src.shape != rec.shape or src.ndim != 1:
            raise ValueError("src and rec must be 1-D arrays of the same length")
        self._h = C.c_void_p()
        lib().fxc_pairplan_create(ctx.handle, _ptr(src), _ptr(rec), src.size, nchan,
                                  C.byref(self._h))
        self.npairs = int(src.size)
        self.nchan = nchan
        self.src = src
        self.rec = rec

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def ntiles(self) -> int:
        return int(lib().fxc_pairplan_ntiles(self._h))

    def set_layout(self, layout: int) -> None:
        """Contraction layout preference (FXC_XC_LAYOUT_*; fxc_pairplan_set_layout)."""
        lib().fxc_pairplan_set_layout(self._h, layout)

    def layouts(self, nwin: int) -> tuple[int, int]:
        """(admitted layouts as a bit mask of 1 << FXC_XC_LAYOUT_*, the layout
        a run of nwin windows takes)."""
        a, e = C.c_int32(), C.c_int32()
        lib().fxc_pairplan_layouts(self._h, nwin, C.byref(a), C.byref(e))
        return int(a.value), int(e.value)

    def close(self):
        if self._h:
            lib().fxc_pairplan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def xc_shape(nspec: int, nstep: int, dt: float, cc_length: float) -> XcShape:
    """finalize_shape (native/xc/io/input.cu:1033-1054)."""
    s = XcShape()
    lib().fxc_xc_shape_init(nspec, nstep, dt, cc_length, C.byref(s))
    return s


class Graph:
    """A recorded launch sequence of one context (fxc_graph_*)."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle

    def launch(self) -> None:
        lib().fxc_graph_launch(self.ctx.handle, self.handle)

    def close(self) -> None:
        if self.handle:
            lib().fxc_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
