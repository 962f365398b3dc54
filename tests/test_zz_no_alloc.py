"""The allocation-free xc entry point (fxc_xc_run_noalloc) against fxc_xc_run.

fxc_xc_run_noalloc serves callers that cannot call cudaMalloc (a host
framework that owns all device memory, or a job whose device footprint is
fixed at start-up): it keeps its scratch in a fixed 64 MiB device array
compiled into the library. This file is collected last so that a run that
stops at its first failure has already run every other test. It builds its
own context, so it passes alone in a fresh process as well as after the
other tests.

Checks: two calls in a row against fxc_xc_run and against the FP64 oracle
(oracle/xc_oracle.py, the reference's stack + finalize restated); a third
call with a new transform length and a new pair list leaves the device's
free memory unchanged (cudaMemGetInfo); oversized requests are refused.

Tolerance: the same NCF bound as the xc parity tests (relative L2 1e-5).
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NCF_RTOL = 1e-5


def _pairs(nsta, ncomp=3):
    src, rec = [], []
    for s in range(nsta):
        for t in range(s + 1, nsta):
            for i in range(ncomp):
                for j in range(ncomp):
                    src.append(s * ncomp + i)
                    rec.append(t * ncomp + j)
    return np.array(src, np.int32), np.array(rec, np.int32)


def _oracle(spec, src, rec, nspec, dt, cc, scale):
    from oracle import xc_oracle as xo

    return xo.xc_run(spec[:, :, :nspec], src, rec, scale, xo.finalize_shape(nspec, spec.shape[0], dt, cc))


def _rel(got, ref):
    return np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)


def _run_both(torch, ctx, spec, src, rec, nspec, dt, cc, scale):
    from fastxc_gb300._lib import lib
    from fastxc_gb300.core import PairPlan, xc_shape

    nwin, nchan, pitch = spec.shape
    shape = xc_shape(nspec, nwin, dt, cc)
    d_spec = torch.from_numpy(spec).cuda()
    ref = torch.empty((src.size, shape.cc_size), dtype=torch.float32, device="cuda")
    got = torch.full((src.size, shape.cc_size), float("nan"), dtype=torch.float32, device="cuda")
    plan = PairPlan(ctx, src, rec, nchan)
    ctx.xc_run(plan, d_spec, nwin, nchan, pitch, None, scale, shape, ref)
    lib().fxc_xc_run_noalloc(ctx.handle, src.ctypes.data, rec.ctypes.data, src.size, d_spec.data_ptr(),
                             nwin, nchan, pitch, None, scale, C.byref(shape), got.data_ptr())
    ctx.synchronize()
    plan.close()
    return got.cpu().numpy(), ref.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastxc_gb300 import build

    build.build()
    from fastxc_gb300.core import Context

    with Context(0) as ctx:
        rng = np.random.default_rng(42)
        # call 1: 4 stations, nspec 18523 (the 37 044-point production transform)
        nwin, nsta, nspec = 6, 4, 18523
        spec = (rng.standard_normal((nwin, 3 * nsta, nspec)) + 1j * rng.standard_normal((nwin, 3 * nsta, nspec))).astype(np.complex64)
        src, rec = _pairs(nsta)
        got, ref = _run_both(torch, ctx, spec, src, rec, nspec, 0.1, 100.0, 1.0 / nwin)
        assert np.all(np.isfinite(got))
        assert _rel(got, ref).max() < NCF_RTOL
        assert _rel(got, _oracle(spec, src, rec, nspec, 0.1, 100.0, 1.0 / nwin)).max() < NCF_RTOL
        # call 2 right after, different shape and pair list: the array keeps the
        # previous call's contents and must not leak into this result
        nwin, nsta, nspec = 9, 6, 1001
        spec = (rng.standard_normal((nwin, 3 * nsta, nspec)) + 1j * rng.standard_normal((nwin, 3 * nsta, nspec))).astype(np.complex64)
        src, rec = _pairs(nsta)
        src, rec = src[::-1].copy(), rec[::-1].copy()
        got, ref = _run_both(torch, ctx, spec, src, rec, nspec, 0.1, 20.0, 1.0 / nwin)
        assert np.all(np.isfinite(got))
        assert _rel(got, ref).max() < NCF_RTOL
        assert _rel(got, _oracle(spec, src, rec, nspec, 0.1, 20.0, 1.0 / nwin)).max() < NCF_RTOL


def test_noalloc_call_leaves_free_device_memory_unchanged():
    """A call whose transform length and pair list the process has not seen
    (the case where the allocating path would add FFT tables and scratch)
    leaves cudaMemGetInfo's free bytes exactly as they were."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastxc_gb300 import build

    build.build()
    from fastxc_gb300._lib import lib
    from fastxc_gb300.core import Context, xc_shape

    with Context(0) as ctx:
        rng = np.random.default_rng(7)

        def call(nwin, nsta, nspec, cc, reverse):
            spec = (rng.standard_normal((nwin, 3 * nsta, nspec)) +
                    1j * rng.standard_normal((nwin, 3 * nsta, nspec))).astype(np.complex64)
            src, rec = _pairs(nsta)
            if reverse:
                src, rec = src[::-1].copy(), rec[::-1].copy()
            shape = xc_shape(nspec, nwin, 0.1, cc)
            d_spec = torch.from_numpy(spec).cuda()
            d_ncf = torch.empty((src.size, shape.cc_size), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            lib().fxc_xc_run_noalloc(ctx.handle, src.ctypes.data, rec.ctypes.data, src.size, d_spec.data_ptr(),
                                     nwin, 3 * nsta, nspec, None, 1.0 / nwin, C.byref(shape), d_ncf.data_ptr())
            ctx.synchronize()
            free1 = torch.cuda.mem_get_info()[0]
            got = d_ncf.cpu().numpy()
            assert _rel(got, _oracle(spec, src, rec, nspec, 0.1, cc, 1.0 / nwin)).max() < NCF_RTOL
            return free0, free1

        call(5, 3, 1001, 20.0, False)  # warm-up: the set-up lookup and first kernel loads
        free0, free1 = call(7, 5, 1201, 30.0, True)  # nfft 2400, new pair list
        assert free0 == free1, (free0, free1)


def test_noalloc_rejects_oversized_requests():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastxc_gb300 import FxcError, build

    build.build()
    from fastxc_gb300._lib import lib
    from fastxc_gb300.core import Context, xc_shape

    with Context(0) as ctx:
        nsta, nspec, nwin = 12, 18523, 1  # 594 pairs x 148 KB > 64 MiB
        src, rec = _pairs(nsta)
        shape = xc_shape(nspec, nwin, 0.1, 100.0)
        d_spec = torch.zeros((nwin, 3 * nsta, nspec), dtype=torch.complex64, device="cuda")
        d_ncf = torch.zeros((src.size, shape.cc_size), dtype=torch.float32, device="cuda")
        with pytest.raises(FxcError, match="64 MiB"):
            lib().fxc_xc_run_noalloc(ctx.handle, src.ctypes.data, rec.ctypes.data, src.size, d_spec.data_ptr(),
                                     nwin, 3 * nsta, nspec, None, 1.0, C.byref(shape), d_ncf.data_ptr())
