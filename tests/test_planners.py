"""Memory planners (CPU, no GPU): the byte models and the binary searches.

fxc_xc_host_bytes / fxc_plan_xc_pairs size the pair blocks of xc_fast and
fxc_stack_batch_bytes / fxc_plan_stack_traces the stacking batches of
ncf_pws / ncf_tfpws, under -M or 0.9 x free device memory (the reference's
budgets: native/xc/memory/memory.cu:112-399,
native/tfpws/include/tfpws_schedule.hpp:149-217). Each model is restated
here from the buffers its call reserves, and each plan must be the largest
count that fits.
"""

import ctypes as C

import pytest

from fastxc_gb300 import FxcError
from fastxc_gb300._lib import FXC_XC_PLAIN, FXC_XC_TENSOR, lib
from fastxc_gb300.core import xc_shape


def al(x):
    return (x + 255) // 256 * 256


def xc_bytes_model(npairs, nwin, nchan, pitch, nspec, cc, tensor, mask):
    """The buffers of one fxc_xc_run_host call: a ring of three 64-window
    chunks, the mask, the NCF staging, the stacked spectra (pitch rounded to
    4 bins), on the tensor path one chunk's packed bf16 hi/lo operands and
    the bin-major rows, plus 64 bytes of pair tables per pair."""
    b = al(8 * nchan * pitch * 64) * 3
    if mask:
        b += al(nwin * nchan)
    b += al(4 * npairs * cc)
    b += 8 * ((nspec + 3) // 4 * 4) * npairs
    if tensor:
        nkb = (min(nwin, 64) + 31) // 32
        b += 16 * nspec * 4 * nkb * 4 * ((nchan + 7) // 8 * 8)  # 4 planes x k-blocks x 4 chunks per row
        b += 8 * ((npairs + 3) // 4 * 4) * nspec
    return b + 64 * npairs


def xc_bytes(npairs, nwin, nchan, pitch, shape, method, mask):
    out = C.c_int64()
    lib().fxc_xc_host_bytes(npairs, nwin, nchan, pitch, C.byref(shape), method, mask, C.byref(out))
    return out.value


@pytest.mark.parametrize("method", [FXC_XC_PLAIN, FXC_XC_TENSOR])
@pytest.mark.parametrize("nchan,nwin,nspec,mask", [(192, 24, 18523, 0), (1500, 48, 9601, 1), (12, 6, 1001, 0)])
def test_xc_bytes_model(built_lib, method, nchan, nwin, nspec, mask):
    shape = xc_shape(nspec, nwin, 0.1, 20.0)
    for npairs in (1, 17, 18144):
        got = xc_bytes(npairs, nwin, nchan, nspec, shape, method, mask)
        want = xc_bytes_model(npairs, nwin, nchan, nspec, nspec, shape.cc_size, method == FXC_XC_TENSOR, mask)
        assert got == want, (npairs, got, want)


@pytest.mark.parametrize("method", [FXC_XC_PLAIN, FXC_XC_TENSOR])
def test_xc_pair_plan_is_the_largest_fitting_block(built_lib, method):
    nchan, nwin, nspec, total = 192, 24, 18523, 18144
    shape = xc_shape(nspec, nwin, 0.1, 100.0)
    one = xc_bytes(1, nwin, nchan, nspec, shape, method, 0)
    full = xc_bytes(total, nwin, nchan, nspec, shape, method, 0)
    for budget in (one, one + 10_000_000, (one + full) // 2, full - 1, full, 4 * full):
        p, b = C.c_int64(), C.c_int64()
        lib().fxc_plan_xc_pairs(total, nwin, nchan, nspec, C.byref(shape), method, 0, budget, C.byref(p), C.byref(b))
        assert 1 <= p.value <= total
        assert b.value == xc_bytes(p.value, nwin, nchan, nspec, shape, method, 0) <= budget
        if p.value < total:
            assert xc_bytes(p.value + 1, nwin, nchan, nspec, shape, method, 0) > budget
    with pytest.raises(FxcError, match="budget"):
        p = C.c_int64()
        lib().fxc_plan_xc_pairs(total, nwin, nchan, nspec, C.byref(shape), method, 0, one - 1, C.byref(p), None)


def stack_bytes_model(mode, ntraces, npairs, ngroups, max_groups, n):
    """The stacking executables' batch buffers (traces, groups, weights,
    linear, out, offset staging) plus the library scratch: PWS partial sums
    of npairs x chunks x n complex, TF-PWS analytic spectra of every group
    and linear stack, output spectra and the Gaussian table."""
    tr, pairs = 4 * ntraces * n, 4 * npairs * n
    b = al(tr) + al(tr) + al(4 * ntraces) + al(pairs) + al(pairs) + al(16 * npairs) + 256
    if mode == 0:
        want = max(1, (7680 + npairs - 1) // max(npairs, 1))
        chunks = max(1, min(want, (max_groups + 1) // 2))
        b += 8 * n * npairs * chunks
    else:
        nfreq = n // 2 + 1
        b += al(8 * npairs) + al(4 * npairs) + al(8 * ngroups * n) + al(8 * npairs * n) * 2 + al(4 * nfreq * n)
    return b


def stack_bytes(mode, ntraces, npairs, ngroups, max_groups, n):
    out = C.c_int64()
    lib().fxc_stack_batch_bytes(mode, ntraces, npairs, ngroups, max_groups, n, C.byref(out))
    return out.value


@pytest.mark.parametrize("mode", [0, 1])
def test_stack_bytes_model(built_lib, mode):
    for ntr, npairs, n, b in ((720, 1, 2001, 10), (720 * 256, 256, 2001, 1), (30 * 7, 7, 4001, 3)):
        ng = npairs * ((ntr // npairs + b - 1) // b)
        mg = (ntr // npairs + b - 1) // b
        assert stack_bytes(mode, ntr, npairs, ng, mg, n) == stack_bytes_model(mode, ntr, npairs, ng, mg, n)


@pytest.mark.parametrize("mode,substack", [(0, 1), (0, 10), (1, 10), (1, 1)])
def test_stack_plan_is_the_largest_fitting_batch(built_lib, mode, substack):
    n, tpp = 2001, 720
    g = (tpp + substack - 1) // substack

    def bytes_of(npairs):
        return stack_bytes(mode, npairs * tpp, npairs, npairs * g, g, n)

    for budget in (bytes_of(1), bytes_of(3) + 5, bytes_of(40), 200 << 30):
        mt, bb = C.c_int64(), C.c_int64()
        lib().fxc_plan_stack_traces(mode, n, tpp, substack, budget, C.byref(mt), C.byref(bb))
        npairs = mt.value // tpp
        assert mt.value % tpp == 0 and npairs >= 1
        assert bb.value == bytes_of(npairs) <= budget < bytes_of(npairs + 1)
    with pytest.raises(FxcError, match="budget"):
        lib().fxc_plan_stack_traces(mode, n, tpp, substack, bytes_of(1) - 1, C.byref(C.c_int64()), None)
