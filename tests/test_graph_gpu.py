"""CUDA-graph capture of a day's launch sequence (fxc_graph_*).

One day of correlation (pack -> tensor-core contraction -> finalize, and
the plain stack -> finalize) is run directly once (sizing the context's
scratch and FFT tables), then recorded into a graph and replayed twice; the
replayed NCFs are bit-identical to the direct ones. A context on the legacy
default stream refuses to record.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_graph_replay_equals_direct_run(built_lib, torch_cuda):
    torch = torch_cuda
    from fastxc_gb300 import _lib as L
    from fastxc_gb300.core import Context, PairPlan, xc_shape
    from fastxc_gb300.synthetic import cross_station_pairs, spectra_device, station_array

    stream = torch.cuda.Stream()
    nsta, nwin, nspec = 9, 24, 4001
    arr = station_array(nsta, seed=2)
    with torch.cuda.stream(stream):
        spec, mask = spectra_device(torch, nwin, arr, nspec, 0.1, seed=2, gap_frac=0.1)
    stream.synchronize()
    d_mask = torch.from_numpy(mask).cuda()
    src, rec = cross_station_pairs(nsta)
    shape = xc_shape(nspec, nwin, 0.1, 50.0)
    pitch = (nspec + 3) // 4 * 4
    with Context(0, stream.cuda_stream) as ctx:
        plan = PairPlan(ctx, src, rec, arr.nchan)
        packed = torch.empty((Context.xc_packed_bytes(arr.nchan, nwin, nspec) // 16, 4), dtype=torch.int32,
                             device="cuda")
        stack = torch.empty((src.size, pitch), dtype=torch.complex64, device="cuda")
        out = {m: torch.empty((src.size, shape.cc_size), dtype=torch.float32, device="cuda") for m in (0, 1)}

        def day():
            ctx.xc_pack(spec, nwin, arr.nchan, nspec, nspec, d_mask, packed)
            ctx.xc_stack_packed(plan, packed, nwin, nspec, 1.0 / nwin, stack, pitch)
            ctx.xc_finalize(stack, src.size, pitch, shape, out[1])
            ctx.xc_stack(plan, spec, nwin, arr.nchan, nspec, nspec, d_mask, 1.0 / nwin, stack, pitch, L.FXC_XC_PLAIN)
            ctx.xc_finalize(stack, src.size, pitch, shape, out[0])

        day()
        ctx.synchronize()
        direct = {m: o.cpu().numpy().copy() for m, o in out.items()}
        ctx.graph_begin()
        day()
        g = ctx.graph_end()
        for _ in range(2):
            for o in out.values():
                o.fill_(float("nan"))
            stream.synchronize()
            g.launch()
            ctx.synchronize()
            for m, o in out.items():
                assert np.array_equal(o.cpu().numpy(), direct[m]), m
        g.close()
        plan.close()


def test_graph_needs_a_non_default_stream(built_lib, torch_cuda):
    from fastxc_gb300 import FxcError
    from fastxc_gb300.core import Context

    with Context(0) as ctx, pytest.raises(FxcError, match="non-default stream"):
        ctx.graph_begin()
