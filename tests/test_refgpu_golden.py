"""Parity against frozen outputs of the reference's own CUDA kernels.

``tests/golden/refgpu_golden.npz`` holds what the reference's kernels and
cuFFT produced on a GB300 for the cases of ``tests/golden/refgpu_cases.py``
(made by ``tests/golden/make_ref_gpu_golden.py`` through
``oracle/ref_gpu.py``). The inputs are rebuilt here from their seeds, run
through this library, and compared with the stored outputs, so this file
needs neither the reference tree nor its built kernels.

Tolerances as in ``tests/test_refgpu_parity.py``: relative L2 1e-5 (one-bit
1e-3; phase-only on bins above 1e-2 of the row peak; the settings whose
whitening reaches the Nyquist frequency within twice the reference's own
distance to FP64, which the fixture stores, x3 against the frozen reference).
"""

import hashlib
import json
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
sys.path.insert(0, str(HERE))
import refgpu_cases as cases  # noqa: E402

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cases.golden_path().exists(), reason="refgpu_golden.npz not generated")]


@pytest.fixture(scope="module")
def gold():
    z = np.load(cases.golden_path())
    data = {k: z[k] for k in z.files if k not in ("meta", "sha256")}
    meta = json.loads(str(z["meta"]))
    sha = json.loads(str(z["sha256"]))
    for k, v in data.items():
        assert hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() == sha[k], k
    return data, meta


def rel_rows(got, ref):
    got = np.asarray(got).reshape(-1, np.asarray(got).shape[-1])
    ref = np.asarray(ref).reshape(-1, np.asarray(ref).shape[-1])
    return np.linalg.norm(got - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-30)


@pytest.mark.parametrize("name,filter_file,delta,whiten,normalize,phase_only,tol", cases.S2S_CASES,
                         ids=[c[0] for c in cases.S2S_CASES])
def test_sac2spec_matches_frozen_reference(ctx, torch_cuda, gold, name, filter_file, delta, whiten, normalize,
                                           phase_only, tol):
    from test_refgpu_parity import s2s_ours

    data, meta = gold
    ours, _, _ = s2s_ours(ctx, torch_cuda, filter_file, delta, whiten, normalize, phase_only, cases.S2S_STEPS,
                          cases.S2S_NSTA)
    row = ours[cases.GOLDEN_STEP, cases.GOLDEN_CHAN]
    ref = data[f"s2s_{name}"]
    if phase_only:
        amp, _, _ = s2s_ours(ctx, torch_cuda, filter_file, delta, whiten, normalize, 0, cases.S2S_STEPS,
                             cases.S2S_NSTA)
        a = np.abs(amp[cases.GOLDEN_STEP, cases.GOLDEN_CHAN])
        keep = a > 1e-2 * a.max()
        row, ref = np.where(keep, row, 0), np.where(keep, ref, 0)
    e = rel_rows(row, ref).max()
    print(f"{name}: vs frozen reference {e:.2e} (reference vs FP64 {meta[f's2s_{name}_ref_vs_fp64']:.2e})")
    bound = 3.0 * meta[f"s2s_{name}_ref_vs_fp64"] + 1e-6 if tol is None else tol
    assert e < bound, (e, bound)


@pytest.mark.parametrize("chain", list(cases.CHAINS))
def test_chained_ncfs_match_frozen_reference(ctx, torch_cuda, gold, chain):
    torch = torch_cuda
    from fastxc_gb300 import _lib as L
    from fastxc_gb300 import synthetic as sy
    from fastxc_gb300.core import PairPlan, xc_shape
    from test_refgpu_parity import s2s_ours

    data, meta = gold
    p = cases.CHAINS[chain]
    spec, _, _ = s2s_ours(ctx, torch, p["filter_file"], p["delta"], p["whiten"], p["normalize"], p["phase_only"],
                          p["steps"], p["nsta"], lag=p["lag"])
    src, rec = sy.cross_station_pairs(p["nsta"])
    nwin, nchan, nspec = spec.shape
    shape = xc_shape(nspec, nwin, p["delta"], p["lag"])
    ref64 = meta[f"{chain}_ncf_ref_vs_fp64"]
    bound = 2.0 * ref64 + 1e-6 if p["tol"] is None else p["tol"]
    plan = PairPlan(ctx, src, rec, nchan)
    d_spec = torch.from_numpy(spec).cuda()
    try:
        for method in (L.FXC_XC_PLAIN, L.FXC_XC_TENSOR):
            d_ncf = torch.empty((len(src), shape.cc_size), dtype=torch.float32, device="cuda")
            ctx.xc_run(plan, d_spec, nwin, nchan, nspec, None, 1.0 / nwin, shape, d_ncf, method)
            ctx.synchronize()
            e = rel_rows(d_ncf.cpu().numpy(), data[f"{chain}_ncf"])
            print(f"{chain} NCFs method {method}: max {e.max():.2e} (reference vs FP64 {ref64:.2e})")
            assert e.max() < bound, (e.max(), bound)
    finally:
        plan.close()


def _prestacked(ctx, torch, tr, substack, mode):
    from fastxc_gb300 import stack

    npairs, nt, n = tr.shape
    d_tr = torch.from_numpy(np.ascontiguousarray(tr.reshape(npairs * nt, n))).cuda()
    offs = np.arange(npairs, dtype=np.int64) * nt
    return stack.prestack(ctx, torch, d_tr, offs, [nt] * npairs, n, substack, mode)


@pytest.mark.parametrize("n,substack", cases.PWS_CASES)
def test_pws_matches_frozen_reference(ctx, torch_cuda, gold, n, substack):
    torch = torch_cuda
    from fastxc_gb300 import stack

    data, _ = gold
    tr = cases.pws_traces(n, substack)
    g, w, lin, goff, gcnt = _prestacked(ctx, torch, tr, substack, stack.MODE_PWS)
    out = torch.empty((tr.shape[0], n), dtype=torch.float32, device="cuda")
    stack.pws(ctx, g, w, goff, gcnt, lin, n, out, 1.0)
    ctx.synchronize()
    e = rel_rows(out.cpu().numpy(), data[f"pws_{n}_{substack}"])
    assert e.max() < 1e-5, e


@pytest.mark.parametrize("n,substack,band", cases.TFPWS_CASES)
def test_tfpws_matches_frozen_reference(ctx, torch_cuda, gold, n, substack, band):
    torch = torch_cuda
    from fastxc_gb300 import stack

    data, _ = gold
    tr = cases.tfpws_traces(n, substack)
    g, w, lin, goff, gcnt = _prestacked(ctx, torch, tr, substack, stack.MODE_TFPWS)
    out = torch.empty((tr.shape[0], n), dtype=torch.float32, device="cuda")
    stack.tfpws(ctx, g, w, goff, gcnt, lin, n, out, cases.TFPWS_DELTA, band=None if band is None else band[:2],
                taper_hz=-1.0 if band is None else band[2], power=1.0)
    ctx.synchronize()
    e = rel_rows(out.cpu().numpy(), data[f"tfpws_{n}_{substack}_{'band' if band else 'full'}"])
    assert e.max() < 1e-5, e
