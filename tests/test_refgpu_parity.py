"""Parity against the reference's own CUDA kernels on the same GPU.

``oracle/ref_gpu.py`` runs the reference's kernel sources (compiled with its
release flags, -O3 --use_fast_math) and cuFFT in the reference's host order.
These tests put this library's output beside that reference output on the
same seeded inputs, and state both against the FP64 oracle:

  * sac2spec spectra for every whitening / normalisation mode, including the
    RUN-ABS-MF band set of the reference's 1 Hz public smoke configuration
    (bands 0.2/0.4 0.1/0.2, whiten after, lag 100 s);
  * the NCFs of the plain configuration (4 stations x 3 components, one day
    at 0.1 s, 24 windows of 3600 s, RAM, whiten after, lag 100 s, 54
    component pairs) chained sac2spec -> xc in both implementations;
  * xc on synthetic spectra with gap windows, plain and tensor-core paths;
  * PWS and TF-PWS (with and without the band blend) on the same prestacks.

Tolerances: relative L2 1e-5 per row / NCF / stack against the reference
(one-bit spectra 1e-3: signs of samples within FP32 rounding of zero flip in
either implementation; phase-only spectra on bins above 1e-2 of the row
peak, the others being unit phasors of rounding noise).

One setting is ill-conditioned for any FP32 implementation: RUN-ABS-MF at
0.2 s with the 0.1-1 / 0.5-2 Hz bands, whose 2 Hz upper edge sits close to
the 2.5 Hz Nyquist frequency. The prefilter's zero at Nyquist leaves bins of
rounding noise there, which the whitening divides by their own smoothed
amplitude and brings back to O(1). The reference kernels themselves sit
2e-5 to 7e-5 from FP64 on it, and the exact figure moves with any change
of FFT rounding order; the bar is that this library stays within twice the
reference's FP64 distance of FP64, and within three times of the reference.

The reference kernels are device code built beside the reference tree; where
they are not present the tests skip (the frozen fixtures of
``tests/golden/refgpu_golden.npz`` cover the same cases without them, see
``test_refgpu_golden.py``).
"""

import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import refgpu_cases as cases  # noqa: E402
from oracle import ref_gpu
from oracle import sac2spec_oracle as so
from oracle import stack_oracle as sto
from oracle import xc_oracle as xo

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(), reason="reference kernels not built (oracle/build_ref.py)")]
G = Path(__file__).resolve().parent / "golden"


def rel_rows(got, ref):
    got = np.asarray(got).reshape(-1, np.asarray(got).shape[-1])
    ref = np.asarray(ref).reshape(-1, np.asarray(ref).shape[-1])
    num = np.linalg.norm(got - ref, axis=1)
    den = np.maximum(np.linalg.norm(ref, axis=1), 1e-30)
    return num / den


def s2s_ours(ctx, torch, filter_file, delta, whiten, normalize, phase_only, steps, nsta=2, win=3600.0, lag=100.0):
    """This library's sac2spec of the case's seeded series: (spectra
    [steps][rows][nspec], filter responses, series)."""
    from fastxc_gb300 import sac2spec as s2s

    F = s2s.read_filter_file(G / filter_file)
    plan = s2s.plan(86400, win, win, lag, delta, F, whiten, normalize, phase_only)
    resp = s2s.filter_response(plan, F)
    series = cases.s2s_series(filter_file, delta, nsta, win, lag)
    assert series.shape[1] == plan.npts
    nrows = series.shape[0]
    d_series = torch.from_numpy(series).cuda()
    d_resp = torch.from_numpy(resp).cuda()
    d_out = torch.zeros((len(steps), nrows, plan.nspec), dtype=torch.complex64, device="cuda")
    s2s.run(ctx, plan, d_series, plan.npts, plan.npts, nrows, 3, steps, d_resp, d_out, plan.nspec)
    ctx.synchronize()
    return d_out.cpu().numpy(), resp, series


def s2s_both(ctx, torch, filter_file, delta, whiten, normalize, phase_only, steps, nsta=2, win=3600.0, lag=100.0):
    """This library's sac2spec and the reference kernels' on the same series;
    returns (ours, reference, fp64 oracle, plan)."""
    ours, resp, series = s2s_ours(ctx, torch, filter_file, delta, whiten, normalize, phase_only, steps, nsta, win,
                                  lag)
    op = so.make_plan(86400, win, win, lag, delta, so.read_filter_file(G / filter_file), whiten, normalize,
                      phase_only)
    wins = so.windows(series, op, steps).astype(np.float32)
    ref = ref_gpu.sac2spec_rows(wins, op, resp, 3)
    fp64 = so.run_rows(wins.astype(np.float64), op, 3)
    return ours, ref, fp64, op


@pytest.mark.parametrize("name,filter_file,delta,whiten,normalize,phase_only,tol", cases.S2S_CASES,
                         ids=[c[0] for c in cases.S2S_CASES])
def test_sac2spec_matches_reference_kernels(ctx, torch_cuda, name, filter_file, delta, whiten, normalize, phase_only,
                                            tol):
    steps = cases.S2S_STEPS
    ours, ref, fp64, _ = s2s_both(ctx, torch_cuda, filter_file, delta, whiten, normalize, phase_only, steps,
                                  cases.S2S_NSTA)
    assert np.all(np.isfinite(ours)) and np.all(np.isfinite(ref))
    if phase_only:
        _, amp, _, _ = s2s_both(ctx, torch_cuda, filter_file, delta, whiten, normalize, 0, steps)
        a = np.abs(amp)
        keep = a > 1e-2 * a.max(axis=-1, keepdims=True)
        ours, ref, fp64 = (np.where(keep, v, 0) for v in (ours, ref, fp64))
        assert keep.mean() > 0.3
    e_ref = rel_rows(ours, ref)
    e_ours64, e_ref64 = rel_rows(ours, fp64).max(), rel_rows(ref, fp64).max()
    print(f"sac2spec vs reference kernels: max {e_ref.max():.2e}; vs FP64: ours {e_ours64:.2e}, "
          f"reference {e_ref64:.2e}")
    if tol is None:  # ill-conditioned: held to the reference's own FP32 error
        assert e_ours64 <= 2.0 * e_ref64 + 1e-6, (e_ours64, e_ref64)
        assert e_ref.max() <= 3.0 * e_ref64 + 1e-6, (e_ref.max(), e_ref64)
    else:
        assert e_ref.max() < tol, e_ref


@pytest.mark.parametrize("chain", list(cases.CHAINS))
def test_chained_ncfs_match_reference_kernels(ctx, torch_cuda, chain):
    """4 stations x 3 components, one day: sac2spec then xc in each
    implementation; every one of the 54 NCFs within 1e-5 of the reference's."""
    torch = torch_cuda
    from fastxc_gb300 import _lib as L
    from fastxc_gb300 import synthetic as sy
    from fastxc_gb300.core import PairPlan, xc_shape

    p = cases.CHAINS[chain]
    ours_spec, ref_spec, fp64_spec, op = s2s_both(ctx, torch, p["filter_file"], p["delta"], p["whiten"],
                                                  p["normalize"], p["phase_only"], p["steps"], p["nsta"],
                                                  lag=p["lag"])
    src, rec = sy.cross_station_pairs(p["nsta"])
    nwin, nchan, nspec = ours_spec.shape
    shape = xc_shape(nspec, nwin, p["delta"], p["lag"])
    ref_ncf = ref_gpu.xc_run(ref_spec, src, rec, shape.nfft, shape.half_cc, shape.dt)
    fp64_ncf = xo.xc_run(fp64_spec, src, rec, 1.0 / nwin, xo.finalize_shape(nspec, nwin, p["delta"], p["lag"]))
    e_ref64 = rel_rows(ref_ncf, fp64_ncf).max()
    plan = PairPlan(ctx, src, rec, nchan)
    d_spec = torch.from_numpy(ours_spec).cuda()
    try:
        for method in (L.FXC_XC_PLAIN, L.FXC_XC_TENSOR):
            d_ncf = torch.empty((len(src), shape.cc_size), dtype=torch.float32, device="cuda")
            ctx.xc_run(plan, d_spec, nwin, nchan, nspec, None, 1.0 / nwin, shape, d_ncf, method)
            ctx.synchronize()
            ours = d_ncf.cpu().numpy()
            e = rel_rows(ours, ref_ncf)
            e64 = rel_rows(ours, fp64_ncf).max()
            print(f"{chain} NCFs method {method}: vs reference kernels max {e.max():.2e}; vs FP64 ours "
                  f"{e64:.2e}, reference {e_ref64:.2e}")
            if p["tol"] is None:
                assert e64 <= 1.5 * e_ref64 + 1e-6, (e64, e_ref64)
                assert e.max() <= 2.0 * e_ref64 + 1e-6, (e.max(), e_ref64)
            else:
                assert e.max() < p["tol"], e.max()
    finally:
        plan.close()


def test_sac2spec_large_offset_matches_reference_kernels(ctx, torch_cuda):
    """A large DC offset and a steep trend over 72 000-sample windows: the
    reference's FP64-summed detrend against this library's compensated FP32
    one, both checked against FP64."""
    torch = torch_cuda
    from fastxc_gb300 import sac2spec as s2s
    from fastxc_gb300 import synthetic as sy

    delta, ff = 0.05, "filter_d0.05_0.05-5.txt"
    F = s2s.read_filter_file(G / ff)
    plan = s2s.plan(86400, 3600, 3600, 100, delta, F, so.WHITEN_AFTER, so.NORM_RUNABS, False)
    resp = s2s.filter_response(plan, F)
    series = sy.station_series(sy.station_array(1, seed=3), plan.npts, delta, seed=3).astype(np.float64)
    series = (series + 1.0e4 + 50.0 * np.arange(plan.npts)[None, :] / plan.npts).astype(np.float32)
    steps = [0, 11]
    d_out = torch.zeros((len(steps), 3, plan.nspec), dtype=torch.complex64, device="cuda")
    s2s.run(ctx, plan, torch.from_numpy(series).cuda(), plan.npts, plan.npts, 3, 3, steps,
            torch.from_numpy(resp).cuda(), d_out, plan.nspec)
    ctx.synchronize()
    ours = d_out.cpu().numpy()
    op = so.make_plan(86400, 3600, 3600, 100, delta, so.read_filter_file(G / ff), so.WHITEN_AFTER, so.NORM_RUNABS, 0)
    wins = so.windows(series, op, steps).astype(np.float32)
    ref = ref_gpu.sac2spec_rows(wins, op, resp, 3)
    fp64 = so.run_rows(wins.astype(np.float64), op, 3)
    e, e64, r64 = rel_rows(ours, ref).max(), rel_rows(ours, fp64).max(), rel_rows(ref, fp64).max()
    print(f"large offset: vs reference kernels {e:.2e}; vs FP64 ours {e64:.2e}, reference {r64:.2e}")
    assert e < 1e-5 and e64 < 1e-5


@pytest.mark.parametrize("nsta,nwin,nspec,lag", [(4, 24, 18523, 100.0), (7, 48, 9262, 50.0), (3, 5, 1001, 20.0)])
def test_xc_matches_reference_kernels(ctx, torch_cuda, nsta, nwin, nspec, lag):
    """Synthetic spectra with gap windows (zeroed); plain and tensor paths
    against accumulateStepXc2DKernel + finalize_xc_batch."""
    torch = torch_cuda
    from fastxc_gb300 import _lib as L
    from fastxc_gb300 import synthetic as sy
    from fastxc_gb300.core import PairPlan, xc_shape

    arr = sy.station_array(nsta, seed=nsta)
    d_spec, mask = sy.spectra_device(torch, nwin, arr, nspec, 0.1, seed=nsta, gap_frac=0.1)
    src, rec = sy.cross_station_pairs(nsta, auto=True)
    shape = xc_shape(nspec, nwin, 0.1, lag)
    ref = ref_gpu.xc_run(None, src, rec, shape.nfft, shape.half_cc, shape.dt, d_spec=d_spec)
    plan = PairPlan(ctx, src, rec, arr.nchan)
    try:
        for method in (L.FXC_XC_PLAIN, L.FXC_XC_TENSOR):
            d_ncf = torch.empty((len(src), shape.cc_size), dtype=torch.float32, device="cuda")
            ctx.xc_run(plan, d_spec, nwin, arr.nchan, nspec, None, 1.0 / nwin, shape, d_ncf, method)
            ctx.synchronize()
            e = rel_rows(d_ncf.cpu().numpy(), ref)
            print(f"xc {nsta} sta {nwin} win method {method}: max {e.max():.2e}")
            assert e.max() < 1e-5, e.max()
    finally:
        plan.close()


def _prestacked(ctx, torch, tr, substack, mode):
    from fastxc_gb300 import stack

    npairs, nt, n = tr.shape
    d_tr = torch.from_numpy(np.ascontiguousarray(tr.reshape(npairs * nt, n))).cuda()
    offs = np.arange(npairs, dtype=np.int64) * nt
    return stack.prestack(ctx, torch, d_tr, offs, [nt] * npairs, n, substack, mode)


@pytest.mark.parametrize("n,substack", cases.PWS_CASES)
def test_pws_matches_reference_kernels(ctx, torch_cuda, n, substack):
    torch = torch_cuda
    from fastxc_gb300 import stack

    tr = cases.pws_traces(n, substack)
    npairs = tr.shape[0]
    g, w, lin, goff, gcnt = _prestacked(ctx, torch, tr, substack, stack.MODE_PWS)
    out = torch.empty((npairs, n), dtype=torch.float32, device="cuda")
    stack.pws(ctx, g, w, goff, gcnt, lin, n, out, 1.0)
    ctx.synchronize()
    ours = out.cpu().numpy()
    ngroups = int(np.sum(gcnt))
    ref = ref_gpu.pws_run(g.cpu().numpy()[:ngroups], w.cpu().numpy()[:ngroups], gcnt, lin.cpu().numpy())
    fp64 = np.stack([sto.pws(tr[p], substack, 1.0) for p in range(npairs)])
    e = rel_rows(ours, ref)
    print(f"pws n={n} B={substack}: vs reference kernels {e.max():.2e}; vs FP64 ours {rel_rows(ours, fp64).max():.2e}"
          f", reference {rel_rows(ref, fp64).max():.2e}")
    assert e.max() < 1e-5, e


@pytest.mark.parametrize("n,substack,band", cases.TFPWS_CASES)
def test_tfpws_matches_reference_kernels(ctx, torch_cuda, n, substack, band):
    torch = torch_cuda
    from fastxc_gb300 import stack

    tr = cases.tfpws_traces(n, substack)
    npairs = tr.shape[0]
    g, w, lin, goff, gcnt = _prestacked(ctx, torch, tr, substack, stack.MODE_TFPWS)
    out = torch.empty((npairs, n), dtype=torch.float32, device="cuda")
    stack.tfpws(ctx, g, w, goff, gcnt, lin, n, out, cases.TFPWS_DELTA, band=None if band is None else band[:2],
                taper_hz=-1.0 if band is None else band[2], power=1.0)
    ctx.synchronize()
    ours = out.cpu().numpy()
    gh, wh, lh = g.cpu().numpy(), w.cpu().numpy(), lin.cpu().numpy()
    ref = np.stack([ref_gpu.tfpws_run(gh[goff[p]: goff[p] + gcnt[p]], wh[goff[p]: goff[p] + gcnt[p]], lh[p],
                                      cases.TFPWS_DELTA, band=band) for p in range(npairs)])
    fp64 = np.stack([sto.tfpws(tr[p], substack, 1.0, band=None if band is None else band[:2], delta=cases.TFPWS_DELTA,
                               taper_hz=-1.0 if band is None else band[2]) for p in range(npairs)])
    e = rel_rows(ours, ref)
    print(f"tfpws n={n} B={substack} band={band}: vs reference kernels {e.max():.2e}; vs FP64 ours "
          f"{rel_rows(ours, fp64).max():.2e}, reference {rel_rows(ref, fp64).max():.2e}")
    assert e.max() < 1e-5, e
