"""CPU checks against fixtures generated from the reference itself
(tests/golden/make_golden.py): sac2spec planning and filter responses from
the reference's C, filter files from the reference's Python designer, the
xc pair/task list from the reference's scheduler, and the reference's
cross-day linear stack."""

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import sac2spec_oracle as so
from oracle import xc_oracle as xo

G = Path(__file__).resolve().parent / "golden"
PLANS = json.loads((G / "plan_golden.json").read_text())


@pytest.mark.parametrize("case", range(len(PLANS)))
def test_oracle_plan_matches_reference_c(case):
    p = PLANS[case]
    flt = so.read_filter_file(G / p["filter_file"])
    op = so.make_plan(p["sac_len"], p["win_len"], p["shift_len"], p["xcorr_lag"], p["delta"], flt)
    for k in ("npts", "segment_pts", "shift_pts", "nstep", "output_nfft", "nspec", "filter_padding", "filter_nfft"):
        assert getattr(op, k) == p[k], k


@pytest.mark.parametrize("case", range(len(PLANS)))
def test_library_plan_and_responses_match_reference_c(built_lib, case):
    from fastxc_gb300 import sac2spec as s2s

    p = PLANS[case]
    F = s2s.read_filter_file(G / p["filter_file"])
    assert np.allclose(F.b, np.array(p["b"]), rtol=0, atol=0)
    assert np.allclose(F.a, np.array(p["a"]), rtol=0, atol=0)
    assert np.array_equal(F.freq_low, np.array(p["freq_low"], np.float32))
    plan = s2s.plan(p["sac_len"], p["win_len"], p["shift_len"], p["xcorr_lag"], p["delta"], F)
    for k in ("npts", "segment_pts", "shift_pts", "nstep", "output_nfft", "nspec", "filter_padding", "filter_nfft"):
        assert getattr(plan, k) == p[k], k
    got = s2s.filter_response(plan, F)
    ref = np.load(G / "response_golden.npz")
    for k in range(F.n):
        r = ref[f"case{case}_filter{k}"]
        assert got.shape[1] == r.size
        # same double-precision formula as the reference, rounded once to float
        assert np.max(np.abs(got[k].view(np.int32) - r.view(np.int32))) <= 1


@pytest.mark.parametrize("name,delta,bands", [
    ("filter_d0.1_0.1-2.txt", 0.1, "0.1/2"),
    ("filter_d1.0_0.2-0.4_0.1-0.2.txt", 1.0, "0.2/0.4 0.1/0.2"),
    ("filter_d0.05_0.05-5.txt", 0.05, "0.05/5"),
])
def test_oracle_filter_design_matches_reference_python(name, delta, bands):
    ref = so.read_filter_file(G / name)
    got = so.design_filters(delta, bands)
    assert len(ref) == len(got)
    for r, g in zip(ref, got):
        assert r.freq_low == pytest.approx(g.freq_low) and r.freq_high == pytest.approx(g.freq_high)
        # scipy's butter on another platform (libm, BLAS) may differ in the
        # last bits of the double coefficients
        assert np.allclose(r.b, g.b, rtol=1e-12, atol=1e-18)
        assert np.allclose(r.a, g.a, rtol=1e-12, atol=1e-18)


@pytest.mark.parametrize("case", range(5))
def test_oracle_tasks_match_reference_scheduler(case):
    c = json.loads((G / "xc_tasks_golden.json").read_text())[case]
    pids = {xo.make_allowed_path_id(a, b) for a, b in c["paths"]}
    got = []
    for j, job in enumerate(xo.build_jobs(len(c["gnsl"]), c["block_size"])):
        tasks, _ = xo.build_tasks_for_job(c["gnsl"], pids, job)
        got += [(t.src_meta_idx, t.rec_meta_idx, t.path_id, int(t.is_autocorr), j) for t in tasks]
    ref = list(zip(c["src"], c["rec"], c["path_id"], c["auto"], c["job"]))
    assert got == ref


def test_oracle_linear_stack_matches_reference_python():
    from oracle import stack_oracle

    d = np.load(G / "linear_stack_golden.npz")
    got = stack_oracle.linear_stack(d["traces"])
    assert got.dtype == np.float32
    assert np.array_equal(got, d["stacked"])
