"""sac2spec parity: library output spectra against the FP64 oracle on seeded
synthetic series (noise + a shared band-limited source delayed per station,
NaNs and a zero-filled gap), for every whitening / normalisation mode.

Tolerance: relative L2 1e-5 per output row (FP32 GPU vs FP64 oracle); the
one-bit mode can flip the sign of samples within FP32 rounding of zero, so
its rows are held to 1e-3.
"""

from pathlib import Path

import numpy as np
import pytest

from oracle import sac2spec_oracle as so

pytestmark = pytest.mark.gpu
G = Path(__file__).resolve().parent / "golden"


def synth_series(nsta, ncomp, npts, delta, seed=0):
    rng = np.random.default_rng(seed)
    from scipy.signal import butter, sosfiltfilt

    sos = butter(4, [0.1, 2.0], "bandpass", fs=1 / delta, output="sos")
    src = sosfiltfilt(sos, rng.standard_normal(npts + 4000))
    x = np.empty((nsta * ncomp, npts), np.float32)
    for s in range(nsta):
        lag = 300 + 150 * s
        for c in range(ncomp):
            x[s * ncomp + c] = (rng.standard_normal(npts) + 3.0 * src[lag: lag + npts] * (1 + 0.2 * c)).astype(np.float32)
    x[1, 1000:1003] = np.nan
    x[2, 50000:50010] = np.inf
    x[3, 200000:240000] = 0.0  # a gap inside window 5/6
    return x


def run_case(ctx, torch, filter_file, delta, whiten, normalize, phase_only, steps, nsta=2, ncomp=3,
             npts_days=1.0, short_by=0):
    from fastxc_gb300 import sac2spec as s2s

    sac_len = 86400 * npts_days
    F = s2s.read_filter_file(G / filter_file)
    plan = s2s.plan(sac_len, 3600, 3600, 100, delta, F, whiten, normalize, phase_only)
    resp = s2s.filter_response(plan, F)
    npts = plan.npts
    series = synth_series(nsta, ncomp, npts, delta)
    nvalid = npts - short_by
    d_series = torch.from_numpy(series).cuda()
    d_resp = torch.from_numpy(resp).cuda()
    nrows = nsta * ncomp
    d_out = torch.zeros((len(steps), nrows, plan.nspec), dtype=torch.complex64, device="cuda")
    s2s.run(ctx, plan, d_series, npts, nvalid, nrows, ncomp, steps, d_resp, d_out, plan.nspec)
    ctx.synchronize()
    got = d_out.cpu().numpy()

    flt = so.read_filter_file(G / filter_file)
    op = so.make_plan(sac_len, 3600, 3600, 100, delta, flt, whiten, normalize, phase_only)
    ser = series.astype(np.float64).copy()
    if short_by:
        ser[:, nvalid:] = 0.0
    wins = so.windows(ser, op, steps)
    ref = so.run_rows(wins, op, ncomp)
    return got, ref


def row_err(got, ref):
    num = np.linalg.norm((got - ref).reshape(-1, got.shape[-1]), axis=1)
    den = np.maximum(np.linalg.norm(ref.reshape(-1, ref.shape[-1]), axis=1), 1e-30)
    return num / den


@pytest.mark.parametrize("whiten,normalize,phase_only,tol", [
    (so.WHITEN_AFTER, so.NORM_RUNABS, 0, 1e-5),
    (so.WHITEN_NONE, so.NORM_RUNABS, 0, 1e-5),
    (so.WHITEN_BEFORE, so.NORM_RUNABS, 0, 1e-5),
    (so.WHITEN_BOTH, so.NORM_NONE, 1, 1e-5),
    (so.WHITEN_AFTER, so.NORM_ONEBIT, 0, 1e-3),
    (so.WHITEN_NONE, so.NORM_NONE, 0, 1e-5),
])
def test_sac2spec_modes_match_oracle(ctx, torch_cuda, whiten, normalize, phase_only, tol):
    got, ref = run_case(ctx, torch_cuda, "filter_d0.1_0.1-2.txt", 0.1, whiten, normalize, phase_only, [0, 5, 23])
    err = row_err(got, ref)
    assert np.all(np.isfinite(got))
    assert err.max() < tol, err


def test_sac2spec_runabs_mf_matches_oracle(ctx, torch_cuda):
    got, ref = run_case(ctx, torch_cuda, "filter_d0.2_0.1-1_0.5-2.txt", 0.2, so.WHITEN_AFTER, so.NORM_RUNABS_MF, 0,
                        [0, 11])
    assert row_err(got, ref).max() < 1e-5


def test_sac2spec_short_series_zero_padded(ctx, torch_cuda):
    """A series shorter than sac_len is zero-padded (read_sac_buffer)."""
    got, ref = run_case(ctx, torch_cuda, "filter_d0.1_0.1-2.txt", 0.1, so.WHITEN_AFTER, so.NORM_RUNABS, 0, [22, 23],
                        short_by=50000)
    assert row_err(got, ref).max() < 1e-5


def test_sac2spec_rejects_bad_steps(ctx, torch_cuda):
    from fastxc_gb300 import FxcError

    with pytest.raises(FxcError):
        run_case(ctx, torch_cuda, "filter_d0.1_0.1-2.txt", 0.1, so.WHITEN_AFTER, so.NORM_RUNABS, 0, [24])
