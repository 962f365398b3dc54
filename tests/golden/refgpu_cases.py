"""Cases of the reference-kernel parity tests, shared by the live tests
(tests/test_refgpu_parity.py), the frozen-fixture tests
(tests/test_refgpu_golden.py) and the script that freezes the reference
kernels' outputs (tests/golden/make_ref_gpu_golden.py). Inputs are rebuilt
from seeds by fastxc_gb300.synthetic, so the fixture holds outputs only."""

from __future__ import annotations

from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

WHITEN_NONE, WHITEN_BEFORE, WHITEN_AFTER, WHITEN_BOTH = 0, 1, 2, 3
NORM_NONE, NORM_RUNABS_MF, NORM_ONEBIT, NORM_RUNABS = 0, 1, 2, 3

# (name, filter file, delta, whiten, normalize, phase_only, tolerance); a
# tolerance of None marks a case measured ill-conditioned for any FP32
# implementation, held to the reference's own FP32 error (see
# tests/test_refgpu_parity.py): RUN-ABS-MF at 0.2 s with the 0.1-1 / 0.5-2 Hz
# band set, whose 2 Hz upper edge sits close to the 2.5 Hz Nyquist frequency,
# where the prefilter's zero leaves bins of rounding noise that whitening
# brings back to O(1) (the reference kernels themselves sit 2e-5 to 7e-5
# from FP64 there)
S2S_CASES = [
    ("ram_after", "filter_d0.1_0.1-2.txt", 0.1, WHITEN_AFTER, NORM_RUNABS, 0, 1e-5),
    ("ram_before", "filter_d0.1_0.1-2.txt", 0.1, WHITEN_BEFORE, NORM_RUNABS, 0, 1e-5),
    ("plain", "filter_d0.1_0.1-2.txt", 0.1, WHITEN_NONE, NORM_NONE, 0, 1e-5),
    ("phase_both", "filter_d0.1_0.1-2.txt", 0.1, WHITEN_BOTH, NORM_NONE, 1, 1e-5),
    ("onebit_after", "filter_d0.1_0.1-2.txt", 0.1, WHITEN_AFTER, NORM_ONEBIT, 0, 1e-3),
    ("mf_after", "filter_d0.2_0.1-1_0.5-2.txt", 0.2, WHITEN_AFTER, NORM_RUNABS_MF, 0, None),
    ("mf_both", "filter_d0.2_0.1-1_0.5-2.txt", 0.2, WHITEN_BOTH, NORM_RUNABS_MF, 0, None),
    ("mf_1hz_smoke", "filter_d1.0_0.2-0.4_0.1-0.2.txt", 1.0, WHITEN_AFTER, NORM_RUNABS_MF, 0, 1e-5),
    ("ram_after_0.05", "filter_d0.05_0.05-5.txt", 0.05, WHITEN_AFTER, NORM_RUNABS, 0, 1e-5),
]
S2S_STEPS = [0, 7, 23]
S2S_NSTA = 2
# the fixture keeps one spectrum row per case: window S2S_STEPS[1], channel 1
GOLDEN_STEP, GOLDEN_CHAN = 1, 1

# chained sac2spec -> xc cases (4 stations x 3 components, one day, 24
# windows of 3600 s, every cross-station component pair): the plain
# configuration (0.1 s, RAM, whiten after, lag 100 s), and the reference's
# 1 Hz public smoke settings (bands 0.2/0.4 0.1/0.2 -> RUN-ABS-MF, whiten
# after, lag 100 s) on the same synthetic station model; tol as in S2S_CASES
CHAINS = {
    "plain": dict(filter_file="filter_d0.1_0.1-2.txt", delta=0.1, whiten=WHITEN_AFTER, normalize=NORM_RUNABS,
                  phase_only=0, nsta=4, steps=list(range(24)), lag=100.0, tol=1e-5),
    "smoke_1hz": dict(filter_file="filter_d1.0_0.2-0.4_0.1-0.2.txt", delta=1.0, whiten=WHITEN_AFTER,
                      normalize=NORM_RUNABS_MF, phase_only=0, nsta=4, steps=list(range(24)), lag=100.0, tol=1e-5),
}
PLAIN = CHAINS["plain"]

# (nsamples, substack) for PWS on 4 pairs of 40 traces
PWS_CASES = [(2001, 1), (2001, 10), (2000, 3), (4001, 5)]
PWS_PAIRS, PWS_TRACES = 4, 40
# (nsamples, substack, band) for TF-PWS on 2 pairs of 30 traces; band =
# (fmin, fmax, taper_hz), taper_hz < 0 selects 5 % of the band
TFPWS_CASES = [(2001, 10, None), (2001, 10, (0.05, 2.0, -1.0)), (1001, 3, None), (401, 2, (0.2, 1.5, 0.1))]
TFPWS_PAIRS, TFPWS_TRACES = 2, 30
TFPWS_DELTA = 0.1


def s2s_series(filter_file: str, delta: float, nsta: int, win: float = 3600.0, lag: float = 100.0, seed: int = 0):
    """(plan-independent) input series for a sac2spec case: float32
    [3*nsta][npts] of one day at ``delta``."""
    from fastxc_gb300 import synthetic as sy

    npts = int(round(86400 / delta))
    arr = sy.station_array(nsta, seed=seed)
    return sy.station_series(arr, npts, delta, seed=seed)


def pws_traces(n: int, substack: int) -> np.ndarray:
    from fastxc_gb300 import synthetic as sy

    return sy.ncf_traces(PWS_PAIRS, PWS_TRACES, n, seed=n + substack)


def tfpws_traces(n: int, substack: int) -> np.ndarray:
    from fastxc_gb300 import synthetic as sy

    return sy.ncf_traces(TFPWS_PAIRS, TFPWS_TRACES, n, seed=n + substack)


def golden_path() -> Path:
    return HERE / "refgpu_golden.npz"
