"""Real data through the drop-in executables, against the reference.

One day of the reference's public smoke-test data (4 anonymised 1 Hz
stations, E/N/Z; tests/golden/example_1hz_sac.npz, copied from its
example/data by tests/golden/make_example_subset.py) with the settings of
its example/config.ini (win_len 3600 s, bands 0.2/0.4 0.1/0.2 -> RUN-ABS-MF,
whiten after, max_lag 100 s). This build's sac2spec and xc_fast executables
produce the 54 NCFs of the 6 station pairs; they are compared with the
reference's own kernels on the same data: live when those kernels are
built (oracle/ref_gpu.py), and against the frozen reference NCFs of
tests/golden/example_1hz_ref.npz.

Tolerance: relative L2 per NCF within max(1e-5, 2 x r64 + 1e-6) of the
reference, where r64 is the reference's own largest distance to the FP64
oracle on this data, and no further from the FP64 oracle than
max(1e-5, 1.5 x r64). RUN-ABS-MF on this day is ill-conditioned for any
FP32 implementation: the reference's kernels themselves sit about 2e-5 from
FP64, so two FP32 implementations cannot agree to 1e-5 unless they round
alike; the FP64 bound is the one that says which is closer to the exact
result.
"""

import hashlib
import json
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
import example_case as ex  # noqa: E402

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("method", ["plain", "tensor"])
def test_example_data_matches_frozen_reference(tmp_path, built_lib, torch_cuda, method):
    if not ex.GOLDEN.exists():
        pytest.skip("example_1hz_ref.npz not generated")
    z = np.load(ex.GOLDEN)
    sha = json.loads(str(z["sha256"]))
    r64 = json.loads(str(z["meta"]))["ref_vs_fp64"]
    sac = ex.load_sac()
    ours = ex.run_ours(tmp_path, sac, method)
    fp64 = ex.fp64_ncfs(sac)
    assert len(ours) == 54
    worst, e64 = 0.0, 0.0
    for k, v in ours.items():
        ref = z[ex.key_text(k)]
        assert hashlib.sha256(np.ascontiguousarray(ref).tobytes()).hexdigest() == sha[ex.key_text(k)]
        assert v.shape == ref.shape == (201,)
        worst = max(worst, rel(v, ref))
        e64 = max(e64, rel(v, fp64[k]))
    print(f"example data ({method}): max rel-L2 vs frozen reference {worst:.2e}; vs FP64 ours {e64:.2e}, "
          f"reference {r64:.2e}")
    assert worst < max(1e-5, 2 * r64 + 1e-6)
    assert e64 < max(1e-5, 1.5 * r64)


def test_example_data_matches_reference_kernels(tmp_path, built_lib, torch_cuda):
    from oracle import ref_gpu

    if not ref_gpu.available():
        pytest.skip("reference kernels not built")
    sac = ex.load_sac()
    ours = ex.run_ours(tmp_path, sac, "plain")
    ref, fp64 = ex.reference_ncfs(sac)
    assert set(ours) == set(ref)
    e = max(rel(ours[k], ref[k]) for k in ref)
    e64 = max(rel(ours[k], fp64[k]) for k in ref)
    r64 = max(rel(ref[k], fp64[k]) for k in ref)
    print(f"example data: vs reference kernels {e:.2e}; vs FP64 ours {e64:.2e}, reference {r64:.2e}")
    assert e < max(1e-5, 2 * r64 + 1e-6)
    assert e64 < max(1e-5, 1.5 * r64)
