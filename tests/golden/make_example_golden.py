"""Freezes the reference kernels' NCFs of the example_case.py workload.

Runs where a GPU and the reference's kernels (oracle/_ref/ref_*.cubin) are:

    python tests/golden/make_example_golden.py [output.npz]

Writes example_1hz_ref.npz: the 54 reference NCFs keyed "STA.C-STA.C", the
largest distance of the reference to the FP64 oracle, and a sha256 of every
array.
"""

from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
sys.path.insert(0, str(HERE))

import example_case as ex  # noqa: E402


def main(out: Path) -> None:
    ref, fp64 = ex.reference_ncfs(ex.load_sac())
    data = {ex.key_text(k): v.astype(np.float32) for k, v in ref.items()}
    e = max(float(np.linalg.norm(ref[k] - fp64[k]) / np.linalg.norm(fp64[k])) for k in ref)
    sha = {k: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() for k, v in data.items()}
    np.savez_compressed(out, meta=json.dumps({"ref_vs_fp64": e}), sha256=json.dumps(sha), **data)
    print("wrote", out, len(data), "NCFs; reference vs FP64", e)


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else ex.GOLDEN)
