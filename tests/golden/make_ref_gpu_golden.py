"""Freezes the reference kernels' outputs on the cases of refgpu_cases.py.

Runs where a GPU and the reference's kernels (oracle/_ref/ref_*.cubin, built
by oracle/build_ref.py beside the reference tree) are present:

    python tests/golden/make_ref_gpu_golden.py [output.npz]

and writes refgpu_golden.npz (default: next to this script): for every
sac2spec case one spectrum row, the 54 NCFs of each chained sac2spec -> xc
case, and the PWS / TF-PWS stacks, all computed by
oracle/ref_gpu.py (the reference's kernels + cuFFT in the reference's host
order). The distance of each to the FP64 oracle is stored beside it, and a
sha256 of every array in the ``sha256`` entry.
"""

from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

import refgpu_cases as cases  # noqa: E402
from oracle import ref_gpu  # noqa: E402
from oracle import sac2spec_oracle as so  # noqa: E402
from oracle import stack_oracle as sto  # noqa: E402
from oracle import xc_oracle as xo  # noqa: E402


def rel(a, b):
    a = np.asarray(a).reshape(-1, np.asarray(a).shape[-1])
    b = np.asarray(b).reshape(-1, np.asarray(b).shape[-1])
    return float((np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-30)).max())


def sac2spec_ref(filter_file, delta, whiten, normalize, phase_only, steps, nsta, lag=100.0):
    flt = so.read_filter_file(HERE / filter_file)
    op = so.make_plan(86400, 3600, 3600, lag, delta, flt, whiten, normalize, phase_only)
    series = cases.s2s_series(filter_file, delta, nsta)
    wins = so.windows(series, op, steps).astype(np.float32)
    ref = ref_gpu.sac2spec_rows(wins, op, op.responses, 3)
    fp64 = so.run_rows(wins.astype(np.float64), op, 3)
    return ref, fp64, op


def main(out: Path) -> None:
    data: dict[str, np.ndarray] = {}
    meta: dict[str, float] = {}
    for name, ff, delta, wh, nm, ph, _tol in cases.S2S_CASES:
        ref, fp64, _ = sac2spec_ref(ff, delta, wh, nm, ph, cases.S2S_STEPS, cases.S2S_NSTA)
        data[f"s2s_{name}"] = ref[cases.GOLDEN_STEP, cases.GOLDEN_CHAN].astype(np.complex64)
        meta[f"s2s_{name}_ref_vs_fp64"] = rel(ref, fp64)
        print(name, meta[f"s2s_{name}_ref_vs_fp64"])
    from fastxc_gb300 import synthetic as sy

    for chain, p in cases.CHAINS.items():
        ref, fp64, _ = sac2spec_ref(p["filter_file"], p["delta"], p["whiten"], p["normalize"], p["phase_only"],
                                    p["steps"], p["nsta"], p["lag"])
        src, rec = sy.cross_station_pairs(p["nsta"])
        nwin, _, nspec = ref.shape
        shape = xo.finalize_shape(nspec, nwin, p["delta"], p["lag"])
        ncf = ref_gpu.xc_run(ref, src, rec, shape.nfft, shape.half_cc, shape.dt)
        ncf64 = xo.xc_run(fp64, src, rec, 1.0 / nwin, shape)
        data[f"{chain}_ncf"] = ncf.astype(np.float32)
        meta[f"{chain}_ncf_ref_vs_fp64"] = rel(ncf, ncf64)
        print(chain, "ncf", meta[f"{chain}_ncf_ref_vs_fp64"])
    for n, b in cases.PWS_CASES:
        tr = cases.pws_traces(n, b)
        gs, ws, ls, cnt = [], [], [], []
        for q in range(tr.shape[0]):
            g, w, lin = sto.pws_prestack(tr[q], b)
            gs.append(g)
            ws.append(w)
            ls.append(lin)
            cnt.append(len(w))
        out_ref = ref_gpu.pws_run(np.concatenate(gs).astype(np.float32), np.concatenate(ws).astype(np.float32), cnt,
                                  np.stack(ls).astype(np.float32))
        data[f"pws_{n}_{b}"] = out_ref
        meta[f"pws_{n}_{b}_ref_vs_fp64"] = rel(out_ref, np.stack([sto.pws(tr[q], b, 1.0) for q in range(tr.shape[0])]))
    for n, b, band in cases.TFPWS_CASES:
        tr = cases.tfpws_traces(n, b)
        outs = []
        for q in range(tr.shape[0]):
            g, w, lin = sto.tfpws_prestack(tr[q], b)
            outs.append(ref_gpu.tfpws_run(g.astype(np.float32), w.astype(np.float32), lin.astype(np.float32),
                                          cases.TFPWS_DELTA, band=band))
        key = f"tfpws_{n}_{b}_{'band' if band else 'full'}"
        data[key] = np.stack(outs)
        fp = np.stack([sto.tfpws(tr[q], b, 1.0, band=None if band is None else band[:2], delta=cases.TFPWS_DELTA,
                                 taper_hz=None if band is None else band[2]) for q in range(tr.shape[0])])
        meta[f"{key}_ref_vs_fp64"] = rel(data[key], fp)
    sha = {k: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() for k, v in data.items()}
    np.savez_compressed(out, meta=json.dumps(meta), sha256=json.dumps(sha), **data)
    print("wrote", out, json.dumps(meta, indent=1))


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else cases.golden_path())
