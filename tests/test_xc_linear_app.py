"""xc_linear (one pass from stepack to the cross-timestamp linear stack)
against the chain it replaces: xc_fast per timestamp -> SourcePack
materializer -> linear stack of SourcePack records (whose outputs are pinned
to the reference's own operators in test_operators*.py).

Three timestamps; one station is missing on the second, so some groups
average fewer records. Index rows, _SUCCESS texts and SAC headers must be
identical (stack folders aside); samples agree to float32 rounding (one
inverse transform of the summed stacks instead of an FP64 mean of
per-timestamp transforms)."""

from __future__ import annotations

import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
BIN = ROOT / "fastxc_gb300" / "bin"
NCF_RTOL = 1e-5


def make_days(tmp: Path, nspec=1001, nstep=6, seed=4):
    from fastxc_gb300 import formats

    rng = np.random.default_rng(seed)
    nsl = [3, 7, 12, 20]
    sp = tmp / "stepack"
    dt, df = 0.1, 1.0 / (2 * (nspec - 1) * 0.1)
    for d, ts in enumerate(("2020.123.0000", "2020.124.0000", "2020.125.0000")):
        chans = []
        for s, g in enumerate(nsl):
            if d == 1 and g == 12:
                continue  # station 12 is missing on the second day
            for c in "ENZ":
                chans.append(dict(timestamp=ts, nsl_id=g, network="XX", station=f"ST{g:02d}", location="00",
                                  component=f"BH{c}", stla=30.0 + s, stlo=100.0 + s))
        spec = (rng.standard_normal((nstep, len(chans), nspec)) +
                1j * rng.standard_normal((nstep, len(chans), nspec))).astype(np.complex64)
        formats.write_stepack(sp, 0, d, chans, spec, dt, df, group_count=len(chans) // 3)
    rows = [(a, b, 0.5, 55.5 + a, 10.0 + b, 190.0) for a in nsl for b in nsl if a < b and not (a == 3 and b == 20)]
    rows.append((7, 7, 0.0, 0.0, 0.0, 0.0))
    formats.write_allowed_paths(tmp / "allowed_paths.tsv", rows)


def read_pack(path: Path, npts: int):
    raw = path.read_bytes()
    rec = 632 + 4 * npts
    return ([raw[k:k + 632] for k in range(0, len(raw), rec)],
            np.stack([np.frombuffer(raw[k + 632:k + rec], "<f4") for k in range(0, len(raw), rec)]))


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["plain", "tensor"])
def test_xc_linear_equals_xc_fast_materializer_linear_stack(tmp_path, built_lib, ctx, method):
    from fastxc_gb300 import linear, sourcepack

    tmp = tmp_path.resolve()
    make_days(tmp)
    env = dict(os.environ, FASTXC_XC_METHOD=method, FASTXC_LOG_LEVEL="warn")
    common = ["-I", str(tmp / "stepack"), "-P", str(tmp / "allowed_paths.tsv"), "-O", str(tmp / "ncf"), "-C", "20"]
    r = subprocess.run([str(BIN / "xc_fast"), *common], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    sourcepack.build_sourcepack(tmp / "ncf", tmp / "sourcepack")
    chain = linear.linear_stack_sourcepack_indexes(sourcepack.discover_sourcepack_indexes(tmp / "sourcepack"),
                                                   tmp / "stack_chain", ctx=ctx)
    prog = tmp / "lin_progress.tsv"
    r = subprocess.run([str(BIN / "xc_linear"), *common, "-S", str(tmp / "stack_fused"), "--progress", str(prog)],
                       env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert prog.read_text().splitlines()[1].split("\t")[:4] == ["xc_linear", "DONE", "3", "3"]

    a = tmp / "stack_chain" / "linearstack_sourcepack" / "STACK"
    b = tmp / "stack_fused" / "linearstack_sourcepack" / "STACK"
    norm = lambda p, d: p.read_text().replace(str(d), "{STACK}")  # noqa: E731
    assert norm(b / "sourcepack_index.tsv", tmp / "stack_fused") == norm(a / "sourcepack_index.tsv", tmp / "stack_chain")
    assert norm(b / "_SUCCESS", tmp / "stack_fused") == norm(a / "_SUCCESS", tmp / "stack_chain")
    npts = chain[0].sample_count
    ha, da = read_pack(a / "linearstack.pack", npts)
    hb, db = read_pack(b / "linearstack.pack", npts)
    assert hb == ha  # headers (first record's header, user0 = record count)
    assert sorted({r.segment_count for r in chain}) == [2, 3]
    err = np.linalg.norm(db.astype(np.float64) - da, axis=1) / np.linalg.norm(da.astype(np.float64), axis=1)
    assert err.max() < NCF_RTOL


@pytest.mark.gpu
def test_xc_linear_rejects_bad_command_lines(tmp_path, built_lib, torch_cuda):
    exe = str(BIN / "xc_linear")
    assert subprocess.run([exe], capture_output=True).returncode == 1
    assert subprocess.run([exe, "-I", str(tmp_path), "-C", "20"], capture_output=True).returncode == 1
    assert subprocess.run([exe, "--bogus"], capture_output=True).returncode == 1
    assert subprocess.run([exe, "-h"], capture_output=True).returncode == 0
