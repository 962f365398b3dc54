"""End-to-end drop-in check of the xc_fast executable: stepack batches in,
xcpack records out, run through the reference's command line.

Checks: the record order equals the reference scheduler's task order
(restated bit-exactly in oracle.xc_oracle); file naming, markers and TSV
columns; SAC header fields of every record (SacheadProcess +
build_sac_header_for_task); NCF data within relative L2 1e-5 of the FP64
oracle; exit codes of bad command lines.
"""

import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import xc_oracle as xo

ROOT = Path(__file__).resolve().parents[1]
EXE = ROOT / "fastxc_gb300" / "bin" / "xc_fast"


def make_inputs(tmp, nsta=4, nstep=6, nspec=1001, split=True, seed=0):
    from fastxc_gb300 import formats

    rng = np.random.default_rng(seed)
    nsl = [3, 7, 12, 20][:nsta]
    comps = ["E", "N", "Z"]
    chans = []
    for s, g in enumerate(nsl):
        for c in comps:
            chans.append(dict(timestamp="2020.123.0000", nsl_id=g, network="XX", station=f"ST{g:02d}", location="00",
                              component=f"BH{c}", stla=30.0 + s, stlo=100.0 + s))
    spec = (rng.standard_normal((nstep, len(chans), nspec)) + 1j * rng.standard_normal((nstep, len(chans), nspec))).astype(np.complex64)
    sp = tmp / "stepack"
    dt, df = 0.1, 1.0 / (2 * (nspec - 1) * 0.1)
    if split:
        # two batches, out of NSL order, to exercise the merge + stable sort
        half = 6
        formats.write_stepack(sp, 0, 1, chans[half:], np.ascontiguousarray(spec[:, half:]), dt, df, group_count=2)
        formats.write_stepack(sp, 0, 0, chans[:half], np.ascontiguousarray(spec[:, :half]), dt, df, group_count=2)
    else:
        formats.write_stepack(sp, 0, 0, chans, spec, dt, df, group_count=nsta)
    rows = []
    for a in nsl:
        for b in nsl:
            if a < b and not (a == 3 and b == 20):  # one station pair not allowed
                rows.append((a, b, 0.5, 55.5, 10.0, 190.0))
    rows.append((7, 7, 0.0, 0.0, 0.0, 0.0))  # one autocorrelation path
    formats.write_allowed_paths(tmp / "allowed_paths.tsv", rows)
    return chans, spec, rows


@pytest.mark.gpu
@pytest.mark.parametrize("method,block", [("plain", None), ("tensor", None), ("plain", "5"), ("auto", None)])
def test_xc_fast_end_to_end(tmp_path, built_lib, torch_cuda, method, block):
    import os

    from fastxc_gb300 import formats

    chans, spec, rows = make_inputs(tmp_path)
    env = dict(os.environ, FASTXC_XC_METHOD=method, FASTXC_LOG_LEVEL="warn")
    if block:
        env["FASTXC_XC_BLOCK"] = block
    out = tmp_path / "ncf"
    prog = tmp_path / "xc_progress.tsv"
    r = subprocess.run([str(EXE), "-I", str(tmp_path / "stepack"), "-P", str(tmp_path / "allowed_paths.tsv"), "-O",
                        str(out), "-C", "20", "-G", "0", "--progress", str(prog)], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    root = out / "xcpack"
    assert (root / "_SUCCESS").read_text() == "DONE\n"
    assert (root / "2020.123.0000.done").exists()
    assert prog.read_text().splitlines()[1].split("\t")[1] == "DONE"
    recs = formats.read_xcpack_dir(root)

    # expected task order: reference scheduler over the merged, sorted channels
    gnsl = [c["nsl_id"] for c in chans]
    pids = {xo.make_allowed_path_id(a, b) for a, b, *_ in rows}
    bs = int(block) if block else len(chans)
    expected = []
    for j in xo.build_jobs(len(chans), bs):
        tasks, _ = xo.build_tasks_for_job(gnsl, pids, j)
        expected += [(j, t) for t in tasks]
    assert len(recs) == len(expected)
    nstep, nspec = spec.shape[0], spec.shape[2]
    shape = xo.finalize_shape(nspec, nstep, 0.1, 20.0)
    src = np.array([t.src_meta_idx for _, t in expected])
    rec = np.array([t.rec_meta_idx for _, t in expected])
    ref = xo.xc_run(spec, src, rec, 1.0 / nstep, shape)
    for k, (rrow, (job, t)) in enumerate(zip(recs, expected)):
        s, rc = chans[t.src_meta_idx], chans[t.rec_meta_idx]
        assert rrow["tsv"] == f"2020.123.0000.i{job.anchor_block:06d}.j{job.target_begin_block:06d}.w000.p000.tsv"
        assert int(rrow["src_id"]) == s["nsl_id"] and int(rrow["rec_id"]) == rc["nsl_id"]
        assert rrow["src_component"] == s["component"] and rrow["rec_component"] == rc["component"]
        assert int(rrow["npts"]) == shape.cc_size and int(rrow["anchor_block"]) == job.anchor_block
        assert rrow["final_pair_path"].endswith(f"XX-XX.{s['station']}-{rc['station']}.{s['component']}-{rc['component']}.sac")
        h = rrow["header"]
        assert h["npts"] == shape.cc_size and h["iftype"] == 1 and h["leven"] == 1 and h["unused27"] == 1
        assert h["nvhdr"] == 6 and h["nzyear"] == 2020 and h["nzjday"] == 123 and h["nzhour"] == 0
        assert h["b"] == pytest.approx(-shape.half_cc * 0.1, rel=1e-6) and h["e"] == pytest.approx(shape.half_cc * 0.1, rel=1e-6)
        assert h["user0"] == s["nsl_id"] and h["user1"] == rc["nsl_id"] and h["user2"] == t.path_id
        assert h["evla"] == pytest.approx(s["stla"]) and h["stla"] == pytest.approx(rc["stla"])
        assert h["kcmpnm"] == f"{s['component']}-{rc['component']}"[:8].ljust(8)
        assert h["kstnm"] == rc["station"].ljust(8) and h["kevnm"] == f"XX.{s['station']}".ljust(16)
        err = np.linalg.norm(rrow["data"] - ref[k]) / np.linalg.norm(ref[k])
        assert err < 1e-5, (k, err)


def test_xc_fast_command_line_errors(tmp_path, built_lib):
    r = subprocess.run([str(EXE)], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([str(EXE), "-h"], capture_output=True, text=True)
    assert r.returncode == 0
    r = subprocess.run([str(EXE), "-I", "x", "-O", "y"], capture_output=True, text=True)
    assert r.returncode == 1 and "required_argument_missing" in r.stderr
    r = subprocess.run([str(EXE), "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1 and "argument_unknown" in r.stderr


@pytest.mark.gpu
def test_xc_fast_emits_sourcepack_index(tmp_path, built_lib, torch_cuda):
    """xc_fast --sourcepack writes each timestamp's SourcePack index while it
    runs; the files equal, byte for byte, what the materializer builds
    afterwards from the same xcpack output."""
    import os

    from fastxc_gb300 import sourcepack

    make_inputs(tmp_path)
    out = tmp_path / "ncf"
    emitted = tmp_path / "sp_emitted"
    r = subprocess.run([str(EXE), "-I", str(tmp_path / "stepack"), "-P", str(tmp_path / "allowed_paths.tsv"), "-O",
                        str(out), "-C", "20", "--sourcepack", str(emitted)],
                       env=dict(os.environ, FASTXC_LOG_LEVEL="warn"), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    built = sourcepack.build_sourcepack(out, tmp_path / "sp_built")
    assert built.index_paths and built.record_count > 0
    for idx in built.index_paths:
        mine = emitted / idx.parent.name
        assert (mine / "sourcepack_index.tsv").read_bytes() == idx.read_bytes()
        assert (mine / "_SUCCESS").read_bytes() == (idx.parent / "_SUCCESS").read_bytes()


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["plain", "tensor"])
def test_xc_fast_memory_budget_pair_blocks(tmp_path, built_lib, torch_cuda, method):
    """-M below one timestamp's footprint splits its pairs into blocks
    (fxc_plan_xc_pairs); the records are byte-identical to one whole run."""
    import ctypes as C
    import os

    from fastxc_gb300._lib import FXC_XC_PLAIN, FXC_XC_TENSOR, lib
    from fastxc_gb300.core import xc_shape

    nspec, nstep, nch = 8001, 6, 12
    make_inputs(tmp_path, nspec=nspec, nstep=nstep)
    env = dict(os.environ, FASTXC_XC_METHOD=method, FASTXC_LOG_LEVEL="info")

    def run(out, extra):
        r = subprocess.run([str(EXE), "-I", str(tmp_path / "stepack"), "-P", str(tmp_path / "allowed_paths.tsv"),
                            "-O", str(out), "-C", "20", *extra], env=env, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        return r.stderr

    run(tmp_path / "whole", [])
    tsv = next((tmp_path / "whole" / "xcpack").glob("*.tsv"))
    npairs = len(tsv.read_text().splitlines()) - 1
    shape = xc_shape(nspec, nstep, 0.1, 20.0)
    m = FXC_XC_TENSOR if method == "tensor" else FXC_XC_PLAIN

    def nbytes(p):
        out = C.c_int64()
        lib().fxc_xc_host_bytes(p, nstep, nch, nspec, C.byref(shape), m, 0, C.byref(out))
        return out.value

    mib = (nbytes(1) + nbytes(npairs)) // 2 >> 20
    per = C.c_int64()
    lib().fxc_plan_xc_pairs(npairs, nstep, nch, nspec, C.byref(shape), m, 0, mib << 20, C.byref(per), None)
    assert 1 <= per.value < npairs, (per.value, npairs)
    log = run(tmp_path / "blocks", ["-M", str(mib)])
    assert "xc_pair_blocks" in log
    a, b = tmp_path / "whole" / "xcpack", tmp_path / "blocks" / "xcpack"
    for f in sorted(a.glob("*.xcpack")):
        assert (b / f.name).read_bytes() == f.read_bytes(), f.name
    for f in sorted(a.glob("*.tsv")):
        assert (b / f.name).read_text().replace(str(tmp_path / "blocks"), "@") == \
            f.read_text().replace(str(tmp_path / "whole"), "@")
