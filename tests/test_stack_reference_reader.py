"""The reference's own readers on the stacked SourcePack outputs this build
writes.

``tests/golden/stack_sample`` holds this build's ncf_pws (two worker shards
+ merged index), ncf_tfpws and RTZ-rotation outputs for the nine-component
case of tests/golden/stack_case.py (made on a GPU by
tests/golden/make_stack_sample.py). Here, on the CPU:

  * the reference's SourcePack unpacker
    (fastxc/operators/sourcepack/unpack.py:28) reads the merged index and
    each PWS worker shard index and writes one SAC file per stacked pair;
    every file equals its record's bytes, the reference's SAC decoder
    (fastxc/io/sac_binary.py:225) reads it back, and its samples lie within
    relative L2 1e-5 of the FP64 oracle's PWS / TF-PWS of the same inputs
    (regenerated here from the case's seed);
  * the reference's rotation of stacked outputs
    (fastxc/operators/rotation/python_rotate.py:264, the step that follows
    stacking) reads the PWS and TF-PWS folders, and its RTZ index equals
    the committed one of this build's rotation column by column, its SAC
    headers byte for byte (up to the last bit of the float32 geometry
    fields) and its traces within 1e-6 of their largest sample.

The reference tree is read where it exists (its root from
$FXC_REFERENCE_ROOT or the default of oracle/build_ref.py); elsewhere these
checks skip.
"""

import csv
import importlib
import shutil
import sys
import types
from pathlib import Path

import numpy as np
import pytest

from oracle import stack_oracle as sto

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
import stack_case as sc  # noqa: E402

# reference modules and the bare packages they import through (the
# packages' own __init__ files pull in the whole controller)
_BARE = ("fastxc", "fastxc.inventory", "fastxc.operators", "fastxc.operators.rotation",
         "fastxc.operators.sourcepack")


@pytest.fixture
def ref():
    from oracle.build_ref import reference_root

    root = reference_root()
    if not (root / "fastxc" / "operators" / "rotation" / "python_rotate.py").exists():
        pytest.skip(f"reference tree not present ({root})")
    pytest.importorskip("tqdm")
    saved = {k: v for k, v in sys.modules.items() if k == "fastxc" or k.startswith("fastxc.")}
    for k in saved:
        del sys.modules[k]
    for name in _BARE:
        m = types.ModuleType(name)
        m.__path__ = [str(root / name.replace(".", "/"))]
        sys.modules[name] = m
    try:
        yield types.SimpleNamespace(
            unpack=importlib.import_module("fastxc.operators.sourcepack.unpack"),
            rotate=importlib.import_module("fastxc.operators.rotation.python_rotate"),
            sac=importlib.import_module("fastxc.io.sac_binary"))
    finally:
        for k in [k for k in sys.modules if k == "fastxc" or k.startswith("fastxc.")]:
            del sys.modules[k]
        sys.modules.update(saved)


def _relocate(dest: Path) -> Path:
    """Copy of the sample under dest with its relative record and final
    paths joined to dest (the tools write them absolute)."""
    dest = dest.resolve()
    shutil.copytree(sc.SAMPLE / "stack", dest / "stack")
    for tsv in dest.rglob("*.tsv"):
        with tsv.open(newline="") as fh:
            rd = csv.DictReader(fh, delimiter="\t")
            head, rows = rd.fieldnames, list(rd)
        for r in rows:
            for col in ("record_path", "final_pair_path"):
                if r[col] and not Path(r[col]).is_absolute():
                    r[col] = str(dest / r[col])
        with tsv.open("w", newline="") as fh:
            wr = csv.DictWriter(fh, fieldnames=head, delimiter="\t", lineterminator="\n")
            wr.writeheader()
            wr.writerows(rows)
    return dest


def _index(path: Path) -> list:
    with path.open(newline="") as fh:
        return list(csv.DictReader(fh, delimiter="\t"))


def _record(row) -> bytes:
    with open(row["record_path"], "rb") as fh:
        fh.seek(int(row["record_offset"]))
        return fh.read(int(row["bytes"]))


def _oracle(method: str, x: np.ndarray) -> np.ndarray:
    if method == "pws":
        return sto.pws(x, sc.PWS_SUB)
    return sto.tfpws(x, sc.TFPWS_SUB, band=sc.TFPWS_BAND, delta=sc.DELTA)


def _key(row) -> tuple:
    return row["path_id"], row["src_component"][-1], row["rec_component"][-1]


def _rel(a, b) -> float:
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_sample_layout():
    stack = sc.SAMPLE / "stack"
    assert sorted(p.name for p in (stack / "pws_sourcepack" / "STACK").iterdir()) == [
        "_SUCCESS", "pws.w000.pack", "pws.w000.tsv", "pws.w001.pack", "pws.w001.tsv", "sourcepack_index.tsv"]
    assert sorted(p.name for p in (stack / "tfpws_sourcepack" / "STACK").iterdir()) == [
        "_SUCCESS", "sourcepack_index.tsv", "tfpws.w000.pack", "tfpws.w000.tsv"]
    for m in ("pws", "tfpws"):
        merged = _index(stack / f"{m}_sourcepack" / "STACK" / "sourcepack_index.tsv")
        assert [_key(r) for r in merged] == sc.groups_order()
        assert {r["storage_kind"] for r in merged} == {f"{m}_pack"}
        assert {r["timestamp"] for r in merged} == {"STACK"}
        rtz = _index(stack / f"rtz_{m}_sourcepack" / "STACK" / "sourcepack_index.tsv")
        assert len(rtz) == 9 * len(sc.PAIRS) and {r["storage_kind"] for r in rtz} == {f"rtz_{m}_pack"}


@pytest.mark.parametrize("method", ["pws", "tfpws"])
def test_reference_unpacker_reads_stacked_output(tmp_path, ref, method):
    out = _relocate(tmp_path / "out")
    stack = out / "stack" / f"{method}_sourcepack" / "STACK"
    merged = _index(stack / "sourcepack_index.tsv")
    res = ref.unpack.unpack_sourcepack(stack, tmp_path / "sac")
    assert res.record_count == res.file_count == len(merged) == 9 * len(sc.PAIRS)
    assert res.bytes_written == sum(int(r["bytes"]) for r in merged)
    inputs = sc.traces()
    for row in merged:
        f = (tmp_path / "sac" / f"XX.{row['src_station']}" / f"XX.{row['rec_station']}" /
             f"XX-XX.{row['src_station']}-{row['rec_station']}.{row['src_component']}-{row['rec_component']}"
             ".ncf.SAC")
        assert f.read_bytes() == _record(row)
        hd, data = ref.sac.read_sac(f)
        assert hd.npts == sc.NSAMPLES and np.isclose(hd.get_float("delta"), sc.DELTA)
        assert hd.get_float("user0") == sc.NTS
        assert _rel(data.astype(np.float64), _oracle(method, inputs[_key(row)])) < 1e-5, _key(row)
    if method == "pws":
        # each worker shard index on its own: the groups dealt round-robin
        for w in (0, 1):
            shard = _index(stack / f"pws.w{w:03d}.tsv")
            assert [_key(r) for r in shard] == sc.groups_order()[w::2]
            r2 = ref.unpack.unpack_sourcepack(stack / f"pws.w{w:03d}.tsv", tmp_path / f"w{w}")
            assert r2.record_count == len(shard)


@pytest.mark.parametrize("method", ["pws", "tfpws"])
def test_reference_rotation_of_stacked_output(tmp_path, ref, method):
    out = _relocate(tmp_path / "out")
    ours_dir = out / "stack" / f"rtz_{method}_sourcepack" / "STACK"
    ours = _index(ours_dir / "sourcepack_index.tsv")
    ours_rec = [_record(r) for r in ours]
    shutil.rmtree(ours_dir)
    res = ref.rotate.rotate_sourcepack_stack(out, method)
    assert len(res) == len(sc.PAIRS)
    theirs = _index(ours_dir / "sourcepack_index.tsv")
    assert len(theirs) == len(ours)
    for a, b, rec in zip(ours, theirs, ours_rec):
        for col in a:
            if col != "record_path":
                assert a[col] == b[col], (col, a[col], b[col])
        assert Path(b["record_path"]).name == Path(a["record_path"]).name
        got = _record(b)
        assert len(got) == len(rec)
        ha, hb = np.frombuffer(rec[:280], "<f4"), np.frombuffer(got[:280], "<f4")
        assert np.allclose(ha, hb, rtol=2e-7, atol=0), np.nonzero(ha != hb)
        assert rec[280:632] == got[280:632]
        da, db = np.frombuffer(rec[632:], "<f4"), np.frombuffer(got[632:], "<f4")
        assert np.max(np.abs(da - db)) <= 1e-6 * np.max(np.abs(db))
