"""GPU operators after xc_fast, against the reference's own outputs on the
seeded workspace of tests/golden/operators_case.py: the SourcePack ->
linear stack -> ENZ->RTZ rotation chain (index files, _SUCCESS texts and SAC
headers byte for byte; the linear-stack pack bit for bit; rotated samples
within float32 summation-order tolerance), and the rotation kernel against
an FP64 product."""

from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
import operators_case as oc  # noqa: E402

pytestmark = pytest.mark.gpu
GOLD = json.loads((HERE / "golden" / "operators_golden.json").read_text())
# float32 rotation: nine products per sample, summation order differs from
# numpy's matmul -> relative to the trace's peak
ROT_RTOL = 1e-6


def test_sourcepack_linear_rotate_chain_matches_reference(ctx, tmp_path):
    from fastxc_gb300 import linear, rotate, sourcepack

    root = tmp_path.resolve()
    ncf = oc.make_xc_workspace(root)
    sourcepack.build_sourcepack(ncf, root / "sourcepack")
    indexes = sourcepack.discover_sourcepack_indexes(root / "sourcepack")
    res = linear.linear_stack_sourcepack_indexes(indexes, root / "stack", ctx=ctx)
    assert [[oc.normalize(str(r.input_path), root), oc.normalize(str(r.output_path), root), r.segment_count,
             r.sample_count] for r in res] == GOLD["linear"]["results"]
    ldir = root / "stack" / "linearstack_sourcepack" / "STACK"
    assert oc.normalize((ldir / "sourcepack_index.tsv").read_text(), root) == GOLD["linear"]["index"]
    assert oc.normalize((ldir / "_SUCCESS").read_text(), root) == GOLD["linear"]["success"]
    assert hashlib.sha256((ldir / "linearstack.pack").read_bytes()).hexdigest() == GOLD["linear"]["pack_sha256"]

    rres = rotate.rotate_linearstack_sourcepack(root, ctx=ctx)
    assert len(rres) == GOLD["rotate"]["pairs"]
    rdir = root / "stack" / "rtz_linearstack_sourcepack" / "STACK"
    assert oc.normalize((rdir / "sourcepack_index.tsv").read_text(), root) == GOLD["rotate"]["index"]
    assert oc.normalize((rdir / "_SUCCESS").read_text(), root) == GOLD["rotate"]["success"]
    raw = (rdir / "rtz_linearstack.pack").read_bytes()
    rec = 632 + 4 * oc.NPTS
    assert [raw[k:k + 632].hex() for k in range(0, len(raw), rec)] == GOLD["rotate"]["headers"]
    got = np.stack([np.frombuffer(raw[k + 632:k + rec], "<f4") for k in range(0, len(raw), rec)])
    ref = np.load(HERE / "golden" / "operators_rtz.npz")["data"]
    assert got.shape == ref.shape
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert np.all(np.abs(got - ref) <= ROT_RTOL * scale)


def test_linear_stack_dry_run_and_empty(ctx, tmp_path):
    from fastxc_gb300 import linear, sourcepack

    root = tmp_path.resolve()
    ncf = oc.make_xc_workspace(root)
    sourcepack.build_sourcepack(ncf, root / "sourcepack")
    indexes = sourcepack.discover_sourcepack_indexes(root / "sourcepack")
    dry = linear.linear_stack_sourcepack_indexes(indexes, root / "stack", dry_run=True)
    assert [r.segment_count for r in dry] == [r[2] for r in GOLD["linear"]["results"]]
    assert not (root / "stack").exists()
    empty = root / "empty.tsv"
    empty.write_text("\t".join(sourcepack.SOURCEPACK_INDEX_HEADER) + "\r\n")
    assert linear.linear_stack_sourcepack_indexes([empty], root / "stack2", ctx=ctx) == []
    assert not (root / "stack2" / "linearstack_sourcepack" / "STACK").exists()


@pytest.mark.parametrize("npairs,npts", [(1, 1), (3, 2001), (70000, 33)])
def test_rotation_kernel_matches_fp64(ctx, torch_cuda, npairs, npts):
    """Random geometries and traces; 70 000 pairs exceed one grid column."""
    from fastxc_gb300 import rotate

    rng = np.random.default_rng(npairs)
    enz = rng.standard_normal((npairs, 9, npts)).astype(np.float32)
    az = rng.uniform(0, 360, npairs)
    baz = rng.uniform(0, 360, npairs)
    mats = np.stack([rotate.build_rotate_matrix(a, b) for a, b in zip(az, baz)])
    got = rotate._Rotator(ctx)(enz, mats)
    ref = np.einsum("prc,pct->prt", mats.astype(np.float64), enz.astype(np.float64))
    assert np.abs(got - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())


def test_rotate_sac_files_roundtrip(ctx, tmp_path):
    """Nine ENZ SAC files in, nine RTZ files out; a pure-Z pair stays put."""
    from fastxc_gb300 import rotate, sacbin

    rng = np.random.default_rng(3)
    ins, outs = [], []
    data = rng.standard_normal((9, 101)).astype(np.float32)
    for k, tag in enumerate(rotate.ENZ_ORDER):
        h = sacbin.Header(bytes(632), "<")
        for f in sacbin.FLOATS:
            h.set_float(f, sacbin.NULL_VALUE)
        h.set_int("nvhdr", 6)
        h.set_int("iftype", 1)
        h.set_int("npts", 101)
        h.set_float("delta", 0.1)
        h.set_float("az", 40.0)
        h.set_float("baz", 220.5)
        p = tmp_path / f"in.{tag}.sac"
        sacbin.write_file(p, h, data[k])
        ins.append(p)
        outs.append(tmp_path / "out" / f"o.{rotate.RTZ_ORDER[k]}.sac")
    r = rotate.rotate_sac_files(ins, outs, ctx=ctx)
    assert r.sample_count == 101
    m = rotate.build_rotate_matrix(40.0, 220.5)
    for k, p in enumerate(outs):
        h, d = sacbin.read_file(p)
        assert h.get_text("kcmpnm") == rotate.SAC_COMPONENT_NAMES[k]
        assert abs(h.get_float("cmpaz") - 40.5) < 1e-4 and h.get_float("cmpinc") == 90.0
        np.testing.assert_allclose(d, (m.astype(np.float64) @ data.astype(np.float64))[k], rtol=0, atol=1e-5)
    np.testing.assert_array_equal(sacbin.read_file(outs[8])[1], data[8])
