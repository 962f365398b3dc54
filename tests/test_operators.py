"""Host-side operators after xc_fast: SourcePack materializer, rotation
matrices and geodesic, pinned against the reference's own Python run on the
seeded workspace of tests/golden/operators_case.py (operators_golden.json).
No GPU: the GPU parts of the linear stack and the rotation are in
test_operators_gpu.py."""

from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
import operators_case as oc  # noqa: E402

GOLD = json.loads((HERE / "golden" / "operators_golden.json").read_text())


def _tree(root: Path, sub: str) -> dict:
    base = root / sub
    return {p.relative_to(root).as_posix(): oc.normalize(p.read_text(), root)
            for p in sorted(base.rglob("*")) if p.is_file()}


def test_materializer_matches_reference(tmp_path):
    from fastxc_gb300 import sourcepack

    ncf = oc.make_xc_workspace(tmp_path)
    progress = tmp_path / "progress.tsv"
    res = sourcepack.build_sourcepack(ncf, tmp_path / "sourcepack", progress_file=progress)
    assert [res.record_count, res.source_count, res.bytes_indexed] == GOLD["materializer"]["result"]
    assert _tree(tmp_path.resolve(), "sourcepack") == GOLD["materializer"]["files"]
    lines = progress.read_text().splitlines()
    assert lines[0] == "task\tstatus\tcompleted\ttotal\tunit\tdetail"
    assert lines[1] == "overall\tDONE\t2\t2\ttimestamps\tsource index ready"


def test_async_materializer_and_single_timestamp(tmp_path):
    from fastxc_gb300 import sourcepack

    ncf = oc.make_xc_workspace(tmp_path)
    m = sourcepack.AsyncSourcePackMaterializer(ncf, tmp_path / "sp", poll_interval_sec=0.5)
    m.start()
    res = m.finish()
    assert res.record_count == GOLD["materializer"]["result"][0]
    got = _tree(tmp_path.resolve(), "sp")
    ok = {k.replace("sourcepack/", "sp/"): v.replace("{ROOT}/sourcepack/", "{ROOT}/sp/")
          for k, v in GOLD["materializer"]["files"].items()}
    success = got.pop("sp/_SUCCESS")
    assert got == ok
    assert success.startswith(f"timestamps\t2\nrecords\t{res.record_count}\n")
    one = sourcepack.build_sourcepack_timestamp(ncf, tmp_path / "one", oc.TIMESTAMPS[1])
    assert one.index_paths[0].read_text() == (tmp_path / "sp" / oc.TIMESTAMPS[1] / "sourcepack_index.tsv").read_text()


def test_materializer_rejects_bad_tsv(tmp_path):
    from fastxc_gb300 import sourcepack

    ncf = oc.make_xc_workspace(tmp_path)
    tsv = sorted((ncf / "xcpack").glob("*.tsv"))[0]
    tsv.write_text(tsv.read_text().replace("\tbytes\t", "\tsize\t", 1))
    with pytest.raises(ValueError, match="missing fields"):
        sourcepack.build_sourcepack(ncf, tmp_path / "sp")


def test_rotation_matrices_and_geodesic_match_reference():
    from fastxc_gb300 import rotate

    for key, ref in GOLD["matrices"].items():
        az, baz = (float(x) for x in key.split("_"))
        assert np.array_equal(rotate.build_rotate_matrix(az, baz), np.asarray(ref, np.float32)), key
    geos = ((101.0, 31.0, 101.9, 31.4), (100.6, 30.2, 101.0, 31.0), (0.0, 0.0, 10.0, 0.0),
            (-70.5, -33.4, 151.2, -33.9), (10.0, 90.0, 20.0, 45.0))
    for g, ref in zip(geos, GOLD["rudoe"]):
        assert list(rotate.distkm_az_baz_rudoe(*g)) == ref


def test_rotation_matrix_c_abi_matches_numpy():
    """fxc_rotate_matrix (host C, libm float32 sine/cosine) against the numpy
    construction: identical structure, values within one float32 ulp."""
    from fastxc_gb300 import rotate
    from fastxc_gb300._lib import lib

    out = (C.c_float * 81)()
    for az, baz in ((0.0, 180.0), (37.5, 219.25), (90.0, 270.0), (301.1, 120.7), (359.99, 0.01)):
        lib().fxc_rotate_matrix(az, baz, out)
        got = np.frombuffer(out, np.float32).reshape(9, 9)
        ref = rotate.build_rotate_matrix(az, baz)
        assert np.array_equal(got == 0, ref == 0)
        assert np.allclose(got, ref, rtol=2.5e-7, atol=1e-7)


def test_rotation_geometry_from_header_fallback():
    from fastxc_gb300 import rotate, sacbin

    h = sacbin.Header(bytes(632), "<")
    for k in sacbin.FLOATS:
        h.set_float(k, sacbin.NULL_VALUE)
    h.set_int("nvhdr", 6)
    h.set_float("az", 12.5)
    h.set_float("baz", 193.0)
    h.set_float("gcarc", 0.25)
    h.set_float("dist", 27.0)
    assert rotate.geometry_from_header(h) == (0.25, 12.5, 193.0, 27.0)
    h.set_float("az", sacbin.NULL_VALUE)
    with pytest.raises(ValueError):
        rotate.geometry_from_header(h)
