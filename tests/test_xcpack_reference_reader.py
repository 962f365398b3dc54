"""The reference's own readers on files this build writes.

``tests/golden/xcpack_sample`` is an xcpack output of this build's xc_fast
(made on a GPU by ``tests/golden/make_xcpack_sample.py``). Here, on the CPU:

  * the reference's NCF extractor (fastxc/tools/extract_ncf.py:38) finds
    every record of the sample by (timestamp, source, receiver, component
    pair), directly from the xcpack TSV and through a SourcePack index that
    this build's materializer wrote; the bytes it extracts equal the record
    bytes, and the reference's SAC decoder (fastxc/io/sac_binary.py) reads
    them back as a 401-sample NCF with this build's header fields;
  * the sample's TSV carries every column the reference's SourcePack
    reader requires (checked through the materializer, which rejects a
    TSV that lacks one).

The reference tree is read where it exists (its root from
$FXC_REFERENCE_ROOT or the default of oracle/build_ref.py); elsewhere the
reference-reader checks skip.
"""

import importlib.util
import shutil
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
SAMPLE = HERE / "golden" / "xcpack_sample"


def _reference_module(rel: str, name: str):
    from oracle.build_ref import reference_root

    path = reference_root() / rel
    if not path.exists():
        pytest.skip(f"reference tree not present ({path})")
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def _rows():
    tsv = next(SAMPLE.glob("*.tsv"))
    lines = tsv.read_text().splitlines()
    head = lines[0].split("\t")
    return tsv, [dict(zip(head, ln.split("\t"))) for ln in lines[1:] if ln]


def _record(row) -> bytes:
    with (SAMPLE / row["pack_path"]).open("rb") as fh:
        fh.seek(int(row["offset"]))
        return fh.read(int(row["bytes"]))


def test_reference_extractor_reads_our_xcpack(tmp_path):
    ex = _reference_module("fastxc/tools/extract_ncf.py", "ref_extract_ncf")
    sac = _reference_module("fastxc/io/sac_binary.py", "ref_sac_binary")
    ws = tmp_path / "ncf"
    shutil.copytree(SAMPLE, ws / "xcpack")
    _, rows = _rows()
    assert len(rows) > 20
    for k, row in enumerate(rows):
        out = tmp_path / f"r{k}.sac"
        res = ex.extract_ncf(input_path=ws / "xcpack", timestamp=row["timestamp"], source=row["src_station"],
                             receiver=row["rec_station"],
                             component_pair=f"{row['src_component']}-{row['rec_component']}", output=out)
        assert res.record_offset == int(row["offset"]) and res.record_bytes == int(row["bytes"])
        data = out.read_bytes()
        assert data == _record(row)
        # the reference's decoder: header-implied record size, float32 payload
        hdr, samples = sac.read_sac_record(ws / "xcpack" / row["pack_path"], int(row["offset"]), int(row["bytes"]))
        assert samples.size == int(row["npts"])
        assert np.array_equal(samples, np.frombuffer(data[632:], "<f4"))
        _, whole = sac.read_sac(out)
        assert np.array_equal(whole, samples)
    # a record's payload is the 401-sample NCF after the 632-byte header
    from fastxc_gb300 import sacbin

    h = sacbin.Header(_record(rows[0])[:632], "<")
    assert h.get_int("npts") == int(rows[0]["npts"]) == 401
    payload = np.frombuffer(_record(rows[0])[632:], "<f4")
    assert payload.size == 401 and np.all(np.isfinite(payload))


def test_reference_extractor_reads_our_sourcepack_index(tmp_path):
    ex = _reference_module("fastxc/tools/extract_ncf.py", "ref_extract_ncf")
    from fastxc_gb300 import sourcepack

    ws = tmp_path / "ws"
    shutil.copytree(SAMPLE, ws / "ncf" / "xcpack")
    res = sourcepack.build_sourcepack(ws / "ncf", ws / "sourcepack")
    assert res.record_count == len(_rows()[1])
    for row in _rows()[1][::7]:
        out = tmp_path / "x.sac"
        ex.extract_ncf(workspace=ws, timestamp=row["timestamp"], source=row["src_station"],
                       receiver=row["rec_station"], component_pair=f"{row['src_component']}-{row['rec_component']}",
                       output=out)
        assert out.read_bytes() == _record(row)
