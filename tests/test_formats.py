"""File formats of the drop-in executables against the reference's own
readers/encoders (fixtures in golden/formats_golden.json, made by
golden/make_golden.py): the stepack batch layout as parsed by
fastxc/tools/extract_stepack.py, and the SAC header field table of
fastxc/io/sac_binary.py."""

import csv
import importlib.util
import json
from pathlib import Path

import numpy as np
import pytest

from fastxc_gb300 import formats

GOLDEN = Path(__file__).resolve().parent / "golden"


def _make_golden_module():
    spec = importlib.util.spec_from_file_location("fxc_make_golden", GOLDEN / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def golden():
    return json.loads((GOLDEN / "formats_golden.json").read_text())


def test_stepack_writer_matches_reference_reader(tmp_path, golden):
    mg = _make_golden_module()
    chans, spec = mg.formats_case()
    pack = formats.write_stepack(tmp_path, 2, 5, chans, spec, 0.1, 0.05, group_count=2, start_group=4)
    raw = pack.read_bytes()
    h = formats.STEPACK_HDR.unpack_from(raw, 0)
    gh = golden["header"]
    mine = dict(version=h[1], header_size=h[2], nslc_entry_size=h[3], layout=h[4], batch_seq=h[5], start_group=h[6],
                group_count=h[7], worker_id=h[8], nstep=h[9], nslc_count=h[10], nspec=h[11], payload_offset=h[15],
                payload_bytes=h[16], pitch_step_bytes=h[17], first_timestamp=h[18].rstrip(b"\0").decode())
    assert mine == gh
    with (tmp_path / "w002.b000005.tsv").open() as fh:
        rows = list(csv.DictReader(fh, delimiter="\t"))
    assert len(rows) == len(golden["fragments"])
    for r, g in zip(rows, golden["fragments"]):
        for k, v in g.items():
            got = r[k]
            assert (float(got) == pytest.approx(v, rel=1e-7)) if isinstance(v, float) else (type(v)(got) == v), k
    for e in golden["entries"]:
        i = e["file_index"]
        ent = formats.STEPACK_NSLC.unpack_from(raw, gh["header_size"] + i * gh["nslc_entry_size"])
        assert ent[0] == i and ent[1] == e["nsl_id"]
        assert ent[2] == pytest.approx(e["stla"]) and ent[3] == pytest.approx(e["stlo"])
        key = ".".join(x.rstrip(b"\0").decode() for x in ent[4:8])
        assert key == e["key"]
        sp = spec[:, i, :].astype(np.complex128)
        assert sp.real.sum() == pytest.approx(e["sum_re"], abs=1e-9)
        assert sp.imag.sum() == pytest.approx(e["sum_im"], abs=1e-9)


def test_sac_header_table_matches_reference_encoder(golden):
    mg = _make_golden_module()
    raw = bytes.fromhex(golden["sac_header_hex"])
    assert len(raw) == formats.SAC_HEADER_BYTES
    h = formats.parse_sac_header(raw)
    for k, v in mg.SAC_PIN_FLOATS.items():
        assert h[k] == pytest.approx(v), k
    for k, v in mg.SAC_PIN_INTS.items():
        assert h[k] == v, k
    for k, v in mg.SAC_PIN_TEXT.items():
        assert h[k].rstrip() == v, k
    assert h["nvhdr"] == 6
