"""Generates the golden fixtures in this directory from the reference itself.

Run in a container where the reference tree exists (it is read there, never
copied):  python tests/golden/make_golden.py [reference root]
The reference root is the argument, else $FXC_REFERENCE_ROOT, else the
default of oracle/build_ref.py.

  filter_*.txt          fastxc/operators/filter_design.py:design_filter (the
                        reference's own Python, scipy butter) for the band
                        sets of the benchmark configurations;
  plan_golden.json      segment / FFT lengths and filter padding from the
                        reference's C (native/sac2spec/fft_length.c,
                        core/filter_response.c) compiled by oracle/build_ref.py;
  response_golden.npz   processButterworthFilters power responses (float32);
  xc_tasks_golden.json  build_jobs + build_tasks_for_job of the reference's
                        scheduler (native/xc/worker/scheduler.cu) on small
                        station layouts;
  linear_stack_golden.npz  _linear_stack_group of
                        fastxc/operators/stacking/linear_stack.py on seeded
                        records;
  formats_golden.json   a stepack batch written by fastxc_gb300.formats as
                        parsed by the reference's fastxc/tools/extract_stepack.py,
                        and a SAC header encoded by fastxc/io/sac_binary.py;
  operators_golden.json / operators_rtz.npz
                        the reference's SourcePack materializer
                        (fastxc/operators/sourcepack/builder.py), linear stack
                        (fastxc/operators/stacking/linear_stack.py) and ENZ->RTZ
                        rotation (fastxc/operators/rotation/python_rotate.py)
                        run in sequence on the seeded workspace of
                        operators_case.py; absolute paths become {ROOT}.
"""

from __future__ import annotations

import ctypes as C
import importlib.util
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
from oracle.build_ref import reference_root  # noqa: E402

REF_ROOT = reference_root(sys.argv[1] if len(sys.argv) > 1 else None)

FILTER_SETS = [
    ("filter_d0.1_0.1-2.txt", 0.1, "0.1/2"),
    ("filter_d1.0_0.2-0.4_0.1-0.2.txt", 1.0, "0.2/0.4 0.1/0.2"),
    ("filter_d0.05_0.05-5.txt", 0.05, "0.05/5"),
    ("filter_d0.2_0.1-1_0.5-2.txt", 0.2, "0.1/1 0.5/2"),
]

PLAN_CASES = [
    # sac_len, win_len, shift, lag, delta, filter file
    (86400, 3600, 3600, 100, 0.1, "filter_d0.1_0.1-2.txt"),
    (86400, 1800, 1800, 100, 0.1, "filter_d0.1_0.1-2.txt"),
    (86400, 3600, 3600, 50, 0.1, "filter_d0.1_0.1-2.txt"),
    (86400, 3600, 3600, 200, 0.1, "filter_d0.1_0.1-2.txt"),
    (86400, 3600, 1800, 100, 0.05, "filter_d0.05_0.05-5.txt"),
    (86400, 3600, 3600, 100, 0.2, "filter_d0.2_0.1-1_0.5-2.txt"),
    (86400, 7200, 3600, 500, 1.0, "filter_d1.0_0.2-0.4_0.1-0.2.txt"),
    (3600, 7200, 0, 100, 0.1, "filter_d0.1_0.1-2.txt"),
    (86400, 3601.3, 3600, 97.7, 0.1, "filter_d0.1_0.1-2.txt"),
]


def load_module(path: Path, name: str):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod  # dataclasses look their module up while the class body runs
    spec.loader.exec_module(mod)
    return mod


class RefButterworth(C.Structure):
    _fields_ = [("freq_low", C.c_float), ("freq_high", C.c_float), ("b", C.c_double * 5), ("a", C.c_double * 5)]


class RefResp(C.Structure):
    _fields_ = [("freq_low", C.c_float), ("response", C.POINTER(C.c_float))]


def ref_sac2spec_lib():
    from oracle import build_ref

    libs = build_ref.build(root=REF_ROOT)
    lib = C.CDLL(str(libs["sac2spec"]))
    lib.readButterworthFilters.restype = C.POINTER(RefButterworth)
    lib.readButterworthFilters.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
    lib.estimateButterworthFilterPadding.restype = C.c_int
    lib.estimateButterworthFilterPadding.argtypes = [C.POINTER(RefButterworth), C.c_int, C.c_int]
    lib.processButterworthFilters.restype = C.POINTER(RefResp)
    lib.processButterworthFilters.argtypes = [C.POINTER(RefButterworth), C.c_int, C.c_float, C.c_int]
    lib.segment_length_from_seconds.restype = C.c_int
    lib.segment_length_from_seconds.argtypes = [C.c_float, C.c_int, C.c_float]
    lib.next_even_smooth_2357_length.restype = C.c_int
    lib.next_even_smooth_2357_length.argtypes = [C.c_int]
    lib.next_smooth_2357_length.restype = C.c_int
    lib.next_smooth_2357_length.argtypes = [C.c_int]
    return lib


def ref_plan(lib, sac_len, win_len, shift, lag, delta, fpath):
    """The planning arithmetic of native/sac2spec/cuda.main.cu:203-296 driven
    through the reference's compiled functions."""
    d = np.float32(delta)
    npts = int(np.floor(abs(float(np.float32(sac_len)) / float(d)) + 0.5))
    seg = lib.segment_length_from_seconds(float(np.float32(win_len)), npts, float(d))
    shift_pts = int(np.floor(float(np.float32(shift)) / float(d) + 0.5))
    if shift_pts < 1:
        shift_pts = seg
    nstep = max((npts - seg) // shift_pts + 1, 1) if seg <= npts else 1
    keep = min(int(np.floor(float(np.float32(lag)) / float(d) + 0.5)), seg)
    out_nfft = min(lib.next_even_smooth_2357_length(seg + keep), 2 * seg)
    cnt = C.c_int(0)
    flt = lib.readButterworthFilters(str(fpath).encode(), C.byref(cnt))
    pad = lib.estimateButterworthFilterPadding(flt, cnt.value, seg)
    fnfft = min(lib.next_even_smooth_2357_length(seg + pad), 2 * seg)
    return dict(npts=npts, segment_pts=seg, shift_pts=shift_pts, nstep=nstep, output_nfft=out_nfft,
                nspec=out_nfft // 2 + 1, filter_padding=pad, filter_nfft=fnfft, nfilters=cnt.value,
                freq_low=[flt[i].freq_low for i in range(cnt.value)],
                freq_high=[flt[i].freq_high for i in range(cnt.value)],
                b=[list(flt[i].b) for i in range(cnt.value)], a=[list(flt[i].a) for i in range(cnt.value)]), flt, cnt.value


def main() -> None:
    if not REF_ROOT.exists():
        raise SystemExit("reference tree not present; goldens are generated where it is mounted")
    fd = load_module(REF_ROOT / "fastxc" / "operators" / "filter_design.py", "ref_filter_design")
    for name, delta, bands in FILTER_SETS:
        fd.design_filter(delta, bands, HERE / name)

    lib = ref_sac2spec_lib()
    plans = []
    responses = {}
    for i, (sl, wl, sh, lag, delta, fname) in enumerate(PLAN_CASES):
        p, flt, cnt = ref_plan(lib, sl, wl, sh, lag, delta, HERE / fname)
        p.update(dict(sac_len=sl, win_len=wl, shift_len=sh, xcorr_lag=lag, delta=delta, filter_file=fname))
        plans.append(p)
        resp = lib.processButterworthFilters(flt, cnt, C.c_float(0.0), p["filter_nfft"])
        half = p["filter_nfft"] // 2
        for k in range(cnt):
            responses[f"case{i}_filter{k}"] = np.ctypeslib.as_array(resp[k].response, shape=(half + 1,)).copy()
    (HERE / "plan_golden.json").write_text(json.dumps(plans, indent=1))
    np.savez_compressed(HERE / "response_golden.npz", **responses)

    # xc scheduler
    from oracle import build_ref

    xlib = C.CDLL(str(build_ref.build(root=REF_ROOT)["xc"]))
    xlib.ref_xc_tasks.restype = C.c_int
    cases = []
    rng = np.random.default_rng(0)
    layouts = [
        (np.repeat(np.arange(1, 5), 3), "all", 12),
        (np.repeat(np.arange(1, 5), 3), "all", 4),
        (np.repeat(np.arange(1, 8), 3), "sparse", 5),
        (np.repeat([3, 1, 7, 2], [3, 3, 3, 3]), "all", 7),
        (np.repeat(np.arange(1, 6), 1), "auto", 2),
    ]
    for gnsl, mode, block in layouts:
        ids = sorted(set(int(g) for g in gnsl))
        paths = []
        for a in ids:
            for b in ids:
                if a > b:
                    continue
                if mode == "sparse" and a != b and rng.random() < 0.4:
                    continue
                if mode != "auto" and a == b and mode != "sparse":
                    continue
                paths.append((a, b))
        n = len(gnsl)
        mx = 4 * n * n + 16
        bufs = [np.zeros(mx, np.int32) for _ in range(5)]
        g = np.ascontiguousarray(gnsl, np.int32)
        ps = np.ascontiguousarray([p[0] for p in paths], np.int32)
        pr = np.ascontiguousarray([p[1] for p in paths], np.int32)
        cnt = xlib.ref_xc_tasks(g.ctypes.data_as(C.c_void_p), n, ps.ctypes.data_as(C.c_void_p),
                                pr.ctypes.data_as(C.c_void_p), len(paths), block,
                                *[b.ctypes.data_as(C.c_void_p) for b in bufs], mx)
        cases.append(dict(gnsl=[int(x) for x in gnsl], paths=paths, block_size=block,
                          src=bufs[0][:cnt].tolist(), rec=bufs[1][:cnt].tolist(), path_id=bufs[2][:cnt].tolist(),
                          auto=bufs[3][:cnt].tolist(), job=bufs[4][:cnt].tolist()))
    (HERE / "xc_tasks_golden.json").write_text(json.dumps(cases))

    # linear stack: the reference's own _linear_stack_group over seeded SAC
    # records written with its own encoder (the package __init__ pulls in
    # the inventory and pandas, so its sub-packages are loaded directly)
    import importlib
    import tempfile
    import types

    sys.path.insert(0, str(REF_ROOT))
    for name, path in (("fastxc", "fastxc"), ("fastxc.operators", "fastxc/operators"),
                       ("fastxc.operators.stacking", "fastxc/operators/stacking")):
        if name not in sys.modules:
            m = types.ModuleType(name)
            m.__path__ = [str(REF_ROOT / path)]
            sys.modules[name] = m
    ls = importlib.import_module("fastxc.operators.stacking.linear_stack")
    sacio = importlib.import_module("fastxc.io")
    rng = np.random.default_rng(7)
    traces = (rng.standard_normal((7, 2001)) * 1e3).astype(np.float32)
    with tempfile.TemporaryDirectory() as td:
        pack = Path(td) / "x.pack"
        records = []
        with pack.open("wb") as fh:
            for i, tr in enumerate(traces):
                hd = sacio.SacHeader.empty()
                hd.set_float("delta", 0.1)
                hd.set_float("b", -100.0)
                hd.set_int("npts", tr.size)
                blob = sacio.encode_sac_record(hd, tr)
                records.append(ls.SourceIndexRecord(row={"timestamp": f"2020.{i:03d}"}, record_path=pack,
                                                    record_offset=fh.tell(), record_bytes=len(blob)))
                fh.write(blob)
        _, stacked = ls._linear_stack_group(records)
    np.savez_compressed(HERE / "linear_stack_golden.npz", traces=traces, stacked=np.asarray(stacked, np.float32))

    # file formats: a stepack written by fastxc_gb300.formats, read back by the
    # reference's own stepack reader (fastxc/tools/extract_stepack.py); a SAC
    # header written by the reference's encoder (fastxc/io/sac_binary.py)
    sys.path.insert(0, str(HERE.parents[1]))
    from fastxc_gb300 import formats

    es = load_module(REF_ROOT / "fastxc" / "tools" / "extract_stepack.py", "ref_extract_stepack")
    chans, spec = formats_case()
    with tempfile.TemporaryDirectory() as td:
        formats.write_stepack(td, 2, 5, chans, spec, 0.1, 0.05, group_count=2, start_group=4)
        frags = es.discover_stepack_fragments(td)
        out = {"fragments": [], "entries": []}
        for fr in frags:
            out["fragments"].append({k: (str(getattr(fr, k)) if k in ("tsv_path", "pack_path") else getattr(fr, k))
                                     for k in ("timestamp", "nslc_start", "nslc_count", "batch_nslc_count", "nspec",
                                               "nstep", "dt", "df", "payload_offset", "pitch_step_bytes",
                                               "nslc_step_bytes")})
            for e in es.read_fragment_nslc_entries(fr):
                sp = es.read_entry_spectra(e)
                out["entries"].append({"file_index": e.file_index, "nsl_id": e.nsl_id, "stla": e.stla, "stlo": e.stlo,
                                       "key": e.key, "sum_re": float(np.real(sp).astype(np.float64).sum()),
                                       "sum_im": float(np.imag(sp).astype(np.float64).sum()), "shape": list(sp.shape)})
        hdr = es.read_stepack_header(Path(td) / "w002.b000005.stepack")
        out["header"] = {k: getattr(hdr, k) for k in ("version", "header_size", "nslc_entry_size", "layout", "batch_seq",
                                                      "start_group", "group_count", "worker_id", "nstep", "nslc_count",
                                                      "nspec", "payload_offset", "payload_bytes", "pitch_step_bytes",
                                                      "first_timestamp")}
    for fr in out["fragments"]:
        fr.pop("tsv_path", None)
        fr.pop("pack_path", None)
    sac = importlib.import_module("fastxc.io.sac_binary")
    hd = sac.SacHeader.empty()
    for k, v in SAC_PIN_FLOATS.items():
        hd.set_float(k, v)
    for k, v in SAC_PIN_INTS.items():
        hd.set_int(k, v)
    for k, v in SAC_PIN_TEXT.items():
        hd.set_text(k, v)
    raw = sac.encode_sac_record(hd, np.zeros(SAC_PIN_INTS["npts"], dtype=np.float32))
    out["sac_header_hex"] = raw[:632].hex()
    (HERE / "formats_golden.json").write_text(json.dumps(out, indent=1))
    print("goldens written to", HERE)


SAC_PIN_FLOATS = {"delta": 0.1, "b": -100.0, "e": 100.0, "o": 0.0, "stla": 31.5, "stlo": 101.25, "evla": 30.5,
                  "evlo": 100.75, "user0": 7.0, "user1": 12.0, "user2": 70012.0, "dist": 55.5, "az": 10.0,
                  "baz": 190.0, "gcarc": 0.5}
SAC_PIN_INTS = {"nzyear": 2020, "nzjday": 123, "nzhour": 4, "nzmin": 5, "nzsec": 0, "nzmsec": 0, "npts": 2001,
                "iftype": 1, "leven": 1, "unused27": 1}
SAC_PIN_TEXT = {"kstnm": "ST12", "kevnm": "XX.ST07", "kcmpnm": "BHE-BHN", "knetwk": "XX-XX"}


def formats_case():
    """Seeded channels + spectra of the stepack pin (two timestamps in one batch)."""
    rng = np.random.default_rng(11)
    chans = []
    for t, ts in enumerate(("2020.123.0000", "2020.123.0100")):
        for s, g in enumerate((3, 9)):
            for c in "EN":
                chans.append(dict(timestamp=ts, nsl_id=g, network="XX", station=f"ST{g:02d}", location="00",
                                  component=f"BH{c}", stla=30.0 + s + t, stlo=100.5 - s))
    spec = (rng.standard_normal((3, len(chans), 17)) + 1j * rng.standard_normal((3, len(chans), 17))).astype(np.complex64)
    return chans, spec


def ref_packages():
    """The reference's Python sub-packages, loaded without the top-level
    package __init__ (which pulls in the inventory and pandas)."""
    import importlib
    import types

    sys.path.insert(0, str(REF_ROOT))
    for name in ("fastxc", "fastxc.operators", "fastxc.inventory"):
        if name not in sys.modules:
            m = types.ModuleType(name)
            m.__path__ = [str(REF_ROOT / name.replace(".", "/"))]
            sys.modules[name] = m
    return (importlib.import_module("fastxc.operators.sourcepack.builder"),
            importlib.import_module("fastxc.operators.stacking.linear_stack"),
            importlib.import_module("fastxc.operators.rotation.python_rotate"))


def operators_golden() -> None:
    import hashlib
    import tempfile

    sys.path.insert(0, str(HERE))
    import operators_case as oc

    builder, linear, rotate = ref_packages()
    out: dict = {}
    with tempfile.TemporaryDirectory() as td:
        root = Path(td).resolve()
        ncf = oc.make_xc_workspace(root)
        res = builder.build_sourcepack(ncf, root / "sourcepack")
        out["materializer"] = {
            "result": [res.record_count, res.source_count, res.bytes_indexed],
            "files": {p.relative_to(root).as_posix(): oc.normalize(p.read_text(), root)
                      for p in sorted((root / "sourcepack").rglob("*")) if p.is_file()},
        }
        indexes = sorted((root / "sourcepack").glob("*/sourcepack_index.tsv"))
        lres = linear.linear_stack_sourcepack_indexes(indexes, root / "stack")
        ldir = root / "stack" / "linearstack_sourcepack" / "STACK"
        out["linear"] = {
            "results": [[oc.normalize(str(r.input_path), root), oc.normalize(str(r.output_path), root),
                         r.segment_count, r.sample_count] for r in lres],
            "index": oc.normalize((ldir / "sourcepack_index.tsv").read_text(), root),
            "success": oc.normalize((ldir / "_SUCCESS").read_text(), root),
            "pack_sha256": hashlib.sha256((ldir / "linearstack.pack").read_bytes()).hexdigest(),
        }
        rres = rotate.rotate_linearstack_sourcepack(root)
        rdir = root / "stack" / "rtz_linearstack_sourcepack" / "STACK"
        raw = (rdir / "rtz_linearstack.pack").read_bytes()
        rec = 632 + 4 * oc.NPTS
        headers = [raw[k:k + 632].hex() for k in range(0, len(raw), rec)]
        data = np.stack([np.frombuffer(raw[k + 632:k + rec], "<f4") for k in range(0, len(raw), rec)])
        out["rotate"] = {
            "pairs": len(rres),
            "index": oc.normalize((rdir / "sourcepack_index.tsv").read_text(), root),
            "success": oc.normalize((rdir / "_SUCCESS").read_text(), root),
            "headers": headers,
        }
        # the rotation matrices of a few geometries, for the CPU pin
        out["matrices"] = {f"{az}_{baz}": rotate.build_rotate_matrix(az, baz).tolist()
                           for az, baz in ((0.0, 180.0), (37.5, 219.25), (90.0, 270.0), (301.1, 120.7))}
        out["rudoe"] = [list(rotate.distkm_az_baz_rudoe(*g)) for g in
                        ((101.0, 31.0, 101.9, 31.4), (100.6, 30.2, 101.0, 31.0), (0.0, 0.0, 10.0, 0.0),
                         (-70.5, -33.4, 151.2, -33.9), (10.0, 90.0, 20.0, 45.0))]
        np.savez_compressed(HERE / "operators_rtz.npz", data=data)
    (HERE / "operators_golden.json").write_text(json.dumps(out, indent=1))
    print("operator goldens written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "operators":
        operators_golden()
        raise SystemExit(0)
    main()
    operators_golden()
