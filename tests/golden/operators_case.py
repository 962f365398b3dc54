"""Seeded xc_fast-style output workspace for the SourcePack, linear-stack and
rotation operator tests (and for make_golden.py, which runs the reference's
own operators on it). Deterministic: the same bytes on every machine.

Layout under `root`:
  ncf/xcpack/<ts>.i000000.j000000.w000.p000.{xcpack,tsv}, <ts>.done
for two timestamps, three stations (XX.ST00-ST02) and their three station
pairs x 9 component pairs, except that pair ST00-ST02 exists on the first
timestamp only and pair ST01-ST02 lacks its Z-E component on both (so its
rotation is skipped). Records are SAC (632-byte header + 201 float32).
"""

from __future__ import annotations

from pathlib import Path

import numpy as np

TIMESTAMPS = ("2020.123.0000", "2020.124.0000")
STATIONS = (("ST00", 31.0, 101.0), ("ST01", 31.4, 101.9), ("ST02", 30.2, 100.6))
COMPONENTS = ("E", "N", "Z")  # the single-letter names the rotation keys on
NPTS = 201
DELTA = 0.5

TSV_COLUMNS = ("timestamp", "worker_id", "anchor_block", "target_begin_block", "target_end_block", "block_size",
               "anchor_begin", "anchor_end", "target_begin", "target_end", "pack_path", "offset", "bytes", "src_id",
               "rec_id", "src_network", "src_station", "src_location", "src_component", "rec_network", "rec_station",
               "rec_location", "rec_component", "npts", "dt", "dist", "az", "baz", "final_pair_path")


def _header(sacbin, src, rec, comp_s, comp_r, ts_index):
    h = sacbin.Header(bytes(632), "<")
    for k in sacbin.FLOATS:
        h.set_float(k, sacbin.NULL_VALUE)
    for k in ("nzyear", "nzjday", "nzhour", "nzmin", "nzsec", "nzmsec"):
        h.set_int(k, 0)
    h.set_int("nvhdr", 6)
    h.set_int("iftype", sacbin.ITIME)
    h.set_int("leven", 1)
    h.set_int("npts", NPTS)
    h.set_float("delta", DELTA)
    h.set_float("b", -DELTA * (NPTS // 2))
    h.set_float("e", DELTA * (NPTS // 2))
    h.set_float("evla", src[1])
    h.set_float("evlo", src[2])
    h.set_float("stla", rec[1])
    h.set_float("stlo", rec[2])
    h.set_int("nzyear", 2020)
    h.set_int("nzjday", 123 + ts_index)
    h.set_text("kevnm", f"XX.{src[0]}")
    h.set_text("kstnm", rec[0])
    h.set_text("knetwk", "XX-XX")
    h.set_text("kcmpnm", f"{comp_s[-1]}{comp_r[-1]}")
    return h


def make_xc_workspace(root) -> Path:
    """Writes the workspace; returns its ncf folder."""
    import sys

    sys.path.insert(0, str(Path(__file__).resolve().parents[2]))
    from fastxc_gb300 import sacbin

    root = Path(root)
    ncf = root / "ncf"
    xcpack = ncf / "xcpack"
    xcpack.mkdir(parents=True, exist_ok=True)
    rng = np.random.default_rng(2024)
    for t, ts in enumerate(TIMESTAMPS):
        name = f"{ts}.i000000.j000000.w000.p000"
        rows = []
        with (xcpack / f"{name}.xcpack").open("wb") as pack:
            for i in range(len(STATIONS)):
                for j in range(i + 1, len(STATIONS)):
                    if (i, j) == (0, 2) and t == 1:
                        continue
                    s, r = STATIONS[i], STATIONS[j]
                    for cs in COMPONENTS:
                        for cr in COMPONENTS:
                            if (i, j) == (1, 2) and (cs, cr) == ("Z", "E"):
                                continue
                            data = (rng.standard_normal(NPTS) * (1.0 + i + 2 * j)).astype(np.float32)
                            blob = sacbin.encode_record(_header(sacbin, s, r, cs, cr, t), data)
                            off = pack.tell()
                            pack.write(blob)
                            fpp = (f"{ncf.as_posix()}/XX.{s[0]}/XX.{r[0]}/XX-XX.{s[0]}-{r[0]}.{cs}-{cr}.sac")
                            rows.append([ts, "0", "0", "0", "1", "64", "0", "3", "0", "3", f"{name}.xcpack", str(off),
                                         str(len(blob)), str(i), str(j), "XX", s[0], "00", cs, "XX", r[0], "00", cr,
                                         str(NPTS), f"{DELTA:.9g}", f"{10.0 * (i + j):.9g}",
                                         f"{30.0 + i:.9g}", f"{210.0 + j:.9g}", fpp])
        with (xcpack / f"{name}.tsv").open("w") as fh:
            fh.write("\t".join(TSV_COLUMNS) + "\n")
            for row in rows:
                fh.write("\t".join(row) + "\n")
        (xcpack / f"{ts}.done").write_text("DONE\n")
    return ncf


def normalize(text: str, root) -> str:
    return text.replace(Path(root).resolve().as_posix(), "{ROOT}")
