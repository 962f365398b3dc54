"""Python readers/writers of the file formats the drop-in executables use
(stepack v3 batches + TSV, xcpack records + TSV, SAC headers, allowed-path
tables). Byte layouts follow native/sac2spec/io/stepack_writer.c,
native/xc/pack_io/pack_writer.cu and native/xc/include/sac.h."""

from __future__ import annotations

import csv
import struct
from pathlib import Path

import numpy as np

SAC_HEADER_BYTES = 632
STEPACK_HDR = struct.Struct("<8sIIIIQQQIIIIffQQQQ64s64s")
STEPACK_NSLC = struct.Struct("<IIff16s32s16s16s32s")
STEPACK_TSV_COLUMNS = [
    "timestamp", "worker_id", "batch_seq", "start_group", "group_count", "pack_path", "offset", "bytes",
    "version", "layout", "nstep", "nslc_start", "nslc_count", "batch_nslc_count", "nspec", "dt", "df",
    "nslc_table_bytes", "payload_offset", "payload_bytes", "batch_payload_bytes", "step_bytes",
    "pitch_step_bytes", "nslc_step_bytes", "first_nsl_id", "last_nsl_id",
]


def write_stepack(root, worker_id: int, batch_seq: int, channels, spectra: np.ndarray, dt: float, df: float,
                  group_count: int = 0, start_group: int = 0) -> Path:
    """One stepack batch. channels: list of dicts (timestamp, nsl_id, network,
    station, location, component, stla, stlo) in payload order; spectra
    complex64 [nstep][nslc][nspec]."""
    root = Path(root).resolve()
    root.mkdir(parents=True, exist_ok=True)
    nstep, n, nspec = spectra.shape
    pack = root / f"w{worker_id:03d}.b{batch_seq:06d}.stepack"
    tsv = root / f"w{worker_id:03d}.b{batch_seq:06d}.tsv"
    table = n * STEPACK_NSLC.size
    nslc_step = nspec * 8
    pitch = n * nslc_step
    payload = nstep * pitch
    poff = STEPACK_HDR.size + table
    hdr = STEPACK_HDR.pack(b"FXCSTPK\0", 3, STEPACK_HDR.size, STEPACK_NSLC.size, 2, batch_seq, start_group,
                           group_count, worker_id, nstep, n, nspec, dt, df, table, poff, payload, pitch,
                           channels[0]["timestamp"].encode().ljust(64, b"\0"), b"\0" * 64)
    with pack.open("wb") as fh:
        fh.write(hdr)
        for i, c in enumerate(channels):
            fh.write(STEPACK_NSLC.pack(i, c["nsl_id"], c.get("stla", 0.0), c.get("stlo", 0.0),
                                       c["network"].encode(), c["station"].encode(), c.get("location", "").encode(),
                                       c["component"].encode(), b"\0" * 32))
        fh.write(np.ascontiguousarray(spectra, np.complex64).tobytes())
    num_ch = n // group_count if group_count and n % group_count == 0 else 0
    rows = []
    b = 0
    while b < n:
        e = b + 1
        while e < n and channels[e]["timestamp"] == channels[b]["timestamp"]:
            e += 1
        rc = e - b
        sg, gc = start_group, group_count
        if num_ch and b % num_ch == 0 and rc % num_ch == 0:
            sg, gc = start_group + b // num_ch, rc // num_ch
        rows.append([channels[b]["timestamp"], worker_id, batch_seq, sg, gc, str(pack), 0, STEPACK_HDR.size + table + payload,
                     3, 2, nstep, b, rc, n, nspec, f"{dt:.9g}", f"{df:.9g}", table, poff, nstep * rc * nslc_step,
                     payload, rc * nslc_step, pitch, nslc_step, channels[b]["nsl_id"], channels[e - 1]["nsl_id"]])
        b = e
    with tsv.open("w") as fh:
        fh.write("\t".join(STEPACK_TSV_COLUMNS) + "\n")
        for r in rows:
            fh.write("\t".join(str(x) for x in r) + "\n")
    return pack


def write_allowed_paths(path, rows) -> None:
    """rows: (src_nsl, rec_nsl, gcarc, dist, az, baz) with src <= rec; 9-column
    layout read by load_allowed_path_table (native/xc/io/path_table.c:82-180)."""
    with open(path, "w") as fh:
        fh.write("path_id\tsrc_id\trec_id\tsrc_key\trec_key\tgcarc\tdist\taz\tbaz\n")
        for s, r, g, d, a, b in rows:
            fh.write(f"{s * 10000 + r}\t{s}\t{r}\tS{s}\tS{r}\t{g}\t{d}\t{a}\t{b}\n")


SAC_FLOAT = {"delta": 0, "b": 5, "e": 6, "o": 7, "stla": 31, "stlo": 32, "evla": 35, "evlo": 36, "user0": 40,
             "user1": 41, "user2": 42, "dist": 50, "az": 51, "baz": 52, "gcarc": 53}
SAC_INT = {"nzyear": 0, "nzjday": 1, "nzhour": 2, "nzmin": 3, "nzsec": 4, "nzmsec": 5, "nvhdr": 6, "npts": 9,
           "iftype": 15, "leven": 35, "unused27": 39}
SAC_STR = {"kstnm": (440, 8), "kevnm": (448, 16), "kcmpnm": (600, 8), "knetwk": (608, 8)}


def parse_sac_header(raw: bytes) -> dict:
    f = np.frombuffer(raw[:280], "<f4")
    i = np.frombuffer(raw[280:440], "<i4")
    out = {k: float(f[v]) for k, v in SAC_FLOAT.items()}
    out.update({k: int(i[v]) for k, v in SAC_INT.items()})
    out.update({k: raw[o:o + n].decode("ascii", "replace") for k, (o, n) in SAC_STR.items()})
    return out


def read_xcpack_dir(root) -> list[dict]:
    """Every record of every xcpack TSV under root, in file and row order:
    the TSV row plus 'header' (parsed SAC header) and 'data' (float32)."""
    out = []
    for tsv in sorted(Path(root).glob("*.tsv")):
        with tsv.open() as fh:
            for row in csv.DictReader(fh, delimiter="\t"):
                with open(row["pack_path"], "rb") as pf:
                    pf.seek(int(row["offset"]))
                    raw = pf.read(int(row["bytes"]))
                row["header"] = parse_sac_header(raw[:SAC_HEADER_BYTES])
                row["data"] = np.frombuffer(raw[SAC_HEADER_BYTES:], "<f4").copy()
                row["tsv"] = tsv.name
                out.append(row)
    return out


SOURCEPACK_COLUMNS = [
    "timestamp", "path_id", "component_slot", "source_key", "receiver_key", "src_id", "rec_id",
    "src_network", "src_station", "src_location", "src_component", "rec_network", "rec_station",
    "rec_location", "rec_component", "npts", "dt", "dist", "az", "baz", "record_path", "record_offset",
    "bytes", "storage_kind", "final_pair_path",
]


def sac_header_bytes(npts: int, delta: float, b: float = 0.0, **fields) -> bytes:
    """632-byte little-endian SAC header: SAC null values (-12345, "-12345  ")
    except version 6, npts, delta, b, iftype 1, leven 1 and `fields`
    (names of SAC_FLOAT / SAC_INT / SAC_STR)."""
    f = np.full(70, -12345.0, "<f4")
    i = np.full(40, -12345, "<i4")
    f[0], f[5] = delta, b
    i[6], i[9], i[15], i[35] = 6, npts, 1, 1
    s = bytearray(b"-12345  " * 24)
    s[8:24] = b"-12345".ljust(16)  # kevnm is 16 characters wide
    for k, v in fields.items():
        if k in SAC_FLOAT:
            f[SAC_FLOAT[k]] = v
        elif k in SAC_INT:
            i[SAC_INT[k]] = v
        else:
            o, n = SAC_STR[k]
            s[o - 440:o - 440 + n] = str(v).encode()[:n].ljust(n)
    return f.tobytes() + i.tobytes() + bytes(s)


def write_sourcepack(root, name: str, rows) -> Path:
    """One SourcePack shard: <name>.pack of SAC records and <name>.tsv index.
    rows: dicts with the index columns (except record_path, record_offset,
    bytes, npts, dt) plus 'data' (float32 trace), 'delta' and optionally
    'sac' (extra header fields for sac_header_bytes)."""
    root = Path(root).resolve()
    root.mkdir(parents=True, exist_ok=True)
    pack, tsv = root / f"{name}.pack", root / f"{name}.tsv"
    with pack.open("wb") as fh, tsv.open("w") as th:
        th.write("\t".join(SOURCEPACK_COLUMNS) + "\n")
        for r in rows:
            data = np.ascontiguousarray(r["data"], "<f4")
            blob = sac_header_bytes(data.size, r["delta"], b=-(data.size // 2) * r["delta"],
                                    **r.get("sac", {})) + data.tobytes()
            off = fh.tell()
            fh.write(blob)
            row = dict(r, record_path=str(pack), record_offset=off, bytes=len(blob), npts=data.size,
                       dt=f"{r['delta']:g}", storage_kind=r.get("storage_kind", "xcpack"))
            th.write("\t".join(str(row.get(c, "")) for c in SOURCEPACK_COLUMNS) + "\n")
    return tsv


def read_sourcepack_index(path) -> list[dict]:
    """Rows of a SourcePack index with their SAC records ('header', 'data')."""
    out = []
    with open(path) as fh:
        for row in csv.DictReader(fh, delimiter="\t"):
            with open(row["record_path"], "rb") as pf:
                pf.seek(int(row["record_offset"]))
                raw = pf.read(int(row["bytes"]))
            row["header"] = parse_sac_header(raw[:SAC_HEADER_BYTES])
            row["raw_header"] = raw[:SAC_HEADER_BYTES]
            row["data"] = np.frombuffer(raw[SAC_HEADER_BYTES:], "<f4").copy()
            out.append(row)
    return out


def read_stepack(pack) -> dict:
    """Header fields, NSLC entries and payload (complex64 [nstep][nslc][nspec])
    of one stepack batch file."""
    raw = Path(pack).read_bytes()
    h = STEPACK_HDR.unpack_from(raw, 0)
    names = ["magic", "version", "header_size", "nslc_entry_size", "layout", "batch_seq", "start_group",
             "group_count", "worker_id", "nstep", "nslc_count", "nspec", "dt", "df", "nslc_table_bytes",
             "payload_offset", "payload_bytes", "pitch_step_bytes", "first_timestamp", "reserved"]
    hd = dict(zip(names, h))
    hd["magic"] = hd["magic"].rstrip(b"\0").decode()
    hd["first_timestamp"] = hd["first_timestamp"].rstrip(b"\0").decode()
    ents = []
    for i in range(hd["nslc_count"]):
        e = STEPACK_NSLC.unpack_from(raw, hd["header_size"] + i * hd["nslc_entry_size"])
        ents.append(dict(file_index=e[0], nsl_id=e[1], stla=e[2], stlo=e[3],
                         network=e[4].rstrip(b"\0").decode(), station=e[5].rstrip(b"\0").decode(),
                         location=e[6].rstrip(b"\0").decode(), component=e[7].rstrip(b"\0").decode()))
    pay = np.frombuffer(raw, np.complex64, count=hd["nstep"] * hd["nslc_count"] * hd["nspec"],
                        offset=hd["payload_offset"]).reshape(hd["nstep"], hd["nslc_count"], hd["nspec"])
    return {"header": hd, "entries": ents, "payload": pay}


def write_sac(path, data: np.ndarray, delta: float, **fields) -> None:
    """A SAC file: header (sac_header_bytes) + float32 samples."""
    data = np.ascontiguousarray(data, "<f4")
    Path(path).write_bytes(sac_header_bytes(data.size, delta, **fields) + data.tobytes())
