"""SourcePack materializer: per-timestamp source-grouped indexes over the
xcpack output of xc_fast.

Drop-in for fastxc/operators/sourcepack/builder.py (build_sourcepack :163-245,
build_sourcepack_timestamp :248-271, AsyncSourcePackMaterializer :27-159).
No NCF bytes are copied: each ``<sourcepack>/<timestamp>/sourcepack_index.tsv``
row points at a record inside an xcpack file. The index columns, row order,
``_SUCCESS`` texts and progress sidecar are the reference's, byte for byte
(tab-separated, CRLF row ends as Python's csv writer produces them).

Row order within a timestamp (``sort_within_source``): (path_id,
component_slot, source_key, receiver_key, input sequence), where the input
sequence numbers the rows of the timestamp's xcpack TSVs read in sorted
file-name order. This materializer ranks components E/1=0, N/2=1, Z/3=2,
R=3, T=4 (builder.py:403-405); the linear stack ranks R with E and T with N
-- both are kept as the reference has them.
"""

from __future__ import annotations

import csv
import re
import shutil
import threading
from dataclasses import dataclass
from pathlib import Path

SOURCEPACK_INDEX_HEADER = [
    "timestamp", "path_id", "component_slot", "source_key", "receiver_key", "src_id", "rec_id",
    "src_network", "src_station", "src_location", "src_component", "rec_network", "rec_station",
    "rec_location", "rec_component", "npts", "dt", "dist", "az", "baz", "record_path", "record_offset",
    "bytes", "storage_kind", "final_pair_path",
]

XCPACK_REQUIRED = {
    "timestamp", "pack_path", "offset", "bytes", "src_id", "rec_id", "src_network", "src_station",
    "src_location", "src_component", "rec_network", "rec_station", "rec_location", "rec_component",
    "npts", "dt", "dist", "az", "baz",
}

PROGRESS_HEADER = ["task", "status", "completed", "total", "unit", "detail"]


@dataclass(frozen=True)
class XcPackRecord:
    sequence: int
    timestamp: str
    pack_path: Path
    offset: int
    bytes: int
    row: dict

    @property
    def source_key(self) -> str:
        return station_key(self.row, "src")

    @property
    def receiver_key(self) -> str:
        return station_key(self.row, "rec")


@dataclass(frozen=True)
class SourcePackBuildResult:
    output_dir: Path
    index_paths: list
    record_count: int
    source_count: int
    bytes_indexed: int


def station_key(row: dict, prefix: str) -> str:
    return f"{row[prefix + '_network']}.{row[prefix + '_station']}.{row[prefix + '_location']}"


def write_progress_file(progress_file, status: str, completed: int, total: int, unit: str, detail: str,
                        task: str = "overall") -> None:
    """Atomic two-line progress sidecar (fastxc/runtime/progress.py:15-42)."""
    if progress_file is None:
        return
    path = Path(progress_file).expanduser().resolve()
    path.parent.mkdir(parents=True, exist_ok=True)
    clean = [str(v).replace("\t", " ").replace("\r", " ").replace("\n", " ")
             for v in (task, status, completed, total, unit, detail)]
    tmp = path.with_name(path.name + ".tmp")
    tmp.write_text("\t".join(PROGRESS_HEADER) + "\n" + "\t".join(clean) + "\n", encoding="utf-8")
    tmp.replace(path)


def read_xcpack_tsv(tsv_path: Path, first_sequence: int) -> list:
    """Rows of one xcpack TSV (fastxc/io/sourcepack.py:119-156): pack paths
    resolved against the TSV's folder and required to exist."""
    out: list = []
    resolved: dict = {}
    with Path(tsv_path).open("r", encoding="utf-8-sig", newline="") as fh:
        reader = csv.DictReader(fh, delimiter="\t")
        if reader.fieldnames is None:
            return out
        missing = XCPACK_REQUIRED.difference(reader.fieldnames)
        if missing:
            raise ValueError(f"XC pack TSV missing fields {sorted(missing)}: {tsv_path}")
        for row in reader:
            text = row["pack_path"]
            pack = resolved.get(text)
            if pack is None:
                pack = Path(text).expanduser()
                if not pack.is_absolute():
                    pack = Path(tsv_path).parent / pack
                if not pack.is_file():
                    raise FileNotFoundError(f"XC pack file is missing for {tsv_path}: {pack}")
                resolved[text] = pack
            try:
                offset, size = int(row["offset"]), int(row["bytes"])
            except ValueError as exc:
                raise ValueError(f"Invalid XC pack numeric field in {tsv_path}: {row}") from exc
            if offset < 0 or size <= 0:
                raise ValueError(f"Invalid XC pack offset/bytes in {tsv_path}: {row}")
            out.append(XcPackRecord(first_sequence + len(out), row["timestamp"], pack, offset, size, row))
    return out


def _component_rank(component: str) -> int:
    tail = component.upper()[-1:] if component else ""
    return {"E": 0, "1": 0, "N": 1, "2": 1, "Z": 2, "3": 2, "R": 3, "T": 4}.get(tail, 100)


def component_slot(src_component: str, rec_component: str) -> int:
    return _component_rank(src_component) * 3 + _component_rank(rec_component)


def path_id_text(row: dict) -> str:
    pid = row.get("path_id", "").strip()
    if pid:
        return pid.zfill(8) if pid.isdigit() else pid
    return f"{int(row['src_id']) * 10000 + int(row['rec_id']):08d}"


def _safe_name(text: str) -> str:
    return re.sub(r"[^0-9A-Za-z._:-]+", "-", text).strip("-") or "item"


def _xcpack_dir_of(root: Path) -> Path:
    return root if root.name == "xcpack" else root / "xcpack"


def _existing_xcpack_dir(root: Path) -> Path:
    d = _xcpack_dir_of(root)
    if d.is_dir():
        return d
    raise FileNotFoundError(f"XC pack directory not found: {root} or {d}")


def _inventory_timestamps(xcpack_dir: Path) -> list:
    ws = xcpack_dir.parent.parent if xcpack_dir.parent.name == "ncf" else xcpack_dir.parent
    index = ws / "manifest" / "timestamp_index.tsv"
    if not index.is_file():
        return []
    with index.open("r", encoding="utf-8-sig", newline="") as fh:
        reader = csv.DictReader(fh, delimiter="\t")
        if not reader.fieldnames or "timestamp" not in reader.fieldnames:
            return []
        found = {row.get("timestamp", "").strip() for row in reader}
    return sorted(t for t in found if t)


def _done_timestamps(xcpack_dir: Path) -> list:
    return [p.name[:-len(".done")] for p in xcpack_dir.glob("*.done") if not p.name.startswith("_")]


def _index_row(rec: XcPackRecord) -> dict:
    row = rec.row
    return {
        "timestamp": rec.timestamp,
        "path_id": path_id_text(row),
        "component_slot": str(component_slot(row["src_component"], row["rec_component"])),
        "source_key": rec.source_key,
        "receiver_key": rec.receiver_key,
        **{k: row[k] for k in ("src_id", "rec_id", "src_network", "src_station", "src_location", "src_component",
                               "rec_network", "rec_station", "rec_location", "rec_component", "npts", "dt",
                               "dist", "az", "baz")},
        "record_path": rec.pack_path.as_posix(),
        "record_offset": str(rec.offset),
        "bytes": str(rec.bytes),
        "storage_kind": "xcpack",
        "final_pair_path": row.get("final_pair_path", ""),
    }


def _write_timestamp_index(timestamp: str, records: list, output_dir: Path,
                           sort_within_source: bool) -> SourcePackBuildResult:
    """<output_dir>/<safe timestamp>/{sourcepack_index.tsv,_SUCCESS}, written
    in a dot-prefixed temporary folder and renamed into place."""
    target = output_dir / _safe_name(timestamp)
    tmp = output_dir / f".{_safe_name(timestamp)}.tmp"
    if tmp.exists():
        shutil.rmtree(tmp)
    tmp.mkdir(parents=True)
    if sort_within_source:
        records = sorted(records, key=lambda r: (path_id_text(r.row),
                                                 component_slot(r.row["src_component"], r.row["rec_component"]),
                                                 r.source_key, r.receiver_key, r.sequence))
    else:
        records = sorted(records, key=lambda r: r.sequence)
    sources = set()
    nbytes = 0
    with (tmp / "sourcepack_index.tsv").open("w", encoding="utf-8", newline="") as fh:
        writer = csv.DictWriter(fh, fieldnames=SOURCEPACK_INDEX_HEADER, delimiter="\t")
        writer.writeheader()
        for rec in records:
            sources.add(rec.source_key)
            nbytes += rec.bytes
            writer.writerow(_index_row(rec))
    (tmp / "_SUCCESS").write_text(
        f"timestamp\t{timestamp}\nrecords\t{len(records)}\nsources\t{len(sources)}\nbytes_indexed\t{nbytes}\n",
        encoding="utf-8")
    if target.exists():
        shutil.rmtree(target)
    tmp.replace(target)
    return SourcePackBuildResult(target, [target / "sourcepack_index.tsv"], len(records), len(sources), nbytes)


def build_sourcepack(xc_output_root, sourcepack_dir=None, *, sort_within_source: bool = True,
                     progress_file=None) -> SourcePackBuildResult:
    """Index every timestamp of an xc_fast output (default output folder:
    ``<xcpack>/../sourcepack``)."""
    xcpack_dir = _existing_xcpack_dir(Path(xc_output_root).expanduser().resolve())
    out = (Path(sourcepack_dir).expanduser().resolve() if sourcepack_dir is not None
           else xcpack_dir.parent / "sourcepack")
    out.mkdir(parents=True, exist_ok=True)
    by_ts: dict = {}
    seq = 0
    for tsv in sorted(xcpack_dir.glob("*.tsv")):
        for rec in read_xcpack_tsv(tsv, seq):
            by_ts.setdefault(rec.timestamp, []).append(rec)
            seq += 1
    stamps = sorted(set(by_ts) | set(_inventory_timestamps(xcpack_dir)) | set(_done_timestamps(xcpack_dir)))
    if not stamps:
        raise FileNotFoundError(f"No XC pack timestamps found in {xcpack_dir}")
    write_progress_file(progress_file, "RUNNING", 0, len(stamps), "timestamps", "source index build")
    paths: list = []
    nrec = nsrc = nbytes = 0
    for i, ts in enumerate(stamps, start=1):
        r = _write_timestamp_index(ts, by_ts.get(ts, []), out, sort_within_source)
        paths.extend(r.index_paths)
        nrec += r.record_count
        nsrc += r.source_count
        nbytes += r.bytes_indexed
        write_progress_file(progress_file, "RUNNING", i, len(stamps), "timestamps", f"{ts}: {r.record_count} records")
    write_progress_file(progress_file, "DONE", len(stamps), len(stamps), "timestamps", "source index ready")
    return SourcePackBuildResult(out, paths, nrec, nsrc, nbytes)


def build_sourcepack_timestamp(xc_output_root, sourcepack_dir, timestamp: str, *,
                               sort_within_source: bool = True) -> SourcePackBuildResult:
    """Index one timestamp: its own TSVs (file names starting with the
    timestamp), or every TSV when none does."""
    xcpack_dir = _existing_xcpack_dir(Path(xc_output_root).expanduser().resolve())
    out = Path(sourcepack_dir).expanduser().resolve()
    tsvs = sorted(p for p in xcpack_dir.glob("*.tsv") if p.name.startswith(timestamp)) or \
        sorted(xcpack_dir.glob("*.tsv"))
    seq = 0
    recs: list = []
    for tsv in tsvs:
        for rec in read_xcpack_tsv(tsv, seq):
            seq += 1
            if rec.timestamp == timestamp:
                recs.append(rec)
    return _write_timestamp_index(timestamp, recs, out, sort_within_source)


class AsyncSourcePackMaterializer:
    """Indexes each timestamp as soon as xc_fast writes its ``<ts>.done``
    marker, on a polling thread; finish() indexes what is left, writes the
    global ``_SUCCESS`` and the progress sidecar."""

    def __init__(self, xc_output_root, sourcepack_dir, *, sort_within_source: bool = True, progress_file=None,
                 poll_interval_sec: float = 5.0):
        self.xcpack_dir = _xcpack_dir_of(Path(xc_output_root).expanduser().resolve())
        self.output_dir = Path(sourcepack_dir).expanduser().resolve()
        self.sort_within_source = sort_within_source
        self.progress_file = progress_file
        self.poll_interval_sec = max(0.5, float(poll_interval_sec))
        self._stop = threading.Event()
        self._thread = None
        self._done: set = set()
        self._errors: list = []
        self._lock = threading.Lock()
        self._records = self._sources = self._bytes = 0
        inv = _inventory_timestamps(self.xcpack_dir)
        self._expected = len(inv) if inv else (len(_done_timestamps(self.xcpack_dir)) if self.xcpack_dir.is_dir()
                                               else 0)

    def start(self) -> None:
        self.output_dir.mkdir(parents=True, exist_ok=True)
        write_progress_file(self.progress_file, "RUNNING", 0, self._expected, "timestamps", "async source index build")
        self._thread = threading.Thread(target=self._run, name="sourcepack-materializer", daemon=True)
        self._thread.start()

    def _run(self) -> None:
        while not self._stop.is_set():
            try:
                self._scan_once()
            except BaseException as exc:  # reported by finish()
                self._errors.append(exc)
                self._stop.set()
                return
            self._stop.wait(self.poll_interval_sec)

    def _scan_once(self) -> None:
        if not self.xcpack_dir.is_dir():
            return
        for done in sorted(self.xcpack_dir.glob("*.done")):
            if done.name.startswith("_"):
                continue
            ts = done.name[:-len(".done")]
            with self._lock:
                if ts in self._done:
                    continue
            r = build_sourcepack_timestamp(self.xcpack_dir, self.output_dir, ts,
                                           sort_within_source=self.sort_within_source)
            with self._lock:
                self._done.add(ts)
                self._records += r.record_count
                self._sources += r.source_count
                self._bytes += r.bytes_indexed
                n = len(self._done)
            write_progress_file(self.progress_file, "RUNNING", n, self._expected, "timestamps",
                                f"{ts}: {r.record_count} records")

    def finish(self, *, mark_success: bool = True, status_message: str | None = None) -> SourcePackBuildResult:
        self._stop.set()
        if self._thread is not None:
            self._thread.join()
        self._scan_once()
        if self._errors:
            write_progress_file(self.progress_file, "FAILED", len(self._done), self._expected, "timestamps",
                                str(self._errors[0]))
            raise RuntimeError("async SourcePack materialization failed") from self._errors[0]
        paths = sorted(self.output_dir.glob("*/sourcepack_index.tsv"))
        success = self.output_dir / "_SUCCESS"
        total = self._expected or len(paths)
        if mark_success:
            success.write_text(f"timestamps\t{len(paths)}\nrecords\t{self._records}\n"
                               f"sources\t{self._sources}\nbytes_indexed\t{self._bytes}\n", encoding="utf-8")
            write_progress_file(self.progress_file, "DONE", len(paths), total, "timestamps", "source index ready")
        else:
            success.unlink(missing_ok=True)
            write_progress_file(self.progress_file, "FAILED", len(paths), total, "timestamps",
                                status_message or "upstream XC did not complete; global success marker withheld")
        return SourcePackBuildResult(self.output_dir, paths, self._records, self._sources, self._bytes)


def discover_sourcepack_indexes(sourcepack_input) -> list:
    """An index file, a folder holding one, or a folder of per-timestamp
    index folders (fastxc/io/sourcepack.py:75-91)."""
    path = Path(sourcepack_input).expanduser().resolve()
    if path.is_file():
        return [path]
    if not path.is_dir():
        raise FileNotFoundError(f"SourcePack input not found: {path}")
    direct = path / "sourcepack_index.tsv"
    if direct.is_file():
        return [direct]
    found = sorted(p for p in path.glob("*/sourcepack_index.tsv") if p.is_file())
    if not found:
        raise FileNotFoundError(f"No sourcepack_index.tsv found under {path}")
    return found
