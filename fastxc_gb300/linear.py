"""Cross-timestamp linear stack of SourcePack records, on the GPU.

Drop-in for linear_stack_sourcepack_indexes
(fastxc/operators/stacking/linear_stack.py:312-391). Records of all input
indexes are merged by (path_id, component_slot) group key in one streaming
k-way merge (:163-189); a group's records are read in (timestamp,
record_path, offset) order and averaged in FP64 (the sum runs in that
order, then one division by the record count, then float32, :228-247) by
fxc_linear_stack -- the same operations in the same order, so the stacked
samples are bit-identical to the reference's. The outputs are the
reference's: ``<stack_dir>/linearstack_sourcepack/STACK/{linearstack.pack,
sourcepack_index.tsv,_SUCCESS}`` built in a ``STACK.tmp`` folder and renamed
into place, SAC headers from each group's first record with npts, iftype,
user0 = record count and the fixed reference time of :81-92.
"""

from __future__ import annotations

import csv
import heapq
import shutil
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import sacbin
from .sourcepack import SOURCEPACK_INDEX_HEADER


@dataclass(frozen=True)
class StackResult:
    input_path: Path
    output_path: Path
    segment_count: int
    sample_count: int


@dataclass(frozen=True)
class IndexRecord:
    row: dict
    record_path: Path
    record_offset: int
    record_bytes: int


def linear_sourcepack_dir(stack_dir) -> Path:
    return Path(stack_dir).expanduser().resolve() / "linearstack_sourcepack" / "STACK"


def linear_output_path(final_pair_path, stack_dir) -> Path:
    parts = Path(final_pair_path).name.split(".")
    if parts and parts[-1].lower() == "sac":
        parts = parts[:-1]
    if len(parts) < 3:
        raise ValueError(f"Unexpected final pair path: {Path(final_pair_path).name}")
    pair = f"{parts[0]}.{parts[1]}"
    return Path(stack_dir).expanduser().resolve() / "linearstack" / pair / f"{pair}.{parts[2]}.linearstack.sac"


def _rank(component: str) -> int:
    # the linear stack's own ranking: R with E, T with N
    tail = component.upper()[-1:] if component else ""
    return {"E": 0, "1": 0, "R": 0, "N": 1, "2": 1, "T": 1, "Z": 2, "3": 2}.get(tail, 100)


def _path_id(row: dict) -> str:
    pid = row.get("path_id", "").strip()
    if pid:
        return pid.zfill(8) if pid.isdigit() else pid
    try:
        return f"{int(row['src_id']) * 10000 + int(row['rec_id']):08d}"
    except (KeyError, ValueError):
        return ""


def _slot(row: dict) -> int:
    text = row.get("component_slot", "").strip()
    if text.isdigit():
        return int(text)
    return _rank(row.get("src_component", "")) * 3 + _rank(row.get("rec_component", ""))


def _group_key(rec: IndexRecord) -> tuple:
    return (_path_id(rec.row), _slot(rec.row))


def _final_pair(rec: IndexRecord) -> str:
    row = rec.row
    fp = row.get("final_pair_path")
    if fp:
        return fp
    return (f"{row['src_network']}-{row['rec_network']}.{row['src_station']}-{row['rec_station']}."
            f"{row['src_component']}-{row['rec_component']}.sac")


_REQUIRED = {"source_key", "receiver_key", "record_path", "record_offset", "bytes", "src_component", "rec_component"}


def _index_records(path: Path, fh):
    reader = csv.DictReader(fh, delimiter="\t")
    if reader.fieldnames is None:
        return
    missing = _REQUIRED.difference(reader.fieldnames)
    if missing:
        raise ValueError(f"Source index missing fields {sorted(missing)}: {path}")
    for row in reader:
        rp = Path(row["record_path"]).expanduser()
        if not rp.is_absolute():
            rp = path.parent / rp
        yield IndexRecord(row, rp, int(row["record_offset"]), int(row["bytes"]))


def stream_groups(indexes):
    """(group key, records) in ascending key order over all indexes; the
    records of a group sorted by (timestamp, record_path, offset)."""
    files = []
    heap = []
    tick = 0
    try:
        for index in indexes:
            path = Path(index).expanduser().resolve()
            fh = path.open("r", encoding="utf-8-sig", newline="")
            files.append(fh)
            it = _index_records(path, fh)
            first = next(it, None)
            if first is not None:
                heapq.heappush(heap, (_group_key(first), tick, first, it))
                tick += 1
        while heap:
            key = heap[0][0]
            group = []
            while heap and heap[0][0] == key:
                _, _, rec, it = heapq.heappop(heap)
                group.append(rec)
                nxt = next(it, None)
                if nxt is not None:
                    heapq.heappush(heap, (_group_key(nxt), tick, nxt, it))
                    tick += 1
            group.sort(key=lambda r: (r.row.get("timestamp", ""), r.record_path.as_posix(), r.record_offset))
            yield key, group
    finally:
        for fh in reversed(files):
            fh.close()


def _stacked_header(first: sacbin.Header, count: int, divisor: int) -> sacbin.Header:
    h = first.copy()
    h.set_int("npts", int(count))
    h.set_int("iftype", sacbin.ITIME)
    h.set_float("user0", float(divisor))
    for name, value in (("nzyear", 2010), ("nzjday", 214), ("nzhour", 0), ("nzmin", 0), ("nzsec", 0),
                        ("nzmsec", 0)):
        h.set_int(name, value)
    return h


def _index_row(template: dict, pack_path: Path, offset: int, nbytes: int, final_path: Path,
               hd: sacbin.Header) -> dict:
    row = {f: "" for f in SOURCEPACK_INDEX_HEADER}
    for key in ("path_id", "component_slot", "source_key", "receiver_key", "src_id", "rec_id", "src_network",
                "src_station", "src_location", "src_component", "rec_network", "rec_station", "rec_location",
                "rec_component", "dist", "az", "baz"):
        row[key] = template.get(key, "")
    row.update({
        "timestamp": "STACK",
        "npts": str(hd.npts),
        "dt": f"{hd.get_float('delta'):.9g}",
        "record_path": pack_path.as_posix(),
        "record_offset": str(offset),
        "bytes": str(nbytes),
        "storage_kind": "linearstack_pack",
        "final_pair_path": final_path.as_posix(),
    })
    return row


class _GpuMean:
    """FP64 group means of float32 traces through fxc_linear_stack."""

    def __init__(self, ctx=None):
        import torch

        from .core import Context

        if not torch.cuda.is_available():
            raise RuntimeError("the GPU linear stack needs a CUDA device")
        self.torch = torch
        self.ctx = ctx or Context(torch.cuda.current_device(), torch.cuda.current_stream().cuda_stream)

    def __call__(self, traces: np.ndarray, counts: np.ndarray) -> np.ndarray:
        from .stack import linear_stack

        torch = self.torch
        nsamples = traces.shape[1]
        offsets = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
        d_tr = torch.from_numpy(np.ascontiguousarray(traces)).cuda()
        d_out = torch.empty((counts.size, nsamples), dtype=torch.float32, device=d_tr.device)
        linear_stack(self.ctx, d_tr, offsets, counts.astype(np.int32), nsamples, d_out)
        self.ctx.synchronize()
        return d_out.cpu().numpy()


def linear_stack_sourcepack_indexes(indexes, stack_dir, *, dry_run: bool = False, ctx=None,
                                    batch_bytes: int = 1 << 30) -> list:
    indexes = list(indexes)
    out_dir = linear_sourcepack_dir(stack_dir)
    pack_path = out_dir / "linearstack.pack"
    index_path = out_dir / "sourcepack_index.tsv"
    if dry_run:
        return [StackResult(Path(_final_pair(g[0])), pack_path, len(g), 0) for _, g in stream_groups(indexes)]

    tmp = out_dir.with_name(out_dir.name + ".tmp")
    if tmp.exists():
        shutil.rmtree(tmp)
    tmp.mkdir(parents=True, exist_ok=True)
    mean = _GpuMean(ctx)
    results: list = []
    handles: dict = {}

    def read(rec: IndexRecord):
        fh = handles.get(rec.record_path)
        if fh is None:
            fh = handles[rec.record_path] = rec.record_path.open("rb")
        return sacbin.read_record_from(fh, rec.record_path, rec.record_offset, rec.record_bytes)

    try:
        with (tmp / "linearstack.pack").open("wb") as pack, \
                (tmp / "sourcepack_index.tsv").open("w", encoding="utf-8", newline="") as idx:
            writer = csv.DictWriter(idx, fieldnames=SOURCEPACK_INDEX_HEADER, delimiter="\t")
            writer.writeheader()
            batch = []  # (records, first header, traces [n][count])
            batch_len = 0

            def flush():
                nonlocal batch_len
                if not batch:
                    return
                traces = np.concatenate([b[2] for b in batch], axis=0)
                counts = np.array([b[2].shape[0] for b in batch], np.int64)
                stacked = mean(traces, counts)
                for (recs, first, tr), data in zip(batch, stacked):
                    hd = _stacked_header(first, tr.shape[1], tr.shape[0])
                    off = pack.tell()
                    blob = sacbin.encode_record(hd, data)
                    pack.write(blob)
                    final = _final_pair(recs[0])
                    lpath = linear_output_path(final, stack_dir)
                    writer.writerow(_index_row(recs[0].row, pack_path, off, len(blob), lpath, hd))
                    results.append(StackResult(Path(final), lpath, len(recs), hd.data_count))
                batch.clear()
                batch_len = 0

            for _, recs in stream_groups(indexes):
                first, data0 = read(recs[0])
                count = first.data_count
                delta = first.get_float("delta")
                tr = np.empty((len(recs), count), np.float32)
                tr[0] = data0
                for i, rec in enumerate(recs[1:], start=1):
                    hd, data = read(rec)
                    if hd.data_count != count:
                        raise ValueError(f"{rec.record_path}: data_count mismatch ({hd.data_count} vs {count})")
                    if not np.isclose(hd.get_float("delta"), delta, rtol=0.0, atol=1.0e-7):
                        raise ValueError(f"{rec.record_path}: delta mismatch ({hd.get_float('delta')} vs {delta})")
                    tr[i] = data
                if batch and batch[0][2].shape[1] != count:
                    flush()  # one trace length per GPU batch
                batch.append((recs, first, tr))
                batch_len += tr.nbytes
                if batch_len >= batch_bytes or len(batch) == 65535:  # the kernel's per-call group limit
                    flush()
            flush()
    finally:
        for fh in handles.values():
            fh.close()

    if not results:
        shutil.rmtree(tmp, ignore_errors=True)
        return []
    (tmp / "_SUCCESS").write_text(f"records\t{len(results)}\npack\t{pack_path}\nindex\t{index_path}\n",
                                  encoding="utf-8")
    if out_dir.exists():
        shutil.rmtree(out_dir)
    tmp.replace(out_dir)
    return results
