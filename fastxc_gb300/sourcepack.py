"""SourcePack materializer: Python entry points over the library's native
index builder (``fxc_sourcepack_build`` / ``fxc_sourcepack_async_*`` in
``csrc/sourcepack_index.cpp``).

The names, arguments and results are those the reference's pipeline calls
(fastxc/operators/sourcepack/builder.py: build_sourcepack,
build_sourcepack_timestamp, AsyncSourcePackMaterializer; and
fastxc/io/sourcepack.py: discover_sourcepack_indexes), so the pipeline can
import them unchanged. All parsing, ordering and file writing happens in
C++; ``xc_fast --sourcepack DIR`` emits the same per-timestamp indexes
itself, right after each timestamp's records are written.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

from ._lib import FXC_ERR_INVALID, FXC_ERR_NOTFOUND, FXC_OK, lib
from ._lib import SourcePackTotals as Totals

# Columns of sourcepack_index.tsv, in file order (fastxc/io/sourcepack.py:30-56).
SOURCEPACK_INDEX_HEADER = [
    "timestamp", "path_id", "component_slot", "source_key", "receiver_key", "src_id", "rec_id",
    "src_network", "src_station", "src_location", "src_component", "rec_network", "rec_station",
    "rec_location", "rec_component", "npts", "dt", "dist", "az", "baz", "record_path", "record_offset",
    "bytes", "storage_kind", "final_pair_path",
]


@dataclass(frozen=True)
class SourcePackBuildResult:
    output_dir: Path
    index_paths: list
    record_count: int
    source_count: int
    bytes_indexed: int


def _native():
    """(library, raw entry points): statuses are mapped to Python exceptions here."""
    L = lib()
    return L, type("Raw", (), {k: getattr(L, "_raw_" + k) for k in (
        "fxc_sourcepack_build", "fxc_sourcepack_async_start", "fxc_sourcepack_async_finish")})


def _enc(p) -> bytes | None:
    return None if p is None else str(Path(p).expanduser()).encode()


def _raise(status: int, L, what: str):
    msg = L.last_error()
    if status == FXC_ERR_NOTFOUND:
        raise FileNotFoundError(msg)
    if status == FXC_ERR_INVALID:
        raise ValueError(f"{what}: {msg}")
    raise ValueError(msg) if "TSV" in msg else OSError(f"{what}: {msg}")


def _index_paths(out_dir: Path) -> list:
    return sorted(p for p in out_dir.glob("*/sourcepack_index.tsv") if p.is_file())


def _build(xc_output_root, sourcepack_dir, timestamp, sort_within_source, progress_file, what):
    """One native build; returns (output folder, indexed folder names, totals)."""
    L, cd = _native()
    t = Totals()
    out = C.create_string_buffer(4096)
    names = C.create_string_buffer(1 << 22)
    st = cd.fxc_sourcepack_build(_enc(xc_output_root), _enc(sourcepack_dir),
                                 None if timestamp is None else timestamp.encode(), 1 if sort_within_source else 0,
                                 _enc(progress_file), C.byref(t), out, len(out), names, len(names))
    if st != FXC_OK:
        _raise(st, L, what)
    return Path(out.value.decode()), names.value.decode().splitlines(), t


def build_sourcepack(xc_output_root, sourcepack_dir=None, *, sort_within_source: bool = True,
                     progress_file=None) -> SourcePackBuildResult:
    """Index every timestamp of an xc output (default output folder:
    ``<xcpack>/../sourcepack``); no NCF bytes are copied."""
    out, names, t = _build(xc_output_root, sourcepack_dir, None, sort_within_source, progress_file,
                           "build_sourcepack")
    return SourcePackBuildResult(out, [out / n / "sourcepack_index.tsv" for n in names], t.records, t.sources,
                                 t.bytes_indexed)


def build_sourcepack_timestamp(xc_output_root, sourcepack_dir, timestamp: str, *,
                               sort_within_source: bool = True) -> SourcePackBuildResult:
    """Index one timestamp from its own TSVs (names starting with the
    timestamp; every TSV when none does)."""
    out, names, t = _build(xc_output_root, sourcepack_dir, timestamp, sort_within_source, None,
                           "build_sourcepack_timestamp")
    target = out / names[0]
    return SourcePackBuildResult(target, [target / "sourcepack_index.tsv"], t.records, t.sources, t.bytes_indexed)


class AsyncSourcePackMaterializer:
    """Indexes each timestamp once xc_fast has written its ``<ts>.done``
    marker, from a native polling thread; ``finish`` indexes what is left and
    writes the global ``_SUCCESS``."""

    def __init__(self, xc_output_root, sourcepack_dir, *, sort_within_source: bool = True, progress_file=None,
                 poll_interval_sec: float = 5.0):
        self.xc_output_root = xc_output_root
        self.output_dir = Path(sourcepack_dir).expanduser().resolve()
        self.sort_within_source = sort_within_source
        self.progress_file = progress_file
        self.poll_interval_sec = max(0.5, float(poll_interval_sec))
        self._handle = None

    def start(self) -> None:
        L, cd = _native()
        h = C.c_void_p()
        st = cd.fxc_sourcepack_async_start(_enc(self.xc_output_root), _enc(self.output_dir),
                                           1 if self.sort_within_source else 0, _enc(self.progress_file),
                                           self.poll_interval_sec, C.byref(h))
        if st != FXC_OK:
            _raise(st, L, "AsyncSourcePackMaterializer.start")
        self._handle = h

    def finish(self, *, mark_success: bool = True, status_message: str | None = None) -> SourcePackBuildResult:
        L, cd = _native()
        if self._handle is None:
            self.start()
        t = Totals()
        st = cd.fxc_sourcepack_async_finish(self._handle, 1 if mark_success else 0,
                                            status_message.encode() if status_message else None, C.byref(t))
        self._handle = None
        if st != FXC_OK:
            raise RuntimeError(f"async SourcePack indexing failed: {L.last_error()}")
        return SourcePackBuildResult(self.output_dir, _index_paths(self.output_dir), t.records, t.sources,
                                     t.bytes_indexed)


def discover_sourcepack_indexes(sourcepack_input) -> list:
    """An index file, a folder holding one, or a folder of per-timestamp
    index folders (fastxc/io/sourcepack.py:75-91)."""
    path = Path(sourcepack_input).expanduser().resolve()
    if path.is_file():
        return [path]
    if not path.is_dir():
        raise FileNotFoundError(f"no SourcePack index at {path}")
    if (path / "sourcepack_index.tsv").is_file():
        return [path / "sourcepack_index.tsv"]
    found = _index_paths(path)
    if not found:
        raise FileNotFoundError(f"{path} holds no */sourcepack_index.tsv")
    return found
