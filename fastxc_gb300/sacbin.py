"""SAC binary records (632-byte header + float32 samples) for the stacking,
rotation and SourcePack operators.

The header layout is the SAC standard: 70 floats, 40 ints, 24 text fields
(fastxc/io/sac_binary.py:11-101 names the same slots). A header keeps its
original bytes and byte order; only the fields a caller sets are rewritten,
so records pass through these operators unchanged apart from those fields
(the behaviour of SacHeader, fastxc/io/sac_binary.py:141-215).
"""

from __future__ import annotations

import struct
import sys
from pathlib import Path
from typing import BinaryIO

import numpy as np

HEADER_BYTES = 632
NFLOAT = 70
NINT = 40
ITIME = 1
IXY = 4
NULL_VALUE = -12345.0

# float slot index by name
FLOATS = {
    "delta": 0, "depmin": 1, "depmax": 2, "scale": 3, "odelta": 4, "b": 5, "e": 6, "o": 7, "a": 8,
    "stla": 31, "stlo": 32, "stel": 33, "stdp": 34, "evla": 35, "evlo": 36, "evel": 37, "evdp": 38,
    "user0": 40, "user1": 41, "user2": 42, "user3": 43, "user4": 44, "user5": 45, "user6": 46,
    "user7": 47, "user8": 48, "user9": 49, "dist": 50, "az": 51, "baz": 52, "gcarc": 53, "depmen": 56,
    "cmpaz": 57, "cmpinc": 58, "scmpaz": 68, "scmpinc": 69,
}
# int slot index by name (after the 70 floats)
INTS = {
    "nzyear": 0, "nzjday": 1, "nzhour": 2, "nzmin": 3, "nzsec": 4, "nzmsec": 5, "nvhdr": 6, "npts": 9,
    "iftype": 15, "leven": 35, "lpspol": 36, "lovrok": 37, "lcalda": 38,
}
# text fields: (byte offset, width)
TEXTS = {
    "kstnm": (440, 8), "kevnm": (448, 16), "khole": (464, 8), "ko": (472, 8), "ka": (480, 8),
    "kcmpnm": (600, 8), "knetwk": (608, 8), "kinst": (624, 8),
}

_NATIVE = "<" if sys.byteorder == "little" else ">"


def _byte_order(raw: bytes) -> str:
    # nvhdr is 6 (or 7) in a valid header; otherwise the order in which only
    # one reading gives a plausible npts and a finite delta; otherwise native
    # (the rule of _detect_endian, fastxc/io/sac_binary.py:104-128)
    for order in ("<", ">"):
        if struct.unpack_from(order + "i", raw, (NFLOAT + INTS["nvhdr"]) * 4)[0] in (6, 7):
            return order
    ok = {}
    for order in ("<", ">"):
        n = struct.unpack_from(order + "i", raw, (NFLOAT + INTS["npts"]) * 4)[0]
        d = struct.unpack_from(order + "f", raw, 0)[0]
        ok[order] = 0 < n < 1_000_000_000 and np.isfinite(d)
    if ok["<"] != ok[">"]:
        return "<" if ok["<"] else ">"
    return _NATIVE


class Header:
    """A mutable SAC header over its original bytes."""

    __slots__ = ("raw", "order")

    def __init__(self, raw: bytes | bytearray, order: str | None = None):
        if len(raw) != HEADER_BYTES:
            raise ValueError(f"SAC header must be {HEADER_BYTES} bytes, got {len(raw)}")
        self.raw = bytearray(raw)
        self.order = order or _byte_order(self.raw)

    def copy(self) -> "Header":
        return Header(bytes(self.raw), self.order)

    def get_float(self, name: str) -> float:
        return struct.unpack_from(self.order + "f", self.raw, FLOATS[name] * 4)[0]

    def set_float(self, name: str, value: float) -> None:
        struct.pack_into(self.order + "f", self.raw, FLOATS[name] * 4, float(value))

    def get_int(self, name: str) -> int:
        return struct.unpack_from(self.order + "i", self.raw, (NFLOAT + INTS[name]) * 4)[0]

    def set_int(self, name: str, value: int) -> None:
        struct.pack_into(self.order + "i", self.raw, (NFLOAT + INTS[name]) * 4, int(value))

    def get_text(self, name: str) -> str:
        off, width = TEXTS[name]
        return bytes(self.raw[off:off + width]).decode("ascii", errors="ignore").strip()

    def set_text(self, name: str, value: str) -> None:
        off, width = TEXTS[name]
        self.raw[off:off + width] = value.encode("ascii", errors="replace")[:width].ljust(width, b" ")

    @property
    def npts(self) -> int:
        return self.get_int("npts")

    @property
    def data_count(self) -> int:
        n = self.npts
        if n <= 0:
            raise ValueError(f"invalid SAC npts {n}")
        return 2 * n if self.get_int("iftype") == IXY else n

    @property
    def dtype(self) -> np.dtype:
        return np.dtype(self.order + "f4")


def read_record_from(fp: BinaryIO, path, offset: int, size: int | None = None) -> tuple[Header, np.ndarray]:
    """One record at `offset` of an open pack; `size` (when given) must equal
    the header's record size."""
    if offset < 0:
        raise ValueError(f"{path}: negative SAC record offset {offset}")
    fp.seek(offset)
    raw = fp.read(HEADER_BYTES)
    if len(raw) != HEADER_BYTES:
        raise EOFError(f"{path}: short SAC header at offset {offset}")
    hd = Header(raw)
    nbytes = hd.data_count * 4
    if size is not None and int(size) != HEADER_BYTES + nbytes:
        raise ValueError(f"{path}: record size {size} differs from the header's {HEADER_BYTES + nbytes}")
    body = fp.read(nbytes)
    if len(body) != nbytes:
        raise EOFError(f"{path}: short SAC data at offset {offset}")
    return hd, np.frombuffer(body, dtype=hd.dtype).astype(np.float32)


def read_record(path, offset: int = 0, size: int | None = None) -> tuple[Header, np.ndarray]:
    with open(path, "rb") as fp:
        return read_record_from(fp, path, offset, size)


def encode_record(hd: Header, data: np.ndarray) -> bytes:
    arr = np.asarray(data, dtype=np.float32)
    if arr.size != hd.data_count:
        raise ValueError(f"SAC header expects {hd.data_count} samples, got {arr.size}")
    return bytes(hd.raw) + arr.astype(hd.dtype, copy=False).tobytes()


def write_file(path, hd: Header, data: np.ndarray) -> None:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    path.write_bytes(encode_record(hd, data))


def read_file(path) -> tuple[Header, np.ndarray]:
    return read_record(path, 0, None)
