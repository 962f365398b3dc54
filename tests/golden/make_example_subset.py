"""Copies one day of the reference's public smoke-test data into a fixture.

The reference ships 84 anonymised 1 Hz SAC files (4 stations x E/N/Z x 7
days, example/data, with example/config.ini). This keeps one day
(2022.138, the first with no zero-filled gap on any station) of all four
stations -- 12 files, byte for byte -- in example_1hz_sac.npz:

    python tests/golden/make_example_subset.py [reference root]

(the root defaults to $FXC_REFERENCE_ROOT, else oracle/build_ref.py's
default). Each entry is a file's raw bytes; `names` lists the file names.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
from oracle.build_ref import reference_root  # noqa: E402

STATIONS = ("A7K2", "B4Q8", "C9M3", "D2X6")
DAY = "2022.138.0000"


def main(root: Path) -> None:
    data = root / "example" / "data"
    names, blobs = [], {}
    for sta in STATIONS:
        for comp in "ENZ":
            f = data / sta / "2022" / f"{sta}.{DAY}.{comp}.sac"
            names.append(f.name)
            blobs[f"f{len(names) - 1}"] = np.frombuffer(f.read_bytes(), np.uint8)
    np.savez_compressed(HERE / "example_1hz_sac.npz", names=np.array(names), **blobs)
    print("wrote", HERE / "example_1hz_sac.npz", len(names), "files")


if __name__ == "__main__":
    main(reference_root(sys.argv[1] if len(sys.argv) > 1 else None))
