"""Writes a small xc_fast output for the reference-reader readback test.

Runs where a GPU and the built executables are present:

    python tests/golden/make_xcpack_sample.py [output folder]

It builds the stepack input of tests/test_xc_fast_app.py (4 stations x 3
components at 0.1 s, 6 windows, nspec 1001, two out-of-order batches, one
disallowed station pair, one autocorrelation path), runs
``xc_fast -C 20`` on it and copies the resulting xcpack folder (records,
TSVs, markers) to the output folder (default: tests/golden/xcpack_sample).
The TSVs' pack_path column (absolute where xc_fast wrote it) becomes the pack
file's name, which readers resolve against the TSV's folder, so the copy is
self-contained.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from test_xc_fast_app import EXE, make_inputs  # noqa: E402


def main(dest: Path) -> None:
    with tempfile.TemporaryDirectory() as d:
        tmp = Path(d)
        make_inputs(tmp)
        out = tmp / "ncf"
        r = subprocess.run([str(EXE), "-I", str(tmp / "stepack"), "-P", str(tmp / "allowed_paths.tsv"), "-O", str(out),
                            "-C", "20"], env=dict(os.environ, FASTXC_LOG_LEVEL="warn", FASTXC_XC_METHOD="plain"),
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise SystemExit(r.stderr)
        if dest.exists():
            shutil.rmtree(dest)
        shutil.copytree(out / "xcpack", dest)
    for tsv in dest.glob("*.tsv"):
        lines = tsv.read_text().splitlines(keepends=True)
        col = lines[0].rstrip("\r\n").split("\t").index("pack_path")
        fixed = [lines[0]]
        for ln in lines[1:]:
            end = ln[len(ln.rstrip("\r\n")):]
            f = ln.rstrip("\r\n").split("\t")
            f[col] = Path(f[col]).name
            fixed.append("\t".join(f) + end)
        tsv.write_text("".join(fixed))
    print("wrote", dest, sorted(p.name for p in dest.iterdir()))


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else HERE / "xcpack_sample")
