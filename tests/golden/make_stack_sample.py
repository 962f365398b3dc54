"""Writes the stacked-output sample for the reference-reader readback test.

Runs where a GPU and the built executables are present:

    python tests/golden/make_stack_sample.py [output folder]

On the inputs of tests/golden/stack_case.py (two station pairs x nine E/N/Z
component pairs, 5 NCFs of 201 lags) it runs, through the reference's
command lines and folder layout,

  * ``ncf_pws -B 3 -G 0,0`` into ``stack/pws_sourcepack/STACK`` (two worker
    shards ``pws.w000`` / ``pws.w001`` and the merged index),
  * ``ncf_tfpws -B 2 -F 0.2/1.5`` into ``stack/tfpws_sourcepack/STACK``,
  * this build's RTZ rotation of both (``rotate_sourcepack_stack``) into
    ``stack/rtz_{pws,tfpws}_sourcepack/STACK``,

and copies the ``stack`` folder to the output folder (default:
tests/golden/stack_sample). Paths the tools wrote absolute (record_path,
final_pair_path, the _SUCCESS lines) become relative to the output folder,
so the copy is self-contained; a reader relocates them by joining.
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
sys.path.insert(0, str(HERE))

import stack_case as sc  # noqa: E402

BIN = ROOT / "fastxc_gb300" / "bin"


def _relativize(path: Path, base: Path) -> None:
    text = path.read_text()
    path.write_text(text.replace(str(base) + "/", ""))


def main(dest: Path) -> None:
    from fastxc_gb300 import rotate

    env = dict(os.environ, FASTXC_LOG_LEVEL="warn")
    with tempfile.TemporaryDirectory() as d:
        tmp = Path(d).resolve()
        lst = sc.write_inputs(tmp)
        out = tmp / "out"
        pws = out / "stack" / "pws_sourcepack" / "STACK"
        tfpws = out / "stack" / "tfpws_sourcepack" / "STACK"
        for cmd in ([str(BIN / "ncf_pws"), "--index-list", str(lst), "--output-dir", str(pws), "-B", str(sc.PWS_SUB),
                     "-G", "0,0"],
                    [str(BIN / "ncf_tfpws"), "-I", str(lst), "-O", str(tfpws), "-B", str(sc.TFPWS_SUB),
                     "-F", "%g/%g" % sc.TFPWS_BAND]):
            r = subprocess.run(cmd, env=env, capture_output=True, text=True)
            if r.returncode != 0:
                raise SystemExit(r.stderr)
        for method in ("pws", "tfpws"):
            res = rotate.rotate_sourcepack_stack(out, method)
            assert len(res) == len(sc.PAIRS), res
        if dest.exists():
            shutil.rmtree(dest)
        shutil.copytree(out / "stack", dest / "stack")
        for f in dest.rglob("*"):
            if f.suffix == ".tsv" or f.name == "_SUCCESS":
                _relativize(f, out)
    print("wrote", dest, sorted(str(p.relative_to(dest)) for p in dest.rglob("*") if p.is_file()))


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else sc.SAMPLE)
