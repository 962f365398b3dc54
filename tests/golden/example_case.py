"""One day of the reference's public smoke-test data (4 anonymised Kansas
stations, 1 Hz, E/N/Z; example_1hz_sac.npz) run through this build's
executables and through the reference's kernels, with the settings of the
reference's example/config.ini: win_len 3600 s, bands 0.2/0.4 0.1/0.2
(RUN-ABS-MF), whiten after, max_lag 100 s, every station pair."""

from __future__ import annotations

import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
BIN = ROOT / "fastxc_gb300" / "bin"
FILTER = HERE / "filter_d1.0_0.2-0.4_0.1-0.2.txt"
TS = "2022.138.0000"
STATIONS = ("A7K2", "B4Q8", "C9M3", "D2X6")
COMPS = ("E", "N", "Z")
SAC_LEN, WIN, LAG, DELTA = 86400.0, 3600.0, 100.0, 1.0
WHITEN_AFTER, NORM_RUNABS_MF = 2, 1
GOLDEN = HERE / "example_1hz_ref.npz"


def load_sac():
    """{(station, component): raw SAC file bytes}."""
    z = np.load(HERE / "example_1hz_sac.npz")
    out = {}
    for i, name in enumerate(z["names"]):
        sta, _, _, _, comp, _ = str(name).split(".")
        out[(sta, comp)] = z[f"f{i}"].tobytes()
    return out


def series(sac) -> np.ndarray:
    """float32 [12][npts], rows station-major in index order."""
    return np.stack([np.frombuffer(sac[(s, c)][632:], "<f4") for s in STATIONS for c in COMPS])


def write_inputs(tmp: Path, sac) -> tuple[Path, Path]:
    d = tmp / "sac"
    d.mkdir(parents=True, exist_ok=True)
    lines = ["timestamp\tnsl_id\tnetwork\tstation\tlocation\tcomponent\tsac_path"]
    for k, s in enumerate(STATIONS):
        for c in COMPS:
            p = d / f"{s}.{TS}.{c}.sac"
            p.write_bytes(sac[(s, c)])
            lines.append(f"{TS}\t{k + 1:04d}\tKS\t{s}\t00\t{c}\t{p}")
    idx = tmp / "sac_index.tsv"
    idx.write_text("\n".join(lines) + "\n")
    from fastxc_gb300 import formats

    rows = [(a + 1, b + 1, 0.06 * (b - a), 6.5 * (b - a), 90.0, 270.0) for a in range(4) for b in range(a + 1, 4)]
    formats.write_allowed_paths(tmp / "allowed_paths.tsv", rows)
    return idx, tmp / "allowed_paths.tsv"


def run_ours(tmp: Path, sac, method: str = "plain") -> dict:
    """{(src station, src comp, rec station, rec comp): NCF} from this
    build's sac2spec and xc_fast executables."""
    from fastxc_gb300 import formats

    idx, paths = write_inputs(tmp, sac)
    env = dict(os.environ, FASTXC_LOG_LEVEL="error", FASTXC_XC_METHOD=method)
    r = subprocess.run([str(BIN / "sac2spec"), "-I", str(idx), "-O", str(tmp / "ws"), "-L",
                        f"{SAC_LEN:g}/{WIN:g}/{WIN:g}/{LAG:g}", "-B", str(FILTER), "-C", "3",
                        "-W", f"{WHITEN_AFTER}/0", "-N", str(NORM_RUNABS_MF), "-T", "4"],
                       env=env, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    r = subprocess.run([str(BIN / "xc_fast"), "-I", str(tmp / "ws" / "stepack"), "-P", str(paths), "-O",
                        str(tmp / "ncf"), "-C", f"{LAG:g}"], env=env, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    out = {}
    for rec in formats.read_xcpack_dir(tmp / "ncf" / "xcpack"):
        key = (rec["src_station"], rec["src_component"], rec["rec_station"], rec["rec_component"])
        out[key] = np.asarray(rec["data"], np.float32)
    return out


def pairs():
    """(keys, src rows, rec rows) of the 54 component pairs."""
    keys, src, rec = [], [], []
    for a in range(4):
        for b in range(a + 1, 4):
            for i in range(3):
                for j in range(3):
                    keys.append((STATIONS[a], COMPS[i], STATIONS[b], COMPS[j]))
                    src.append(3 * a + i)
                    rec.append(3 * b + j)
    return keys, np.array(src), np.array(rec)


def fp64_ncfs(sac) -> dict:
    """The FP64 oracle's NCFs of the same data: {key: NCF}."""
    from oracle import sac2spec_oracle as so
    from oracle import xc_oracle as xo

    op = so.make_plan(SAC_LEN, WIN, WIN, LAG, DELTA, so.read_filter_file(FILTER), WHITEN_AFTER, NORM_RUNABS_MF, 0)
    wins = so.windows(series(sac), op, list(range(op.nstep))).astype(np.float32)
    spec = so.run_rows(wins.astype(np.float64), op, 3)
    keys, src, rec = pairs()
    nwin, _, nspec = spec.shape
    shape = xo.finalize_shape(nspec, nwin, DELTA, LAG)
    out = xo.xc_run(spec, src, rec, 1.0 / nwin, shape)
    return {k: out[i] for i, k in enumerate(keys)}


def reference_ncfs(sac) -> tuple[dict, dict]:
    """The reference's kernels (oracle/ref_gpu.py) and the FP64 oracle on the
    same data: ({key: NCF}, {key: FP64 NCF})."""
    from oracle import ref_gpu
    from oracle import sac2spec_oracle as so
    from oracle import xc_oracle as xo

    op = so.make_plan(SAC_LEN, WIN, WIN, LAG, DELTA, so.read_filter_file(FILTER), WHITEN_AFTER, NORM_RUNABS_MF, 0)
    x = series(sac)
    wins = so.windows(x, op, list(range(op.nstep))).astype(np.float32)
    ref_spec = ref_gpu.sac2spec_rows(wins, op, op.responses, 3)
    fp64_spec = so.run_rows(wins.astype(np.float64), op, 3)
    keys, src, rec = pairs()
    nwin, _, nspec = ref_spec.shape
    shape = xo.finalize_shape(nspec, nwin, DELTA, LAG)
    ref = ref_gpu.xc_run(ref_spec, src, rec, shape.nfft, shape.half_cc, shape.dt)
    fp64 = xo.xc_run(fp64_spec, src, rec, 1.0 / nwin, shape)
    return {k: ref[i] for i, k in enumerate(keys)}, {k: fp64[i] for i, k in enumerate(keys)}


def key_text(k) -> str:
    return f"{k[0]}.{k[1]}-{k[2]}.{k[3]}"
