"""End-to-end drop-in check of the sac2spec executable: a SAC index and SAC
files in, stepack batches out, through the reference's command line.

Checks: index grouping (header/comment lines skipped, an incomplete group
dropped, nsl_id text kept), SAC length contract (a short file zero-padded, a
long one truncated), -Q window skipping, the stepack header / NSLC table /
TSV rows (first/last_nsl_id as written in the index), per-timestamp and
final _SUCCESS markers, the progress sidecar, and every output spectrum row
within relative L2 1e-5 of the FP64 oracle (rows that are exactly zero in
the oracle must be exactly zero); argv errors.
"""

import csv
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from fastxc_gb300 import formats
from oracle import sac2spec_oracle as so

ROOT = Path(__file__).resolve().parents[1]
EXE = ROOT / "fastxc_gb300" / "bin" / "sac2spec"
G = Path(__file__).resolve().parent / "golden"
DELTA = 0.1
SAC_LEN, WIN, LAG = 7200.0, 1800.0, 100.0


def synth(npts, seed):
    rng = np.random.default_rng(seed)
    from scipy.signal import butter, sosfiltfilt

    sos = butter(4, [0.1, 2.0], "bandpass", fs=1 / DELTA, output="sos")
    src = sosfiltfilt(sos, rng.standard_normal(npts + 3000))
    return (rng.standard_normal(npts) + 3.0 * src[1000:1000 + npts]).astype(np.float32)


def make_inputs(tmp):
    npts = int(round(SAC_LEN / DELTA))
    sac_dir = tmp / "sac"
    sac_dir.mkdir()
    lines = ["timestamp\tnsl_id\tnetwork\tstation\tlocation\tcomponent\tsac_path", "# comment"]
    series = {}
    k = 0
    for ts in ("2020.100.0000", "2020.101.0000"):
        for nsl, sta in (("0007", "AA"), ("0012", "BB"), ("0031", "CC")):
            for comp in ("BHE", "BHN", "BHZ"):
                x = synth(npts, k)
                if (ts, sta, comp) == ("2020.100.0000", "BB", "BHN"):
                    x = x[: npts - 18000]  # short by exactly one window: zero-padded
                if (ts, sta, comp) == ("2020.101.0000", "CC", "BHZ"):
                    x = np.concatenate([x, synth(500, 99)])  # long: truncated
                p = sac_dir / f"{ts}.{sta}.{comp}.sac"
                formats.write_sac(p, x, DELTA, stla=30.0 + k * 0.01, stlo=100.0 - k * 0.01)
                full = np.zeros(npts, np.float32)
                full[: min(npts, x.size)] = x[:npts]
                series[(ts, nsl, comp)] = full
                lines.append(f"{ts}\t{nsl}\tXX\t{sta}\t00\t{comp}\t{p}")
                k += 1
        # an incomplete group (2 of 3 components) is skipped with a warning
        for comp in ("BHE", "BHN"):
            p = sac_dir / f"{ts}.DD.{comp}.sac"
            formats.write_sac(p, synth(npts, 500 + k), DELTA)
            lines.append(f"{ts}\t0040\tXX\tDD\t00\t{comp}\t{p}")
            k += 1
    idx = tmp / "sac_index.tsv"
    idx.write_text("\n".join(lines) + "\n")
    return idx, series


@pytest.mark.gpu
@pytest.mark.parametrize("whiten,normalize", [(2, 3), (0, 2)])
def test_sac2spec_end_to_end(tmp_path, built_lib, torch_cuda, whiten, normalize):
    idx, series = make_inputs(tmp_path)
    out = tmp_path / "work"
    filt = G / "filter_d0.1_0.1-2.txt"
    env = dict(os.environ, FASTXC_LOG_LEVEL="error")
    r = subprocess.run([str(EXE), "-I", str(idx), "-O", str(out), "-L", f"{SAC_LEN:g}/{WIN:g}/{WIN:g}/{LAG:g}",
                        "-B", str(filt), "-C", "3", "-W", f"{whiten}/0", "-N", str(normalize), "-Q", "2,-1",
                        "-T", "3"], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    st = out / "stepack"
    assert (st / "_SUCCESS").read_text() == "DONE\n"
    for ts in ("2020.100.0000", "2020.101.0000"):
        assert (st / ts / "_SUCCESS").read_text() == f"timestamp\t{ts}\ngroups\t3\n"
    prog = (out / "progress" / "sac2spec_progress.tsv").read_text().splitlines()
    assert prog[1].split("\t")[:5] == ["overall", "DONE", "18", "18", "sac_rows"]

    flt = so.read_filter_file(filt)
    plan = so.make_plan(SAC_LEN, WIN, WIN, LAG, DELTA, flt, whiten, normalize, 0)
    steps = [s for s in range(plan.nstep) if s != 2]
    packs = sorted(st.glob("*.stepack"))
    assert packs
    rows_seen = 0
    for pack in packs:
        d = formats.read_stepack(pack)
        h = d["header"]
        assert h["magic"] == "FXCSTPK" and h["version"] == 3 and h["layout"] == 2
        assert h["nstep"] == len(steps) and h["nspec"] == plan.nspec
        assert h["dt"] == np.float32(DELTA)
        assert h["df"] == np.float32(np.float32(1.0) / (np.float32(plan.output_nfft) * np.float32(DELTA)))
        assert h["nslc_count"] == 3 * h["group_count"]
        with open(pack.with_suffix(".tsv")) as fh:
            trows = list(csv.DictReader(fh, delimiter="\t"))
        for t in trows:
            b, n = int(t["nslc_start"]), int(t["nslc_count"])
            assert t["first_nsl_id"] == f"{d['entries'][b]['nsl_id']:04d}"
            assert t["last_nsl_id"] == f"{d['entries'][b + n - 1]['nsl_id']:04d}"
        ts_of = {}
        for t in trows:
            for i in range(int(t["nslc_start"]), int(t["nslc_start"]) + int(t["nslc_count"])):
                ts_of[i] = t["timestamp"]
        ents = d["entries"]
        for g in range(h["group_count"]):
            e0 = ents[3 * g]
            ts = ts_of[3 * g]
            x = np.stack([series[(ts, f"{e0['nsl_id']:04d}", ents[3 * g + c]["component"])] for c in range(3)])
            ref = so.run_rows(so.windows(x.astype(np.float64), plan, steps), plan, 3)
            got = d["payload"][:, 3 * g: 3 * g + 3, :]
            for s in range(len(steps)):
                for c in range(3):
                    a, b = got[s, c], ref[s, c]
                    nb = np.linalg.norm(b)
                    if nb == 0:
                        assert not np.any(a), (ts, g, s, c)
                    else:
                        assert np.linalg.norm(a - b) / nb < 1e-5, (ts, g, s, c)
            rows_seen += 3
    assert rows_seen == 18


def test_sac2spec_command_line_errors(tmp_path, built_lib):
    r = subprocess.run([str(EXE)], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([str(EXE), "-h"], capture_output=True, text=True)
    assert r.returncode == 0
    base = ["-I", "x", "-O", str(tmp_path / "o"), "-B", "f"]
    r = subprocess.run([str(EXE), *base], capture_output=True, text=True)
    assert r.returncode == 1 and "-L sac_len/win_len/shift_len/xcorr_lag is required" in r.stderr
    r = subprocess.run([str(EXE), *base, "-L", "1/2/3"], capture_output=True, text=True)
    assert r.returncode == 1 and "-L expects" in r.stderr
    r = subprocess.run([str(EXE), *base, "-L", "86400/3600/3600/100", "-W", "4/0"], capture_output=True, text=True)
    assert r.returncode == 1 and "whiten_type must be" in r.stderr
    r = subprocess.run([str(EXE), *base, "-L", "86400/3600/3600/100", "-G", "0", "-M", "1,2"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "-M count must match -G count" in r.stderr
    r = subprocess.run([str(EXE), *base, "-L", "86400/3600/3600/100", "-X"], capture_output=True, text=True)
    assert r.returncode == 1 and "Unknown option -X" in r.stderr
    # a non-empty stepack directory is refused before any GPU work
    (tmp_path / "o" / "stepack").mkdir(parents=True)
    (tmp_path / "o" / "stepack" / "old.tsv").write_text("x")
    r = subprocess.run([str(EXE), *base, "-L", "86400/3600/3600/100"], capture_output=True, text=True)
    assert r.returncode == 1 and "stepack_dir_not_empty" in r.stderr


@pytest.mark.gpu
def test_sac2spec_then_xc_fast_chain(tmp_path, built_lib, torch_cuda):
    """The two drop-ins chained as fastxc runs them: sac2spec's stepack
    output is xc_fast's input; every NCF matches the FP64 oracle run on the
    oracle's own spectra (relative L2 1e-5)."""
    from oracle import xc_oracle as xo

    idx, series = make_inputs(tmp_path)
    out = tmp_path / "work"
    filt = G / "filter_d0.1_0.1-2.txt"
    env = dict(os.environ, FASTXC_LOG_LEVEL="error")
    r = subprocess.run([str(EXE), "-I", str(idx), "-O", str(out), "-L", f"{SAC_LEN:g}/{WIN:g}/{WIN:g}/{LAG:g}",
                        "-B", str(filt), "-C", "3", "-W", "2/0", "-N", "3"], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    paths = [(7, 12, 0.5, 55.5, 10.0, 190.0), (7, 31, 0.6, 66.6, 20.0, 200.0), (12, 31, 0.7, 77.7, 30.0, 210.0)]
    formats.write_allowed_paths(tmp_path / "allowed_paths.tsv", paths)
    r = subprocess.run([str(ROOT / "fastxc_gb300" / "bin" / "xc_fast"), "-I", str(out / "stepack"), "-P",
                        str(tmp_path / "allowed_paths.tsv"), "-O", str(tmp_path / "ncf"), "-C", str(LAG)],
                       env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    recs = formats.read_xcpack_dir(tmp_path / "ncf" / "xcpack")
    assert len(recs) == 2 * 3 * 9
    flt = so.read_filter_file(filt)
    plan = so.make_plan(SAC_LEN, WIN, WIN, LAG, DELTA, flt, 2, 3, 0)
    steps = list(range(plan.nstep))
    shape = xo.finalize_shape(plan.nspec, plan.nstep, DELTA, LAG)
    spec_cache = {}
    for rec in recs:
        ts = rec["timestamp"]
        if ts not in spec_cache:
            keys = [(ts, nsl, c) for nsl in ("0007", "0012", "0031") for c in ("BHE", "BHN", "BHZ")]
            x = np.stack([series[k] for k in keys]).astype(np.float64)
            sp = so.run_rows(so.windows(x, plan, steps), plan, 3)  # [step][row][nspec]
            spec_cache[ts] = (sp, {(k[1], k[2]): i for i, k in enumerate(keys)})
        sp, pos = spec_cache[ts]
        s = pos[(f"{int(rec['src_id']):04d}", rec["src_component"])]
        q = pos[(f"{int(rec['rec_id']):04d}", rec["rec_component"])]
        ref = xo.xc_run(sp, np.array([s]), np.array([q]), 1.0 / plan.nstep, shape)[0]
        err = np.linalg.norm(rec["data"] - ref) / np.linalg.norm(ref)
        assert err < 1e-5, (rec["src_id"], rec["rec_id"], err)
