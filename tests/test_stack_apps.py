"""End-to-end drop-in checks of the ncf_pws and ncf_tfpws executables:
SourcePack indexes in, stacked SourcePack shards + merged index out, run
through the reference's command lines.

Checks: grouping by (path_id as a string, component_slot) across several
index files with each group's records in timestamp order; round-robin
dealing to the -G workers and their shard files; the merged index order and
columns; _SUCCESS contents; the output SAC headers (configure_output_header
+ update_output_stats for PWS, configure_tfpws_output_header for TF-PWS);
stacked traces within relative L2 1e-5 of the FP64 oracle; argv errors.
"""

import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from fastxc_gb300 import formats
from fastxc_gb300.synthetic import ncf_traces
from oracle import stack_oracle as sto

ROOT = Path(__file__).resolve().parents[1]
BIN = ROOT / "fastxc_gb300" / "bin"
# path ids whose string order differs from their numeric order
PATHS = ["9", "10", "100", "27"]
SLOTS = [0, 4]
NTS = 7


def make_sourcepack(tmp, nsamples=2001, delta=0.1, seed=0):
    """Two index files (timestamps split between them); returns the list
    file and {(path_id, slot): traces in timestamp order}."""
    tr = ncf_traces(len(PATHS) * len(SLOTS), NTS, nsamples, delta=delta, seed=seed)
    groups = {}
    rows = [[], []]
    k = 0
    for pid in sorted(PATHS):  # index files are sorted by (path_id, slot)
        for slot in SLOTS:
            groups[(pid, slot)] = tr[k]
            for t in range(NTS):
                rows[t % 2].append(dict(
                    timestamp=f"2020.{100 + t:03d}.0000", path_id=pid, component_slot=slot,
                    source_key=f"XX.S{pid}", receiver_key=f"XX.R{pid}", src_id=pid, rec_id=str(int(pid) + 1),
                    src_network="XX", src_station=f"S{pid}", src_location="00", src_component="BHZ",
                    rec_network="XX", rec_station=f"R{pid}", rec_location="00", rec_component=f"BH{slot}",
                    dist="55.5", az="10", baz="190", data=tr[k][t], delta=delta,
                    final_pair_path=f"stack/XX-XX.S{pid}-R{pid}.BHZ-BH{slot}.sac"))
            k += 1
    # the second file lists its records in reverse timestamp order inside a group
    for part in (0, 1):
        rows[part].sort(key=lambda r: (r["path_id"], r["component_slot"], r["timestamp"] if part == 0 else
                                       "".join(chr(255 - ord(c)) for c in r["timestamp"])))
    idx = [formats.write_sourcepack(tmp / "in", f"part{i}", rows[i]) for i in (0, 1)]
    lst = tmp / "list.txt"
    lst.write_text("# sourcepack indexes\n" + "\n".join(str(p) for p in idx) + "\n\n")
    return lst, groups


def expected_order():
    return [(p, s) for p in sorted(PATHS) for s in SLOTS]


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.gpu
def test_ncf_pws_end_to_end(tmp_path, built_lib, torch_cuda):
    lst, groups = make_sourcepack(tmp_path)
    out = tmp_path / "pws"
    prog = tmp_path / "prog.tsv"
    env = dict(os.environ, FASTXC_LOG_LEVEL="warn")
    r = subprocess.run([str(BIN / "ncf_pws"), "--index-list", str(lst), "--output-dir", str(out), "-B", "3",
                        "-G", "0,0", "--progress", str(prog)], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    order = expected_order()
    # round-robin dealing: group k -> worker k % 2, rows in group order
    for w in (0, 1):
        shard = formats.read_sourcepack_index(out / f"pws.w{w:03d}.tsv")
        assert [(x["path_id"], int(x["component_slot"])) for x in shard] == order[w::2]
        assert all(x["record_path"] == str(out / f"pws.w{w:03d}.pack") for x in shard)
    merged = formats.read_sourcepack_index(out / "sourcepack_index.tsv")
    assert [(x["path_id"], int(x["component_slot"])) for x in merged] == order
    succ = (out / "_SUCCESS").read_text().splitlines()
    assert succ[:3] == [f"records\t{len(order)}", "workers\t2", f"index\t{out / 'sourcepack_index.tsv'}"]
    assert succ[3:] == [f"pack\t{out / 'pws.w000.pack'}", f"pack\t{out / 'pws.w001.pack'}"]
    assert prog.read_text().splitlines()[1].split("\t")[:4] == ["overall", "DONE", str(len(order)), str(len(order))]
    for x in merged:
        key = (x["path_id"], int(x["component_slot"]))
        tr = groups[key]
        assert x["timestamp"] == "STACK" and x["storage_kind"] == "pws_pack"
        assert x["final_pair_path"].endswith(f"BHZ-BH{key[1]}.pws.sac")
        assert x["npts"] == "2001" and x["dt"] == "0.1" and x["dist"] == "55.5"
        h = x["header"]
        assert h["npts"] == 2001 and h["iftype"] == 1 and h["leven"] == 1
        assert h["user0"] == NTS and h["user1"] == 3 and h["user2"] == 3
        assert h["nzyear"] == 2010 and h["nzjday"] == 214 and h["nzhour"] == 0 and h["nzsec"] == 0
        assert h["e"] == np.float32(np.float32(-1000 * np.float32(0.1)) + np.float32(2000) * np.float32(0.1))
        raw = x["raw_header"]
        assert raw[576:600] == b"NTRACE  NGROUP  SUBSTK  "
        f = np.frombuffer(raw[:280], "<f4")
        d = x["data"]
        assert f[1] == d.min() and f[2] == d.max()
        acc = 0.0
        for v in d.tolist():  # sequential double sum, as update_output_stats
            acc += v
        assert f[56] == np.float32(acc / d.size)
        ref = sto.pws(tr, 3)
        assert rel(d, ref) < 1e-5, key


@pytest.mark.gpu
def test_ncf_tfpws_end_to_end(tmp_path, built_lib, torch_cuda):
    lst, groups = make_sourcepack(tmp_path, nsamples=401, seed=4)
    out = tmp_path / "tfpws"
    env = dict(os.environ, FASTXC_LOG_LEVEL="warn")
    r = subprocess.run([str(BIN / "ncf_tfpws"), "-I", str(lst), "-O", str(out), "-B", "2", "-F", "0.2/1.5",
                        "-S", "001"], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    merged = formats.read_sourcepack_index(out / "sourcepack_index.tsv")
    assert [(x["path_id"], int(x["component_slot"])) for x in merged] == expected_order()
    assert (out / "_SUCCESS").read_text().splitlines()[1] == "workers\t1"
    for x in merged:
        key = (x["path_id"], int(x["component_slot"]))
        assert x["storage_kind"] == "tfpws_pack" and x["final_pair_path"].endswith(".tfpws.sac")
        h = x["header"]
        assert h["npts"] == 401 and h["iftype"] == 1 and h["user0"] == NTS
        assert h["nzyear"] == 2010 and h["nzjday"] == 214 and h["nzmin"] == 0
        assert h["nzsec"] == -12345  # TF-PWS leaves nzsec as read
        ref = sto.tfpws(groups[key], 2, band=(0.2, 1.5), delta=0.1)
        assert rel(x["data"], ref) < 1e-5, key


def test_stack_apps_command_line_errors(tmp_path, built_lib):
    for exe in ("ncf_pws", "ncf_tfpws"):
        r = subprocess.run([str(BIN / exe)], capture_output=True, text=True)
        assert r.returncode == 1
    r = subprocess.run([str(BIN / "ncf_pws"), "--index-list", "x"], capture_output=True, text=True)
    assert r.returncode == 1 and "missing_sourcepack_io" in r.stderr
    r = subprocess.run([str(BIN / "ncf_tfpws"), "-I", "x", "-O", "y", "-S", "010"], capture_output=True, text=True)
    assert r.returncode == 1 and "invalid_stack_selector" in r.stderr
    r = subprocess.run([str(BIN / "ncf_tfpws"), "-I", "x", "-O", "y", "-F", "2/1"], capture_output=True, text=True)
    assert r.returncode == 1 and "invalid_band_argument" in r.stderr
    r = subprocess.run([str(BIN / "ncf_pws"), "--index-list", str(tmp_path / "none.txt"), "--output-dir",
                        str(tmp_path / "o")], capture_output=True, text=True)
    assert r.returncode == 1 and "sourcepack_list_open_failed" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("exe,args,mode,sub", [("ncf_pws", ["-B", "3"], 0, 3),
                                               ("ncf_tfpws", ["-B", "2", "-F", "0.2/1.5"], 1, 2)])
def test_stack_apps_memory_budget_batches(tmp_path, built_lib, torch_cuda, exe, args, mode, sub):
    """-M below the whole job's device footprint splits the groups into
    several batches (fxc_stack_batch_bytes); every output byte equals the
    one-batch run's."""
    import ctypes as C

    from fastxc_gb300._lib import lib

    n = 2001
    lst, groups = make_sourcepack(tmp_path, nsamples=n, seed=5)
    ng = (NTS + sub - 1) // sub

    def nbytes(npairs):
        out = C.c_int64()
        lib().fxc_stack_batch_bytes(mode, npairs * NTS, npairs, npairs * ng, ng, n, C.byref(out))
        return out.value

    total = len(groups)
    mib = -(-nbytes(3) // (1 << 20))
    assert nbytes(total) > mib << 20, "budget must split the job"
    flag = ["--gpu-memory-mib"] if exe == "ncf_pws" else ["-M"]
    out_dirs = []
    for tag, extra in (("whole", []), ("split", flag + [str(mib)])):
        out = tmp_path / tag
        cmd = [str(BIN / exe), "--index-list" if exe == "ncf_pws" else "-I", str(lst),
               "--output-dir" if exe == "ncf_pws" else "-O", str(out), *args, *extra]
        r = subprocess.run(cmd, env=dict(os.environ, FASTXC_LOG_LEVEL="warn"), capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out_dirs.append(out)
    a, b = out_dirs
    files = sorted(p.relative_to(a) for p in a.rglob("*") if p.is_file())
    assert files == sorted(p.relative_to(b) for p in b.rglob("*") if p.is_file())
    for f in files:
        if f.suffix in (".tsv",) or f.name == "_SUCCESS":
            assert (b / f).read_text().replace(str(b), "@") == (a / f).read_text().replace(str(a), "@"), f
        else:
            assert (b / f).read_bytes() == (a / f).read_bytes(), f
