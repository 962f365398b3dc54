"""Build recipe of the native library ``libfastxc_gb300.so`` (sm_103a only).

Every ``csrc/*.cu`` translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into one shared
library inside the package (``fastxc_gb300/lib/``); the C++ drop-in
executables are linked against it. Nothing is installed into site-packages.

Usage: ``python -m fastxc_gb300.build`` (or ``__graft_entry__.build()``).
"""

from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libfastxc_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC",
    "--expt-relaxed-constexpr",
    "-I" + str(INCLUDE),
]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build fastxc_gb300")


APPS = PKG / "apps"
BINDIR = PKG / "bin"


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _build_apps(nvcc: str, force: bool) -> list[Path]:
    """Drop-in executables (C++ host code linked against the library)."""
    BINDIR.mkdir(exist_ok=True)
    out = []
    hdr = _headers_digest()
    for src in sorted(APPS.glob("*.cpp")):
        exe = BINDIR / src.stem
        stamp = BUILD / f"app_{src.stem}.stamp"
        key = hashlib.sha256((src.read_bytes().decode("utf-8", "replace") + hdr + LIB.name).encode()).hexdigest()[:16]
        if force or not exe.exists() or not stamp.exists() or stamp.read_text() != key or \
                exe.stat().st_mtime < LIB.stat().st_mtime:
            cmd = [nvcc, "-O2", "-std=c++17", "-I" + str(INCLUDE), "-I" + str(CSRC), str(src), "-o", str(exe),
                   "-L" + str(LIBDIR), "-lfastxc_gb300", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN/../lib"]
            proc = subprocess.run(cmd, capture_output=True, text=True)
            if proc.returncode != 0:
                raise RuntimeError(f"app build failed for {src.name}:\n{' '.join(cmd)}\n{proc.stderr}")
            stamp.write_text(key)
        out.append(exe)
    return out


def _headers_digest() -> str:
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")) +
                    list(APPS.glob("*.h"))):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    return h.hexdigest()[:16]


def _compile(nvcc: str, src: Path, obj: Path, extra: list[str]) -> tuple[Path, str]:
    cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    return obj, proc.stderr


def build(verbose: bool = False, force: bool = False, extra: list[str] | None = None) -> Path:
    """Compile the library if any source changed; return the .so path."""
    nvcc = nvcc_path()
    extra = list(extra or [])
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    hdr = _headers_digest()
    objs = []
    jobs = []
    for src in _sources():
        key = hashlib.sha256((src.read_bytes().decode("utf-8", "replace") + hdr + " ".join(extra)).encode()).hexdigest()[:16]
        obj = BUILD / f"{src.stem}.{key}.o"
        objs.append(obj)
        if force or not obj.exists():
            jobs.append((src, obj))
    if jobs:
        workers = min(len(jobs), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            futs = [ex.submit(_compile, nvcc, s, o, extra) for s, o in jobs]
            for f in cf.as_completed(futs):
                obj, err = f.result()
                if verbose and err.strip():
                    print(err, file=sys.stderr)
    stamp = BUILD / "link.stamp"
    link_key = "|".join(o.name for o in objs)
    if force or not LIB.exists() or not stamp.exists() or stamp.read_text() != link_key:
        cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(LIB), *map(str, objs)]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
        stamp.write_text(link_key)
    # drop stale objects of earlier source versions
    keep = {o.name for o in objs}
    for o in BUILD.glob("*.o"):
        if o.name not in keep:
            o.unlink()
    _build_apps(nvcc, force)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
