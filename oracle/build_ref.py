"""Recipe that compiles parts of the reference (wangkingh/FastXC) for the CPU
as test oracles (TEST INFRASTRUCTURE ONLY).

Compiled from the sources where they lie in the read-only reference tree
(nothing is copied into this repository); outputs go to ``oracle/_ref/``
(git-ignored):
  * libref_sac2spec.so: native/sac2spec/fft_length.c,
    native/sac2spec/core/filter_response.c, native/sac2spec/logger.c
    (segment / FFT-length planning, Butterworth filter file reader, impulse
    padding estimate, zero-phase power response);
  * libref_xc.so: native/xc/worker/scheduler.cu (host C++ only, compiled as
    C++ against the CUDA headers), native/xc/io/path_table.c,
    native/xc/logger.c plus oracle/ref_xc_shim.cpp (row-batch jobs, the
    XcTask pair list, allowed-path lookups).
  * ref_sac2spec.cubin, ref_xc.cubin, ref_pws.cubin, ref_tfpws.cubin: the
    reference's CUDA kernel sources (native/<stage>/kernels/*.cu) compiled as
    device code for sm_103 with the reference's release flags
    (native/common.mk:21,77: -std=c++17 -O3 --use_fast_math) through
    oracle/ref_kernels.cu, which gives each kernel an extern "C" entry point.
    oracle/ref_gpu.py loads them and restates the host call order. A cubin is
    device code, so it runs on the GPU host although it is built here.
The reference root is taken from the FXC_REFERENCE_ROOT environment variable
or the first command-line argument (default: the read-only reference mount of
the build container). When the reference tree is absent (e.g. on a GPU host),
build() does nothing and the tests that need these artefacts skip.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
CUDA_INC = "/usr/local/cuda/include"
DEFAULT_ROOT = "/root/reference"
REF_STAGES = ("sac2spec", "xc", "pws", "tfpws")


def reference_root(root: str | os.PathLike | None = None) -> Path:
    """The reference project's root: ``root``, else $FXC_REFERENCE_ROOT, else
    the container's default mount."""
    return Path(root or os.environ.get("FXC_REFERENCE_ROOT") or DEFAULT_ROOT)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"reference oracle build failed:\n{' '.join(cmd)}\n{proc.stderr}")


def lib_paths() -> dict[str, Path]:
    return {"sac2spec": OUT / "libref_sac2spec.so", "xc": OUT / "libref_xc.so"}


def cubin_paths() -> dict[str, Path]:
    return {st: OUT / f"ref_{st}.cubin" for st in REF_STAGES}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def build_kernels(ref: Path, force: bool = False) -> dict[str, Path]:
    """The reference's kernels as sm_103 cubins (device code only)."""
    outs = cubin_paths()
    shim = HERE / "ref_kernels.cu"
    for st, out in outs.items():
        if not force and out.exists() and out.stat().st_mtime >= shim.stat().st_mtime:
            continue
        src = ref / st
        _run([_nvcc(), "-cubin", "-gencode", "arch=compute_103,code=sm_103", "-O3", "--use_fast_math",
              "-std=c++17", f"-DFXC_REF_{st.upper()}", f"-I{src}", f"-I{src / 'include'}", f"-I{src / 'kernels'}",
              str(shim), "-o", str(out)])
    return outs


def build(force: bool = False, root: str | os.PathLike | None = None) -> dict[str, Path]:
    libs = lib_paths()
    REF = reference_root(root) / "native"
    if not REF.exists():
        return {k: v for k, v in libs.items() if v.exists()}
    OUT.mkdir(exist_ok=True)
    cc = shutil.which("gcc") or "gcc"
    cxx = shutil.which("g++") or "g++"
    s2s = REF / "sac2spec"
    if force or not libs["sac2spec"].exists():
        _run([cc, "-O2", "-shared", "-fPIC", "-w", f"-I{s2s}", f"-I{s2s / 'include'}", f"-I{s2s / 'core'}",
              str(s2s / "fft_length.c"), str(s2s / "core" / "filter_response.c"), str(s2s / "logger.c"),
              "-o", str(libs["sac2spec"]), "-lm"])
    xc = REF / "xc"
    if force or not libs["xc"].exists():
        objs = []
        for src, lang in ((xc / "io" / "path_table.c", "c"), (xc / "logger.c", "c")):
            obj = OUT / (src.stem + "_xc.o")
            _run([cc, "-O2", "-fPIC", "-w", "-c", f"-I{xc}", f"-I{xc / 'include'}", f"-I{xc / 'io'}", str(src),
                  "-o", str(obj)])
            objs.append(str(obj))
        _run([cxx, "-O2", "-shared", "-fPIC", "-w", "-std=c++17", f"-I{xc}", f"-I{xc / 'include'}",
              f"-I{xc / 'io'}", f"-I{xc / 'worker'}", f"-I{CUDA_INC}", "-x", "c++", str(xc / "worker" / "scheduler.cu"),
              "-x", "c++", str(HERE / "ref_xc_shim.cpp"), "-x", "none", *objs, "-o", str(libs["xc"]), "-lpthread"])
    libs.update({f"cubin_{st}": path for st, path in build_kernels(REF, force).items()})
    return libs


if __name__ == "__main__":
    print(build(force=True, root=sys.argv[1] if len(sys.argv) > 1 else None))
