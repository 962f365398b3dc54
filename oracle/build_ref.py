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
The reference's GPU kernels and cuFFT calls are not built here. When the
reference tree is absent (e.g. on a GPU host), build() does nothing and the
tests that need these libraries skip.
"""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

REF = Path("/root/reference/native")
HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
CUDA_INC = "/usr/local/cuda/include"


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"reference oracle build failed:\n{' '.join(cmd)}\n{proc.stderr}")


def lib_paths() -> dict[str, Path]:
    return {"sac2spec": OUT / "libref_sac2spec.so", "xc": OUT / "libref_xc.so"}


def build(force: bool = False) -> dict[str, Path]:
    libs = lib_paths()
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
    return libs


if __name__ == "__main__":
    print(build(force=True))
