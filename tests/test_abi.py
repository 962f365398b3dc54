"""CPU-side checks of the C ABI: the library builds, loads without a GPU and
exports every function that include/*.h declares; the ctypes table matches."""

import re
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def header_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?\**\s*\**(fxc_[a-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(built_lib):
    from fastxc_gb300._lib import LIB_PATH

    out = subprocess.run(["nm", "-D", "--defined-only", str(LIB_PATH)], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    declared = header_functions()
    assert declared, "no declarations parsed"
    missing = sorted(declared - exported)
    assert not missing, f"declared but not exported: {missing}"


def test_ctypes_table_matches_header(built_lib):
    from fastxc_gb300._lib import declared_symbols

    assert set(declared_symbols()) == header_functions()


def test_loads_without_gpu_and_reports_no_device(built_lib):
    import ctypes

    from fastxc_gb300._lib import lib

    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    assert lib().fxc_version() >= 100
    if not has_gpu:
        h = ctypes.c_void_p()
        st = lib()._raw_fxc_ctx_create(0, None, ctypes.byref(h))
        assert st != 0
        assert lib().last_error()
