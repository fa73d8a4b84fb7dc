"""The C ABI library builds, loads and exports every entry point that
include/transopt.h declares (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    txt = (ROOT / "include" / "transopt.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(to_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_header(lib_built):
    lib = C.CDLL(str(lib_built))
    names = declared_symbols()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(lib_built):
    from transportoptimiser_gb300 import _capi
    names = declared_symbols()
    assert sorted(_capi.SIGNATURES) == names


def test_status_strings_without_gpu(lib_built):
    from transportoptimiser_gb300 import _capi
    lib = _capi.load()
    assert lib.to_status_string(0) == b"ok"
    n = C.c_int(-1)
    assert lib.to_device_count(C.byref(n)) == 0 and n.value >= 0
