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


def test_header_builds_c_and_cpp_callers(lib_built, tmp_path):
    """A C11 and a C++17 caller compile against include/transopt.h with
    warnings as errors, link the library and run its GPU-free calls, as a
    host program replacing the reference's SimulateGPU layer would."""
    import shutil
    import subprocess
    src = r'''
#include "transopt.h"
#include <stdio.h>
#include <string.h>
int main(void) {
    to_mte_problem p;
    memset(&p, 0, sizeof(p));
    int n = -1;
    if (to_device_count(&n) != TO_OK || n < 0) return 1;
    if (strcmp(to_status_string(TO_OK), "ok") != 0) return 2;
    /* invalid arguments are refused before any device work */
    if (to_simulate_mte(NULL, &p, NULL, NULL) == TO_OK) return 3;
    printf("%d\n", (int)sizeof(p));
    return 0;
}
'''
    lib_dir = Path(lib_built).parent
    built = 0
    for cc, ext, std in (("gcc", "c", "-std=c11"), ("g++", "cpp", "-std=c++17")):
        exe = shutil.which(cc)
        if exe is None:
            continue
        f = tmp_path / f"caller.{ext}"
        f.write_text(src)
        out = tmp_path / f"caller_{ext}"
        subprocess.run([exe, std, "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-I", str(ROOT / "include"), str(f), "-o", str(out),
                        "-L", str(lib_dir), "-ltransopt", f"-Wl,-rpath,{lib_dir}"],
                       check=True, capture_output=True, text=True)
        r = subprocess.run([str(out)], capture_output=True, text=True)
        assert r.returncode == 0, (cc, r.returncode, r.stderr)
        built += 1
    assert built >= 1
