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


def test_ctypes_structs_match_the_header(tmp_path):
    """Every ctypes mirror of a struct in include/transopt.h has the C
    compiler's size and field offsets (a mismatch would pass garbage across
    the boundary without any error)."""
    import shutil
    import subprocess
    from transportoptimiser_gb300 import _capi
    from transportoptimiser_gb300.adjoint import AdjointProblem
    pairs = {"to_habitat": _capi.Habitat, "to_species_in": _capi.SpeciesIn,
             "to_species_out": _capi.SpeciesOut, "to_mte_species": _capi.MteSpecies,
             "to_mte_problem": _capi.MteProblem, "to_mte_stats": _capi.MteStats,
             "to_mte_device_problem": _capi.MteDeviceProblem,
             "to_exp_pv_params": _capi.ExpPvParams, "to_species_desc": _capi.SpeciesDesc,
             "to_scene": _capi.Scene, "to_eval_opts": _capi.EvalOpts,
             "to_rov_species": _capi.RovSpecies, "to_rov_problem": _capi.RovProblem,
             "to_rov_result": _capi.RovResult, "to_adjoint_problem": AdjointProblem}
    cc = shutil.which("gcc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "transopt.h"', 'int main(void) {']
    for cname, py in pairs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ['return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True,
                               text=True).stdout.splitlines():
        name, field, val = line.split()
        got[(name, field)] = int(val)
    for cname, py in pairs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
