"""Builds the in-tree CUDA library and the CPU oracle.

``build()`` compiles every ``csrc/*.cu`` for sm_103a with nvcc (in
parallel, one -gencode) and links ``_lib/libtransopt.so``.  The oracle
(test infrastructure under ``oracle/``) is built by ``build_oracle()``; the
reference-on-CPU pin library by ``oracle/build_ref.sh`` when the reference
tree is mounted.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libtransopt.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
    "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills",
]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found")
    return cand


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    objdir = LIBDIR / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "transopt.h"]
    jobs = []
    for src in sources:
        obj = objdir / (src.stem + ".o")
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    if jobs:
        workers = min(len(jobs), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            for f in [ex.submit(_run, j) for j in jobs]:
                f.result()
    objs = [objdir / (s.stem + ".o") for s in sources]
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"])
    if verbose:
        print("built", LIB)
    return LIB


def build_oracle(force: bool = False) -> Path:
    srcs = [ORACLE_DIR / "oracle.c", ORACLE_DIR / "oracle_rov.c", ORACLE_DIR / "oracle_mlp.c",
            ORACLE_DIR / "oracle_adjoint.c", ORACLE_DIR / "oracle_interp.c",
            ORACLE_DIR / "oracle_sample.c"]
    deps = srcs + [ORACLE_DIR / "oracle.h", ORACLE_DIR / "oracle_rov.h", ORACLE_DIR / "oracle_mlp.h",
                   ORACLE_DIR / "oracle_adjoint.h", ORACLE_DIR / "oracle_interp.h",
                   ORACLE_DIR / "oracle_sample.h",
                   CSRC / "to_math.h", CSRC / "to_math_tables.h", CSRC / "to_lsm_math.h"]
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    if force or _stale(ORACLE_LIB, deps):
        cc = shutil.which("gcc") or "cc"
        _run([cc, "-O3", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared",
              "-pthread", *map(str, srcs), "-o", str(ORACLE_LIB), "-lm"])
    return ORACLE_LIB


def build_reference_pin() -> None:
    """oracle/_ref from the reference tree: the recipe (oracle/build_ref.sh)
    knows where the tree is mounted (TO_REFERENCE_DIR) and skips the build
    where it is absent."""
    script = ORACLE_DIR / "build_ref.sh"
    if script.exists():
        _run(["sh", str(script)])


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    build_oracle(force="--force" in sys.argv)
    build_reference_pin()
