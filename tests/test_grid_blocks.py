"""The host check that the reference's coarse-block loop stays inside the
grid (csrc/to_grid.h), compiled as plain C++ on the CPU: every square grid
passes, non-square grids whose last blocks would leave the grid are
refused."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _blocks(W, H, res):
    xres = res if W % res == 0 else res + 1
    yres = res if H % res == 0 else res + 1
    return (W - 1) // res, (H - 1) // res, xres, yres


def _inside_py(W, H, skpx, skpy, xres, yres):
    """The cells the kernels' loop visits, enumerated."""
    xs = [bx * skpx + ii for bx in range(xres)
          for ii in range(skpx if (bx + 1) * skpx <= H else H - bx * skpx)]
    ys = [by * skpy + jj for by in range(yres)
          for jj in range(skpy if (by + 1) * skpy <= W else W - by * skpy)]
    if not xs or not ys:
        return True
    return max(xs) < W and max(ys) < H


def test_blocks_inside_matches_enumeration(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cases = []
    for W in (1, 2, 7, 37, 64, 100, 128, 199, 200, 201):
        for H in (W, W + 1, W + 13, max(1, W - 9), 2 * W):
            for res in (1, 2, 3, 4, 7, 10, 16):
                cases.append((W, H) + _blocks(W, H, res))
    cases += [(64, 64, 30, 30, 3, 3), (50, 80, 10, 10, 6, 6), (80, 50, 10, 10, 6, 6)]
    src = tmp_path / "t.cpp"
    src.write_text('#include <cstdio>\n#include "to_grid.h"\nint main() {\n' + "".join(
        f'std::printf("%d\\n", (int)to_blocks_inside({W}, {H}, {a}, {b}, {c}, {d}));\n'
        for (W, H, a, b, c, d) in cases) + "return 0;\n}\n")
    exe = tmp_path / "t"
    subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-I",
                    str(ROOT / "transportoptimiser_gb300" / "csrc"), str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    for case, g in zip(cases, got):
        assert bool(g) == _inside_py(*case), case
    # square grids at every resolution are always inside
    for (W, H, *_), g in zip(cases, got):
        if W == H:
            assert g == 1, (W, H)
    # and some non-square layouts are refused
    assert not all(got)
