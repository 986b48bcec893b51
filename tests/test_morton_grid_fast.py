"""The 64-bit Morton grid coordinate from float pieces (morton_floor_fast in
obvhs_gb300/csrc/morton_grid.h, used by the Morton kernels) against the
double-precision value it stands for, sat_u32(RN(RN(c * S) + O)), the
reference's `(c * scale + offset) * 2^21 ... as u32`
(src/ploc/mod.rs:782-785), on the CPU.

tests/morton_grid_check.cpp compiles the same header for the host (every
float operation rounded on its own, -ffp-contract=off) and draws scenes
around the origin and far from it, centres inside them, the bounds, centres
a few ulps from every kind of grid line, and values the fast path must leave
to double precision (zeros, subnormals, infinities, NaN).  Every coordinate
the fast path decides must equal the double-precision one; for scenes near
the origin almost all of them must be decided."""
import json
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "obvhs_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("mg") / "morton_grid_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "morton_grid_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_fast_grid_coordinate_equals_double_precision(checker, seed):
    p = subprocess.run([checker, str(seed), "1500", "4000"], capture_output=True, text=True)
    r = json.loads(p.stdout)
    assert p.returncode == 0 and r["mismatches"] == 0, (r, p.stderr[:2000])
    assert r["decided"] > 0.95 * r["cases"], r
    assert r["in_range_decided"] > 0.999 * r["in_range_cases"], r
