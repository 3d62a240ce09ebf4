"""The plan's FP32 shortcut for the cell geometry of GRDH2D/GRDDEH2D (sde_gb300/csrc/geom.cuh,
geom_near_identity) against the DOUBLE arithmetic it stands in for (geom_dd), on the host:
random grids, cell sizes, near-identity SHIFT diagonals and uv points, plus points placed on
every rounding boundary either routine has.  Wherever the shortcut decides a visibility, all
outputs must be identical; the DOUBLE arithmetic itself is checked against the oracle by the
GPU plan tests."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def geom_check(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("geom") / "geom_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "sde_gb300", "csrc"),
                    os.path.join(HERE, "geom_check.cpp"), "-o", exe, "-lm"], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 7, 12345])
def test_shortcut_matches_double(geom_check, seed):
    out = subprocess.run([geom_check, "10000000", str(seed)], capture_output=True, text=True)
    cases, taken, bad = (int(x) for x in out.stdout.split())
    assert bad == 0, out.stderr
    assert out.returncode == 0
    # most points are decided by the shortcut, including a share of the boundary placements
    assert taken > 0.85 * cases
