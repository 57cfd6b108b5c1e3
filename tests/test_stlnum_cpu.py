"""The device STL reader's exact decimal converter (csrc/stl_number.h),
compiled here as host code, against strtod: every string it converts must
give strtod's bits (strtod rounds correctly like the reference's
istream >> double, GeometryReader.cpp:33-117), and it must stop where
strtod stops.  Random decimal strings, printf %e/%f/%.17g forms, halfway
integers above 2^53 and decimal exponents up to +-60."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("stlnum") / "stlnum_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "pv2013_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "stlnum", "stlnum_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2])
def test_exact_converter_equals_strtod(checker, seed):
    out = subprocess.run([checker, "400000", str(seed)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    parts = out.stdout.split()
    checked, exact = int(parts[1]), int(parts[3])
    assert checked >= 400000
    # the exact scope covers nearly every generated string
    assert exact / checked > 0.95
