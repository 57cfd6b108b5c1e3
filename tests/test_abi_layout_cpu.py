"""The ctypes structures of the Python binding (pv2013_gb300/_capi.py) have the
C header's layout: for every struct of include/lbm_gb300.h the binding
mirrors, a C++ program compiled against the header prints sizeof and the
offset of each field, and they must equal the ctypes ones.  Guards the ABI
against a field added on one side only."""
import ctypes
import os
import shutil
import subprocess

import pytest

from pv2013_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PAIRS = [("Tri", "lbm_tri"), ("Grid", "lbm_grid"), ("Predicate", "lbm_bc_predicate"),
         ("GeometryInfo", "lbm_geometry_info"), ("ListBC", "lbm_list_bc"), ("SimParams", "lbm_sim_params"),
         ("TuneEntry", "lbm_tune_entry"), ("VtuArray", "lbm_vtu_array"), ("SimInfo", "lbm_sim_info"),
         ("Monitors", "lbm_monitors")]


def test_ctypes_structs_match_the_header(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    lines = ['#include <cstddef>', '#include <cstdio>', '#include "lbm_gb300.h"', "int main() {"]
    expect = []
    for py, c in PAIRS:
        cls = getattr(_capi, py)
        lines.append(f'    std::printf("%s size %zu\\n", "{c}", sizeof({c}));')
        expect.append(f"{c} size {ctypes.sizeof(cls)}")
        for name, _ in cls._fields_:
            lines.append(f'    std::printf("%s.%s %zu\\n", "{c}", "{name}", offsetof({c}, {name}));')
            expect.append(f"{c}.{name} {getattr(cls, name).offset}")
    lines.append("    return 0;\n}")
    src = tmp_path / "layout.cpp"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    got = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    assert [g for g in got if g] == expect
