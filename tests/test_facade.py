"""The header-only C++ facade (include/pv2013/pv2013.hpp): compiles with the
reference's driver calls and, on a GPU, gives the Python API's results."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "pv2013_gb300", "_lib")


def _build(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "facade_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "facade", "facade_check.cpp"), "-L", LIB, "-llbm_gb300",
                    f"-Wl,-rpath,{LIB}", "-o", exe], check=True)
    return exe


def _stl(tmp_path):
    import golden_pv2013 as G
    from pv2013_gb300 import Reader
    _, tris, _ = G.load()
    path = str(tmp_path / "pv2013.stl")
    Reader.writeSTLASCII(path, tris)
    return path


def test_facade_compiles_and_reports_no_device(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (covered by the GPU test)")
    exe = _build(tmp_path)
    out = subprocess.run([exe, _stl(tmp_path), "3"], capture_output=True, text=True, check=True).stdout
    assert out.strip() == "nodev"


@pytest.mark.gpu
def test_facade_matches_python_api(tmp_path):
    from pv2013_gb300 import BoundarySpec, Geometry, Reader, Simulation, _capi, pv2013_predicates
    exe = _build(tmp_path)
    stl = _stl(tmp_path)
    out = subprocess.run([exe, stl, "5"], capture_output=True, text=True, check=True).stdout.split()
    nf, nwall, mass = int(out[0]), int(out[1]), float(out[2])
    geom = Geometry(Reader.readSTLASCII(stl), 0.1, predicates=pv2013_predicates())
    kinds = [_capi.BC_VEL_NEGY, _capi.BC_PRESS_NEGY, _capi.BC_PRESS_POSY, _capi.BC_PRESS_POSX, _capi.BC_PRESS_POSX,
             _capi.BC_PRESS_POSX, _capi.BC_PRESS_POSZ]
    specs = [BoundarySpec(0, kinds[0], dir=(0.0, -1.0, 0.0), amp=np.array([0.1]))]
    specs += [BoundarySpec(l, kinds[l], rho=1.01) for l in range(1, 7)]
    sim = Simulation(geom, 0.66, specs, precision="f64", pattern="pull")
    sim.step(5)
    _, rho, _ = sim.fields(f=False)
    assert nf == geom.info.n_fluid and nwall == len(geom.WallboundaryPoints)
    # the facade sums rho left to right in FP64: the same order as cumsum
    assert mass == float(np.cumsum(rho)[-1])
