"""A run file with boundary blocks reproduces the Python-built straight pipe
bit for bit (FP64), from the pipe's surface written as an STL file; the
reference's pulsatile waveform preset drives a run."""
import numpy as np
import pytest

from pv2013_gb300 import Reader, Simulation, cases, runfile
from pv2013_gb300.__main__ import build_problem

pytestmark = pytest.mark.gpu


def pipe_run_file(c, stl, waveform="constant"):
    (cx, cz), r = c.inlet.center, c.inlet.radius
    (mx, my, mz), (nx, ny, nz) = c.grid
    inlet, outlet = c.predicates
    half = r + 3
    return f"""# the straight pipe of pv2013_gb300.cases.pipe
stl {stl}
spacing {c.spacing!r}
box {mx!r} {my!r} {mz!r} {nx} {ny} {nz}
tau {c.tau!r}
boundary 0
  axis y
  plane {inlet.plane!r}
  tol 0.01
  box {cx - half!r} {cx + half!r} nan nan {cz - half!r} {cz + half!r}
  kind vel_negy
  dir 0 -1 0
  u {c.inlet.u_max!r}
  profile parabolic {cx!r} {cz!r} {r!r}
  waveform {waveform}
end
boundary 2
  axis y
  plane {outlet.plane!r}
  box {cx - half!r} {cx + half!r} nan nan {cz - half!r} {cz + half!r}
  kind press_posy
  rho {c.outlet_rho!r}
end
""".splitlines(True)


def test_run_file_reproduces_the_pipe(tmp_path):
    c = cases.pipe()
    stl = str(tmp_path / "pipe.stl")
    Reader.writeSTLASCII(stl, c.triangles)
    cfg, blocks = runfile.parse(pipe_run_file(c, stl))
    g, tau, specs, Q = build_problem(cfg, blocks)
    ref_g = c.geometry()
    assert np.array_equal(g.flags(), ref_g.flags())
    for lid in (0, 2):
        assert np.array_equal(g.list(lid), ref_g.list(lid))
    a = Simulation(g, tau, specs, Q=Q, precision="f64", pattern="pull")
    b = Simulation(ref_g, c.tau, c.boundary_specs(ref_g), precision="f64", pattern="pull")
    a.step(25)
    b.step(25)
    assert np.array_equal(a.fields()[0], b.fields()[0])


def test_pv2013_waveform_drives_the_inlet(tmp_path):
    c = cases.pipe()
    stl = str(tmp_path / "pipe.stl")
    Reader.writeSTLASCII(stl, c.triangles)
    cfg, blocks = runfile.parse(pipe_run_file(c, stl, waveform="pv2013 40"))
    g, tau, specs, Q = build_problem(cfg, blocks)
    sim = Simulation(g, tau, specs, Q=Q, precision="f16s", pattern="aa")
    sim.step(60, graph=True)
    _, rho, u = sim.fields(f=False)
    assert np.isfinite(u).all() and np.abs(u).max() > 0
