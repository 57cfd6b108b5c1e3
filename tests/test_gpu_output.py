"""Wall shear stress and asynchronous snapshots against the oracle and the
synchronous field copies."""
import numpy as np
import pytest

from pv2013_gb300 import Simulation, Snapshot, cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pattern", ["pull", "aa"])
def test_wall_shear_stress_fp64_bit_exact(oracle_mod, pattern):
    """After k steps the GPU's wall shear stress equals the reference's of
    iteration k (ComputeWallShearStress, from the velocities its Collision of
    iteration k stores) bit for bit: the oracle after k + 1 steps."""
    O = oracle_mod
    c = cases.vessel(4002)
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern=pattern)
    sim.step(15)
    w = sim.wall_shear_stress()
    assert len(w) == len(geom.WallboundaryPoints)
    geo = O.geometry(c.triangles, c.spacing, c.grid, c.predicates)
    ref = O.run_case(19, geo, c.tau, {0: (O.BC_VEL_NEGY, 1.0), 2: (O.BC_PRESS_POSY, c.outlet_rho)}, 16,
                     profile=c.inlet_profile(geom), amp=c.amp_table())
    assert np.array_equal(w, ref.wss())
    assert w.max() > 0


def test_wall_shear_stress_reduced_precision():
    c = cases.vessel(4002)
    geom = c.geometry()
    a = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern="aa")
    b = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f16s", pattern="aa")
    a.step(300, graph=True)
    b.step(300, graph=True)
    wa, wb = a.wall_shear_stress(), b.wall_shear_stress()
    assert np.linalg.norm(wb - wa) / np.linalg.norm(wa) < 2e-2


def test_snapshot_is_the_captured_state(tmp_path):
    """capture() returns before the copy completes; the simulation keeps
    stepping on its stream; the snapshot holds the state at capture time."""
    c = cases.pipe()
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f32", pattern="aa")
    snap = Snapshot(sim, fields=True, wss=True)
    sim.step(40, graph=True)
    _, r40, u40 = sim.fields(f=False)
    w40 = sim.wall_shear_stress()
    snap.capture()
    sim.step(30, graph=True)              # enqueued behind the snapshot launch
    rho, u, wss, step = snap.data()
    assert step == 40
    assert np.array_equal(rho, r40) and np.array_equal(u, u40) and np.array_equal(wss, w40)
    snap.capture()                        # a second capture reuses the buffers
    _, r70, u70 = sim.fields(f=False)
    rho2, u2, _, step2 = snap.data()
    assert step2 == 70 and np.array_equal(u2, u70)
    snap.write_fields_vtu(tmp_path / "f.vtu")
    snap.write_wss_vtu(tmp_path / "w.vtu")
    import test_vtu_cpu as T
    _, n, arrs = T._read_vtu(tmp_path / "f.vtu")
    assert n == len(rho2)
    # points in the reference's order: x fastest, then y, then z
    pts = arrs["Points"].reshape(-1, 3).astype(np.int64)
    key = (pts[:, 2] * geom.GeomSize[1] + pts[:, 1]) * geom.GeomSize[0] + pts[:, 0]
    assert np.all(np.diff(key) > 0)
    assert np.allclose(arrs["Pressure"], arrs["Density"] / 3.0)
    # the fields of a point match the x-major output of lbm_sim_fields
    idx = sim.nodes()
    Nx, Ny, Nz = geom.GeomSize
    xm = (pts[:, 0] * Ny + pts[:, 1]) * Nz + pts[:, 2]
    order = np.searchsorted(idx, xm)
    assert np.array_equal(arrs["Density"], r70[order])
    assert np.array_equal(arrs["Velocity"].reshape(-1, 3), u70[order])
    _, nw, w = T._read_vtu(tmp_path / "w.vtu")
    assert nw == len(geom.WallboundaryPoints)
    snap.close()
