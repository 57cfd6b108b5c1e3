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


@pytest.mark.parametrize("precision,pattern", [("f64", "pull"), ("f64", "aa"), ("f16s", "aa"), ("f32", "pull")])
def test_checkpoint_restart_continues_exactly(tmp_path, precision, pattern):
    c = cases.vessel(4001)
    geom = c.geometry()
    a = Simulation(geom, c.tau, c.boundary_specs(geom), precision=precision, pattern=pattern)
    a.step(21)                                        # odd: AA parity and pull buffer index matter
    a.checkpoint(tmp_path / "s.ckpt")
    a.step(30, graph=True)
    b = Simulation(geom, c.tau, c.boundary_specs(geom), precision=precision, pattern=pattern)
    b.restart(tmp_path / "s.ckpt")
    assert b.info().steps_done == 21
    b.step(30, graph=True)
    assert np.array_equal(a.fields()[0], b.fields()[0])


def test_restart_rejects_other_lattices(tmp_path):
    from pv2013_gb300 import _capi
    c1, c2 = cases.vessel(4001), cases.vessel(4002)
    g1, g2 = c1.geometry(), c2.geometry()
    a = Simulation(g1, c1.tau, c1.boundary_specs(g1), precision="f32", pattern="aa")
    a.checkpoint(tmp_path / "a.ckpt")
    b = Simulation(g2, c2.tau, c2.boundary_specs(g2), precision="f32", pattern="aa")
    with pytest.raises(_capi.LbmError) as e:
        b.restart(tmp_path / "a.ckpt")
    assert e.value.status == _capi.ERR_ARG
    c = Simulation(g1, c1.tau, c1.boundary_specs(g1), precision="f16s", pattern="aa")
    with pytest.raises(_capi.LbmError):
        c.restart(tmp_path / "a.ckpt")
    (tmp_path / "junk.ckpt").write_bytes(b"not a checkpoint")
    with pytest.raises(_capi.LbmError) as e:
        a.restart(tmp_path / "junk.ckpt")
    assert e.value.status == 2
    with pytest.raises(_capi.LbmError) as e:
        a.restart(tmp_path / "missing.ckpt")
    assert e.value.status == 1
