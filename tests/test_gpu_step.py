"""Fused GPU step against the FP64 oracle.

FP64 storage is bit-exact (every population, every node) for the pull and
AA patterns, with and without CUDA-graph replay, single and batched.  The
reduced-precision stores are checked against the FP64 oracle with the
tolerances stated in each test (velocity relative L2 error)."""
import numpy as np
import pytest

from pv2013_gb300 import BoundarySpec, Geometry, Simulation, _capi, cases, pv2013_predicates

pytestmark = pytest.mark.gpu


def oracle_run(O, case, geom, steps, Q=19, bcs=None, inlet_dir=(0.0, -1.0, 0.0)):
    geo = O.geometry(case.triangles, case.spacing, case.grid, case.predicates)
    bcs = bcs or {0: (O.BC_VEL_NEGY, 1.0), 2: (O.BC_PRESS_POSY, case.outlet_rho)}
    return geo, O.run_case(Q, geo, case.tau, bcs, steps, profile=case.inlet_profile(geom), amp=case.amp_table(),
                           inlet_dir=inlet_dir)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("staging", [0, 1])
@pytest.mark.parametrize("run_axis", [1, 2])
@pytest.mark.parametrize("pattern", ["pull", "aa"])
@pytest.mark.parametrize("steps", [1, 2, 37])
def test_fp64_pipe_bit_exact(oracle_mod, pattern, steps, run_axis, staging):
    """Both node numberings (runs along y or along z) and both kernels (TMA-staged
    pipeline, direct loads) give the reference's populations; outputs are in the
    reference's x-major node order."""
    O = oracle_mod
    c = cases.pipe()
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern=pattern, run_axis=run_axis,
                     staging=staging)
    assert sim.info().run_axis == run_axis
    sim.step(steps)
    f, rho, u = sim.fields()
    _, ref = oracle_run(O, c, geom, steps)
    fr = ref.f()
    assert np.array_equal(f, fr)
    rr, ur = O.macro(fr)
    assert np.array_equal(rho, rr) and np.array_equal(u, ur)
    assert np.array_equal(sim.nodes(), np.flatnonzero(geom.flags().reshape(-1)))


@pytest.mark.parametrize("pattern", ["pull", "aa"])
def test_fp64_graph_replay_equals_direct(pattern):
    c = cases.pipe()
    geom = c.geometry()
    a = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern=pattern)
    b = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern=pattern)
    a.step(1)
    a.step(131, graph=True)
    b.step(132)
    assert a.info().steps_done == 132
    assert np.array_equal(a.fields()[0], b.fields()[0])


@pytest.mark.parametrize("pattern,run_axis,staging", [("pull", 2, 0), ("aa", 1, 0), ("aa", 0, 0), ("pull", 1, 1)])
def test_fp64_pulsatile_vessel_bit_exact(oracle_mod, pattern, run_axis, staging):
    O = oracle_mod
    c = cases.vessel(4001)
    c.inlet.period = 9
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern=pattern, run_axis=run_axis,
                     staging=staging)
    sim.step(25)
    _, ref = oracle_run(O, c, geom, 25)
    assert np.array_equal(sim.fields()[0], ref.f())


def test_fp64_pv2013_all_reference_boundaries(oracle_mod):
    """PV2013 with the reference's own lists and routines: velocity inlet
    (0,-0.1,0), pressure outlets 1-6 at rho 1.01 (Simulation.cpp:952-1348,
    including the f10 term of outlets 3-5), bounce-back walls; 6 steps."""
    import golden_pv2013 as G
    O = oracle_mod
    meta, tris, lists = G.load()
    geom = Geometry(tris, 0.1, predicates=pv2013_predicates())
    kinds = {0: _capi.BC_VEL_NEGY, 1: _capi.BC_PRESS_NEGY, 2: _capi.BC_PRESS_POSY, 3: _capi.BC_PRESS_POSX,
             4: _capi.BC_PRESS_POSX, 5: _capi.BC_PRESS_POSX, 6: _capi.BC_PRESS_POSZ}
    specs = [BoundarySpec(0, kinds[0], dir=(0.0, -1.0, 0.0), amp=np.array([0.1]))]
    specs += [BoundarySpec(l, kinds[l], rho=1.01) for l in range(1, 7)]
    sim = Simulation(geom, 0.66, specs, precision="f64", pattern="pull")
    steps = 6
    sim.step(steps)
    bb, dims = O.tight_grid(tris, 0.1)
    flags = O.voxelize(tris, bb, 0.1, dims)
    bidx = O.boundary_points(flags)
    tup = G.oracle_tuples()
    pm = O.classify(bidx, dims, bb, 0.1, [t for _, t in tup])
    role = np.where(flags.reshape(-1) > 0, 0, -1).astype(np.int8)
    first = np.ones(len(bidx), dtype=np.int8)
    for k in range(6, -1, -1):
        sel = ((pm >> np.uint64(k)) & np.uint64(1)).astype(bool)
        first[sel] = 2 + k
    role[bidx] = first
    kk = np.zeros(64, dtype=np.int32)
    rr = np.ones(64)
    for l, k in kinds.items():
        kk[l] = k
        rr[l] = 1.01
    ref = O.OracleSim(19, dims, role, kk, rr, 0.66)   # inlet keeps the reference default (0,-0.1,0)
    ref.step(steps)
    assert np.array_equal(sim.fields()[0], ref.f())


def test_batch_equals_individual_runs():
    c1, c2 = cases.pipe(), cases.vessel(4002)
    g1, g2 = c1.geometry(), c2.geometry()
    batch = Simulation([g1, g2], [c1.tau, c2.tau], [c1.boundary_specs(g1), c2.boundary_specs(g2)],
                       precision="f64", pattern="aa", run_axis=1)
    s1 = Simulation(g1, c1.tau, c1.boundary_specs(g1), precision="f64", pattern="aa")
    s2 = Simulation(g2, c2.tau, c2.boundary_specs(g2), precision="f64", pattern="aa")
    for s in (batch, s1, s2):
        s.step(17, graph=True)
    off = batch.instance_offsets()
    fb = batch.fields()[0]
    assert np.array_equal(fb[off[0]:off[1]], s1.fields()[0])
    assert np.array_equal(fb[off[1]:off[2]], s2.fields()[0])
    nodes = batch.nodes()
    assert np.array_equal(nodes[off[0]:off[1]], s1.nodes()) and np.array_equal(nodes[off[1]:off[2]], s2.nodes())


@pytest.mark.parametrize("precision,pattern,tol", [("f32", "pull", 2e-5), ("f32", "aa", 2e-5),
                                                    ("f16s", "aa", 1e-3), ("f16s", "pull", 1e-3),
                                                    ("bf16s", "aa", 3e-2)])
@pytest.mark.parametrize("run_axis", [1, 2])
def test_reduced_precision_velocity_error(oracle_mod, precision, pattern, tol, run_axis):
    """Velocity relative L2 error vs the FP64 oracle after 400 steps of the pipe."""
    O = oracle_mod
    c = cases.pipe()
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision=precision, pattern=pattern, run_axis=run_axis)
    sim.step(400)
    _, rho, u = sim.fields()
    _, ref = oracle_run(O, c, geom, 400)
    rr, ur = O.macro(ref.f())
    err = rel_l2(u, ur)
    assert err < tol, (precision, pattern, err)
    assert abs(rho.sum() / rr.sum() - 1) < 10 * tol


def test_monitors_and_fields_consistent():
    c = cases.pipe()
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern="pull")
    sim.step(50)
    m = sim.monitors()
    f, rho, u = sim.fields()
    assert m["step"] == 50 and not m["nonfinite"]
    assert abs(m["mass"] - rho.sum()) <= 1e-9 * rho.sum()
    assert abs(m["max_speed"] - np.sqrt((u ** 2).sum(1)).max()) <= 1e-12
    assert m["inlet_flux"] > 0 and m["outlet_flux"] > 0


def test_divergence_monitor_reports_status():
    """An unstable run (tau close to 1/2, large inlet speed) is reported as
    LBM_ERR_DIVERGED by the host-side monitor, not as a fault."""
    c = cases.pipe()
    geom = c.geometry()
    specs = [BoundarySpec(0, _capi.BC_VEL_NEGY, amp=np.array([0.4])), BoundarySpec(2, _capi.BC_PRESS_POSY)]
    sim = Simulation(geom, 0.5005, specs, precision="f32", pattern="aa")
    sim.set_divergence_tolerance(1e-3)
    with pytest.raises(_capi.LbmError) as e:
        for _ in range(40):
            sim.step(50, monitor=True)
    assert e.value.status == 5


def test_d3q27_fp64_bit_exact(oracle_mod):
    O = oracle_mod
    c = cases.pipe_x()
    preds = c.predicates[:1]
    geom = Geometry(c.triangles, 1.0, grid=c.grid, predicates=preds)
    prof = c.inlet_profile(geom)
    specs = [BoundarySpec(0, _capi.BC_VEL_POSX, dir=(1.0, 0.0, 0.0), profile=prof, amp=c.amp_table())]
    for pattern in ("pull", "aa"):
        sim = Simulation(geom, c.tau, specs, Q=27, precision="f64", pattern=pattern)
        sim.step(11)
        geo = O.geometry(c.triangles, 1.0, c.grid, preds)
        ref = O.run_case(27, geo, c.tau, {0: (O.BC_VEL_POSX, 1.0)}, 11, profile=prof, amp=c.amp_table(),
                         inlet_dir=(1.0, 0.0, 0.0))
        assert np.array_equal(sim.fields()[0], ref.f()), pattern


@pytest.mark.parametrize("corrections", [1, 2, 3])
@pytest.mark.parametrize("pattern", ["pull", "aa"])
def test_fp64_corrections_bit_exact(oracle_mod, pattern, corrections):
    """The corrected boundary handling (bounce-back of every direction, of
    inlet/outlet nodes too) against the oracle with the same corrections."""
    O = oracle_mod
    c = cases.vessel(4001)
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern=pattern, corrections=corrections)
    sim.step(21)
    geo = O.geometry(c.triangles, c.spacing, c.grid, c.predicates)
    ref = O.run_case(19, geo, c.tau, {0: (O.BC_VEL_NEGY, 1.0), 2: (O.BC_PRESS_POSY, c.outlet_rho)}, 21,
                     profile=c.inlet_profile(geom), amp=c.amp_table(), corrections=corrections)
    assert np.array_equal(sim.fields()[0], ref.f())


def test_corrections_act_on_boundary_nodes_first():
    """Parity and corrected runs differ, most at the boundary nodes (where the
    bounce-back rules differ)."""
    c = cases.pipe()
    geom = c.geometry()
    a = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern="pull")
    b = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern="pull", corrections=3)
    a.step(10)
    b.step(10)
    fa, fb = a.fields()[0], b.fields()[0]
    d = np.abs(fa - fb).max(axis=1)
    assert d.max() > 0
    bnd = set(geom.list(_capi.LIST_BOUNDARY).tolist())
    assert int(a.nodes()[np.argmax(d)]) in bnd


def test_bounded_wait_runs_out_and_the_handle_recovers(tmp_path):
    """The TMA-staged kernel's mbarrier waits are bounded.  With the
    failure-test hook each warp's first stage is never issued (no copy, no
    arrival): its wait, limited to 1000 non-blocking tests, runs out; the warp
    records it, drains its other stages and stops; the next monitor call
    reports LBM_ERR_TIMEOUT, once.  With the hook off, the default limit and
    the state restored from a checkpoint, the run continues bit for bit."""
    c = cases.pipe()
    geom = c.geometry()
    specs = c.boundary_specs(geom)
    ref = Simulation(geom, c.tau, specs, precision="f64", pattern="pull", staging=0)
    sim = Simulation(geom, c.tau, specs, precision="f64", pattern="pull", staging=0)
    ref.step(4)
    sim.step(4)
    path = str(tmp_path / "w.ckpt")
    sim.checkpoint(path)
    sim.set_wait_limit(1000)
    sim.test_stall(True)
    sim.step(2)
    with pytest.raises(_capi.LbmError) as e:
        sim.monitors()
    assert e.value.status == _capi.ERR_TIMEOUT
    sim.monitors()          # reported once: this call succeeds
    sim.test_stall(False)
    sim.set_wait_limit(0)
    sim.restart(path)
    sim.step(6)
    ref.step(6)
    assert np.array_equal(sim.fields()[0], ref.fields()[0])


@pytest.mark.parametrize("precision,pattern,npl", [("f64", "pull", 1), ("f64", "aa", 1), ("f32", "pull", 2),
                                                   ("f32", "aa", 1), ("f16s", "aa", 2), ("f16s", "pull", 2),
                                                   ("bf16s", "aa", 2), ("f16s", "aa", 1)])
def test_ghost_slots_never_reach_results(precision, pattern, npl):
    """Self-check: NaN in every population slot of no fluid node (ghost layer,
    pair padding, array slack), at the start and again mid-run, leaves every
    population of every fluid node bit-identical and finite -- no kernel uses
    a value it must replace (walls, inlet, outlet, graph replay included)."""
    c = cases.vessel(4001)
    c.inlet.period = 9
    geom = c.geometry()
    runs = []
    for poison in (False, True):
        sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision=precision, pattern=pattern,
                         nodes_per_lane=npl, staging=0 if npl == 1 else 1,
                         corrections=_capi.FIX_LIST_NODES if pattern == "pull" else 0)
        if poison:
            sim.poison_ghosts()
        sim.step(5)
        if poison:
            sim.poison_ghosts()
        sim.step(8, graph=True)
        f, rho, u = sim.fields()
        mon = sim.monitors()
        runs.append((f, mon))
    (f0, m0), (f1, m1) = runs
    assert np.isfinite(f1).all() and not m1["nonfinite"]
    assert np.array_equal(f1, f0)


@pytest.mark.parametrize("pattern", ["pull", "aa"])
@pytest.mark.parametrize("precision", ["f64", "f16s"])
def test_prepared_graph_equals_direct_steps(pattern, precision):
    """A graph captured ahead (lbm_sim_prepare_graph), from an aligned and
    from a misaligned state, replays the same steps as direct launches."""
    c = cases.vessel(4001)
    c.inlet.period = 9
    geom = c.geometry()
    a = Simulation(geom, c.tau, c.boundary_specs(geom), precision=precision, pattern=pattern)
    b = Simulation(geom, c.tau, c.boundary_specs(geom), precision=precision, pattern=pattern)
    a.step(3)                       # misaligned: the replay starts with one direct step
    f3 = a.fields()[0]
    a.prepare_graph(70)
    assert a.info().steps_done == 3 and np.array_equal(a.fields()[0], f3)   # the state is untouched
    a.step(70, graph=True)
    a.prepare_graph(40)
    a.step(40, graph=True)
    b.step(113)
    assert np.array_equal(a.fields()[0], b.fields()[0])
