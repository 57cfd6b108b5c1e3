"""Paired step kernel (two adjacent nodes per lane, packed FP32 arithmetic).

The paired kernel performs the same operations as the one-node-per-lane
kernel in FP32 (operation order inside the collision differs), so it is
checked (1) against the FP64 oracle with the reduced-precision tolerances of
test_gpu_step.py (velocity relative L2 error) and (2) against the
one-node-per-lane kernel on the same storage: FP32 state within 1e-6
relative L2 after the test's steps.  Both kernels share the memory layout of
each streaming pattern, so they may alternate within one run."""
import numpy as np
import pytest

from pv2013_gb300 import BoundarySpec, Geometry, Simulation, _capi, cases

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_u(O, case, geom, steps):
    geo = O.geometry(case.triangles, case.spacing, case.grid, case.predicates)
    ref = O.run_case(19, geo, case.tau, {0: (O.BC_VEL_NEGY, 1.0), 2: (O.BC_PRESS_POSY, case.outlet_rho)}, steps,
                     profile=case.inlet_profile(geom), amp=case.amp_table())
    return O.macro(ref.f())


@pytest.mark.parametrize("precision,tol", [("f32", 2e-5), ("f16s", 1e-3), ("bf16s", 3e-2)])
@pytest.mark.parametrize("pattern", ["pull", "aa"])
@pytest.mark.parametrize("run_axis", [1, 2])
def test_pair_kernel_against_fp64_oracle(oracle_mod, precision, tol, pattern, run_axis):
    c = cases.pipe()
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision=precision, pattern=pattern, run_axis=run_axis,
                     nodes_per_lane=2)
    info = sim.info()
    assert info.nodes_per_lane == 2 and info.run_axis == run_axis
    sim.step(400, graph=True)
    _, rho, u = sim.fields()
    rr, ur = oracle_u(oracle_mod, c, geom, 400)
    assert rel_l2(u, ur) < tol, (precision, pattern, rel_l2(u, ur))
    assert abs(rho.sum() / rr.sum() - 1) < 10 * tol


@pytest.mark.parametrize("pattern", ["pull", "aa"])
@pytest.mark.parametrize("seed", [4000, 4005])
def test_pair_kernel_matches_single_kernel_fp32(pattern, seed):
    """Tortuous vessel with a pulsatile inlet: FP32 populations of the paired
    and the one-node-per-lane kernels agree to FP32 rounding."""
    c = cases.vessel(seed)
    geom = c.geometry()
    runs = []
    for npl in (1, 2):
        sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f32", pattern=pattern, nodes_per_lane=npl,
                         staging=1)
        sim.step(120, graph=True)
        runs.append(sim.fields())
    (f1, r1, u1), (f2, r2, u2) = runs
    assert np.isfinite(f2).all()
    assert rel_l2(f2, f1) < 1e-6
    assert rel_l2(u2, u1) < 1e-4


def test_pair_kernel_alternates_with_single_kernel():
    """AA state written by one kernel is read by the other: the layouts agree."""
    c = cases.vessel(4001)
    geom = c.geometry()
    a = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f32", pattern="aa", nodes_per_lane=2)
    b = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f32", pattern="aa", nodes_per_lane=1, staging=1)
    a.step(7)
    b.step(7)
    assert rel_l2(a.fields()[0], b.fields()[0]) < 1e-6


def test_pair_kernel_all_reference_boundaries():
    """PV2013 geometry (its seven predicate lists, every reference boundary
    routine): FP32 paired against FP32 one-node-per-lane."""
    import golden_pv2013 as G
    from pv2013_gb300 import pv2013_predicates
    _, tris, _ = G.load()
    geom = Geometry(tris, 0.1, predicates=pv2013_predicates())
    kinds = {0: _capi.BC_VEL_NEGY, 1: _capi.BC_PRESS_NEGY, 2: _capi.BC_PRESS_POSY, 3: _capi.BC_PRESS_POSX,
             4: _capi.BC_PRESS_POSX, 5: _capi.BC_PRESS_POSX, 6: _capi.BC_PRESS_POSZ}
    specs = [BoundarySpec(0, kinds[0], dir=(0.0, -1.0, 0.0), amp=np.array([0.1]))]
    specs += [BoundarySpec(l, kinds[l], rho=1.01) for l in range(1, 7)]
    steps = 6
    out = {}
    for npl in (1, 2):
        sim = Simulation(geom, 0.66, specs, precision="f32", pattern="pull", nodes_per_lane=npl, staging=1)
        sim.step(steps)
        out[npl] = sim.fields()
    assert rel_l2(out[2][0], out[1][0]) < 1e-6
    assert rel_l2(out[2][2], out[1][2]) < 1e-4


def test_pair_kernel_batch_and_d3q27():
    c1, c2 = cases.pipe(), cases.vessel(4002)
    g1, g2 = c1.geometry(), c2.geometry()
    batch = Simulation([g1, g2], [c1.tau, c2.tau], [c1.boundary_specs(g1), c2.boundary_specs(g2)],
                       precision="f16s", pattern="aa", nodes_per_lane=2)
    s1 = Simulation(g1, c1.tau, c1.boundary_specs(g1), precision="f16s", pattern="aa", nodes_per_lane=2)
    s2 = Simulation(g2, c2.tau, c2.boundary_specs(g2), precision="f16s", pattern="aa", nodes_per_lane=2)
    for s in (batch, s1, s2):
        s.step(30, graph=True)
    off = batch.instance_offsets()
    fb = batch.fields()[0]
    # the instances are independent: a batch member equals its own run
    assert np.array_equal(fb[off[0]:off[1]], s1.fields()[0])
    assert np.array_equal(fb[off[1]:off[2]], s2.fields()[0])

    c = cases.pipe_x()
    geom = Geometry(c.triangles, 1.0, grid=c.grid, predicates=c.predicates[:1])
    specs = [BoundarySpec(0, _capi.BC_VEL_POSX, dir=(1.0, 0.0, 0.0), profile=c.inlet_profile(geom),
                          amp=c.amp_table())]
    res = {}
    for npl in (1, 2):
        sim = Simulation(geom, c.tau, specs, Q=27, precision="f32", pattern="pull", nodes_per_lane=npl, staging=1)
        sim.step(40)
        res[npl] = sim.fields()[0]
    assert rel_l2(res[2], res[1]) < 1e-6


def test_pair_kernel_rejects_fp64():
    c = cases.pipe()
    geom = c.geometry()
    with pytest.raises(_capi.LbmError) as e:
        Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", nodes_per_lane=2)
    assert e.value.status == _capi.ERR_ARG


@pytest.mark.parametrize("pattern", ["pull", "aa"])
def test_autotune_keeps_state_and_results(pattern):
    """The autotuner runs its candidates on a scratch copy: the step count and
    populations are unchanged by it, and the run it tunes agrees with an
    untuned run (FP32 rounding)."""
    c = cases.vessel(4003)
    geom = c.geometry()
    a = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f32", pattern=pattern)
    b = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f32", pattern=pattern)
    a.step(5)
    b.step(5)
    f_before = b.fields()[0]
    res = b.autotune(launches=6)
    # both patterns (an AA state after an even launch converts), one node per
    # lane direct / TMA-staged and two nodes per lane with 8-, 16-, 32-slot
    # pieces, 1-8 warps per block
    assert len(res) == 40 and sum(r[4] for r in res) == 1
    assert {r[5] for r in res} == {"aa", "pull"} and {r[6] for r in res if r[0] == 2} == {8, 16, 32}
    assert all(r[3] > 0 for r in res)
    assert b.info().steps_done == 5
    assert np.array_equal(b.fields()[0], f_before)
    chosen = [r for r in res if r[4]][0]
    info = b.info()
    assert (info.nodes_per_lane, info.warps_per_block) == (chosen[0], chosen[2])
    assert info.pattern == {"pull": _capi.PULL, "aa": _capi.AA}[chosen[5]]
    if chosen[0] == 2:
        assert info.piece_slots == chosen[6]
    a.step(40, graph=True)
    b.step(40, graph=True)
    assert rel_l2(b.fields()[0], a.fields()[0]) < 1e-6


@pytest.mark.parametrize("precision,pattern", [("f16s", "aa"), ("f32", "pull"), ("bf16s", "aa")])
def test_piece_sizes_give_identical_results(precision, pattern):
    """The chunk piece size changes which lanes serve which nodes, not the
    per-node arithmetic: 8-, 16- and 32-slot pieces give the same bits, on a
    pulsatile vessel (walls, inlet and outlet nodes at piece ends) and on a
    two-member batch."""
    c = cases.vessel(4004)
    geom = c.geometry()
    out = {}
    for piece in (8, 16, 32):
        sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision=precision, pattern=pattern,
                         nodes_per_lane=2, piece_slots=piece)
        info = sim.info()
        assert info.piece_slots == piece and info.nodes_per_lane == 2
        sim.step(57, graph=True)
        out[piece] = sim.fields()[0]
    assert np.isfinite(out[16]).all()
    assert np.array_equal(out[8], out[16]) and np.array_equal(out[32], out[16])
    # chunk counts: shorter pieces, more chunks
    c1, c2 = cases.pipe(), cases.vessel(4005)
    g1, g2 = c1.geometry(), c2.geometry()
    runs = {}
    for piece in (8, 32):
        b = Simulation([g1, g2], [c1.tau, c2.tau], [c1.boundary_specs(g1), c2.boundary_specs(g2)],
                       precision=precision, pattern=pattern, piece_slots=piece)
        runs[piece] = (b.info().n_chunks, b)
        b.step(31, graph=True)
    assert runs[8][0] > runs[32][0]
    assert np.array_equal(runs[8][1].fields()[0], runs[32][1].fields()[0])


def test_piece_size_default_and_arguments():
    c = cases.pipe()
    geom = c.geometry()
    assert Simulation(geom, c.tau, c.boundary_specs(geom), precision="f16s", pattern="aa").info().piece_slots == 8
    assert Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64").info().piece_slots == 0
    for bad in (4, 12, 64, -1):
        with pytest.raises(_capi.LbmError) as e:
            Simulation(geom, c.tau, c.boundary_specs(geom), precision="f16s", pattern="aa", piece_slots=bad)
        assert e.value.status == _capi.ERR_ARG


@pytest.mark.parametrize("make", [cases.pipe, lambda: cases.vessel(4006), lambda: cases.vessel(4008)])
def test_automatic_run_axis_has_fewer_chunks(make):
    """run_axis = 0 takes the axis whose chunk table is shorter: the count
    comes straight from the voxel flags and must agree with the tables the
    lattice builder makes for either axis."""
    c = make()
    geom = c.geometry()
    specs = c.boundary_specs(geom)
    n = {}
    for ra in (1, 2):
        n[ra] = Simulation(geom, c.tau, specs, precision="f16s", pattern="aa", run_axis=ra).info().n_chunks
    auto = Simulation(geom, c.tau, specs, precision="f16s", pattern="aa").info()
    assert auto.n_chunks == min(n.values())
    assert n[auto.run_axis] == auto.n_chunks


@pytest.mark.parametrize("precision", ["f16s", "f32", "f64"])
def test_pattern_conversion_keeps_results(precision):
    """lbm_sim_set_pattern: an AA state after an even launch is the pull
    state with its planes permuted, so a run that switches AA -> pull (after
    an odd number of steps) or pull -> AA (any time) continues with the same
    bits as a run that never switched."""
    c = cases.vessel(4002)
    geom = c.geometry()
    specs = c.boundary_specs(geom)
    npl = 1 if precision == "f64" else 2
    mk = lambda pat: Simulation(geom, c.tau, specs, precision=precision, pattern=pat, nodes_per_lane=npl, staging=1)
    ref = mk("aa")
    ref.step(48, graph=True)
    a = mk("aa")
    a.step(7)
    a.set_pattern("pull")
    assert a.info().pattern == _capi.PULL
    a.step(22, graph=True)
    a.set_pattern("aa")              # pull -> AA with the step count odd
    assert a.info().pattern == _capi.AA
    a.step(19, graph=True)
    assert np.array_equal(a.fields()[0], ref.fields()[0])
    b = mk("aa")
    b.step(6)
    with pytest.raises(_capi.LbmError) as e:
        b.set_pattern("pull")        # after an odd launch: not a pull state
    assert e.value.status == _capi.ERR_STATE


@pytest.mark.parametrize("corrections", [0, _capi.FIX_BB_ALL_DIRS | _capi.FIX_LIST_NODES])
@pytest.mark.parametrize("precision", ["f16s", "bf16s"])
def test_pair_kernel_16bit_aa_matches_single_kernel(precision, corrections):
    """16-bit AA storage: the paired kernel's bounce-back, initial values and
    ghost-slot handling against the one-node-per-lane kernel on a tortuous
    vessel with walls, inlet and outlet nodes.  Both compute in FP32 (in a
    different order) and round to the same storage, so the deviations f - w
    agree to a few storage roundings; a wrong bounced or initial value at the
    boundary nodes moves their relative L2 difference above 1e-2."""
    c = cases.vessel(4003)
    geom = c.geometry()
    out = {}
    for npl in (1, 2):
        sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision=precision, pattern="aa",
                         nodes_per_lane=npl, staging=1, corrections=corrections)
        sim.step(9)
        out[npl] = sim.fields()
    from pv2013_gb300.engine import LatticeModel
    w = LatticeModel(19).w
    d1, d2 = out[1][0] - w, out[2][0] - w
    assert np.isfinite(d2).all()
    assert rel_l2(d2, d1) < (2e-3 if precision == "f16s" else 2e-2)
    assert rel_l2(out[2][2], out[1][2]) < (2e-3 if precision == "f16s" else 2e-2)
