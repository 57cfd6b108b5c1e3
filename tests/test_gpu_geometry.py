"""GPU voxelizer + boundary classifier against the oracle and the PV2013
golden lists (bit-exact: same node-type field, same ordered lists)."""
import numpy as np
import pytest

import golden_pv2013 as G
from pv2013_gb300 import Geometry, cases, pv2013_predicates

pytestmark = pytest.mark.gpu


def _check_case(O, case):
    geom = case.geometry()
    geo = O.geometry(case.triangles, case.spacing, case.grid, case.predicates)
    assert np.array_equal(geom.flags(), geo["flags"])
    assert np.array_equal(geom.boundaryPoints, geo["bidx"])
    assert np.array_equal(geom.WallboundaryPoints, geo["lists"]["wall"])
    for lid in {p.list_id for p in case.predicates}:
        assert np.array_equal(geom.list(lid), geo["lists"].get(lid, np.zeros(0, np.int64))), lid
    assert geom.info.n_fluid == int(geo["flags"].sum())
    return geom


def test_pipe_matches_oracle(oracle_mod):
    _check_case(oracle_mod, cases.pipe())


def test_pipe_tight_grid_matches_oracle(oracle_mod):
    """Tight grid: points on the bbox faces get the reference's 0.01 ray nudge."""
    O = oracle_mod
    c = cases.pipe()
    geom = Geometry(c.triangles, 1.0)
    bb, dims = O.tight_grid(c.triangles, 1.0)
    assert geom.GeomSize == list(dims)
    assert np.array_equal(np.array(geom.boundingbox), bb)
    assert np.array_equal(geom.flags(), O.voxelize(c.triangles, bb, 1.0, dims, binned=False))


@pytest.mark.parametrize("seed", [4000, 4001, 4002, 4005])
def test_vessels_match_oracle(oracle_mod, seed):
    _check_case(oracle_mod, cases.vessel(seed))


def test_bifurcation_matches_oracle(oracle_mod):
    _check_case(oracle_mod, cases.bifurcation(nx=128, ny=256, nz=128, r_parent=12, r_child=9, h=1.3))


def test_full_bifurcation_matches_oracle(oracle_mod):
    """The bifurcation workload at its full size (256 x 512 x 256 grid)."""
    _check_case(oracle_mod, cases.bifurcation())


_TREE = {}


def _tree_oracle(O):
    """The benchmark's tree and its oracle geometry, computed once per session."""
    if "geo" not in _TREE:
        c = cases.vascular_tree(h=2.2)
        _TREE["case"] = c
        _TREE["geo"] = O.geometry(c.triangles, c.spacing, c.grid, c.predicates)
    return _TREE["case"], _TREE["geo"]


def test_full_vascular_tree_matches_oracle(oracle_mod):
    """The benchmark's vascular tree (512 x 1024 x 512 grid, 2.07 M triangles,
    32 outlet lists): node-type field, boundary points and every list bit-exact
    with the oracle (about a minute of OpenMP work on the host)."""
    c, geo = _tree_oracle(oracle_mod)
    geom = c.geometry()
    assert np.array_equal(geom.flags(), geo["flags"])
    assert np.array_equal(geom.boundaryPoints, geo["bidx"])
    assert np.array_equal(geom.WallboundaryPoints, geo["lists"]["wall"])
    for lid in {p.list_id for p in c.predicates}:
        assert np.array_equal(geom.list(lid), geo["lists"].get(lid, np.zeros(0, np.int64))), lid
    assert geom.info.n_fluid == int(geo["flags"].sum())


def test_full_vascular_tree_fp64_steps_bit_exact(oracle_mod):
    """FP64 on the benchmark's tree itself (10.27 M fluid nodes, its inlet
    with the parabolic profile and waveform, its outlets and walls): three AA
    steps (even, odd, even launch), every population of every node bit-exact
    with the oracle."""
    from pv2013_gb300 import Simulation
    O = oracle_mod
    c, geo = _tree_oracle(O)
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern="aa")
    sim.step(3)
    f = sim.fields(rho=False, u=False)[0]
    del sim
    ref = O.run_case(19, geo, c.tau, {0: (O.BC_VEL_NEGY, 1.0), 2: (O.BC_PRESS_POSY, c.outlet_rho)}, 3,
                     profile=c.inlet_profile(geom), amp=c.amp_table())
    assert np.array_equal(f, ref.f())


def test_fine_spacing_matches_oracle(oracle_mod):
    """Spacing 0.37 (grid coordinates not representable exactly)."""
    O = oracle_mod
    c = cases.vessel(4003, h=1.0)
    geom = Geometry(c.triangles, 0.37)
    bb, dims = O.tight_grid(c.triangles, 0.37)
    assert np.array_equal(geom.flags(), O.voxelize(c.triangles, bb, 0.37, dims))


def test_pv2013_golden_lists():
    """Full PV2013 pass at spacing 0.1 (421 x 351 x 341 points, 4988 triangles):
    the eight boundary lists equal the reference's VTK files byte for byte."""
    meta, tris, lists = G.load()
    geom = Geometry(tris, 0.1, predicates=pv2013_predicates())
    assert geom.GeomSize == meta["dims"]
    assert np.array_equal(np.array(geom.boundingbox), np.array(meta["bbox"]))
    bb = np.array(meta["bbox"])
    for lid, key in enumerate(G.KEYS[:7]):
        got = geom.list(lid)
        assert np.array_equal(got, lists[key]), key
        assert G.sha256(G.vtk_text(got, meta["dims"], bb, 0.1)) == meta["files"][key]["sha256"], key
    wall = geom.WallboundaryPoints
    assert np.array_equal(wall, lists["wall"])
    assert G.sha256(G.vtk_text(wall, meta["dims"], bb, 0.1)) == meta["files"]["wall"]["sha256"]
    assert geom.info.voxelize_ms > 0


def test_empty_and_degenerate_inputs(oracle_mod):
    """No triangles on an explicit grid -> all NotFluid; a vertical (degenerate
    in xy) triangle alone -> no crossings, as in the reference."""
    g = Geometry(np.zeros((0, 12)), 1.0, grid=((0, 0, 0), (4, 5, 6)))
    assert g.flags().sum() == 0 and g.info.n_boundary == 0
    t = np.array([[1.0, 1.0, 0.0, 1.0, 3.0, 0.0, 1.0, 2.0, 4.0, 1.0, 0.0, 0.0]])
    g = Geometry(t, 1.0, grid=((0, 0, 0), (4, 5, 6)))
    bb, dims = oracle_mod.explicit_grid(((0, 0, 0), (4, 5, 6)), 1.0)
    assert np.array_equal(g.flags(), oracle_mod.voxelize(t, bb, 1.0, dims, binned=False))
