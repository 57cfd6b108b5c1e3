"""The CPU oracle pinned against the reference: the PV2013 golden boundary lists
and the reference's own code compiled from its sources (oracle/_ref)."""
import os
import tempfile

import numpy as np
import pytest

import golden_pv2013 as G
from pv2013_gb300 import Reader, cases


def test_golden_fixture_reproduces_vtk_bytes():
    meta, tris, lists = G.load()
    bb = np.array(meta["bbox"])
    for k in G.KEYS:
        text = G.vtk_text(lists[k], meta["dims"], bb, meta["spacing"])
        assert G.sha256(text) == meta["files"][k]["sha256"], k
        assert len(lists[k]) == meta["files"][k]["points"]


def test_oracle_reproduces_pv2013_golden_lists(oracle_mod):
    O = oracle_mod
    meta, tris, lists = G.load()
    bb, dims = O.tight_grid(tris, 0.1)
    assert list(dims) == meta["dims"]
    assert np.array_equal(bb, np.array(meta["bbox"]))
    flags = O.voxelize(tris, bb, 0.1, dims)
    bidx = O.boundary_points(flags)
    tup = G.oracle_tuples()
    pm = O.classify(bidx, dims, bb, 0.1, [t for _, t in tup])
    for k, (lid, _) in enumerate(tup):
        sel = ((pm >> np.uint64(k)) & np.uint64(1)).astype(bool)
        assert np.array_equal(bidx[sel], lists[G.KEYS[lid]]), G.KEYS[lid]
    assert np.array_equal(bidx[pm == 0], lists["wall"])


def test_oracle_binned_equals_bruteforce(oracle_mod):
    O = oracle_mod
    c = cases.vessel(4002, h=2.0)
    bb, dims = O.explicit_grid(c.grid, 1.0)
    a = O.voxelize(c.triangles, bb, 1.0, dims, binned=True)
    b = O.voxelize(c.triangles, bb, 1.0, dims, binned=False)
    assert a.sum() > 0
    assert np.array_equal(a, b)


def test_oracle_stl_reader_matches_writer(oracle_mod, tmp_path):
    c = cases.pipe()
    p = tmp_path / "pipe.stl"
    Reader.writeSTLASCII(p, c.triangles)
    assert np.array_equal(oracle_mod.read_stl_ascii(p), c.triangles)


ref19 = pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref",
                                                            "pv2013_ref")), reason="reference checker not built")


def _ref_case(O, case, steps, tmp):
    stl = os.path.join(tmp, "case.stl")
    Reader.writeSTLASCII(stl, case.triangles)
    geo = O.geometry(case.triangles, case.spacing, case.grid, case.predicates)
    Nx, Ny, Nz = geo["dims"]
    idx = geo["lists"][0]
    i, k = idx // (Ny * Nz), idx % Nz
    cx, cz = case.inlet.center
    prof = np.maximum(0, 1 - ((i - cx) ** 2 + (k - cz) ** 2) / case.inlet.radius ** 2)
    amp = case.amp_table()
    ref = O.run_reference(stl, case.spacing, grid=case.grid, preds=O.predicate_tuples(case.predicates),
                          tau=case.tau, outlet_rho=case.outlet_rho, steps=steps, profile=prof, amp=amp, workdir=tmp)
    return geo, prof, amp, ref


@ref19
def test_oracle_equals_reference_pipe(oracle_mod):
    O = oracle_mod
    c = cases.pipe()
    with tempfile.TemporaryDirectory() as tmp:
        geo, prof, amp, ref = _ref_case(O, c, 20, tmp)
    assert np.array_equal(ref["flags"], geo["flags"])
    assert np.array_equal(ref["lists"]["boundary"], geo["bidx"])
    assert np.array_equal(ref["lists"][0], geo["lists"][0])
    assert np.array_equal(ref["lists"][2], geo["lists"][2])
    assert np.array_equal(ref["lists"]["wall"], geo["lists"]["wall"])
    sim = O.run_case(19, geo, c.tau, {0: (O.BC_VEL_NEGY, 1.0), 2: (O.BC_PRESS_POSY, c.outlet_rho)}, 20,
                     profile=prof, amp=amp)
    assert sim.zero_hits() == 0
    assert np.array_equal(ref["nodes"], np.flatnonzero(geo["flags"].reshape(-1)))
    assert np.array_equal(sim.f(), ref["f"])     # bit-exact FP64


@ref19
def test_oracle_equals_reference_pulsatile_vessel(oracle_mod):
    """A marching-tetrahedra vessel (tilted walls, many triangles per column)
    with a pulsatile parabolic inlet: geometry and 12 steps bit-exact."""
    O = oracle_mod
    c = cases.vessel(4006, h=3.0)
    c.inlet.period = 7
    with tempfile.TemporaryDirectory() as tmp:
        geo, prof, amp, ref = _ref_case(O, c, 12, tmp)
    assert np.array_equal(ref["flags"], geo["flags"])
    for k in ("boundary", 0, 2, "wall"):
        mine = geo["bidx"] if k == "boundary" else geo["lists"][k]
        assert np.array_equal(ref["lists"][k], mine), k
    sim = O.run_case(19, geo, c.tau, {0: (O.BC_VEL_NEGY, 1.0), 2: (O.BC_PRESS_POSY, c.outlet_rho)}, 12,
                     profile=prof, amp=amp)
    assert np.array_equal(sim.f(), ref["f"])


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref",
                                                    "pv2013_ref27")), reason="reference checker not built")
def test_oracle_equals_reference_d3q27_inlet(oracle_mod):
    """D3Q27 collision (Simulation.cpp:82-152), the D3Q27 x-normal velocity inlet
    (Boundary.cpp:87-123) and bounce-back over all 26 moving directions."""
    O = oracle_mod
    c = cases.pipe_x()
    with tempfile.TemporaryDirectory() as tmp:
        stl = os.path.join(tmp, "x.stl")
        Reader.writeSTLASCII(stl, c.triangles)
        geo = O.geometry(c.triangles, 1.0, c.grid, c.predicates[:1])
        prof = c.inlet_profile_from_indices(geo["lists"][0], geo["dims"])
        ref = O.run_reference(stl, 1.0, grid=c.grid, preds=O.predicate_tuples(c.predicates[:1]), tau=c.tau,
                              steps=8, profile=prof, amp=c.amp_table(), inlet_dir=(1.0, 0.0, 0.0), Q=27, workdir=tmp)
    assert np.array_equal(ref["flags"], geo["flags"])
    sim = O.run_case(27, geo, c.tau, {0: (O.BC_VEL_POSX, 1.0)}, 8, profile=prof, amp=c.amp_table(),
                     inlet_dir=(1.0, 0.0, 0.0))
    assert np.array_equal(sim.f(), ref["f"])
