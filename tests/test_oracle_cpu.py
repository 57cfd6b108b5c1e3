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


def _ref_case(O, case, steps, tmp, wss=False):
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
                          tau=case.tau, outlet_rho=case.outlet_rho, steps=steps, profile=prof, amp=amp, workdir=tmp,
                          wss=wss)
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


def test_face_zou_he_restates_every_reference_routine(oracle_mod):
    """The generic face form of the oracle equals each reference Zou-He routine
    on random populations (to rounding), except the f10 term of outlets 3-5
    (Simulation.cpp:1124-1129), which changes f8 and f9 only."""
    import numpy as np
    O = oracle_mod
    rng = np.random.default_rng(7)
    w19 = np.array([2 / 36] * 6 + [1 / 36] * 12 + [12 / 36])
    w27 = np.array([8 / 27] + [2 / 27] * 6 + [1 / 54] * 12 + [1 / 216] * 8)
    cases = [(19, O.BC_VEL_NEGY, O.BC_FACE_VEL, O.FACE_NEGY, (0.01, -0.05, 0.02), 1.0),
             (19, O.BC_PRESS_NEGY, O.BC_FACE_PRESS, O.FACE_NEGY, (0, 0, 0), 1.01),
             (19, O.BC_PRESS_POSY, O.BC_FACE_PRESS, O.FACE_POSY, (0, 0, 0), 1.01),
             (19, O.BC_PRESS_POSZ, O.BC_FACE_PRESS, O.FACE_POSZ, (0, 0, 0), 0.99),
             (27, O.BC_VEL_POSX, O.BC_FACE_VEL, O.FACE_POSX, (0.04, 0.01, -0.02), 1.0)]
    for Q, ref_kind, face_kind, face, v, rho in cases:
        for _ in range(20):
            f = (w19 if Q == 19 else w27) * (1 + 0.05 * rng.standard_normal(Q))
            a = O.zou_he(Q, ref_kind, f, v, rho)
            b = O.zou_he(Q, face_kind, f, v, rho, face)
            assert np.abs(a - b).max() < 1e-15, (Q, ref_kind)
    f = w19 * (1 + 0.05 * rng.standard_normal(19))
    a = O.zou_he(19, O.BC_PRESS_POSX, f, rho=1.0)
    b = O.zou_he(19, O.BC_FACE_PRESS, f, rho=1.0, face=O.FACE_POSX)
    diff = np.flatnonzero(np.abs(a - b) > 1e-15)
    assert list(diff) == [8, 9]
    # the difference is the f10 - f16 term of Nxz, entering f8 with - and f9 with +
    d = 0.5 * (f[10] - f[16])
    assert abs((a[8] - b[8]) + d) < 1e-15 and abs((a[9] - b[9]) - d) < 1e-15


def _transform(O, Q, role, dims, perm, flip):
    """Role grid and direction map of an axis permutation + reflection:
    new axis a holds old axis perm[a], reversed when flip[a]."""
    r = role.reshape(dims)
    r = np.transpose(r, perm)
    for a in range(3):
        if flip[a]:
            r = np.flip(r, axis=a)
    C = np.array(O_dirs(Q))
    newc = C[:, list(perm)] * np.where(flip, -1, 1)
    dmap = np.array([int(np.flatnonzero((C == newc[q]).all(1))[0]) for q in range(Q)])
    return np.ascontiguousarray(r).reshape(-1), r.shape, dmap


def O_dirs(Q):
    from pv2013_gb300 import LatticeModel
    L = LatticeModel(Q)
    return [L.GetDirection(q) for q in range(Q)]


def _run(O, Q, role, dims, bcs, faces, vel, tau, steps):
    kinds = np.zeros(64, dtype=np.int32)
    rho = np.ones(64)
    for l, (k, r) in bcs.items():
        kinds[l], rho[l] = k, r
    sim = O.OracleSim(Q, dims, role, kinds, rho, tau)
    for l, fc in faces.items():
        sim.set_face(l, fc)
    n = sim.list_size(0)
    sim.set_velocity(0, np.tile(np.asarray(vel, dtype=np.float64), n))
    sim.step(steps)
    return sim.f()


@pytest.mark.parametrize("Q", [19, 27])
def test_face_kinds_are_covariant_under_axis_maps(oracle_mod, Q):
    """The face kinds on a mirrored / axis-swapped lattice reproduce the
    reference routines on the original one (to rounding): the derived
    orientations are the reference's routines with the axes relabelled.
    D3Q19 maps keep +x fixed, because the reference's bounce-back skips
    direction 0 (Simulation.cpp:1361), which no other map preserves."""
    O = oracle_mod
    if Q == 19:
        c = cases.pipe(radius=8.0, length=40.0, segments=32, ny=48, nxz=20)
        geo = O.geometry(c.triangles, 1.0, c.grid, c.predicates)
        base = {0: (O.BC_VEL_NEGY, 1.0), 2: (O.BC_PRESS_POSY, 1.0)}
        vel = (0.0, -0.04, 0.0)
        # inlet unknowns -y, outlet unknowns +y under each map
        maps = [((0, 1, 2), (False, True, False)), ((0, 2, 1), (False, False, False)),
                ((0, 2, 1), (False, False, True))]
    else:
        c = cases.pipe_x(radius=8.0, length=40.0, segments=32, nx=48, nyz=20)
        geo = O.geometry(c.triangles, 1.0, c.grid, c.predicates)
        base = {0: (O.BC_VEL_POSX, 1.0), 2: (O.BC_FACE_PRESS, 1.0)}
        vel = (0.04, 0.0, 0.0)
        maps = [((1, 0, 2), (False, False, False)), ((2, 1, 0), (True, False, False)),
                ((0, 1, 2), (True, False, False))]
    dims = tuple(geo["dims"])
    steps = 30
    base_faces = {2: O.FACE_NEGX} if Q == 27 else {}
    f0 = _run(O, Q, geo["role"], dims, base, base_faces, vel, 0.8, steps)
    C = np.array(O_dirs(Q))
    grid0 = np.full(int(np.prod(dims)), -1)
    grid0[geo["role"] >= 0] = np.arange(int((geo["role"] >= 0).sum()))
    for perm, flip in maps:
        role1, dims1, dmap = _transform(O, Q, geo["role"], dims, perm, flip)
        # faces of the two lists in the new frame: image of the old unknown direction
        def face_of(axis, sign):
            v = np.zeros(3, dtype=int)
            v[axis] = sign
            w = v[list(perm)] * np.where(flip, -1, 1)
            a = int(np.flatnonzero(w)[0])
            return 2 * a + (1 if w[a] < 0 else 0)
        if Q == 19:
            faces = {0: face_of(1, -1), 2: face_of(1, 1)}
        else:
            faces = {0: face_of(0, 1), 2: face_of(0, -1)}
        bcs = {0: (O.BC_FACE_VEL, 1.0), 2: (O.BC_FACE_PRESS, 1.0)}
        vel1 = np.asarray(vel)[list(perm)] * np.where(flip, -1, 1)
        f1 = _run(O, Q, role1, dims1, bcs, faces, vel1, 0.8, steps)
        # node correspondence through the grid map
        g1 = np.transpose(grid0.reshape(dims), perm)
        for a in range(3):
            if flip[a]:
                g1 = np.flip(g1, axis=a)
        ids0 = g1.reshape(-1)[role1 >= 0]          # old node id of every new node, new order
        assert np.abs(f1[:, dmap] - f0[ids0]).max() < 1e-14, (perm, flip)


@ref19
@pytest.mark.parametrize("make,steps", [(cases.pipe, 20), (lambda: cases.vessel(4006, h=3.0), 12)])
def test_oracle_wss_equals_reference(oracle_mod, make, steps):
    """Wall shear stress: the restatement equals the reference's
    ComputeVelocityGradientAtWall + ComputeWallShearStress
    (Simulation.cpp:1374-1421) bit for bit, on the wall nodes in the
    reference's order, after the reference's own steps."""
    O = oracle_mod
    c = make()
    if hasattr(c.inlet, "period") and c.inlet.period > 0:
        c.inlet.period = 7
    with tempfile.TemporaryDirectory() as tmp:
        geo, prof, amp, ref = _ref_case(O, c, steps, tmp, wss=True)
    sim = O.run_case(19, geo, c.tau, {0: (O.BC_VEL_NEGY, 1.0), 2: (O.BC_PRESS_POSY, c.outlet_rho)}, steps,
                     profile=prof, amp=amp)
    assert np.array_equal(ref["wall_nodes"], geo["lists"]["wall"])
    w = sim.wss()
    assert len(w) == len(ref["wss"]) and np.any(w > 0)
    assert np.array_equal(w, ref["wss"])


@ref19
def test_binary_stl_reader_equals_reference(oracle_mod, tmp_path):
    """lbm_stl_read_binary returns the reference's Reader::readSTLBinary
    triangles bit for bit (float vertices; the file's normal renormalised in
    float, GeometryReader.cpp:119-176), on facets with unnormalised normals."""
    from pv2013_gb300 import Reader
    rng = np.random.default_rng(11)
    tris = cases.vessel(4001, h=3.0).triangles.astype(np.float32)
    tris[:, 9:12] *= rng.uniform(0.2, 7.0, size=(len(tris), 1)).astype(np.float32)
    p = tmp_path / "b.stl"
    with open(p, "wb") as fh:
        fh.write(b"solid binary" + b"\0" * 68)
        fh.write(np.uint32(len(tris)).tobytes())
        for t in tris:
            fh.write(t[9:12].tobytes() + t[0:9].tobytes() + b"\0\0")
    mine = Reader.readSTLBinary(str(p))
    ref = oracle_mod.reference_read_stl_binary(str(p), workdir=str(tmp_path))
    assert mine.shape == ref.shape == (len(tris), 12)
    assert np.array_equal(mine, ref)
