"""Zou-He on any face (LBM_BC_VELOCITY / LBM_BC_PRESSURE) against the oracle.

The face kinds restate the reference's routines with the axes relabelled
(checked on the CPU: tests/test_oracle_cpu.py, single-node identities and
covariance under axis maps).  Here the GPU runs them in FP64 and must equal
the oracle bit for bit, for inlets and outlets on x and y faces, D3Q19 and
D3Q27 (the reference has no D3Q27 pressure routine; the face form with the
D3Q27 coefficients is the restatement), both streaming patterns; reduced
storage is checked with the tolerances of the step tests."""
import numpy as np
import pytest

from pv2013_gb300 import BoundarySpec, Geometry, PlanePredicate, Simulation, _capi, cases

pytestmark = pytest.mark.gpu


def _swap_lists(preds):
    """The pipe's predicates with inlet and outlet exchanged: the inlet at the
    bottom (unknowns +y), the outlet at the top (unknowns -y)."""
    out = []
    for p in preds:
        out.append(PlanePredicate(2 if p.list_id == 0 else 0, p.axis, p.plane, p.tol, p.lo, p.hi))
    return out


def _oracle(O, Q, c, preds, bcs, steps, profile, amp, inlet_dir):
    geo = O.geometry(c.triangles, c.spacing, c.grid, preds)
    return O.run_case(Q, geo, c.tau, bcs, steps, profile=profile, amp=amp, inlet_dir=inlet_dir)


@pytest.mark.parametrize("pattern", ["pull", "aa"])
def test_face_kinds_fp64_bit_exact_d3q19(oracle_mod, pattern):
    O = oracle_mod
    c = cases.pipe()
    preds = _swap_lists(c.predicates)
    geom = Geometry(c.triangles, 1.0, grid=c.grid, predicates=preds)
    prof = c.inlet_profile(geom)
    amp = c.amp_table() * np.ones(7)          # a short periodic table
    specs = [BoundarySpec(0, _capi.BC_VELOCITY, dir=(0.0, 1.0, 0.0), profile=prof, amp=amp, face=_capi.FACE_POSY),
             BoundarySpec(2, _capi.BC_PRESSURE, rho=1.0, face=_capi.FACE_NEGY)]
    sim = Simulation(geom, c.tau, specs, precision="f64", pattern=pattern)
    sim.step(23)
    ref = _oracle(O, 19, c, preds, {0: (O.BC_FACE_VEL, 1.0, O.FACE_POSY), 2: (O.BC_FACE_PRESS, 1.0, O.FACE_NEGY)},
                  23, prof, amp, (0.0, 1.0, 0.0))
    assert np.array_equal(sim.fields()[0], ref.f())


@pytest.mark.parametrize("pattern", ["pull", "aa"])
def test_face_kinds_fp64_bit_exact_d3q27(oracle_mod, pattern):
    """D3Q27 pipe along x: the reference's +x velocity inlet and the restated
    pressure outlet (unknowns -x)."""
    O = oracle_mod
    c = cases.pipe_x()
    geom = Geometry(c.triangles, 1.0, grid=c.grid, predicates=c.predicates)
    prof = c.inlet_profile(geom)
    specs = [BoundarySpec(0, _capi.BC_VEL_POSX, dir=(1.0, 0.0, 0.0), profile=prof, amp=c.amp_table()),
             BoundarySpec(2, _capi.BC_PRESSURE, rho=1.0, face=_capi.FACE_NEGX)]
    sim = Simulation(geom, c.tau, specs, Q=27, precision="f64", pattern=pattern)
    sim.step(17)
    ref = _oracle(O, 27, c, c.predicates, {0: (O.BC_VEL_POSX, 1.0), 2: (O.BC_FACE_PRESS, 1.0, O.FACE_NEGX)}, 17,
                  prof, c.amp_table(), (1.0, 0.0, 0.0))
    assert np.array_equal(sim.fields()[0], ref.f())


@pytest.mark.parametrize("precision,tol", [("f32", 2e-5), ("f16s", 1e-3), ("bf16s", 3e-2)])
def test_face_kinds_reduced_precision_d3q27(oracle_mod, precision, tol):
    O = oracle_mod
    c = cases.pipe_x()
    geom = Geometry(c.triangles, 1.0, grid=c.grid, predicates=c.predicates)
    prof = c.inlet_profile(geom)
    specs = [BoundarySpec(0, _capi.BC_VELOCITY, dir=(1.0, 0.0, 0.0), profile=prof, amp=c.amp_table(),
                          face=_capi.FACE_POSX),
             BoundarySpec(2, _capi.BC_PRESSURE, rho=1.0, face=_capi.FACE_NEGX)]
    sim = Simulation(geom, c.tau, specs, Q=27, precision=precision, pattern="aa")
    sim.step(300, graph=True)
    _, rho, u = sim.fields()
    ref = _oracle(O, 27, c, c.predicates, {0: (O.BC_FACE_VEL, 1.0, O.FACE_POSX), 2: (O.BC_FACE_PRESS, 1.0, O.FACE_NEGX)},
                  300, prof, c.amp_table(), (1.0, 0.0, 0.0))
    rr, ur = O.macro(ref.f(), Q=27)
    err = float(np.linalg.norm(u - ur) / np.linalg.norm(ur))
    assert err < tol, (precision, err)


def test_face_kind_arguments_checked():
    c = cases.pipe()
    geom = c.geometry()
    bad = [BoundarySpec(0, _capi.BC_VELOCITY, face=6)]
    with pytest.raises(_capi.LbmError) as e:
        Simulation(geom, c.tau, bad, precision="f64")
    assert e.value.status == _capi.ERR_ARG
    with pytest.raises(_capi.LbmError):
        Simulation(geom, c.tau, [BoundarySpec(0, _capi.BC_VEL_NEGY)], Q=27, precision="f64")
