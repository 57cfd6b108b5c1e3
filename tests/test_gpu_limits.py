"""Argument and size limits, checked before any device work: a call outside
them fails with LBM_ERR_ARG and leaves the handle usable."""
import numpy as np
import pytest

from pv2013_gb300 import Geometry, Simulation, _capi, cases

pytestmark = pytest.mark.gpu


def _arg_error(fn):
    with pytest.raises(_capi.LbmError) as e:
        fn()
    assert e.value.status == _capi.ERR_ARG, e.value


def test_geometry_limits():
    empty = np.zeros((0, 12))
    _arg_error(lambda: Geometry(empty, 1.0, grid=((0, 0, 0), (4, 4, 2049))))    # voxelizer column limit
    _arg_error(lambda: Geometry(empty, 1.0, grid=((0, 0, 0), (0, 4, 4))))       # grid dims >= 1
    _arg_error(lambda: Geometry(empty, 1.0))                                     # tight grid of no triangle
    g = Geometry(empty, 1.0, grid=((0, 0, 0), (4, 4, 2048)))                     # at the limit: fine
    assert g.info.n_fluid == 0


def test_simulation_of_a_lattice_without_fluid():
    g = Geometry(np.zeros((0, 12)), 1.0, grid=((0, 0, 0), (4, 5, 6)))
    _arg_error(lambda: Simulation(g, 0.8, [], precision="f64"))
    _arg_error(lambda: Simulation(g, 0.8, [], precision="f16s", pattern="aa"))


def test_step_count_limits():
    c = cases.pipe()
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f16s", pattern="aa")
    _arg_error(lambda: sim.step(2 ** 32))      # the inlet phase is a 32-bit step count
    _arg_error(lambda: sim.step(-1))
    sim.step(3)
    assert sim.info().steps_done == 3
    _, rho, _ = sim.fields(f=False)
    assert np.isfinite(rho).all()
