"""lbm_sim_fields_noalloc against lbm_sim_fields, through the C ABI.

The no-allocation entry point runs the same snapshot launch as
lbm_sim_fields but writes into the library's fixed device array; its rho and
u must equal lbm_sim_fields' bit for bit (the step tests' tolerance for FP64
state; both calls run the same kernel on the same state).  Checked on two
calls in a row on one handle, then on a second handle (the shared array
holds the first handle's values when the second call starts), and the size
limit is checked to fail cleanly."""
import ctypes as C

import numpy as np
import pytest

from pv2013_gb300 import Simulation, _capi, cases

pytestmark = pytest.mark.gpu

LIMIT = 1 << 19


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _fields_pair(lib, sim):
    n = sim.info().n_nodes
    r0, u0 = np.empty(n), np.empty((n, 3))
    assert lib.lbm_sim_fields(sim._h, _ptr(r0), _ptr(u0), None, n, None) == 0, _capi.last_error()
    r1, u1 = np.full(n, np.nan), np.full((n, 3), np.nan)
    assert lib.lbm_sim_fields_noalloc(sim._h, _ptr(r1), _ptr(u1), n, None) == 0, _capi.last_error()
    return (r0, u0), (r1, u1)


def _check_same(a, b):
    (r0, u0), (r1, u1) = a, b
    assert np.array_equal(r0, r1)
    assert np.array_equal(u0, u1)
    assert np.isfinite(r1).all() and np.isfinite(u1).all()


def test_noalloc_fields_equal_allocating_fields():
    lib = _capi.load()
    c = cases.pipe()
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f64", pattern="pull")
    assert sim.info().n_nodes <= LIMIT
    sim.step(5)
    _check_same(*_fields_pair(lib, sim))       # first call (sets the array up)
    sim.step(3)
    _check_same(*_fields_pair(lib, sim))       # second call in a row, new state

    # another handle, other storage and pattern: the array still holds the pipe's values
    v = cases.vessel(4001)
    gv = v.geometry()
    sv = Simulation(gv, v.tau, v.boundary_specs(gv), precision="f16s", pattern="aa")
    sv.step(4)
    _check_same(*_fields_pair(lib, sv))
    sv.step(1)
    _check_same(*_fields_pair(lib, sv))


def test_noalloc_fields_leave_free_device_memory_unchanged():
    """The promise itself: after a warm-up call, further calls change the
    device's free memory by nothing (cudaMemGetInfo before and after)."""
    import torch
    lib = _capi.load()
    c = cases.pipe()
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f32", pattern="aa")
    sim.step(2)
    n = sim.info().n_nodes
    r, u = np.empty(n), np.empty((n, 3))
    assert lib.lbm_sim_fields_noalloc(sim._h, _ptr(r), _ptr(u), n, None) == 0, _capi.last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        sim.step(1)
        assert lib.lbm_sim_fields_noalloc(sim._h, _ptr(r), _ptr(u), n, None) == 0, _capi.last_error()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0
    assert np.isfinite(r).all()


def test_noalloc_fields_reject_oversized_lattice():
    lib = _capi.load()
    c = cases.pipe(radius=40.0, length=200.0, segments=96, ny=208, nxz=88)
    geom = c.geometry()
    sim = Simulation(geom, c.tau, c.boundary_specs(geom), precision="f16s", pattern="aa")
    n = sim.info().n_nodes
    assert n > LIMIT
    r, u = np.empty(n), np.empty((n, 3))
    assert lib.lbm_sim_fields_noalloc(sim._h, _ptr(r), _ptr(u), n, None) == _capi.ERR_ARG
    assert "exceed" in _capi.last_error()
    # a too-small host capacity is rejected as well
    c2 = cases.pipe()
    g2 = c2.geometry()
    s2 = Simulation(g2, c2.tau, c2.boundary_specs(g2), precision="f64", pattern="pull")
    m = s2.info().n_nodes
    assert lib.lbm_sim_fields_noalloc(s2._h, _ptr(r), _ptr(u), m - 1, None) == _capi.ERR_ARG
