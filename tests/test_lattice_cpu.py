"""Lattice tables and single-node boundary routines (unit level).

* The velocity sets satisfy the lattice identities the BGK equilibrium needs
  (weights sum to 1, first and third moments vanish, second moments are
  c_s^2 = 1/3 times the identity, fourth moments are isotropic), the
  opposite map is an involution with c_opp(q) = -c_q, and the rest
  population is 18 (D3Q19) / 0 (D3Q27) as in LatticeModel.cpp:51-151,
  :208-334.
* The three copies of the tables -- the device tables of the kernels
  (device.cuh, printed by a host-only nvcc build), the C++ facade, the Python
  binding -- are the same numbers.
* Zou-He on one node with a known solution: after a velocity routine the
  node's velocity (the reference's grouped sums) is the imposed one, after a
  pressure routine its density is the imposed one, for every reference
  routine without the f10 quirk and for the face routines on every face."""
import itertools
import os
import shutil
import subprocess

import numpy as np
import pytest

from pv2013_gb300.engine import LatticeModel

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _tables(lines):
    out, cur = {}, None
    for ln in lines:
        p = ln.split()
        if p[0] == "Q":
            cur = int(p[1])
            out[cur] = {"meta": [int(v) for v in p[2:]], "rows": []}
        else:
            out[cur]["rows"].append((int(p[0]), int(p[1]), int(p[2]), int(p[3]), float(p[4])))
    return out


@pytest.mark.parametrize("Q", [19, 27])
def test_lattice_identities(Q):
    L = LatticeModel(Q)
    c, w, opp = L.c.astype(np.float64), L.w, L.opp
    assert abs(w.sum() - 1.0) < 1e-15
    assert np.abs(w @ c).max() < 1e-15
    assert np.abs(np.einsum("q,qa,qb->ab", w, c, c) - np.eye(3) / 3.0).max() < 1e-15
    assert np.abs(np.einsum("q,qa,qb,qc->abc", w, c, c, c)).max() < 1e-15
    m4 = np.einsum("q,qa,qb,qc,qd->abcd", w, c, c, c, c)
    for a, b, cc, d in itertools.product(range(3), repeat=4):
        iso = ((a == b) * (cc == d) + (a == cc) * (b == d) + (a == d) * (b == cc)) / 9.0
        assert abs(m4[a, b, cc, d] - iso) < 1e-15
    assert (opp[opp] == np.arange(Q)).all()
    assert (c[opp] == -c).all()
    rest = 18 if Q == 19 else 0
    assert (c[rest] == 0).all() and (np.abs(c).sum(1) > 0).sum() == Q - 1


def test_device_facade_and_python_tables_agree(tmp_path):
    if shutil.which("nvcc") is None or shutil.which("g++") is None:
        pytest.skip("nvcc or g++ not available")
    dev = str(tmp_path / "lattice_tables")
    r = subprocess.run(["nvcc", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "pv2013_gb300", "csrc"), "--expt-relaxed-constexpr",
                        os.path.join(HERE, "lattice_tables.cu"), "-o", dev], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    fac = str(tmp_path / "facade_tables")
    r = subprocess.run(["g++", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(HERE, "facade_tables.cpp"), "-o", fac], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    td = _tables(subprocess.run([dev], capture_output=True, text=True, check=True).stdout.splitlines())
    tf = _tables(subprocess.run([fac], capture_output=True, text=True, check=True).stdout.splitlines())
    for Q in (19, 27):
        L = LatticeModel(Q)
        py = [(int(L.c[q][0]), int(L.c[q][1]), int(L.c[q][2]), int(L.opp[q]), float(L.w[q])) for q in range(Q)]
        assert td[Q]["rows"] == py, Q
        assert tf[Q]["rows"] == py, Q
        rest, no_bb = td[Q]["meta"]
        assert rest == (18 if Q == 19 else 0)
        # the population the reference's wall loop never writes (it starts at
        # direction 1, Simulation.cpp:1361): opp(0) for D3Q19, none for D3Q27
        # (its direction 0 is the rest population)
        assert no_bb == (int(L.opp[0]) if Q == 19 else -1)


def _near_eq(Q, rng, u=(0.01, -0.02, 0.015), rho=1.0):
    L = LatticeModel(Q)
    c, w = L.c.astype(np.float64), L.w
    cu = c @ np.asarray(u)
    feq = w * rho * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * np.dot(u, u))
    return feq * (1 + 0.02 * rng.standard_normal(Q))


def test_zou_he_recovers_the_imposed_velocity_and_density(oracle_mod):
    O = oracle_mod
    rng = np.random.default_rng(11)
    vel_cases = [(19, O.BC_VEL_NEGY, 0, (0.0, -0.04, 0.0)), (27, O.BC_VEL_POSX, 0, (0.05, 0.0, 0.0))]
    vel_cases += [(Q, O.BC_FACE_VEL, face, v) for Q in (19, 27) for face, v in
                  [(O.FACE_POSX, (0.03, 0.0, 0.0)), (O.FACE_NEGX, (-0.03, 0.0, 0.0)),
                   (O.FACE_POSY, (0.0, 0.02, 0.0)), (O.FACE_NEGY, (0.0, -0.02, 0.0)),
                   (O.FACE_POSZ, (0.0, 0.0, 0.04)), (O.FACE_NEGZ, (0.0, 0.0, -0.04))]]
    for Q, kind, face, v in vel_cases:
        for _ in range(10):
            g = O.zou_he(Q, kind, _near_eq(Q, rng), v, 1.0, face)
            _, u = O.macro(g[None, :], Q)
            assert np.abs(u[0] - np.asarray(v)).max() < 1e-14, (Q, kind, face)
    press_cases = [(19, O.BC_PRESS_NEGY, 0), (19, O.BC_PRESS_POSY, 0), (19, O.BC_PRESS_POSZ, 0)]
    press_cases += [(Q, O.BC_FACE_PRESS, face) for Q in (19, 27) for face in range(6)]
    for Q, kind, face in press_cases:
        for rho in (0.99, 1.0, 1.01):
            g = O.zou_he(Q, kind, _near_eq(Q, rng), (0.0, 0.0, 0.0), rho, face)
            r, _ = O.macro(g[None, :], Q)
            assert abs(r[0] - rho) < 1e-14, (Q, kind, face, rho)
