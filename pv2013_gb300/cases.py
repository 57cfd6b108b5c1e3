"""Seeded synthetic workloads (straight pipe, Y-bifurcation, tortuous vessels,
binary vascular tree) in the form the reference's solver needs: a closed
triangle surface whose inlet and outlet faces are axis-aligned planes, a grid,
plane predicates that pick the inlet/outlet boundary points (the form of
getInOutBP, ComplexGeometry.cpp:579-638) and per-list boundary settings.

Orientation convention (the reference's Zou-He routines are fixed to axes):
vessels run along y; the inlet face is the top (y max) and uses the velocity
routine with unknowns -y (Boundary.cpp:129-148); outlet faces are at the
bottom (y min) and use the pressure routine with unknowns +y
(Simulation.cpp:1029-1083, the reference's outlet list 2).  Lattice units:
spacing 1, grid points at integer coordinates, caps on half-integer planes
so no ray or lattice plane meets a cap.
"""
import math
from dataclasses import dataclass, field
from typing import List

import numpy as np

from . import _capi
from .engine import BoundarySpec, Geometry, PlanePredicate, synth_capsules, synth_cylinder

INLET_LIST = 0
OUTLET_LIST = 2   # the reference's outlet list 2 carries the +y-unknown pressure routine


@dataclass
class Inlet:
    center: tuple          # coordinates of the vessel axis on the two other axes (ascending axis order)
    radius: float
    plane: float           # coordinate of the inlet lattice plane
    u_max: float
    period: int = 0        # pulsation period in steps (0 = steady)
    axis: int = 1          # axis normal to the inlet face


@dataclass
class Case:
    name: str
    triangles: np.ndarray
    grid: tuple            # ((min x,y,z), (Nx,Ny,Nz))
    predicates: List[PlanePredicate]
    inlet: Inlet
    tau: float
    steps: int
    spacing: float = 1.0
    outlet_rho: float = 1.0
    meta: dict = field(default_factory=dict)

    def geometry(self, stream=None):
        return Geometry(self.triangles, self.spacing, grid=self.grid, predicates=self.predicates, stream=stream)

    def inlet_profile(self, geom):
        """Parabolic factor 1 - r^2/R^2 (>= 0) of each inlet-list point, list order."""
        return self.inlet_profile_from_indices(geom.list(INLET_LIST), geom.GeomSize)

    def inlet_profile_from_indices(self, idx, dims):
        Nx, Ny, Nz = (int(v) for v in dims)
        idx = np.asarray(idx, dtype=np.int64)
        ijk = np.stack([idx // (Ny * Nz), (idx // Nz) % Ny, idx % Nz], axis=1).astype(np.float64)
        mn = np.asarray(self.grid[0], dtype=np.float64)
        pts = mn + ijk * self.spacing
        others = [a for a in range(3) if a != self.inlet.axis]
        r2 = (pts[:, others[0]] - self.inlet.center[0]) ** 2 + (pts[:, others[1]] - self.inlet.center[1]) ** 2
        return np.maximum(0.0, 1.0 - r2 / self.inlet.radius ** 2)

    def amp_table(self):
        """Inlet amplitude per step, periodic: u_max (1 + 0.5 sin(2 pi t / T))."""
        if self.inlet.period <= 0:
            return np.array([self.inlet.u_max])
        t = np.arange(self.inlet.period, dtype=np.float64)
        return self.inlet.u_max * (1.0 + 0.5 * np.sin(2.0 * np.pi * t / self.inlet.period))

    def boundary_specs(self, geom):
        return [BoundarySpec(INLET_LIST, _capi.BC_VEL_NEGY, dir=(0.0, -1.0, 0.0), profile=self.inlet_profile(geom),
                             amp=self.amp_table()),
                BoundarySpec(OUTLET_LIST, _capi.BC_PRESS_POSY, rho=self.outlet_rho)]


def _inlet_pred(plane, cx, cz, half):
    return PlanePredicate(INLET_LIST, 1, float(plane), 1e-2, (cx - half, math.nan, cz - half),
                          (cx + half, math.nan, cz + half))


def _outlet_pred(plane, cx, cz, half):
    return PlanePredicate(OUTLET_LIST, 1, float(plane), 1e-2, (cx - half, math.nan, cz - half),
                          (cx + half, math.nan, cz + half))


def pipe(radius=20.0, length=120.0, segments=64, ny=128, nxz=48, tau=0.8, u_max=0.05, steps=2000):
    """Straight cylinder along y (48 x 128 x 48 grid for the defaults)."""
    c = ((nxz - 1) / 2.0, (ny - 1) / 2.0, (nxz - 1) / 2.0)
    tris = synth_cylinder(radius, length, segments, 1, c)
    y_top = c[1] + length / 2.0          # half-integer cap planes
    y_bot = c[1] - length / 2.0
    inlet_plane = math.floor(y_top)
    outlet_plane = math.ceil(y_bot)
    preds = [_inlet_pred(inlet_plane, c[0], c[2], radius + 3), _outlet_pred(outlet_plane, c[0], c[2], radius + 3)]
    return Case("pipe", tris, ((0.0, 0.0, 0.0), (nxz, ny, nxz)), preds,
                Inlet((c[0], c[2]), radius, inlet_plane, u_max), tau, steps,
                meta={"radius": radius, "length": length, "segments": segments})


def pipe_x(radius=12.0, length=80.0, segments=48, nx=88, nyz=32, tau=0.8, u_max=0.04, steps=200):
    """Straight cylinder along x with the inlet on the x-min face: the orientation of
    the reference's D3Q27 velocity routine (unknowns +x, Boundary.cpp:87-123).  The
    x-max face carries an outlet predicate (list 2) for lattices that have one."""
    c = ((nx - 1) / 2.0, (nyz - 1) / 2.0, (nyz - 1) / 2.0)
    tris = synth_cylinder(radius, length, segments, 0, c)
    x_lo, x_hi = c[0] - length / 2.0, c[0] + length / 2.0
    inlet_plane, outlet_plane = math.ceil(x_lo), math.floor(x_hi)
    half = radius + 3
    preds = [PlanePredicate(INLET_LIST, 0, float(inlet_plane), 1e-2, (math.nan, c[1] - half, c[2] - half),
                            (math.nan, c[1] + half, c[2] + half)),
             PlanePredicate(OUTLET_LIST, 0, float(outlet_plane), 1e-2, (math.nan, c[1] - half, c[2] - half),
                            (math.nan, c[1] + half, c[2] + half))]
    return Case("pipe_x", tris, ((0.0, 0.0, 0.0), (nx, nyz, nyz)), preds,
                Inlet((c[1], c[2]), radius, inlet_plane, u_max, 0, axis=0), tau, steps,
                meta={"radius": radius, "length": length})


def bifurcation(nx=256, ny=512, nz=256, r_parent=24.0, r_child=18.0, angle_deg=30.0, h=1.8, seed=0xB1F,
                tau=0.6, u_max=0.04, period=1000, steps=10000):
    """Y-bifurcation: parent along -y from the inlet, daughters at +/-angle in the x-y plane,
    each ending in a straight -y run to its outlet face."""
    cx, cz = nx / 2.0, nz / 2.0
    top = ny - 11.5
    junction = ny * 0.6
    bottom = 10.5
    a = math.radians(angle_deg)
    run = min((nx / 2.0 - r_child - 12) / math.sin(a), (junction - bottom - 60) / math.cos(a))
    seg = [[cx, top + 20, cz, cx, junction, cz, r_parent, 1, top, 1.0]]
    ends = []
    for s in (-1.0, 1.0):
        ex, ey = cx + s * run * math.sin(a), junction - run * math.cos(a)
        seg.append([cx, junction, cz, ex, ey, cz, r_child, -1, 0, 0])
        seg.append([ex, ey, cz, ex, bottom - 20, cz, r_child, 1, bottom, -1.0])
        ends.append(ex)
    tris = synth_capsules(np.array(seg), (0, 0, 0), (nx - 1, ny - 1, nz - 1), h, seed)
    inlet_plane = math.floor(top)
    outlet_plane = math.ceil(bottom)
    preds = [_inlet_pred(inlet_plane, cx, cz, r_parent + 4)]
    preds += [_outlet_pred(outlet_plane, ex, cz, r_child + 4) for ex in ends]
    return Case("bifurcation", tris, ((0.0, 0.0, 0.0), (nx, ny, nz)), preds,
                Inlet((cx, cz), r_parent, inlet_plane, u_max, period), tau, steps,
                meta={"h": h, "seed": seed, "outlets": len(ends)})


def _rotate(v, axis, ang):
    axis = axis / np.linalg.norm(axis)
    return (v * math.cos(ang) + np.cross(axis, v) * math.sin(ang) + axis * np.dot(axis, v) * (1 - math.cos(ang)))


def vascular_tree(nx=512, ny=1024, nz=512, depth=5, r_root=40.0, ratio=0.79, ang=(25.0, 45.0), seed=5,
                  length_factor=7.0, h=1.45, tau=0.6, u_max=0.04, period=1000, steps=20000):
    """Seeded binary tree of tubes growing along -y; every leaf ends in a straight -y run to
    its own outlet face on the bottom plane."""
    rng = np.random.default_rng(seed)
    cx, cz = nx / 2.0, nz / 2.0
    top = ny - 11.5
    bottom = 10.5
    margin = 8.0
    seg = [[cx, top + 30, cz, cx, top - length_factor * r_root, cz, r_root, 1, top, 1.0]]
    leaves = []
    stack = [(np.array([cx, top - length_factor * r_root, cz]), np.array([0.0, -1.0, 0.0]), r_root, 0)]
    while stack:
        p, d, r, lev = stack.pop()
        if lev == depth:
            leaves.append((p, r))
            continue
        rc = r * ratio
        perp = np.cross(d, rng.normal(size=3))
        perp /= np.linalg.norm(perp)
        for side in (1.0, -1.0):
            th = math.radians(rng.uniform(*ang))
            nd = _rotate(d, perp, side * th)
            if nd[1] > -0.35:
                nd = nd + np.array([0.0, -0.6, 0.0])
            nd /= np.linalg.norm(nd)
            L = length_factor * rc
            q = p + L * nd
            for axis, n in ((0, nx), (2, nz)):
                lo, hi = rc + margin, n - 1 - rc - margin
                if q[axis] < lo or q[axis] > hi:
                    nd[axis] = -nd[axis]
                    q = p + L * nd
                    q[axis] = min(max(q[axis], lo), hi)
            q[1] = max(q[1], bottom + 40.0)
            seg.append([*p, *q, rc, -1, 0, 0])
            stack.append((q, nd, rc, lev + 1))
    outlets = []
    for q, r in leaves:
        seg.append([q[0], q[1], q[2], q[0], bottom - 20, q[2], r, 1, bottom, -1.0])
        outlets.append((q[0], q[2], r))
    tris = synth_capsules(np.array(seg), (0, 0, 0), (nx - 1, ny - 1, nz - 1), h, seed)
    inlet_plane = math.floor(top)
    outlet_plane = math.ceil(bottom)
    preds = [_inlet_pred(inlet_plane, cx, cz, r_root + 4)]
    preds += [_outlet_pred(outlet_plane, ox, oz, r + 3) for ox, oz, r in outlets]
    return Case("vascular_tree", tris, ((0.0, 0.0, 0.0), (nx, ny, nz)), preds,
                Inlet((cx, cz), r_root, inlet_plane, u_max, period), tau, steps,
                meta={"h": h, "seed": seed, "outlets": len(outlets), "segments": len(seg)})


def _catmull_rom(pts, n):
    pts = np.asarray(pts, dtype=np.float64)
    ext = np.vstack([pts[0], pts, pts[-1]])
    out = []
    for i in range(1, len(ext) - 2):
        p0, p1, p2, p3 = ext[i - 1], ext[i], ext[i + 1], ext[i + 2]
        for t in np.linspace(0.0, 1.0, n, endpoint=False):
            t2, t3 = t * t, t * t * t
            out.append(0.5 * ((2 * p1) + (-p0 + p2) * t + (2 * p0 - 5 * p1 + 4 * p2 - p3) * t2 +
                              (-p0 + 3 * p1 - 3 * p2 + p3) * t3))
    out.append(pts[-1])
    return np.array(out)


def vessel(seed, h=1.0):
    """One tortuous vessel of the 64-vessel ensemble: a tube along a seeded cubic-spline
    centreline (Catmull-Rom through 4-6 control points) in a box from 32^3 to 128 x 256 x 128."""
    rng = np.random.default_rng(seed)
    nx = int(rng.integers(32, 129))
    nz = int(rng.integers(32, 129))
    ny = int(rng.integers(max(32, nx // 2), 257))
    r = float(rng.uniform(6.0, 24.0))
    r = min(r, (min(nx, nz) - 10) / 2.0 - 1.0)
    # the straight end runs must be longer than the radius so the spherical
    # ends of the inner capsules stay inside the clipped faces
    straight = r + 6.0
    ny = max(ny, int(4 * straight) + 8)
    cx, cz = (nx - 1) / 2.0, (nz - 1) / 2.0
    top, bottom = ny - 3.5, 2.5
    k = int(rng.integers(4, 7))
    ys = np.linspace(top - straight, bottom + straight, k)
    wx, wz = max(0.0, cx - r - 4), max(0.0, cz - r - 4)
    ctrl = [[cx + (rng.uniform(-wx, wx) if 0 < i < k - 1 else 0.0), y,
             cz + (rng.uniform(-wz, wz) if 0 < i < k - 1 else 0.0)] for i, y in enumerate(ys)]
    path = _catmull_rom(ctrl, 6)
    seg = [[cx, top + 10, cz, *path[0], r, 1, top, 1.0]]
    for a, b in zip(path[:-1], path[1:]):
        seg.append([*a, *b, r, -1, 0, 0])
    seg.append([*path[-1], cx, bottom - 10, cz, r, 1, bottom, -1.0])
    tris = synth_capsules(np.array(seg), (0, 0, 0), (nx - 1, ny - 1, nz - 1), h, seed)
    tau = float(rng.uniform(0.55, 1.2))
    amp = float(rng.uniform(0.01, 0.06))
    period = int(rng.integers(500, 2001))
    inlet_plane, outlet_plane = math.floor(top), math.ceil(bottom)
    preds = [_inlet_pred(inlet_plane, cx, cz, r + 3), _outlet_pred(outlet_plane, cx, cz, r + 3)]
    return Case(f"vessel{seed}", tris, ((0.0, 0.0, 0.0), (nx, ny, nz)), preds,
                Inlet((cx, cz), r, inlet_plane, amp, period), tau, 0,
                meta={"seed": seed, "box": (nx, ny, nz), "radius": r})


def ensemble(n=64, first_seed=4000, h=1.0):
    return [vessel(first_seed + i, h) for i in range(n)]
