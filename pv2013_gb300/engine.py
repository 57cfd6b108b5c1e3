"""Python host API over the C ABI (include/lbm_gb300.h).

Names follow the reference's classes: ``Reader`` (GeometryReader.cpp),
``LatticeModel`` (LatticeModel.cpp), ``Geometry`` (ComplexGeometry.cpp),
``Simulation`` (Simulation.cpp, with SubDomain's lattice construction folded
in).  Everything heavy runs in liblbm_gb300.so on the GPU; this module only
marshals arguments and results.
"""
import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _capi
from ._capi import check, load


def _tri_array(ptr, n):
    """Copies a library-owned lbm_tri[n] into an (n, 12) float64 array and frees it."""
    lib = load()
    try:
        if n == 0:
            return np.zeros((0, 12))
        buf = (C.c_double * (12 * n)).from_address(C.addressof(ptr.contents))
        return np.frombuffer(buf, dtype=np.float64).reshape(n, 12).copy()
    finally:
        lib.lbm_free(C.cast(ptr, C.c_void_p))


def _as_tri_ptr(tris):
    tris = np.ascontiguousarray(tris, dtype=np.float64).reshape(-1, 12)
    return tris, tris.ctypes.data_as(C.POINTER(_capi.Tri))


class Reader:
    """STL input/output (GeometryReader.cpp:33-176)."""

    @staticmethod
    def readSTLASCII(path):
        lib = load()
        p = C.POINTER(_capi.Tri)()
        n = C.c_size_t()
        check(lib.lbm_stl_read_ascii(str(path).encode(), C.byref(p), C.byref(n)))
        return _tri_array(p, n.value)

    @staticmethod
    def readSTLASCIIDevice(path, stream=None):
        """readSTLASCII with the parsing on the GPU; returns (triangles,
        on_device) -- on_device False when the file needed the host grammar
        (the triangles are the same either way)."""
        lib = load()
        p = C.POINTER(_capi.Tri)()
        n = C.c_size_t()
        on = C.c_int32()
        check(lib.lbm_stl_read_ascii_device(str(path).encode(), C.c_void_p(stream) if stream else None, C.byref(p),
                                            C.byref(n), C.byref(on)))
        return _tri_array(p, n.value), bool(on.value)

    @staticmethod
    def readSTLBinary(path):
        lib = load()
        p = C.POINTER(_capi.Tri)()
        n = C.c_size_t()
        check(lib.lbm_stl_read_binary(str(path).encode(), C.byref(p), C.byref(n)))
        return _tri_array(p, n.value)

    @staticmethod
    def writeSTLASCII(path, tris, name="lbm_gb300"):
        tris, ptr = _as_tri_ptr(tris)
        check(load().lbm_stl_write_ascii(str(path).encode(), ptr, len(tris), name.encode()))


class LatticeModel:
    """Velocity sets of LatticeModel.cpp: D3Q19 (:51-151, rest population 18)
    and D3Q27 (:208-334, rest population 0)."""

    def __init__(self, Q=19):
        if Q == 19:
            self.c = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [1, 1, 0],
                               [1, -1, 0], [1, 0, 1], [1, 0, -1], [-1, 1, 0], [-1, -1, 0], [-1, 0, 1], [-1, 0, -1],
                               [0, 1, 1], [0, 1, -1], [0, -1, 1], [0, -1, -1], [0, 0, 0]])
            self.w = np.array([2.0 / 36.0] * 6 + [1.0 / 36.0] * 12 + [12.0 / 36.0])
            self.opp = np.array([1, 0, 3, 2, 5, 4, 11, 10, 13, 12, 7, 6, 9, 8, 17, 16, 15, 14, 18])
        elif Q == 27:
            self.c = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                               [1, 1, 0], [1, -1, 0], [-1, 1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1],
                               [-1, 0, -1], [0, 1, 1], [0, 1, -1], [0, -1, 1], [0, -1, -1], [1, 1, 1],
                               [-1, -1, -1], [1, 1, -1], [-1, -1, 1], [1, -1, 1], [-1, 1, -1], [1, -1, -1],
                               [-1, 1, 1]])
            self.w = np.array([8.0 / 27.0] + [2.0 / 27.0] * 6 + [1.0 / 54.0] * 12 + [1.0 / 216.0] * 8)
            self.opp = np.array([0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15, 20, 19, 22, 21,
                                 24, 23, 26, 25])
        else:
            raise ValueError("Q must be 19 or 27")
        self.Q = Q

    def GetWeight(self, d):
        return float(self.w[d])

    def GetDirection(self, d):
        return [int(v) for v in self.c[d]]

    def OppositeDirection(self, d):
        return int(self.opp[d])

    def Get_c_square(self, d=0):
        return 1.0 / 3.0

    def Get_nDirections(self):
        return self.Q


@dataclass
class PlanePredicate:
    """|p[axis] - plane| <= tol and lo < p[other] < hi (getInOutBP form).

    ``plane`` may be a float or a decimal string; strings are split into a
    double-double so long double constants of the reference keep their value.
    """
    list_id: int
    axis: int
    plane: object
    tol: float = 1e-2
    lo: Sequence[float] = (math.nan, math.nan, math.nan)
    hi: Sequence[float] = (math.nan, math.nan, math.nan)

    def to_c(self):
        p = _capi.Predicate()
        p.list_id = self.list_id
        p.axis = self.axis
        if isinstance(self.plane, str):
            from decimal import Decimal, getcontext
            getcontext().prec = 60
            d = Decimal(self.plane)
            hi = float(d)
            lo = float(d - Decimal(hi))
        else:
            hi, lo = float(self.plane), 0.0
        p.plane_hi, p.plane_lo, p.tol = hi, lo, self.tol
        for a in range(3):
            p.lo[a] = self.lo[a]
            p.hi[a] = self.hi[a]
        return p


def pv2013_predicates():
    """The reference's seven hard-coded boundary predicates (ComplexGeometry.cpp:587-633)."""
    lib = load()
    arr = (_capi.Predicate * 7)()
    n = C.c_size_t()
    check(lib.lbm_predicates_pv2013(arr, 7, C.byref(n)))
    return [arr[i] for i in range(n.value)]


class Geometry:
    """GPU voxelization + boundary classification of a triangle surface.

    Mirrors Geometry(FileName, velSet, spacing, mdepth) (ComplexGeometry.cpp:7-32):
    ``triangles`` is an (n, 12) array or an ASCII STL path; ``grid`` is
    (min_xyz, dims_xyz) for an explicit grid, else the tight grid of the
    reference; ``predicates`` select the inlet/outlet lists.
    """

    def __init__(self, triangles, spacing, grid=None, predicates=(), stream=None):
        lib = load()
        if isinstance(triangles, (str, bytes)) or hasattr(triangles, "__fspath__"):
            triangles = Reader.readSTLASCII(triangles)
        self.triangles, tptr = _as_tri_ptr(triangles)
        self.spacing = float(spacing)
        g = None
        if grid is not None:
            g = _capi.Grid()
            for a in range(3):
                g.min[a] = float(grid[0][a])
                g.dims[a] = int(grid[1][a])
        preds = [p.to_c() if isinstance(p, PlanePredicate) else p for p in predicates]
        parr = (_capi.Predicate * max(len(preds), 1))(*preds)
        h = C.c_void_p()
        check(lib.lbm_geometry_create(tptr, len(self.triangles), self.spacing, C.byref(g) if g else None, parr,
                                      len(preds), C.c_void_p(stream) if stream else None, C.byref(h)))
        self._h = h
        info = _capi.GeometryInfo()
        check(lib.lbm_geometry_info_get(h, C.byref(info)))
        self.info = info
        self.GeomSize = [info.dims[0], info.dims[1], info.dims[2]]
        self.boundingbox = [info.bbox[i] for i in range(6)]

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            load().lbm_geometry_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def flags(self):
        """Node-type field, 1 = Fluid, 0 = NotFluid, shape (Nx, Ny, Nz)."""
        out = np.empty(self.info.n_points, dtype=np.uint8)
        check(load().lbm_geometry_flags(self._h, out.ctypes.data_as(C.c_void_p), out.size))
        return out.reshape(self.GeomSize)

    def list(self, list_id):
        """x-major grid indices of a list (LIST_BOUNDARY, LIST_WALL or a predicate list id)."""
        lib = load()
        n = C.c_size_t()
        check(lib.lbm_geometry_list(self._h, list_id, None, 0, C.byref(n)))
        out = np.empty(n.value, dtype=np.int64)
        if n.value:
            check(lib.lbm_geometry_list(self._h, list_id, out.ctypes.data_as(C.c_void_p), out.size, C.byref(n)))
        return out

    def coords(self, idx):
        """Point coordinates min + (i,j,k)*spacing of x-major indices (generatePointsInBoundingBox)."""
        Nx, Ny, Nz = self.GeomSize
        idx = np.asarray(idx, dtype=np.int64)
        i, j, k = idx // (Ny * Nz), (idx // Nz) % Ny, idx % Nz
        bb = self.boundingbox
        return np.stack([bb[0] + i * self.spacing, bb[2] + j * self.spacing, bb[4] + k * self.spacing], axis=-1)

    # reference member names
    @property
    def boundaryPoints(self):
        return self.list(_capi.LIST_BOUNDARY)

    @property
    def WallboundaryPoints(self):
        return self.list(_capi.LIST_WALL)

    @property
    def InletboundaryPoints(self):
        return self.list(0)

    def OutletboundaryPoints(self, k):
        return self.list(k)


@dataclass
class BoundarySpec:
    """Boundary condition of one predicate list (lbm_list_bc)."""
    list_id: int
    kind: int
    rho: float = 1.0
    dir: Sequence[float] = (0.0, -1.0, 0.0)
    profile: Optional[np.ndarray] = None
    amp: Optional[np.ndarray] = None
    face: int = 0                       # lbm_face, for BC_VELOCITY / BC_PRESSURE
    _keep: list = field(default_factory=list, repr=False)

    def to_c(self):
        b = _capi.ListBC()
        b.list_id, b.kind, b.rho = self.list_id, self.kind, float(self.rho)
        b.face = int(self.face)
        for a in range(3):
            b.dir[a] = float(self.dir[a])
        if self.profile is not None:
            p = np.ascontiguousarray(self.profile, dtype=np.float64)
            self._keep.append(p)
            b.profile, b.profile_len = p.ctypes.data_as(C.POINTER(C.c_double)), p.size
        if self.amp is not None:
            a = np.ascontiguousarray(self.amp, dtype=np.float64)
            self._keep.append(a)
            b.amp, b.amp_len = a.ctypes.data_as(C.POINTER(C.c_double)), a.size
        return b


PRECISIONS = {"f64": _capi.F64, "f32": _capi.F32, "f16s": _capi.F16S, "bf16s": _capi.BF16S}
PATTERNS = {"pull": _capi.PULL, "aa": _capi.AA, "auto": _capi.AUTO}


def _params(Q, precision, pattern, tau, bcs, warps_per_block, run_axis=0, staging=0, nodes_per_lane=0,
            corrections=0, piece_slots=0):
    cb = [b.to_c() for b in bcs]
    arr = (_capi.ListBC * max(len(cb), 1))(*cb)
    p = _capi.SimParams()
    p.Q = Q
    p.precision = PRECISIONS[precision] if isinstance(precision, str) else precision
    p.pattern = PATTERNS[pattern] if isinstance(pattern, str) else pattern
    p.tau = float(tau)
    p.bcs = C.cast(arr, C.POINTER(_capi.ListBC))
    p.nbcs = len(cb)
    p.warps_per_block = int(warps_per_block)
    p.run_axis = int(run_axis)
    p.staging = int(staging)
    p.nodes_per_lane = int(nodes_per_lane)
    p.corrections = int(corrections)
    p.piece_slots = int(piece_slots)
    return p, arr


class Simulation:
    """Device lattice + time stepping (SubDomain + Simulation of the reference).

    ``geometry`` may be a Geometry or a list of them (batched ensemble, then
    ``tau`` and ``bcs`` may be per-instance lists).  The keyword arguments are
    the fields of ``lbm_sim_params``: ``precision`` (f64, f32, f16s, bf16s),
    ``pattern`` (pull, aa), ``nodes_per_lane`` (0 = 2 for FP32/16-bit
    storage, 1 for FP64), ``piece_slots`` (8, 16, 32; 0 = 8),
    ``warps_per_block``, ``run_axis`` (0 = the axis with fewer chunks),
    ``staging`` (one node per lane: 0 TMA ring, 1 direct loads) and
    ``corrections`` (``_capi.FIX_*`` bits; 0 = the reference's behaviour).
    """

    def __init__(self, geometry, tau, bcs=(), Q=19, precision="f64", pattern="pull", warps_per_block=0, run_axis=0,
                 staging=0, stream=None, nodes_per_lane=0, corrections=0, piece_slots=0):
        lib = load()
        self._stream = C.c_void_p(stream) if stream else None
        h = C.c_void_p()
        if isinstance(geometry, (list, tuple)):
            n = len(geometry)
            taus = tau if isinstance(tau, (list, tuple, np.ndarray)) else [tau] * n
            bcl = bcs if (len(bcs) and isinstance(bcs[0], (list, tuple))) else [bcs] * n
            keep = []
            params = (_capi.SimParams * n)()
            for i in range(n):
                p, arr = _params(Q, precision, pattern, taus[i], bcl[i], warps_per_block, run_axis, staging, nodes_per_lane,
                                 corrections, piece_slots)
                keep.append((arr, bcl[i]))
                params[i] = p
            geoms = (C.c_void_p * n)(*[g.handle for g in geometry])
            check(lib.lbm_batch_create(geoms, params, n, self._stream, C.byref(h)))
            self.geometries = list(geometry)
        else:
            p, arr = _params(Q, precision, pattern, tau, bcs, warps_per_block, run_axis, staging, nodes_per_lane,
                             corrections, piece_slots)
            check(lib.lbm_sim_create(geometry.handle, C.byref(p), self._stream, C.byref(h)))
            self.geometries = [geometry]
        self._h = h
        self.Q = Q

    def close(self):
        if getattr(self, "_h", None):
            load().lbm_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        i = _capi.SimInfo()
        check(load().lbm_sim_info_get(self._h, C.byref(i)))
        return i

    def step(self, n=1, graph=False, monitor=False):
        flags = (_capi.STEP_GRAPH if graph else 0) | (_capi.STEP_MONITOR if monitor else 0)
        check(load().lbm_sim_step(self._h, int(n), flags, self._stream))

    def prepare_graph(self, n):
        """Captures the CUDA graph that step(n, graph=True) from the current state replays."""
        check(load().lbm_sim_prepare_graph(self._h, int(n), self._stream))

    # reference spelling: Simulation::Iterate runs the time loop
    def Iterate(self, n):
        self.step(n)

    def fields(self, f=True, rho=True, u=True, out=None):
        """FP64 host copies of f (N, Q), rho (N,), u (N, 3) of the current post-boundary state.
        ``out`` = (f, rho, u) caller-owned C-contiguous float64 arrays of those shapes (any may be None), e.g.
        views of pinned host memory, written in place instead of new arrays."""
        n = self.info().n_nodes
        if out is not None:
            fa, ra, ua = out
            for a, shape in ((fa, (n, self.Q)), (ra, (n,)), (ua, (n, 3))):
                if a is not None and (a.dtype != np.float64 or a.shape != shape or not a.flags.c_contiguous):
                    raise ValueError(f"fields: out array must be C-contiguous float64 of shape {shape}")
        else:
            fa = np.empty((n, self.Q)) if f else None
            ra = np.empty(n) if rho else None
            ua = np.empty((n, 3)) if u else None
        ptr = lambda a: a.ctypes.data_as(C.c_void_p) if a is not None else None  # noqa: E731
        check(load().lbm_sim_fields(self._h, ptr(ra), ptr(ua), ptr(fa), n, self._stream))
        return fa, ra, ua

    def nodes(self):
        n = self.info().n_nodes
        out = np.empty(n, dtype=np.int64)
        check(load().lbm_sim_nodes(self._h, out.ctypes.data_as(C.c_void_p), n))
        return out

    def instance_offsets(self):
        k = self.info().n_instances
        out = np.empty(k + 1, dtype=np.int64)
        check(load().lbm_sim_instance_offsets(self._h, out.ctypes.data_as(C.c_void_p), k + 1))
        return out

    def monitors(self):
        m = _capi.Monitors()
        check(load().lbm_sim_monitors(self._h, C.byref(m), self._stream))
        return {"step": m.step, "mass": m.mass, "inlet_flux": m.inlet_flux, "outlet_flux": m.outlet_flux,
                "max_speed": m.max_speed, "nonfinite": bool(m.nonfinite)}

    def autotune(self, launches=20):
        """Times the step-kernel variants (kernel, staging, block size, piece
        size, streaming pattern) on scratch copies of the state and keeps the
        fastest; returns [(nodes_per_lane, staging, warps_per_block,
        ms_per_launch, chosen, pattern, piece_slots)]."""
        ents = (_capi.TuneEntry * 128)()
        n = C.c_size_t()
        check(load().lbm_sim_autotune(self._h, int(launches), self._stream, ents, 128, C.byref(n)))
        return [(e.nodes_per_lane, e.staging, e.warps_per_block, e.ms_per_launch, bool(e.chosen),
                 {_capi.PULL: "pull", _capi.AA: "aa"}[e.pattern], e.piece_slots) for e in ents[:min(n.value, 128)]]

    def set_pattern(self, pattern):
        """Converts the state to another streaming pattern ("pull" or "aa")."""
        check(load().lbm_sim_set_pattern(self._h, {"pull": _capi.PULL, "aa": _capi.AA}[pattern], self._stream))

    def set_divergence_tolerance(self, tol):
        check(load().lbm_sim_set_divergence_tolerance(self._h, float(tol)))

    def set_wait_limit(self, polls):
        """Poll limit of the TMA-staged kernel's bounded waits (0 = default)."""
        check(load().lbm_sim_set_wait_limit(self._h, int(polls)))

    def test_stall(self, enable):
        """Failure-test hook: the TMA-staged kernel's waits on each warp's first stage run out."""
        check(load().lbm_sim_test_stall(self._h, 1 if enable else 0))

    def poison_ghosts(self):
        """Self-check hook: NaN in every population slot of no fluid node (results must not change)."""
        check(load().lbm_sim_poison_ghosts(self._h, self._stream))

    def wall_shear_stress(self):
        """Wall shear stress at every wall node, wall-list order (ComputeWallShearStress)."""
        lib = load()
        n = C.c_size_t()
        check(lib.lbm_sim_wall_shear_stress(self._h, None, 0, C.byref(n), self._stream))
        out = np.empty(n.value)
        check(lib.lbm_sim_wall_shear_stress(self._h, out.ctypes.data_as(C.c_void_p), out.size, C.byref(n),
                                            self._stream))
        return out

    def checkpoint(self, path):
        """Writes the current populations and step count to a file."""
        check(load().lbm_sim_checkpoint(self._h, str(path).encode(), self._stream))

    def restart(self, path):
        """Loads a checkpoint written by a simulation of the same lattice and parameters."""
        check(load().lbm_sim_restart(self._h, str(path).encode(), self._stream))

    # the reference's names (Simulation.cpp:1374-1421)
    def ComputeWallShearStress(self):
        return self.wall_shear_stress()


class Snapshot:
    """Asynchronous snapshot of a simulation (rho, u and/or wall shear stress):
    capture() enqueues the device work and the copy to pinned host memory and
    returns; wait() / data() / write_*_vtu() wait for the copy."""

    def __init__(self, sim, fields=True, wss=True):
        what = (_capi.SNAP_FIELDS if fields else 0) | (_capi.SNAP_WSS if wss else 0)
        h = C.c_void_p()
        check(load().lbm_snapshot_create(sim._h, what, C.byref(h)))
        self._h, self._sim = h, sim

    def capture(self):
        check(load().lbm_snapshot_capture(self._h, self._sim._stream))

    def wait(self):
        check(load().lbm_snapshot_wait(self._h))

    def data(self):
        """(rho, u, wss, step) copies of the last capture (None for fields not captured)."""
        r, u, w = C.POINTER(C.c_double)(), C.POINTER(C.c_double)(), C.POINTER(C.c_double)()
        n, nw, step = C.c_size_t(), C.c_size_t(), C.c_int64()
        check(load().lbm_snapshot_data(self._h, C.byref(r), C.byref(u), C.byref(w), C.byref(n), C.byref(nw),
                                       C.byref(step)))
        take = lambda p, k: np.ctypeslib.as_array(p, shape=(k,)).copy() if p else None  # noqa: E731
        rho = take(r, n.value)
        vel = take(u, 3 * n.value)
        return rho, None if vel is None else vel.reshape(-1, 3), take(w, nw.value), step.value

    def write_fields_vtu(self, path, instance=0):
        check(load().lbm_snapshot_write_fields_vtu(self._h, str(path).encode(), int(instance)))

    def write_wss_vtu(self, path, instance=0):
        check(load().lbm_snapshot_write_wss_vtu(self._h, str(path).encode(), int(instance)))

    def close(self):
        if getattr(self, "_h", None):
            load().lbm_snapshot_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_vtu(path, points, arrays):
    """Point-data .vtu file: points (n, 3); arrays: {name: (n,) or (n, k) float64}."""
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    keep, specs = [], []
    for name, a in arrays.items():
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        v = _capi.VtuArray()
        v.name = name.encode()
        v.components = 1 if a.ndim == 1 else a.shape[1]
        v.data = a.ctypes.data_as(C.POINTER(C.c_double))
        specs.append(v)
    arr = (_capi.VtuArray * max(len(specs), 1))(*specs)
    check(load().lbm_vtu_write(str(path).encode(), len(pts), pts.ctypes.data_as(C.c_void_p), len(specs),
                               C.cast(arr, C.c_void_p)))


def synth_cylinder(radius, length, segments, axis, center):
    lib = load()
    p = C.POINTER(_capi.Tri)()
    n = C.c_size_t()
    c = (C.c_double * 3)(*center)
    check(lib.lbm_synth_cylinder(radius, length, segments, axis, c, C.byref(p), C.byref(n)))
    return _tri_array(p, n.value)


def synth_capsules(segments, lo, hi, h, seed):
    """segments: (n, 10) rows ax,ay,az,bx,by,bz,r,cut_axis,cut_pos,cut_sign."""
    lib = load()
    seg = np.ascontiguousarray(segments, dtype=np.float64).reshape(-1, 10)
    p = C.POINTER(_capi.Tri)()
    n = C.c_size_t()
    lo_ = (C.c_double * 3)(*lo)
    hi_ = (C.c_double * 3)(*hi)
    check(lib.lbm_synth_capsules(seg.ctypes.data_as(C.POINTER(C.c_double)), len(seg), lo_, hi_, float(h),
                                 int(seed), C.byref(p), C.byref(n)))
    return _tri_array(p, n.value)
