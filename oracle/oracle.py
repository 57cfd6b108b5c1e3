"""Python access to the CPU checker.  TEST INFRASTRUCTURE ONLY.

Two checkers live under oracle/:
  * liblbm_oracle.so (oracle/lbm_oracle.cpp): an FP64 restatement of the PV2013
    reference's voxelizer, classifier and time step; fast (OpenMP, SoA);
  * pv2013_ref (oracle/ref): the reference's own C++ sources compiled with a
    single-rank MPI stand-in and driven by a harness; slow (the reference's
    O(points x triangles) voxelizer and pointer-based step).
Only the test suite, the smoke check and the benchmark's CPU-baseline leg use
this module; the engine never imports it.
"""
import ctypes as C
import math
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liblbm_oracle.so")
REF_BIN = {19: os.path.join(HERE, "_ref", "pv2013_ref"), 27: os.path.join(HERE, "_ref", "pv2013_ref27")}

# boundary kinds shared with the engine's lbm_bc_kind numbering
BC_NONE, BC_VEL_NEGY, BC_PRESS_NEGY, BC_PRESS_POSY, BC_PRESS_POSX, BC_PRESS_POSZ, BC_VEL_POSX = range(7)
BC_FACE_VEL, BC_FACE_PRESS = 7, 8
# face of the generic kinds: unknown populations along +x, -x, +y, -y, +z, -z
FACE_POSX, FACE_NEGX, FACE_POSY, FACE_NEGY, FACE_POSZ, FACE_NEGZ = range(6)

_lib = None


class OrcPredicate(C.Structure):
    _fields_ = [("axis", C.c_int), ("plane", C.c_char * 40), ("tol", C.c_double), ("lo", C.c_double * 3),
                ("hi", C.c_double * 3)]


def build():
    """Builds the restatement library (and the reference binaries when their sources are available)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    # the reference binaries: staged from the reference checkout (Makefile's
    # REF_DIR, overridable with PV2013_REF_DIR) or from an earlier staging;
    # where neither exists only the restatement is built
    r = subprocess.run(["make", "-s", "-C", HERE, "ref"], capture_output=True, text=True)
    staged = os.path.exists(os.path.join(HERE, "_ref", "src", ".staged"))
    if r.returncode != 0 and staged:
        raise RuntimeError("building the reference checker failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_read_stl_ascii.restype = C.c_int64
        L.orc_read_stl_ascii.argtypes = [C.c_char_p, C.POINTER(C.POINTER(C.c_double))]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_bbox.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_double]
        L.orc_voxelize.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_double, C.c_void_p, C.c_int, C.c_void_p]
        L.orc_voxelize_cols.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_double, C.c_void_p, C.c_int,
                                        C.c_void_p, C.c_void_p]
        L.orc_boundary_points.restype = C.c_int64
        L.orc_boundary_points.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
        L.orc_classify.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_double,
                                   C.POINTER(OrcPredicate), C.c_int, C.c_void_p]
        L.orc_sim_create.restype = C.c_void_p
        L.orc_sim_create.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_double]
        L.orc_sim_destroy.argtypes = [C.c_void_p]
        L.orc_sim_nodes.restype = C.c_int64
        L.orc_sim_nodes.argtypes = [C.c_void_p]
        L.orc_sim_list_size.restype = C.c_int64
        L.orc_sim_list_size.argtypes = [C.c_void_p, C.c_int]
        L.orc_sim_zero_hits.restype = C.c_int64
        L.orc_sim_zero_hits.argtypes = [C.c_void_p]
        L.orc_sim_set_velocity.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_sim_set_face.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.orc_sim_set_corrections.argtypes = [C.c_void_p, C.c_int]
        L.orc_sim_wss.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_sim_wall_count.restype = C.c_int64
        L.orc_sim_wall_count.argtypes = [C.c_void_p]
        L.orc_zou_he.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_double]
        L.orc_sim_step.argtypes = [C.c_void_p, C.c_int]
        L.orc_sim_get.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_sim_set_f.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_num_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def read_stl_ascii(path):
    L = lib()
    ptr = C.POINTER(C.c_double)()
    n = L.orc_read_stl_ascii(str(path).encode(), C.byref(ptr))
    if n < 0:
        raise OSError(f"cannot open {path}")
    out = np.ctypeslib.as_array(ptr, shape=(max(n, 1) * 12,))[: n * 12].reshape(n, 12).copy()
    L.orc_free(C.cast(ptr, C.c_void_p))
    return out


def tight_grid(tris, spacing):
    """(bbox[6], dims[3]) of GetBoundingbox (ComplexGeometry.cpp:40-73)."""
    tris = np.ascontiguousarray(tris, dtype=np.float64)
    bb = np.zeros(6)
    dims = np.zeros(3, dtype=np.int32)
    lib().orc_bbox(_p(tris), len(tris), _p(bb), _p(dims), float(spacing))
    return bb, dims


def explicit_grid(grid, spacing):
    mn, dims = grid
    bb = np.array([mn[0], mn[0] + (dims[0] - 1) * spacing, mn[1], mn[1] + (dims[1] - 1) * spacing,
                   mn[2], mn[2] + (dims[2] - 1) * spacing], dtype=np.float64)
    return bb, np.array(dims, dtype=np.int32)


def voxelize(tris, bbox, spacing, dims, binned=True):
    tris = np.ascontiguousarray(tris, dtype=np.float64)
    bbox = np.ascontiguousarray(bbox, dtype=np.float64)
    dims = np.ascontiguousarray(dims, dtype=np.int32)
    flags = np.zeros(int(np.prod(dims.astype(np.int64))), dtype=np.uint8)
    lib().orc_voxelize(_p(tris), len(tris), _p(bbox), float(spacing), _p(dims), 1 if binned else 0, _p(flags))
    return flags.reshape(tuple(dims))


def voxelize_columns(tris, bbox, spacing, dims, i0, i1, j0, j1):
    """Voxelizes only the columns i in [i0, i1), j in [j0, j1) of the full grid
    (same rays as the full pass); returns the (i1-i0, j1-j0, Nz) block."""
    tris = np.ascontiguousarray(tris, dtype=np.float64)
    bbox = np.ascontiguousarray(bbox, dtype=np.float64)
    dims = np.ascontiguousarray(dims, dtype=np.int32)
    flags = np.zeros(int(np.prod(dims.astype(np.int64))), dtype=np.uint8)
    cols = np.array([i0, i1, j0, j1], dtype=np.int32)
    lib().orc_voxelize_cols(_p(tris), len(tris), _p(bbox), float(spacing), _p(dims), 1, _p(cols), _p(flags))
    return flags.reshape(tuple(dims))[i0:i1, j0:j1, :].copy()


def boundary_points(flags):
    dims = np.array(flags.shape, dtype=np.int32)
    f = np.ascontiguousarray(flags, dtype=np.uint8)
    n = lib().orc_boundary_points(_p(f), _p(dims), None, 0)
    out = np.zeros(max(n, 1), dtype=np.int64)
    lib().orc_boundary_points(_p(f), _p(dims), _p(out), n)
    return out[:n]


def classify(bidx, dims, bbox, spacing, predicates):
    """predicates: list of (axis, plane_text, tol, lo[3], hi[3]) -> uint64 mask per boundary point."""
    out = np.zeros(len(bidx), dtype=np.uint64)
    for b in range(0, len(predicates), 32):
        m = _classify32(bidx, dims, bbox, spacing, predicates[b:b + 32])
        out |= m.astype(np.uint64) << np.uint64(b)
    return out


def _classify32(bidx, dims, bbox, spacing, predicates):
    arr = (OrcPredicate * max(len(predicates), 1))()
    for i, (axis, plane, tol, lo, hi) in enumerate(predicates):
        arr[i].axis = axis
        arr[i].plane = str(plane).encode()
        arr[i].tol = tol
        for a in range(3):
            arr[i].lo[a] = lo[a]
            arr[i].hi[a] = hi[a]
    bidx = np.ascontiguousarray(bidx, dtype=np.int64)
    mask = np.zeros(len(bidx), dtype=np.uint32)
    lib().orc_classify(_p(bidx), len(bidx), _p(np.asarray(dims, dtype=np.int32)), _p(np.asarray(bbox, np.float64)),
                       float(spacing), arr, len(predicates), _p(mask))
    return mask


def predicate_tuples(preds):
    """Engine PlanePredicate objects -> (list_id, (axis, plane, tol, lo, hi)) for the oracle."""
    out = []
    for p in preds:
        plane = p.plane if isinstance(p.plane, str) else repr(float(p.plane))
        out.append((p.list_id, (p.axis, plane, p.tol, tuple(p.lo), tuple(p.hi))))
    return out


def lists_from_masks(bidx, list_mask):
    """list_mask: per boundary point, bitmask over list ids -> dict list_id -> ordered indices, plus wall."""
    out = {}
    for l in range(64):
        sel = ((list_mask >> np.uint64(l)) & np.uint64(1)).astype(bool)
        if sel.any():
            out[l] = bidx[sel]
    out["wall"] = bidx[list_mask == 0]
    return out


def geometry(tris, spacing, grid, preds):
    """Full reference geometry pass: flags, boundary points, per-list indices, role grid."""
    bb, dims = explicit_grid(grid, spacing) if grid is not None else tight_grid(tris, spacing)
    flags = voxelize(tris, bb, spacing, dims)
    bidx = boundary_points(flags)
    tuples = predicate_tuples(preds)
    pmask = classify(bidx, dims, bb, spacing, [t for _, t in tuples])
    lmask = np.zeros(len(bidx), dtype=np.uint64)
    for k, (lid, _) in enumerate(tuples):
        lmask |= ((pmask >> np.uint64(k)) & np.uint64(1)) << np.uint64(lid)
    lists = lists_from_masks(bidx, lmask)
    role = np.where(flags.reshape(-1) > 0, 0, -1).astype(np.int8)
    first = np.full(len(bidx), 1, dtype=np.int16)
    nz = lmask != 0
    low = (lmask & (~lmask + np.uint64(1)))[nz]
    first[nz] = 2 + np.log2(low.astype(np.float64)).astype(np.int16)
    role[bidx] = first.astype(np.int8)
    return {"bbox": bb, "dims": dims, "flags": flags, "bidx": bidx, "lists": lists, "role": role}


class OracleSim:
    """FP64 restatement of the reference's time loop on a role grid."""

    def __init__(self, Q, dims, role, kinds, list_rho, tau):
        self.L = lib()
        self.Q = Q
        role = np.ascontiguousarray(role, dtype=np.int8)
        kinds = np.ascontiguousarray(kinds, dtype=np.int32)
        rho = np.ascontiguousarray(list_rho, dtype=np.float64)
        self.h = self.L.orc_sim_create(Q, _p(np.asarray(dims, np.int32)), _p(role), len(kinds), _p(kinds), _p(rho),
                                       float(tau))
        self.n = self.L.orc_sim_nodes(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_sim_destroy(self.h)
            self.h = None

    def list_size(self, l):
        return self.L.orc_sim_list_size(self.h, l)

    def set_velocity(self, l, uvw):
        uvw = np.ascontiguousarray(uvw, dtype=np.float64)
        self.L.orc_sim_set_velocity(self.h, l, _p(uvw))

    def set_corrections(self, corr):
        self.L.orc_sim_set_corrections(self.h, int(corr))

    def set_face(self, l, face):
        self.L.orc_sim_set_face(self.h, int(l), int(face))

    def step(self, n=1):
        self.L.orc_sim_step(self.h, int(n))

    def zero_hits(self):
        return self.L.orc_sim_zero_hits(self.h)

    def wss(self):
        """Wall shear stress per wall node (wall-list order) from the last collision's velocities."""
        out = np.empty(self.L.orc_sim_wall_count(self.h))
        self.L.orc_sim_wss(self.h, _p(out))
        return out

    def f(self):
        out = np.empty((self.n, self.Q))
        self.L.orc_sim_get(self.h, _p(out), None, None)
        return out


def zou_he(Q, kind, f, v=(0.0, 0.0, 0.0), rho=1.0, face=0):
    """One node's populations after a Zou-He routine (a copy)."""
    g = np.array(f, dtype=np.float64)
    vv = np.asarray(v, dtype=np.float64)
    lib().orc_zou_he(Q, kind, face, _p(g), _p(vv), float(rho))
    return g


def macro(f, Q=19):
    """rho, u from populations with the reference's grouped sums (Simulation.cpp:32-79)."""
    rho = np.zeros(len(f))
    for q in range(Q):
        rho = rho + f[:, q]
    if Q == 19:
        g = lambda idx: sum_seq(f, idx)  # noqa: E731
        ux = (g([0, 6, 7, 8, 9]) - g([1, 10, 11, 12, 13])) / rho
        uy = (g([2, 6, 10, 14, 15]) - g([3, 7, 11, 16, 17])) / rho
        uz = (g([4, 8, 12, 14, 16]) - g([5, 9, 13, 15, 17])) / rho
    else:
        g = lambda idx: sum_seq(f, idx)  # noqa: E731
        ux = (g([1, 7, 8, 11, 13, 19, 21, 23, 25]) - g([2, 9, 10, 12, 14, 20, 22, 24, 26])) / rho
        uy = (g([3, 7, 9, 15, 16, 19, 21, 24, 26]) - g([4, 8, 10, 17, 18, 20, 22, 23, 25])) / rho
        uz = (g([5, 11, 12, 15, 17, 19, 22, 23, 26]) - g([6, 13, 14, 16, 18, 20, 21, 24, 25])) / rho
    return rho, np.stack([ux, uy, uz], axis=1)


def sum_seq(f, idx):
    s = f[:, idx[0]].copy()
    for i in idx[1:]:
        s = s + f[:, i]
    return s


def run_case(Q, geo, tau, bcs, steps, profile=None, amp=None, inlet_list=0, inlet_dir=(0.0, -1.0, 0.0),
             corrections=0):
    """Runs the restatement on a geometry() result.  bcs: dict list_id -> (kind, rho)
    or (kind, rho, face) for the generic face kinds."""
    nl = 64
    kinds = np.zeros(nl, dtype=np.int32)
    rho = np.ones(nl)
    faces = {}
    for l, spec in bcs.items():
        kinds[l] = spec[0]
        rho[l] = spec[1]
        if len(spec) > 2:
            faces[l] = spec[2]
    sim = OracleSim(Q, geo["dims"], geo["role"], kinds, rho, tau)
    for l, fc in faces.items():
        sim.set_face(l, fc)
    if corrections:
        sim.set_corrections(corrections)
    ninl = sim.list_size(inlet_list)
    prof = np.ones(ninl) if profile is None else np.asarray(profile, dtype=np.float64)
    ampt = np.array([1.0]) if amp is None else np.asarray(amp, dtype=np.float64)
    d = np.asarray(inlet_dir, dtype=np.float64)
    for t in range(steps):
        if kinds[inlet_list] in (BC_VEL_NEGY, BC_VEL_POSX, BC_FACE_VEL):
            s = ampt[t % len(ampt)] * prof
            sim.set_velocity(inlet_list, np.stack([s * d[0], s * d[1], s * d[2]], axis=1).reshape(-1))
        sim.step(1)
    return sim


# ---------------------------------------------------------------------------
# the reference's own code (oracle/_ref)

def ref_available(Q=19):
    return os.path.exists(REF_BIN[Q])


def run_reference(stl_path, spacing, grid=None, preds=(), preset=None, tau=None, outlet_rho=None, steps=0,
                  profile=None, amp=None, inlet_dir=(0.0, -1.0, 0.0), Q=19, vtk_dir=None, workdir=None,
                  flags_path=None, warmup=0, wss=False):
    """Runs the reference harness; returns its outputs as numpy arrays.  With
    flags_path the node-type field of the (explicit) grid is read from that file
    instead of the reference's voxelizer.  With wss the reference's
    ComputeVelocityGradientAtWall + ComputeWallShearStress run after the steps:
    res["wss"] per wall node, res["wall_nodes"] their grid indices
    (Simulation.cpp:1374-1421)."""
    wd = workdir or tempfile.mkdtemp(prefix="pv2013_ref_")
    os.makedirs(wd, exist_ok=True)
    lines = [f"stl {stl_path}", f"spacing {spacing!r}"]
    if flags_path:
        lines.append(f"flags {flags_path}")
    if grid is not None:
        (mx, my, mz), (nx, ny, nz) = grid
        lines.append(f"box {mx!r} {my!r} {mz!r} {nx} {ny} {nz}")
    if preset:
        lines.append(f"preset {preset}")
    for lid, (axis, plane, tol, lo, hi) in preds:
        vals = " ".join("nan" if math.isnan(v) else repr(float(v)) for pair in zip(lo, hi) for v in pair)
        lines.append(f"pred {lid} {axis} {plane} {tol!r} {vals}")
    if vtk_dir:
        lines.append(f"vtk {vtk_dir}")
    if tau is not None:
        lines.append(f"tau {tau!r}")
    if outlet_rho is not None:
        lines.append(f"outlet_rho {outlet_rho!r}")
    lines.append(f"steps {steps}")
    if warmup:
        lines.append(f"warmup {int(warmup)}")
    lines.append("inlet_dir " + " ".join(repr(float(v)) for v in inlet_dir))
    if profile is not None:
        pp = os.path.join(wd, "profile.bin")
        np.asarray(profile, dtype=np.float64).tofile(pp)
        lines.append(f"inlet_profile {pp}")
    if amp is not None:
        ap = os.path.join(wd, "amp.bin")
        np.asarray(amp, dtype=np.float64).tofile(ap)
        lines.append(f"amp_table {ap}")
    if wss:
        lines.append("wss 1")
    out = os.path.join(wd, "ref")
    lines.append(f"out {out}")
    run = os.path.join(wd, "run.txt")
    with open(run, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    subprocess.run([REF_BIN[Q], run], check=True, capture_output=True)
    res = {"flags": np.fromfile(out + ".flags", dtype=np.uint8)}
    meta = open(out + ".meta").read().split()
    res["dims"] = np.array([int(v) for v in meta[:3]], dtype=np.int32)
    res["bbox"] = np.array([float(v) for v in meta[3:9]])
    res["flags"] = res["flags"].reshape(tuple(res["dims"]))
    lst = np.fromfile(out + ".lists", dtype=np.int64)
    counts = lst[:9]
    pos = 9
    names = ["boundary"] + list(range(7)) + ["wall"]
    res["lists"] = {}
    for nm, c in zip(names, counts):
        res["lists"][nm] = lst[pos:pos + c]
        pos += c
    if os.path.exists(out + ".f"):
        res["f"] = np.fromfile(out + ".f", dtype=np.float64).reshape(-1, Q)
        res["nodes"] = np.fromfile(out + ".nodes", dtype=np.int64)
        res["rho"] = np.fromfile(out + ".rho", dtype=np.float64)
        res["u"] = np.fromfile(out + ".u", dtype=np.float64).reshape(-1, 3)
        t = open(out + ".time").read().split()
        res["time"] = {"steps": int(t[0]), "nodes": int(t[1]), "seconds": float(t[2])}
    if os.path.exists(out + ".wss"):
        res["wss"] = np.fromfile(out + ".wss", dtype=np.float64)
        res["wall_nodes"] = np.fromfile(out + ".wallnodes", dtype=np.int64)
    return res


def reference_pulsatile(n, workdir=None):
    """The reference's inlet waveform (pulsatile.h:8-31, selected as in
    Simulation.cpp:875-900) at x = 0.9 s * s / n, s = 0..n-1."""
    wd = workdir or tempfile.mkdtemp(prefix="pv2013_ref_")
    out = os.path.join(wd, "ref")
    run = os.path.join(wd, "run.txt")
    with open(run, "w") as fh:
        fh.write(f"pulsatile {int(n)}\nout {out}\n")
    subprocess.run([REF_BIN[19], run], check=True, capture_output=True)
    return np.fromfile(out + ".pulsatile", dtype=np.float64)


def reference_read_stl_binary(path, workdir=None):
    """Triangles (n, 12) as the reference's Reader::readSTLBinary returns them
    (GeometryReader.cpp:119-176: float vertices, normal renormalised in float)."""
    wd = workdir or tempfile.mkdtemp(prefix="pv2013_ref_")
    out = os.path.join(wd, "ref")
    run = os.path.join(wd, "run.txt")
    with open(run, "w") as fh:
        fh.write(f"stl_binary {path}\nout {out}\n")
    subprocess.run([REF_BIN[19], run], check=True, capture_output=True)
    return np.fromfile(out + ".tris", dtype=np.float64).reshape(-1, 12)
