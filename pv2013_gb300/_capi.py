"""ctypes binding of the C ABI declared in include/lbm_gb300.h.

The shared library is built in-tree (pv2013_gb300/_lib/liblbm_gb300.so) by
``pv2013_gb300.build.build_library``.  Loading fails loudly when it is absent:
there is no fallback implementation.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liblbm_gb300.so")

LBM_OK = 0
ERR_TIMEOUT, ERR_ARG, ERR_STATE = 6, 7, 8
STATUS_NAMES = {
    0: "LBM_OK", 1: "LBM_ERR_IO", 2: "LBM_ERR_PARSE", 3: "LBM_ERR_NOMEM", 4: "LBM_ERR_CUDA",
    5: "LBM_ERR_DIVERGED", 6: "LBM_ERR_TIMEOUT", 7: "LBM_ERR_ARG", 8: "LBM_ERR_STATE", 9: "LBM_ERR_NODEV",
}

# lbm_precision
F64, F32, F16S, BF16S = 0, 1, 2, 3
# lbm_pattern
PULL, AA, AUTO = 0, 1, 2
# lbm_bc_kind
BC_NONE, BC_VEL_NEGY, BC_PRESS_NEGY, BC_PRESS_POSY, BC_PRESS_POSX, BC_PRESS_POSZ, BC_VEL_POSX = range(7)
BC_VELOCITY, BC_PRESSURE = 7, 8
# lbm_face
FACE_POSX, FACE_NEGX, FACE_POSY, FACE_NEGY, FACE_POSZ, FACE_NEGZ = range(6)
LIST_BOUNDARY, LIST_WALL = -1, -2
STEP_GRAPH, STEP_MONITOR = 1, 2
FIX_BB_ALL_DIRS, FIX_LIST_NODES = 1, 2
SNAP_FIELDS, SNAP_WSS = 1, 2


class LbmError(RuntimeError):
    """A C-ABI call returned a status other than LBM_OK."""

    def __init__(self, status, message):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class Tri(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("x1", "y1", "z1", "x2", "y2", "z2", "x3", "y3", "z3", "nx", "ny", "nz")]


class Grid(C.Structure):
    _fields_ = [("min", C.c_double * 3), ("dims", C.c_int32 * 3)]


class Predicate(C.Structure):
    _fields_ = [("list_id", C.c_int32), ("axis", C.c_int32), ("plane_hi", C.c_double), ("plane_lo", C.c_double),
                ("tol", C.c_double), ("lo", C.c_double * 3), ("hi", C.c_double * 3)]


class GeometryInfo(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("bbox", C.c_double * 6), ("spacing", C.c_double),
                ("n_points", C.c_int64), ("n_fluid", C.c_int64), ("n_boundary", C.c_int64), ("n_wall", C.c_int64),
                ("list_size", C.c_int64 * 64), ("n_lists", C.c_int32), ("voxelize_ms", C.c_double),
                ("classify_ms", C.c_double)]


class ListBC(C.Structure):
    _fields_ = [("list_id", C.c_int32), ("kind", C.c_int32), ("rho", C.c_double), ("dir", C.c_double * 3),
                ("profile", C.POINTER(C.c_double)), ("profile_len", C.c_size_t),
                ("amp", C.POINTER(C.c_double)), ("amp_len", C.c_size_t), ("face", C.c_int32),
                ("reserved", C.c_int32)]


class SimParams(C.Structure):
    _fields_ = [("Q", C.c_int32), ("precision", C.c_int32), ("pattern", C.c_int32), ("tau", C.c_double),
                ("bcs", C.POINTER(ListBC)), ("nbcs", C.c_size_t), ("warps_per_block", C.c_int32),
                ("run_axis", C.c_int32), ("staging", C.c_int32), ("nodes_per_lane", C.c_int32),
                ("corrections", C.c_int32), ("piece_slots", C.c_int32)]


class TuneEntry(C.Structure):
    _fields_ = [("nodes_per_lane", C.c_int32), ("staging", C.c_int32), ("warps_per_block", C.c_int32),
                ("chosen", C.c_int32), ("pattern", C.c_int32), ("piece_slots", C.c_int32),
                ("ms_per_launch", C.c_double)]


class VtuArray(C.Structure):
    _fields_ = [("name", C.c_char_p), ("components", C.c_int32), ("reserved", C.c_int32),
                ("data", C.POINTER(C.c_double))]


class SimInfo(C.Structure):
    _fields_ = [("n_nodes", C.c_int64), ("n_instances", C.c_int64), ("steps_done", C.c_int64),
                ("n_chunks", C.c_int64), ("Q", C.c_int32), ("precision", C.c_int32), ("pattern", C.c_int32),
                ("warps_per_block", C.c_int32), ("run_axis", C.c_int32), ("state_bytes", C.c_int64),
                ("algorithmic_bytes_per_update", C.c_double), ("n_lattice_nodes", C.c_int64),
                ("nodes_per_lane", C.c_int32), ("piece_slots", C.c_int32)]


class Monitors(C.Structure):
    _fields_ = [("step", C.c_int64), ("mass", C.c_double), ("inlet_flux", C.c_double),
                ("outlet_flux", C.c_double), ("max_speed", C.c_double), ("nonfinite", C.c_int32)]


# exported symbols and their prototypes: (restype, argtypes)
_P = C.POINTER
PROTOTYPES = {
    "lbm_last_error": (C.c_char_p, []),
    "lbm_status_string": (C.c_char_p, [C.c_int]),
    "lbm_free": (None, [C.c_void_p]),
    "lbm_abi_version": (C.c_int, []),
    "lbm_stl_read_ascii": (C.c_int, [C.c_char_p, _P(_P(Tri)), _P(C.c_size_t)]),
    "lbm_stl_read_binary": (C.c_int, [C.c_char_p, _P(_P(Tri)), _P(C.c_size_t)]),
    "lbm_stl_read_ascii_device": (C.c_int, [C.c_char_p, C.c_void_p, _P(_P(Tri)), _P(C.c_size_t), _P(C.c_int32)]),
    "lbm_stl_write_ascii": (C.c_int, [C.c_char_p, _P(Tri), C.c_size_t, C.c_char_p]),
    "lbm_geometry_create": (C.c_int, [_P(Tri), C.c_size_t, C.c_double, _P(Grid), _P(Predicate), C.c_size_t,
                                      C.c_void_p, _P(C.c_void_p)]),
    "lbm_predicates_pv2013": (C.c_int, [_P(Predicate), C.c_size_t, _P(C.c_size_t)]),
    "lbm_geometry_info_get": (C.c_int, [C.c_void_p, _P(GeometryInfo)]),
    "lbm_geometry_flags": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lbm_geometry_list": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t, _P(C.c_size_t)]),
    "lbm_geometry_destroy": (None, [C.c_void_p]),
    "lbm_sim_create": (C.c_int, [C.c_void_p, _P(SimParams), C.c_void_p, _P(C.c_void_p)]),
    "lbm_batch_create": (C.c_int, [_P(C.c_void_p), _P(SimParams), C.c_size_t, C.c_void_p, _P(C.c_void_p)]),
    "lbm_sim_step": (C.c_int, [C.c_void_p, C.c_int64, C.c_uint32, C.c_void_p]),
    "lbm_sim_info_get": (C.c_int, [C.c_void_p, _P(SimInfo)]),
    "lbm_sim_fields": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "lbm_sim_fields_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "lbm_sim_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "lbm_sim_wall_shear_stress": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    "lbm_vtu_write": (C.c_int, [C.c_char_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p]),
    "lbm_snapshot_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "lbm_snapshot_capture": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_snapshot_wait": (C.c_int, [C.c_void_p]),
    "lbm_snapshot_data": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p]),
    "lbm_snapshot_write_fields_vtu": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int32]),
    "lbm_snapshot_write_wss_vtu": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int32]),
    "lbm_snapshot_destroy": (None, [C.c_void_p]),
    "lbm_sim_checkpoint": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p]),
    "lbm_sim_restart": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p]),
    "lbm_sim_nodes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lbm_sim_instance_offsets": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lbm_sim_monitors": (C.c_int, [C.c_void_p, _P(Monitors), C.c_void_p]),
    "lbm_sim_set_divergence_tolerance": (C.c_int, [C.c_void_p, C.c_double]),
    "lbm_sim_set_wait_limit": (C.c_int, [C.c_void_p, C.c_uint32]),
    "lbm_sim_test_stall": (C.c_int, [C.c_void_p, C.c_int32]),
    "lbm_sim_poison_ghosts": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_sim_prepare_graph": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "lbm_sim_set_pattern": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "lbm_sim_destroy": (None, [C.c_void_p]),
    "lbm_synth_cylinder": (C.c_int, [C.c_double, C.c_double, C.c_int32, C.c_int32, _P(C.c_double),
                                     _P(_P(Tri)), _P(C.c_size_t)]),
    "lbm_synth_capsules": (C.c_int, [_P(C.c_double), C.c_size_t, _P(C.c_double), _P(C.c_double), C.c_double,
                                     C.c_uint64, _P(_P(Tri)), _P(C.c_size_t)]),
}

_lib = None


def load():
    """Loads liblbm_gb300.so once and binds every prototype; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built; run pv2013_gb300.build.build_library() "
                          "(the engine has no fallback path)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    """Message of the last failing call on this thread."""
    msg = load().lbm_last_error()
    return msg.decode() if msg else ""


def check(status):
    """Raises LbmError with the library's message unless status is LBM_OK."""
    if status != LBM_OK:
        msg = load().lbm_last_error()
        raise LbmError(status, msg.decode() if msg else "")
