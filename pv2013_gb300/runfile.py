"""Run files: the reference's ConfigReader format, extended with boundary blocks.

The reference reads `key value` lines and skips empty lines and lines that
start with `#` (ConfigReader.cpp:13-51); its inlet and outlet planes are
compiled in (ComplexGeometry.cpp:579-638).  A run file here has the same
`key value` lines (keys below) plus one block per boundary list, so a user
STL with its own inlet and outlet planes runs from a file:

    stl vessel.stl
    spacing 1.0
    box 0 0 0 48 128 48          # optional explicit grid: min x y z, Nx Ny Nz
    tau 0.8
    boundary 0                   # list id (0..63); lists match in id order
      axis y                     # predicate |p[axis] - plane| <= tol (getInOutBP form)
      plane 107
      tol 0.01
      box 0.5 nan nan nan 0.5 45.5   # lo < p < hi on the other axes: lo_x hi_x lo_y hi_y lo_z hi_z
      kind vel_negy              # or velocity / pressure with a face, or another reference routine
      dir 0 -1 0
      u 0.05
      profile parabolic 23.5 23.5 20   # 1 - r^2/R^2 about (centre on the two other axes), R
      waveform sine 1000 0.5           # u (1 + 0.5 sin(2 pi t / 1000))
    end
    boundary 2
      axis y
      plane 20
      kind press_posy
      rho 1.0
    end

Block keys: axis (x|y|z), plane (decimal string, kept exactly), tol, box,
kind (vel_negy, press_negy, press_posy, press_posx, press_posz, vel_posx,
velocity, pressure), face (+x -x +y -y +z -z: the direction of the unknown
populations, for velocity/pressure), rho, dir, u, profile (uniform |
parabolic c1 c2 R), waveform (constant | sine PERIOD_STEPS REL_AMPLITUDE |
pv2013 STEPS_PER_PERIOD: the reference's three-piece inlet waveform of
pulsatile.h:8-31 over its 0.9 s period, in units of `u`).
"""
import math

import numpy as np

KEYS = {"case": str, "stl": str, "preset": str, "spacing": float, "tau": float, "steps": int, "warmup": int,
        "precision": str, "pattern": str, "Q": int, "u_in": float, "outlet_rho": float, "run_axis": int,
        "staging": int, "warps_per_block": int, "nodes_per_lane": int, "piece_slots": int, "h": float,
        "box": str}

KINDS = {"vel_negy": 1, "press_negy": 2, "press_posy": 3, "press_posx": 4, "press_posz": 5, "vel_posx": 6,
         "velocity": 7, "pressure": 8}
VELOCITY_KINDS = {"vel_negy", "vel_posx", "velocity"}
FACES = {"+x": 0, "-x": 1, "+y": 2, "-y": 3, "+z": 4, "-z": 5}
AXES = {"x": 0, "y": 1, "z": 2}


class RunFileError(ValueError):
    """A run file line the reader cannot use (file:line in the message)."""


class Block:
    """One `boundary <list> ... end` block."""

    def __init__(self, list_id, where):
        self.list_id = list_id
        self.where = where
        self.axis = None
        self.plane = None
        self.tol = 1e-2
        self.lo = [math.nan] * 3
        self.hi = [math.nan] * 3
        self.kind = None
        self.face = None
        self.rho = 1.0
        self.dir = (0.0, -1.0, 0.0)
        self.u = 1.0
        self.profile = ("uniform",)
        self.waveform = ("constant",)


def _num(tok, where):
    try:
        return float(tok)
    except ValueError:
        raise RunFileError(f"{where}: expected a number, got {tok!r}") from None


def _block_line(b, key, vals, where):
    need = {"axis": 1, "plane": 1, "tol": 1, "box": 6, "kind": 1, "face": 1, "rho": 1, "dir": 3, "u": 1}
    if key in need and len(vals) != need[key]:
        raise RunFileError(f"{where}: '{key}' takes {need[key]} value(s)")
    if key == "axis":
        if vals[0] not in AXES:
            raise RunFileError(f"{where}: axis must be x, y or z")
        b.axis = AXES[vals[0]]
    elif key == "plane":
        _num(vals[0], where)
        b.plane = vals[0]                      # decimal string: split into a double-double later
    elif key == "tol":
        b.tol = _num(vals[0], where)
    elif key == "box":
        v = [_num(t, where) for t in vals]
        b.lo = [v[0], v[2], v[4]]
        b.hi = [v[1], v[3], v[5]]
    elif key == "kind":
        if vals[0] not in KINDS:
            raise RunFileError(f"{where}: unknown kind {vals[0]!r}; one of {sorted(KINDS)}")
        b.kind = vals[0]
    elif key == "face":
        if vals[0] not in FACES:
            raise RunFileError(f"{where}: face must be one of {sorted(FACES)}")
        b.face = vals[0]
    elif key == "rho":
        b.rho = _num(vals[0], where)
    elif key == "dir":
        b.dir = tuple(_num(t, where) for t in vals)
    elif key == "u":
        b.u = _num(vals[0], where)
    elif key == "profile":
        if vals == ["uniform"]:
            b.profile = ("uniform",)
        elif len(vals) == 4 and vals[0] == "parabolic":
            b.profile = ("parabolic",) + tuple(_num(t, where) for t in vals[1:])
        else:
            raise RunFileError(f"{where}: profile is 'uniform' or 'parabolic c1 c2 R'")
    elif key == "waveform":
        if vals == ["constant"]:
            b.waveform = ("constant",)
        elif len(vals) == 3 and vals[0] == "sine":
            period = _num(vals[1], where)
            if period < 1 or period != int(period):
                raise RunFileError(f"{where}: the sine period is a whole number of steps >= 1")
            b.waveform = ("sine", int(period), _num(vals[2], where))
        elif len(vals) == 2 and vals[0] == "pv2013":
            n = _num(vals[1], where)
            if n < 1 or n != int(n):
                raise RunFileError(f"{where}: steps per period is a whole number >= 1")
            b.waveform = ("pv2013", int(n))
        else:
            raise RunFileError(f"{where}: waveform is 'constant', 'sine PERIOD REL_AMPLITUDE' or "
                               f"'pv2013 STEPS_PER_PERIOD'")
    else:
        raise RunFileError(f"{where}: unknown boundary key {key!r}")


def _check_block(b):
    if b.axis is None or b.plane is None:
        raise RunFileError(f"{b.where}: boundary {b.list_id} needs 'axis' and 'plane'")
    if b.kind is None:
        raise RunFileError(f"{b.where}: boundary {b.list_id} needs 'kind'")
    if b.kind in ("velocity", "pressure") and b.face is None:
        raise RunFileError(f"{b.where}: kind {b.kind} needs 'face'")


def parse(lines, name="<run file>"):
    """(cfg dict, [Block]) of run-file lines."""
    cfg, blocks, cur = {}, [], None
    for n, line in enumerate(lines, 1):
        line = line.rstrip("\n")
        where = f"{name}:{n}"
        if not line.strip() or line.lstrip()[0] == "#":
            continue
        parts = line.split("#", 1)[0].split()
        key, vals = parts[0], parts[1:]
        if cur is not None:
            if key == "end" and not vals:
                _check_block(cur)
                blocks.append(cur)
                cur = None
            else:
                _block_line(cur, key, vals, where)
            continue
        if key == "boundary":
            if len(vals) != 1 or not vals[0].isdigit() or int(vals[0]) > 63:
                raise RunFileError(f"{where}: 'boundary' takes a list id 0..63")
            lid = int(vals[0])
            if any(b.list_id == lid for b in blocks):
                raise RunFileError(f"{where}: boundary {lid} is defined twice")
            cur = Block(lid, where)
            continue
        if key == "end":
            raise RunFileError(f"{where}: 'end' outside a boundary block")
        if key not in KEYS:
            raise RunFileError(f"{where}: unknown key {key!r}")
        if not vals:
            raise RunFileError(f"{where}: expected 'key value'")
        text = " ".join(vals)
        try:
            cfg[key] = KEYS[key](text)
        except ValueError:
            raise RunFileError(f"{where}: bad value {text!r} for {key!r}") from None
    if cur is not None:
        raise RunFileError(f"{cur.where}: boundary {cur.list_id} has no 'end'")
    return cfg, blocks


def read(path):
    """(cfg dict, [Block]) of a run file."""
    with open(path) as fh:
        return parse(fh, path)


# ---------------------------------------------------------------------------
# waveforms (amplitude per step, periodic; multiplied by the profile and dir)

def pulsatile_pv2013(x):
    """The reference's inlet waveform at time x in [0, 0.9) s: three
    polynomial pieces on [0, 0.09), [0.09, 0.27), [0.27, 0.81), zero after
    (pulsatile.h:8-31, Simulation.cpp:875-900)."""
    period = 0.9
    x = math.fmod(x, period)
    if 0.0 <= x < 0.1 * period:
        return (-8.579e+08 * x ** 8 + 4.059e+08 * x ** 7 - 7.817e+07 * x ** 6 + 7.994e+06 * x ** 5
                - 4.835e+05 * x ** 4 + 1.782e+04 * x ** 3 - 321.6 * x ** 2 + 3.215 * x + 0.1423)
    if 0.1 * period <= x < 0.3 * period:
        return (-4.32e+06 * x ** 8 + 7.94e+06 * x ** 7 - 6.298e+06 * x ** 6 + 2.82e+06 * x ** 5
                - 7.809e+05 * x ** 4 + 1.37e+05 * x ** 3 - 1.484e+04 * x ** 2 + 901.9 * x - 22.87)
    if 0.3 * period <= x < 0.9 * period:
        return -5.123 * x ** 4 + 14.15 * x ** 3 - 14.21 * x ** 2 + 5.865 * x - 0.5696
    return 0.0


def amplitude_table(block):
    """Amplitude per step of a velocity block (its period), times `u`."""
    w = block.waveform
    if w[0] == "constant":
        return np.array([block.u])
    if w[0] == "sine":
        t = np.arange(w[1], dtype=np.float64)
        return block.u * (1.0 + w[2] * np.sin(2.0 * np.pi * t / w[1]))
    n = w[1]                                   # pv2013: n steps per 0.9 s period
    return block.u * np.array([pulsatile_pv2013(0.9 * s / n) for s in range(n)])


def profile_values(block, geom):
    """Profile factor of each node of the block's list, in list order."""
    idx = geom.list(block.list_id)
    if block.profile[0] == "uniform":
        return None
    c1, c2, r = block.profile[1:]
    pts = geom.coords(idx)
    others = [a for a in range(3) if a != block.axis]
    r2 = (pts[:, others[0]] - c1) ** 2 + (pts[:, others[1]] - c2) ** 2
    return np.maximum(0.0, 1.0 - r2 / r ** 2)


def predicates(blocks):
    from .engine import PlanePredicate
    return [PlanePredicate(b.list_id, b.axis, b.plane, b.tol, tuple(b.lo), tuple(b.hi)) for b in blocks]


def boundary_specs(blocks, geom):
    from .engine import BoundarySpec
    specs = []
    for b in blocks:
        kw = {"face": FACES[b.face]} if b.face is not None else {}
        if b.kind in VELOCITY_KINDS:
            specs.append(BoundarySpec(b.list_id, KINDS[b.kind], dir=b.dir, profile=profile_values(b, geom),
                                      amp=amplitude_table(b), **kw))
        else:
            specs.append(BoundarySpec(b.list_id, KINDS[b.kind], rho=b.rho, **kw))
    return specs


def grid_of(cfg):
    """Explicit grid ((min x, y, z), (Nx, Ny, Nz)) of the `box` key, else None."""
    if "box" not in cfg:
        return None
    v = cfg["box"].split()
    if len(v) != 6:
        raise RunFileError("box takes min x y z and Nx Ny Nz")
    return (tuple(float(t) for t in v[:3]), tuple(int(t) for t in v[3:]))
