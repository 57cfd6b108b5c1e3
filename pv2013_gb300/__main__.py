"""Command-line runner: one simulation from a run file or from options.

    python -m pv2013_gb300 [run-file] [--case NAME | --stl FILE --preset pv2013]
                           [--precision f64|f32|f16s|bf16s] [--pattern pull|aa]
                           [--steps N] [--warmup W] [--tau T] [--Q 19|27] ...

The run file uses the reference's ConfigReader format (ConfigReader.cpp:13-51):
one `key value` pair per line, `#` starts a comment line; command-line options
override it.  Keys: case, stl, preset, spacing, box, tau, steps, warmup,
precision, pattern, Q, u_in, outlet_rho, run_axis, staging, warps_per_block,
nodes_per_lane, piece_slots.  `boundary <list> ... end` blocks give each
inlet/outlet list its plane predicate and boundary condition (runfile.py).

Named cases are the seeded synthetic workloads of pv2013_gb300.cases (pipe,
pipe_x, bifurcation, vascular_tree, vessel); `--stl FILE` with boundary blocks
runs any surface (ASCII or binary STL); `--stl FILE --preset pv2013` runs
an STL with the PV2013 inlet/outlet planes (ComplexGeometry.cpp:579-638), the
reference's uniform inlet velocity (0, -u_in, 0) (Boundary.cpp:9, Input.h:7)
and its outlet density 1.01 (Simulation.cpp:954).

Prints one JSON object: lattice size, set-up times, the timed steps' MLUPS
(CUDA events around a graph-replayed step loop) and the monitors.
"""
import argparse
import json
import sys
import time

from . import runfile
from .runfile import KEYS


def read_run_file(path):
    """key/value pairs of a ConfigReader-format file (boundary blocks aside)."""
    return runfile.read(path)[0]


def read_surface(path):
    """Triangles of an ASCII or binary STL (binary when it does not start with 'solid')."""
    from .engine import Reader
    with open(path, "rb") as fh:
        head = fh.read(5)
    return Reader.readSTLASCII(path) if head == b"solid" else Reader.readSTLBinary(path)


def build_problem(cfg, blocks=()):
    """(geometry, tau, boundary specs, Q) for the configuration."""
    from . import _capi, cases
    from .engine import BoundarySpec, Geometry, Reader, pv2013_predicates
    if blocks:
        if cfg.get("stl"):
            tris = read_surface(cfg["stl"])
            grid = runfile.grid_of(cfg)
            tau = cfg.get("tau", 0.8)
        else:
            case = cases.pipe() if cfg.get("case", "pipe") == "pipe" else None
            if case is None:
                raise ValueError("boundary blocks need an STL (or the pipe case)")
            tris, grid, tau = case.triangles, runfile.grid_of(cfg) or case.grid, cfg.get("tau", case.tau)
        g = Geometry(tris, cfg.get("spacing", 1.0), grid=grid, predicates=runfile.predicates(blocks))
        return g, tau, runfile.boundary_specs(blocks, g), cfg.get("Q", 19)
    if cfg.get("stl"):
        if cfg.get("preset", "pv2013") != "pv2013":
            raise ValueError("an STL run needs --preset pv2013 (the only built-in predicate set)")
        tris = Reader.readSTLASCII(cfg["stl"])
        g = Geometry(tris, cfg.get("spacing", 0.1), predicates=pv2013_predicates())
        u_in = cfg.get("u_in", 0.1)
        rho = cfg.get("outlet_rho", 1.01)
        kinds = [_capi.BC_VEL_NEGY, _capi.BC_PRESS_NEGY, _capi.BC_PRESS_POSY, _capi.BC_PRESS_POSX,
                 _capi.BC_PRESS_POSX, _capi.BC_PRESS_POSX, _capi.BC_PRESS_POSZ]
        specs = [BoundarySpec(0, kinds[0], dir=(0.0, -1.0, 0.0), amp=[u_in])]
        specs += [BoundarySpec(l, kinds[l], rho=rho) for l in range(1, 7)]
        return g, cfg.get("tau", 0.66), specs, 19
    name = cfg.get("case", "pipe")
    makers = {"pipe": cases.pipe, "pipe_x": cases.pipe_x, "bifurcation": cases.bifurcation,
              "vascular_tree": cases.vascular_tree, "vessel": lambda **k: cases.vessel(4000, **k)}
    if name not in makers:
        raise ValueError(f"unknown case {name!r}; one of {sorted(makers)}")
    kw = {"h": cfg["h"]} if "h" in cfg and name in ("bifurcation", "vascular_tree", "vessel") else {}
    if name == "vascular_tree" and not kw:
        kw = {"h": 2.2}
    case = makers[name](**kw)
    if name == "pipe_x":   # D3Q27 x-normal inlet (Boundary.cpp:87-123); no D3Q27 outlet routine exists
        g = Geometry(case.triangles, 1.0, grid=case.grid, predicates=case.predicates[:1])
        specs = [BoundarySpec(0, _capi.BC_VEL_POSX, dir=(1.0, 0.0, 0.0), profile=case.inlet_profile(g),
                              amp=case.amp_table())]
        return g, cfg.get("tau", case.tau), specs, 27
    g = case.geometry()
    return g, cfg.get("tau", case.tau), case.boundary_specs(g), cfg.get("Q", 19)


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m pv2013_gb300", description=__doc__.split("\n\n")[0])
    ap.add_argument("run_file", nargs="?")
    for k, t in KEYS.items():
        ap.add_argument("--" + k, type=t)
    a = ap.parse_args(argv)
    cfg, blocks = runfile.read(a.run_file) if a.run_file else ({}, [])
    cfg.update({k: v for k, v in vars(a).items() if k in KEYS and v is not None})

    import torch
    from .engine import Simulation
    torch.cuda.init()
    t0 = time.time()
    g, tau, specs, Q = build_problem(cfg, blocks)
    t_geom = time.time() - t0
    t0 = time.time()
    sim = Simulation(g, tau, specs, Q=Q, precision=cfg.get("precision", "f64"), pattern=cfg.get("pattern", "pull"),
                     warps_per_block=cfg.get("warps_per_block", 0), run_axis=cfg.get("run_axis", 0),
                     staging=cfg.get("staging", 1), nodes_per_lane=cfg.get("nodes_per_lane", 0),
                     piece_slots=cfg.get("piece_slots", 0))
    torch.cuda.synchronize()
    t_build = time.time() - t0
    steps, warmup = cfg.get("steps", 100), cfg.get("warmup", 3)
    sim.step(warmup, graph=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    sim.step(steps, graph=True)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    info = sim.info()
    nf = g.info.n_fluid
    mon = sim.monitors()
    print(json.dumps({
        "case": cfg.get("stl") or cfg.get("case", "pipe"), "Q": info.Q, "precision": cfg.get("precision", "f64"),
        "pattern": cfg.get("pattern", "pull"), "dims": list(g.GeomSize), "fluid_nodes": nf,
        "lattice_nodes": info.n_lattice_nodes, "chunks": info.n_chunks, "run_axis": info.run_axis,
        "nodes_per_lane": info.nodes_per_lane, "piece_slots": info.piece_slots,
        "warps_per_block": info.warps_per_block,
        "geometry_s": t_geom, "voxelize_ms": g.info.voxelize_ms, "lattice_build_s": t_build,
        "steps": steps, "warmup": warmup, "ms_per_step": sec / steps * 1e3, "mlups": nf * steps / sec / 1e6,
        "gbs_algorithmic": info.algorithmic_bytes_per_update * nf * steps / sec / 1e9,
        "monitors": {k: mon[k] for k in ("step", "mass", "max_speed", "nonfinite")}}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
