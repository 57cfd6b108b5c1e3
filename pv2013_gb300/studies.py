"""Accuracy and ensemble studies on the synthetic workloads.

    python -m pv2013_gb300.studies precision --case bifurcation --Q 27 --taus 0.51,0.55,0.8 --steps 10000
    python -m pv2013_gb300.studies ensemble --n 64 --steps 2000
    python -m pv2013_gb300.studies pv2013 --steps 20000 [--stl PV2013.stl]

precision: for each relaxation time, the FP64 run (the reference's
arithmetic, bit-exact with the CPU oracle) and the FP32 / FP16-shifted /
BF16-shifted storage runs (FP32 collision math) advance the same case; the
study reports, per storage, the velocity error relative to FP64 (L2 and max,
relative to the FP64 field's L2 norm and maximum), the largest density
difference, the relative mass change per 1000 steps, and MLUPS.  A run whose
monitors report non-finite values or a mass change above 50 % is reported
as diverged, with the step at which it was detected (checked every 500
steps).

ensemble: n tortuous vessels (cases.vessel, per-instance tau, inlet
amplitude and period) advance together in one launch per step over a packed
node list (FP16-shifted storage, AA pattern, CUDA-graph replay, autotuned
kernel); the study reports the aggregate MLUPS and, for a subset, the
per-instance velocity error against FP64 runs of the same instances.

pv2013: the reference's own production run (PV2013 geometry, spacing 0.1,
tau 0.66, 20 000 iterations) in FP64 (the reference's arithmetic) and
FP16-shifted storage, timed against the reference's recorded run.

Prints one JSON object.
"""
import argparse
import json
import sys
import time

import numpy as np

from . import _capi, cases
from .engine import BoundarySpec, Geometry, Simulation


def _rel(a, b):
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float("nan")


def face_specs(case, geom, Q):
    """Boundary settings valid for either lattice: velocity inlet on the top
    face (unknowns -y) and pressure outlets on the bottom face (unknowns +y),
    through the face kinds (the reference's D3Q19 routines for Q = 19)."""
    if Q == 19:
        return case.boundary_specs(geom)
    return [BoundarySpec(cases.INLET_LIST, _capi.BC_VELOCITY, dir=(0.0, -1.0, 0.0), profile=case.inlet_profile(geom),
                         amp=case.amp_table(), face=_capi.FACE_NEGY),
            BoundarySpec(cases.OUTLET_LIST, _capi.BC_PRESSURE, rho=case.outlet_rho, face=_capi.FACE_POSY)]


def _timed_run(sim, steps, chunk=500):
    """Advances in chunks with the divergence monitor; returns (seconds,
    None) or, when the monitor trips, (seconds, the step count reached)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.time()
    done = 0
    try:
        while done < steps:
            k = min(chunk, steps - done)
            sim.step(k, graph=True, monitor=True)
            done += k
    except _capi.LbmError as e:
        if e.status == 5:
            return time.time() - t0, done + k
        raise
    torch.cuda.synchronize()
    return time.time() - t0, None


def precision_study(case, Q, taus, steps, precisions=("f32", "f16s", "bf16s")):
    geom = case.geometry()
    nf = geom.info.n_fluid
    out = {"case": case.name, "Q": Q, "steps": steps, "fluid_nodes": nf, "dims": list(geom.GeomSize),
           "fp64": "FP64 storage and math (the reference's arithmetic)", "runs": []}
    for tau in taus:
        specs = face_specs(case, geom, Q)
        ref = Simulation(geom, tau, specs, Q=Q, precision="f64", pattern="pull")
        ref.set_divergence_tolerance(0.5)
        sec, div = _timed_run(ref, steps)
        row = {"tau": tau, "f64": {"mlups": nf * (div or steps) / sec / 1e6, "diverged_at": div}}
        if div is None:
            _, r64, u64 = ref.fields(f=False)
        del ref
        for prec in precisions:
            sim = Simulation(geom, tau, face_specs(case, geom, Q), Q=Q, precision=prec, pattern="aa")
            sim.set_divergence_tolerance(0.5)
            m0 = sim.monitors()["mass"]
            sec, d = _timed_run(sim, steps)
            r = {"mlups": nf * (d or steps) / sec / 1e6, "diverged_at": d}
            if d is None and div is None:
                _, rr, uu = sim.fields(f=False)
                m1 = sim.monitors()["mass"]
                r.update({"u_rel_l2": _rel(uu, u64), "u_rel_max": float(np.abs(uu - u64).max() / np.abs(u64).max()),
                          "rho_max_abs": float(np.abs(rr - r64).max()),
                          "mass_change_per_1000_steps": float((m1 - m0) / m0 / steps * 1000)})
            row[prec] = r
            del sim
        out["runs"].append(row)
    return out


def ensemble_study(n, steps, check=4, check_steps=500):
    import torch
    ens = cases.ensemble(n)
    geoms = [c.geometry() for c in ens]
    specs = [c.boundary_specs(g) for c, g in zip(ens, geoms)]
    taus = [c.tau for c in ens]
    nf = sum(g.info.n_fluid for g in geoms)
    sim = Simulation(geoms, taus, specs, precision="f16s", pattern="aa")
    tune = sim.autotune(launches=10)
    sim.step(20, graph=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    sim.step(steps, graph=True)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    info = sim.info()
    del sim
    # per-instance error on a subset: the batch vs FP64 runs of the same instances
    sub = list(range(min(check, n)))
    b16 = Simulation([geoms[i] for i in sub], [taus[i] for i in sub], [specs[i] for i in sub], precision="f16s",
                     pattern="aa")
    b16.step(check_steps, graph=True)
    off = b16.instance_offsets()
    _, _, u16 = b16.fields(f=False)
    errs = []
    for k, i in enumerate(sub):
        s64 = Simulation(geoms[i], taus[i], specs[i], precision="f64", pattern="pull")
        s64.step(check_steps, graph=True)
        _, _, u64 = s64.fields(f=False)
        errs.append({"instance": i, "tau": taus[i], "u_rel_l2": _rel(u16[off[k]:off[k + 1]], u64)})
    return {"instances": n, "fluid_nodes": nf, "steps": steps, "mlups": nf * steps / sec / 1e6,
            "ms_per_step": sec / steps * 1e3, "kernel": {"nodes_per_lane": info.nodes_per_lane,
                                                          "warps_per_block": info.warps_per_block},
            "autotune": [{"nodes_per_lane": t[0], "staging": t[1], "warps_per_block": t[2], "ms_per_launch": t[3],
                          "chosen": t[4]} for t in tune],
            "error_vs_fp64": {"steps": check_steps, "per_instance": errs}}


# The reference's production run (slurm-427156.out): PV2013.stl at spacing
# 0.1, tau 0.66, 20 000 iterations on one rank: 71 568.30 s in total, about
# 2 942 s of set-up and a median of 3.34 s per iteration without output.
REF_PV2013_TOTAL_S = 71568.30
REF_PV2013_SETUP_S = 2942.0
REF_PV2013_STEP_S = 3.34


def pv2013_study(tris, steps, precisions=("f64", "f16s"), output_every=0, outdir=None):
    """The reference's own run: PV2013 geometry (its seven predicate lists),
    spacing 0.1, tau 0.66, velocity inlet (0, -0.1, 0), outlets at rho 1.01."""
    import torch
    from .engine import pv2013_predicates
    out = {"case": "PV2013", "steps": steps, "reference": {"total_s": REF_PV2013_TOTAL_S, "setup_s": REF_PV2013_SETUP_S,
                                                          "step_s": REF_PV2013_STEP_S}, "runs": {}}
    torch.cuda.synchronize()
    t0 = time.time()
    geom = Geometry(tris, 0.1, predicates=pv2013_predicates())
    torch.cuda.synchronize()
    out["geometry_s"] = time.time() - t0
    out["voxelize_ms"] = geom.info.voxelize_ms
    out["dims"] = list(geom.GeomSize)
    out["fluid_nodes"] = geom.info.n_fluid
    kinds = [_capi.BC_VEL_NEGY, _capi.BC_PRESS_NEGY, _capi.BC_PRESS_POSY, _capi.BC_PRESS_POSX, _capi.BC_PRESS_POSX,
             _capi.BC_PRESS_POSX, _capi.BC_PRESS_POSZ]
    specs = [BoundarySpec(0, kinds[0], dir=(0.0, -1.0, 0.0), amp=np.array([0.1]))]
    specs += [BoundarySpec(l, kinds[l], rho=1.01) for l in range(1, 7)]
    for prec in precisions:
        t0 = time.time()
        sim = Simulation(geom, 0.66, specs, precision=prec, pattern="pull" if prec == "f64" else "aa")
        torch.cuda.synchronize()
        t_build = time.time() - t0
        snap = None
        if output_every and outdir:
            import os
            from .engine import Snapshot
            os.makedirs(outdir, exist_ok=True)
            snap = Snapshot(sim, fields=True, wss=True)
        t0 = time.time()
        done = 0
        while done < steps:
            k = min(output_every or steps, steps - done)
            sim.step(k, graph=True)
            done += k
            if snap is not None:
                snap.capture()
                snap.write_fields_vtu(f"{outdir}/{prec}_{done}.vtu")
                snap.write_wss_vtu(f"{outdir}/{prec}_{done}_wall_shear_stress.vtu")
        torch.cuda.synchronize()
        sec = time.time() - t0
        mon = sim.monitors()
        out["runs"][prec] = {"lattice_build_s": t_build, "steps_s": sec, "ms_per_step": sec / steps * 1e3,
                             "mlups": geom.info.n_fluid * steps / sec / 1e6,
                             "speedup_per_step_vs_reference": REF_PV2013_STEP_S / (sec / steps),
                             "total_s": out["geometry_s"] + t_build + sec,
                             "mass": mon["mass"], "max_speed": mon["max_speed"], "nonfinite": mon["nonfinite"]}
        del sim
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m pv2013_gb300.studies")
    sub = ap.add_subparsers(dest="study", required=True)
    p = sub.add_parser("precision")
    p.add_argument("--case", default="bifurcation", choices=["pipe", "bifurcation", "vascular_tree"])
    p.add_argument("--Q", type=int, default=19)
    p.add_argument("--taus", default="0.6")
    p.add_argument("--steps", type=int, default=10000)
    p.add_argument("--h", type=float, default=None)
    v = sub.add_parser("pv2013")
    v.add_argument("--stl", help="PV2013.stl (ASCII); default: the triangles of tests/golden/pv2013_tris.npz")
    v.add_argument("--steps", type=int, default=20000)
    v.add_argument("--output-every", type=int, default=0)
    v.add_argument("--outdir", default=None)
    e = sub.add_parser("ensemble")
    e.add_argument("--n", type=int, default=64)
    e.add_argument("--steps", type=int, default=2000)
    a = ap.parse_args(argv)
    import torch
    torch.cuda.init()
    if a.study == "precision":
        maker = {"pipe": cases.pipe, "bifurcation": cases.bifurcation, "vascular_tree": cases.vascular_tree}[a.case]
        kw = {"h": a.h} if a.h else ({"h": 2.2} if a.case == "vascular_tree" else {})
        case = maker(**kw)
        res = precision_study(case, a.Q, [float(t) for t in a.taus.split(",")], a.steps)
    elif a.study == "pv2013":
        from .engine import Reader
        if a.stl:
            tris = Reader.readSTLASCII(a.stl)
        else:
            import os
            fx = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden",
                              "pv2013_tris.npz")
            tris = np.load(fx)["tris"]
        res = pv2013_study(tris, a.steps, output_every=a.output_every, outdir=a.outdir)
    else:
        res = ensemble_study(a.n, a.steps)
    print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
