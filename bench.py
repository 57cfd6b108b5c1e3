#!/usr/bin/env python3
"""Benchmark: D3Q19 MLUPS and HBM-roofline fraction on the 512x1024x512 vascular tree.

Workload (the configuration the headline metric is quoted on): a seeded
depth-5 binary tree of tubes (root radius 40 lattice units, child/parent
radius 0.79, branch angles 25-45 deg, ~2.07 M triangles, 32 outlets)
voxelized on the GPU into a 512 x 1024 x 512 grid (x, y, z; the tree grows
along -y), D3Q19 BGK, tau 0.6, pulsatile Zou-He inlet
u(t) = 0.04 (1 + 0.5 sin(2 pi t / 1000)) with a parabolic profile, pressure
outlets at rho 1.  Synthetic data (seeded generator, no dataset).

GPU arm (default): one step = one fused collide-stream-boundary launch over
the whole lattice.  `value` is the MLUPS of the FP16-shifted storage path;
the plain FP32 two-lattice path is timed on the same lattice and reported
beside it with the ratio, and the velocity error of the FP16 path against the
FP64 path (bit-exact with the CPU oracle) is stated.  Populations
(> 300 MB) exceed the 129 MB L2, so no flush is needed between steps.

Reference arm (--impl reference): the PV2013 reference's own step loop
(Collision, Streaming, ApplyZouHeBc, ApplyWallBc, ApplyOutletBc), compiled
from its sources, run as one process per host core on a bounded sample of
the same tree (the inlet section), aggregate MLUPS.

Prints one JSON line (rank 0).  Multi-GPU: independent replicas per rank
(weak scaling), value = sum over ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "vascular_tree_512x1024x512_D3Q19"
METRIC = "D3Q19 MLUPS, % HBM roofline: FP16-store & batched vs plain FP32 @ stated err"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic_bytes_per_node():
    """DRAM bytes per fluid node per launch of the step kernel, from an ncu
    capture summarised in profiles/step_kernel_traffic.txt (key = value lines)."""
    p = os.path.join(ROOT, "profiles", "step_kernel_traffic.txt")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            if "=" in line and not line.startswith("#"):
                k, v = line.split("=", 1)
                try:
                    out[k.strip()] = float(v.split()[0])
                except ValueError:
                    pass
    return out


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi (read-only
    queries) while a timed region runs.

    nvidia-smi takes longer to start than a short timed region lasts, so the
    sampler is started first and the region is bracketed with begin()/end();
    only samples that arrive inside the bracket (plus one sampling interval)
    are kept.  A failing query is recorded in the summary, not hidden."""

    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    INTERVAL_MS = 50

    def __init__(self, index=0):
        self.index = index
        self.samples = []          # (arrival time, fields)
        self.proc = None
        self.error = None
        self.t0 = self.t1 = None

    def _cmd(self, loop):
        c = ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits"]
        return c + (["-lms", str(self.INTERVAL_MS)] if loop else [])

    def __enter__(self):
        try:
            r = subprocess.run(self._cmd(False), capture_output=True, text=True, timeout=30)
            if r.returncode != 0 or len(r.stdout.split(",")) < 8:
                self.error = f"nvidia-smi query failed (rc {r.returncode}): {(r.stderr or r.stdout).strip()[:200]}"
                return self
            self.proc = subprocess.Popen(self._cmd(True), stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
            t = time.time()
            while not self.samples and time.time() - t < 20 and self.proc.poll() is None:
                time.sleep(0.01)
            if not self.samples:
                self.error = "nvidia-smi produced no sample within 20 s"
        except (OSError, subprocess.SubprocessError) as e:
            self.error = f"nvidia-smi: {e}"
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.samples.append((time.time(), parts))

    def begin(self):
        self.t0 = time.time()

    def end(self):
        self.t1 = time.time()
        # one more interval, so that a region shorter than the interval still
        # gets the sample taken while it ran
        time.sleep(2.5 * self.INTERVAL_MS / 1000.0)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.error:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [f"unsampled: {self.error}"], "samples": 0}
        lo = self.t0 if self.t0 is not None else 0.0
        hi = (self.t1 if self.t1 is not None else time.time()) + 2 * self.INTERVAL_MS / 1000.0
        inside = [f for t, f in self.samples if lo <= t <= hi]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "samples": 0,
                    "reasons": [f"unsampled: no sample inside the timed region ({len(self.samples)} outside)"]}
        num = lambda v: float(v) if v.replace(".", "", 1).isdigit() else None
        sm = [x for x in (num(f[0]) for f in inside) if x is not None]
        mx = [x for x in (num(f[1]) for f in inside) if x is not None]
        reasons = sorted({n for f in inside for n, v in zip(self.NAMES, f[4:8]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside), "interval_ms": self.INTERVAL_MS}


def max_over_ranks(x, world, device):
    """The largest value over the ranks (the slowest replica's time)."""
    if world <= 1:
        return x
    import torch
    t = torch.tensor([float(x)], device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def time_steps(sim, steps, warmup, torch, clk=None):
    sim.step(warmup, graph=True)
    sim.prepare_graph(steps)            # the graph of the timed call is captured outside it
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if clk:
        clk.begin()
    e0.record()
    sim.step(steps, graph=True)
    e1.record()
    torch.cuda.synchronize()
    if clk:
        clk.end()
    return e0.elapsed_time(e1) / 1000.0


# Per-process step rate of the reference's step loop on the machine's host cores
# (measured: about 1 MLUPS per Grace core); sizes the timed sample so that a
# run of the requested step count takes about REF_SECONDS per process.
REF_MLUPS_PER_CORE = 1.0
REF_SECONDS = 60.0


def reference_sample(levels=40):
    """The bounded sample of the tree workload the reference's step loop runs
    on: the top `levels` (3..40) grid levels of the 96 x 40 x 96-point section
    just below the tree's inlet face (oracle/fixtures/tree_inlet_section.npz,
    node types from the CPU oracle's voxelizer on the full grid's rays).
    Returns (sample, parameters): sample = (flags, origin, dims)."""
    import numpy as np
    fx = np.load(os.path.join(ROOT, "oracle", "fixtures", "tree_inlet_section.npz"))
    flags, origin, dims = fx["flags"], [float(v) for v in fx["origin"]], [int(v) for v in fx["dims"]]
    h = max(3, min(int(levels), dims[1]))
    sub = flags[:, dims[1] - h:, :].copy()
    origin[1] += dims[1] - h
    params = {"inlet_plane": float(fx["inlet_plane"]), "inlet_center": [float(v) for v in fx["inlet_center"]],
              "tau": float(fx["tau"])}
    return (sub, tuple(origin), (dims[0], h, dims[2])), params


def levels_for(steps):
    """Section height whose reference run of `steps` steps takes about REF_SECONDS."""
    nodes_per_level = 4900.0        # fluid points per level of the section (inlet radius 40)
    return int(REF_SECONDS * REF_MLUPS_PER_CORE * 1e6 / (max(steps, 1) * nodes_per_level))


def run_reference_sample(params, sample, steps, workdir, tag, warmup=0):
    """One reference process on the sample; returns (fluid nodes, steps, seconds)."""
    from oracle import oracle as O
    sub, origin, dims = sample
    os.makedirs(workdir, exist_ok=True)
    fpath = os.path.join(workdir, f"flags_{tag}.bin")
    sub.tofile(fpath)
    stl = os.path.join(workdir, "one.stl")
    if not os.path.exists(stl):
        with open(stl, "w") as fh:
            fh.write("solid s\nfacet normal 0 0 1\nouter loop\nvertex 0 0 0\nvertex 1 0 0\nvertex 0 1 0\n"
                     "endloop\nendfacet\nendsolid s\n")
    plane = params["inlet_plane"]
    cx, cz = params["inlet_center"]
    pred = [(0, (1, repr(float(plane)), 1e-2, (cx - 44, math.nan, cz - 44), (cx + 44, math.nan, cz + 44)))]
    res = O.run_reference(stl, 1.0, grid=(origin, dims), preds=pred, tau=params["tau"], outlet_rho=1.0, steps=steps,
                          profile=None, amp=None, workdir=os.path.join(workdir, tag), flags_path=fpath,
                          warmup=warmup)
    t = res["time"]
    return t["nodes"], t["steps"], t["seconds"]


def reference_arm(args):
    """The reference's CPU step loop on all host cores (one process per core),
    `args.steps` timed steps after `args.warmup` untimed ones, on a section of
    the tree sized to that step count (this package's library is not loaded)."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    if not O.ref_available(19):
        try:
            O.build()
        except Exception:
            pass
    if not O.ref_available(19):
        return {"impl": "reference", "unavailable": "the reference checker (oracle/_ref) could not be built here"}
    sample, params = reference_sample(levels_for(args.steps + args.warmup))
    cores = os.cpu_count() or 1
    steps = args.steps
    wd = tempfile.mkdtemp(prefix="pv2013_refarm_")
    for d in range(cores):
        os.makedirs(os.path.join(wd, f"p{d}"), exist_ok=True)
    t0 = time.time()
    with ThreadPoolExecutor(max_workers=cores) as ex:
        res = list(ex.map(lambda d: run_reference_sample(params, sample, steps, wd, f"p{d}", args.warmup),
                          range(cores)))
    wall = time.time() - t0
    mlups = sum(n * s / sec for n, s, sec in res) / 1e6
    nodes = res[0][0]
    return {"metric": METRIC, "value": mlups, "unit": "MLUPS", "impl": "reference", "n_gpus": 0,
            "steps": steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": f"inlet section {sample[2][0]}x{sample[2][1]}x{sample[2][2]} "
                                                       f"points", "processes": cores},
            "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": cores, "kind": "reference",
                             "sample": f"{cores} concurrent reference processes, each {args.warmup} untimed + "
                                       f"{steps} timed steps on the "
                                       f"{nodes}-node inlet section of the tree ({sample[2][1]} of its 40 levels, "
                                       f"sized to the step count; reference voxelizer bypassed: flags from the "
                                       f"oracle); step-loop seconds only; wall {wall:.1f}s"},
            "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def gpu_arm(args, rank, world):
    import numpy as np
    import torch
    from pv2013_gb300 import Geometry, Simulation, cases
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    torch.cuda.init()
    peak, peak_kind = peaks()
    t0 = time.time()
    case = cases.vascular_tree(h=2.2)
    t_mesh = time.time() - t0
    geom = case.geometry()
    nf = geom.info.n_fluid
    specs = case.boundary_specs(geom)

    # --- headline: FP16-shifted storage, AA in-place streaming ---------------
    sim16 = Simulation(geom, case.tau, specs, precision="f16s", pattern=args.pattern, run_axis=0,
                       staging=args.staging, nodes_per_lane=args.nodes_per_lane, piece_slots=args.piece_slots)
    info16 = sim16.info()
    with ClockSampler(dev) as clk:
        if world > 1:
            torch.distributed.barrier()
        sec16 = time_steps(sim16, args.steps, args.warmup, torch, clk)
    sec16 = max_over_ranks(sec16, world, "cuda")
    mon = sim16.monitors()
    ms_step = sec16 / args.steps * 1e3
    mlups16 = nf * args.steps / sec16 / 1e6 * world
    bpu16 = info16.algorithmic_bytes_per_update
    del sim16

    # --- plain FP32 two-lattice pull: the engine's best FP32 kernel for it (two
    # nodes per lane), and the one-node-per-lane kernel beside it ------------
    sim32p = Simulation(geom, case.tau, specs, precision="f32", pattern="pull", run_axis=0, nodes_per_lane=2)
    sec32p = max_over_ranks(time_steps(sim32p, args.steps, args.warmup, torch), world, "cuda")
    mlups32p = nf * args.steps / sec32p / 1e6 * world
    del sim32p
    sim32 = Simulation(geom, case.tau, specs, precision="f32", pattern="pull", run_axis=0, staging=1,
                       nodes_per_lane=1)
    sec32 = max_over_ranks(time_steps(sim32, args.steps, args.warmup, torch), world, "cuda")
    mlups32 = nf * args.steps / sec32 / 1e6 * world
    del sim32

    # --- stated error: FP16 vs FP64 (FP64 is bit-exact with the CPU oracle) ----
    err_steps = args.err_steps
    s64 = Simulation(geom, case.tau, specs, precision="f64", pattern="pull", run_axis=0)
    s64.step(err_steps, graph=True)
    _, r64, u64 = s64.fields(f=False)
    m64 = s64.monitors()["mass"]
    del s64
    s16 = Simulation(geom, case.tau, specs, precision="f16s", pattern=args.pattern, run_axis=0, staging=args.staging,
                     nodes_per_lane=args.nodes_per_lane, piece_slots=args.piece_slots)
    m0 = s16.monitors()["mass"]
    s16.step(err_steps, graph=True)
    _, r16, u16 = s16.fields(f=False)
    m16 = s16.monitors()["mass"]
    del s16
    u_l2 = float(np.linalg.norm(u16 - u64) / np.linalg.norm(u64))
    u_max = float(np.abs(u16 - u64).max() / np.abs(u64).max())
    rho_drift = float(np.abs(r16 - r64).max())
    # open-system mass change of the FP16 run (inflow/outflow transient), and
    # the mass the FP16 storage loses against the FP64 run of the same steps
    mass_change_per_1000 = float((m16 - m0) / m0 / err_steps * 1000)
    mass_vs_fp64_per_1000 = float((m16 - m64) / m64 / err_steps * 1000)

    # --- end to end through the C ABI with host buffers -----------------------
    # the inputs (triangles) and outputs (rho, u) live in pinned host memory,
    # set up before the timed region
    e2e_steps = args.steps
    tris_host = torch.from_numpy(np.ascontiguousarray(case.triangles, dtype=np.float64)).pin_memory().numpy()
    rho_host = torch.empty(nf, dtype=torch.float64).pin_memory().numpy()
    u_host = torch.empty((nf, 3), dtype=torch.float64).pin_memory().numpy()
    torch.cuda.synchronize()
    t0 = time.time()
    g2 = Geometry(tris_host, case.spacing, grid=case.grid, predicates=case.predicates)   # H2D, voxelization, lists
    t1 = time.time()
    specs2 = case.boundary_specs(g2)               # inlet profile (host) from the inlet list
    s2 = Simulation(g2, case.tau, specs2, precision="f16s", pattern=args.pattern, run_axis=0,
                    staging=args.staging, nodes_per_lane=args.nodes_per_lane, piece_slots=args.piece_slots)
    torch.cuda.synchronize()
    t2 = time.time()
    s2.step(e2e_steps, graph=True)
    torch.cuda.synchronize()
    t3 = time.time()
    _, rho_h, u_h = s2.fields(f=False, out=(None, rho_host, u_host))
    torch.cuda.synchronize()
    t4 = time.time()
    e2e_sec = t4 - t0
    e2e_parts = {"geometry_s": t1 - t0, "lattice_build_s": t2 - t1, "steps_s": t3 - t2, "fields_d2h_s": t4 - t3,
                 "geometry_voxelize_ms": g2.info.voxelize_ms, "geometry_classify_ms": g2.info.classify_ms}
    e2e_mlups = nf * e2e_steps / e2e_sec / 1e6 * world
    del s2, g2
    h2d = tris_host.nbytes + 8 * len(case.inlet_profile(geom)) + 8 * len(case.amp_table())
    d2h = rho_h.nbytes + u_h.nbytes

    # --- batched: the 64-vessel ensemble in one launch per step --------------
    batched = None
    if not args.no_batch:
        # the 64 vessels are independent: under torchrun each rank advances its
        # share of them (balanced by fluid nodes, no exchange between ranks)
        from pv2013_gb300.shard import shard
        ens = cases.ensemble(64)
        egeo_all = [c.geometry() for c in ens]
        mine = shard([g.info.n_fluid for g in egeo_all], rank, world)
        ens = [ens[i] for i in mine]
        egeo = [egeo_all[i] for i in mine]
        enf = sum(g.info.n_fluid for g in egeo_all)      # all ranks' nodes
        esim = Simulation(egeo, [c.tau for c in ens], [c.boundary_specs(g) for c, g in zip(ens, egeo)],
                          precision="f16s", pattern=args.pattern, piece_slots=args.piece_slots)
        esim.step(1)                         # after an even launch both patterns are candidates
        tuned = esim.autotune(launches=10)
        esec = max_over_ranks(time_steps(esim, args.batch_steps, args.warmup, torch), world, "cuda")
        einfo = esim.info()
        batched = {"workload": "ensemble of 64 tortuous vessels (seeds 4000-4063), per-instance tau, inlet amplitude "
                               "and period, FP16-shifted AA, one launch per step",
                   "fluid_nodes": enf, "steps": args.batch_steps, "mlups": enf * args.batch_steps / esec / 1e6,
                   "sharding": f"{len(mine)} of 64 vessels on this rank, {world} rank(s), no exchange",
                   "ms_per_step": esec / args.batch_steps * 1e3,
                   "kernel": {"nodes_per_lane": einfo.nodes_per_lane, "piece_slots": einfo.piece_slots,
                              "warps_per_block": einfo.warps_per_block,
                              "pattern": {0: "pull", 1: "aa"}[einfo.pattern],
                              "candidates": len(tuned)}}
        del esim, egeo, egeo_all

    # --- roofline of the step kernel ------------------------------------------
    launch_s = sec16 / args.steps
    achieved = bpu16 * nf / launch_s / 1e9
    tr = profiled_traffic_bytes_per_node()
    traffic = tr.get("f16s_aa_dram_bytes_per_node")
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic * nf if traffic else None,
            "peak_kind": peak_kind, "bytes_per_update": bpu16}

    # --- CPU baseline: the reference's step loop on a bounded sample ----------
    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            from oracle import oracle as O
            if not O.ref_available(19):
                O.build()
            wd = tempfile.mkdtemp(prefix="pv2013_cpu_")
            sample, params = reference_sample(40)
            n, s, sec = run_reference_sample(params, sample, 30, wd, "p0", warmup=3)
            cpu = {"value": n * s / sec / 1e6, "unit": "MLUPS", "cores": 1, "kind": "reference",
                   "sample": f"{s} steps of the reference step loop on the {n}-node inlet section (96x40x96) of "
                             f"the tree, one process"}
        except Exception as e:  # the CPU baseline is reported, never required
            cpu = {"value": None, "unit": "MLUPS", "cores": 1, "kind": "reference", "sample": f"failed: {e}"}

    out = {
        "metric": METRIC, "value": mlups16, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f16-shifted storage, f32 math", "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": [512, 1024, 512], "fluid_nodes": nf, "triangles": len(case.triangles),
                   "precision": "f16s", "pattern": args.pattern, "run_axis": info16.run_axis,
                   "kernel": ("paired: 2 nodes/lane, f32x2 math" if info16.nodes_per_lane == 2 else
                              "1 node/lane, " + ("tma-staged" if args.staging == 0 else "direct loads")),
                   "piece_slots": info16.piece_slots, "warps_per_block": info16.warps_per_block,
                   "chunks": info16.n_chunks,
                   "l2": "populations exceed L2 (no flush needed)", "parallelism": f"replicas x{world}"},
        "fp32_pull_mlups": mlups32p, "f16_over_f32": mlups16 / mlups32p,
        "fp32_pull_plain": "FP32 storage and math, two-lattice pull, the engine's best kernel for it "
                           "(two nodes per lane)",
        "fp32_pull_one_node_mlups": mlups32, "f16_over_f32_one_node": mlups16 / mlups32,
        "error_vs_fp64": {"steps": err_steps, "u_rel_l2": u_l2, "u_rel_max": u_max, "rho_max_abs": rho_drift,
                          "mass_vs_fp64_per_1000_steps": mass_vs_fp64_per_1000,
                          "mass_change_per_1000_steps": mass_change_per_1000},
        "batched": batched,
        "roofline": roof, "cpu_baseline": cpu,
        "e2e": {"value": e2e_mlups, "unit": "MLUPS", "h2d_bytes_per_step": h2d / e2e_steps,
                "d2h_bytes_per_step": d2h / e2e_steps,
                "includes": "STL triangles H2D from pinned host memory, GPU voxelization, lattice build, steps, rho/u D2H into pinned host memory",
                "parts": e2e_parts},
        # kernels of the timed region: graphs of 64 step launches plus the
        # step-counter update, then the remaining steps as direct launches
        "gpu_launches": (args.steps // 64) * 65 + args.steps % 64,
        "voxelize_ms": geom.info.voxelize_ms, "mesh_s": t_mesh,
        "clocks": clk.summary(), "monitors_after": {k: mon[k] for k in ("mass", "max_speed", "nonfinite")},
    }
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--pattern", default="aa", choices=["aa", "pull"])
    ap.add_argument("--staging", type=int, default=1, help="0 = TMA-staged pipeline, 1 = direct loads")
    ap.add_argument("--nodes-per-lane", type=int, default=0, help="0 = engine default (paired), 1 or 2")
    ap.add_argument("--piece-slots", type=int, default=0, help="paired kernel: 8, 16 or 32 node slots per chunk "
                                                                   "piece; 0 = engine default (8)")
    ap.add_argument("--err-steps", type=int, default=2000,
                    help="steps of the FP16-vs-FP64 error statement (two inlet pulsation periods)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-vessel ensemble line")
    ap.add_argument("--batch-steps", type=int, default=1000)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(reference_arm(args)))
        return 0
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    out = gpu_arm(args, rank, world)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
