#!/usr/bin/env python3
"""Benchmark: cell-RK3-steps/s of the AFAR stage on the Mach 3 forward-facing-step workload.

Workload (one GPU): channel [0,3]x[0,1] with the step [0.6,3]x[0,0.2] removed, Delaunay
triangulation of ~1M seeded jittered points (jitter 0.3h), RCM-renumbered (--order hilbert: cells
along a Hilbert curve instead): about 2.0M triangles,
3.0M internal faces.  Inflow rho=1.4, p=1, u=3 (label 3), slip walls (label 2), outflow (label 4),
edge-neighbour stencils, R = 1/1.4, Cv = R/0.4, CFL 0.2, device-side CFL step every step.
Synthetic, seeded inputs; the working set (~1.5 GB) is larger than L2, so no L2 flush is needed.

Our arm (default): K timed steps per precision policy, graph-replayed, CUDA events on the solver's
stream; `value` is the mixed policy (FP32 reconstruction/flux, FP64 accumulation); the fp64 and ref
policies are reported beside it.  `e2e` is the same metric through the reference-shaped C ABI
(adjustTimeStep + GPUevolve each step, state uploaded from pinned host memory before and the
fields copied back after).  `cpu_baseline` is the CPU oracle (the reference's algorithm restated
in C, OpenMP on all host cores) on a bounded sample.  `reference_gpu` is the reference's own CUDA
kernels (compiled from its sources) on the same inputs.

--impl reference: the reference arm.  The reference has no CPU implementation of this path, so it
times the CPU restatement (oracle, ref policy, all host cores), a bounded number of steps per run.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-RK3-steps/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
PROFILE_STEPS = 10
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one mixed-policy reconstruct launch
# (tile-staged) per cell, by cell order, from ncu captures of the 500,094-cell version of this
# workload (traffic grows with the cells of the tile stream); None when no capture matches the
# current kernels (the tensor-map fetch; Hilbert order not captured with it).
RECON_TRAFFIC_BYTES_PER_CELL = {"rcm": 398.2, "hilbert": None}
# FP64 work per internal face of the fp64 policy's flux, averaged over a step's three launches (the
# first also reduces the Courant step), from the ncu instruction counts
# smsp__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum of the three launches on the
# 500,094-cell version of this workload (748,881 internal faces): instructions (DFMA + DADD + DMUL,
# divisions and square roots counted as the DFMA sequences they run as) and floating-point
# operations (2 per DFMA).  The FP64 pipe issues one such instruction per lane per cycle at its peak.
FP64_FLUX_INST_PER_FACE = 243.77
FP64_FLUX_FLOPS_PER_FACE = 360.17


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--points", type=int, default=1_000_000)
    ap.add_argument("--cfl", type=float, default=0.2)
    ap.add_argument("--chunk", type=int, default=50,
                    help="timed steps per chunk; every chunk restarts from the same post-warm-up state")
    ap.add_argument("--policies", default="mixed,fp64,ref")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the mixed-vs-FP64 accuracy pass of the main line")
    ap.add_argument("--floor-in-bench", action="store_true",
                    help="main line: also the FP64 policy against itself from a 1-ulp perturbed start")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--mesh", default="step", choices=["step", "riemann_mixed", "vortex"],
                    help="step: the metric's workload; riemann_mixed: the 4M-cell mixed quad/triangle case; "
                         "vortex: the 256^2 isentropic vortex in an outlet box (the small case without periodic "
                         "faces, which the reference's kernels also run)")
    ap.add_argument("--mixed-n", type=int, default=1766)
    ap.add_argument("--order", default="rcm", choices=["rcm", "hilbert"],
                    help="cell order of the workload's mesh: reverse Cuthill-McKee or a Hilbert curve")
    ap.add_argument("--recon", default="auto", choices=["auto", "tile", "register"],
                    help="mixed reconstruct variant: autotuned (default) or forced")
    ap.add_argument("--serve", action="store_true",
                    help="the serving workload instead: Poisson arrivals of solves through afar_server_*")
    ap.add_argument("--batch", action="store_true",
                    help="the batched workload instead: many independent solves stepped by one graph")
    ap.add_argument("--batch-solves", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=500)
    ap.add_argument("--batch-no-solo", action="store_true",
                    help="--batch: skip timing the solves one after another (e.g. for a launch list of the batch kernels)")
    ap.add_argument("--setup", action="store_true",
                    help="time the precompute of the workload's mesh on the host and with its RBF stage on the GPU")
    ap.add_argument("--accuracy", default="",
                    help="instead of timing: the mixed policy against the FP64 policy on the configs listed "
                         "(comma-separated: vortex, step, riemann_mixed, batch), L1/Linf of density and switch flips")
    ap.add_argument("--acc-steps", type=int, default=100, help="--accuracy step: RK3 steps of the Mach 3 start")
    ap.add_argument("--acc-sample", type=int, default=8, help="--accuracy batch: solves of the batch re-run")
    ap.add_argument("--floor", action="store_true",
                    help="--accuracy: also the FP64 policy against itself, on the same mesh in another cell order "
                         "(Hilbert curve instead of RCM: another summation order), from a 1-ulp perturbed start, and "
                         "from the start rounded to float")
    ap.add_argument("--cache-mesh", default="", help=argparse.SUPPRESS)  # helper: build the workload, save it
    ap.add_argument("--cpu-sample", default="", help=argparse.SUPPRESS)  # helper: time the oracle on a saved mesh
    ap.add_argument("--cpu-policy", default="ref", help=argparse.SUPPRESS)
    ap.add_argument("--cpu-threads", type=int, default=0, help=argparse.SUPPRESS)
    ap.add_argument("--sample-steps", type=int, default=5, help=argparse.SUPPRESS)
    ap.add_argument("--serve-requests", type=int, default=60)
    ap.add_argument("--serve-rate", type=float, default=50.0, help="arrivals per second")
    return ap.parse_args()


# ------------------------------------------------------------------------------------ distributed
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")  # host-side barrier and max only; no data-path collective
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ------------------------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return

        def reader():
            for line in self.proc.stdout:
                self.rows.append([x.strip() for x in line.split(",")])

        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        sm = []
        smax = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------------------------ workload
WORKLOADS = {
    "step": ("mach3_forward_step_tri", "synthetic (seeded Delaunay mesh, uniform Mach 3 inflow)"),
    "riemann_mixed": ("riemann4_mixed_quad_tri", "synthetic (quads with a seeded triangulated disk, four-quadrant "
                                                   "Riemann states)"),
    "vortex": ("isentropic_vortex_256x256_outlet_box", "synthetic (isentropic vortex, strength 5, free stream 1, "
                                                       "on 256 x 256 quads of [-7, 9]^2, outlets)"),
}


def make_workload(points: int, seed: int, cfl: float, kind: str = "step", mixed_n: int = 1766,
                  order: str = "rcm"):
    """step: the Mach 3 forward step (about points/2 x 4 triangles); riemann_mixed: the unit square
    of mixed_n^2 quads with the cells of a central disk (r = 0.3) split into seeded triangles (about
    4.0M cells at 1766), four-quadrant Riemann states, outlets all round; vortex: the isentropic
    vortex (strength 5, free stream 1) on 256 x 256 quads of [-7, 9]^2 with outlets all round."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh, precompute

    t0 = time.time()
    if kind == "riemann_mixed":
        m = mesh.riemann_mixed(mixed_n, seed=seed, renumber=order)
        W, Wb = mesh.riemann_fields(m)
    elif kind == "vortex":
        m = mesh.vortex_box(256, renumber=order)
        W = mesh.vortex_fields(m.cell_centres(), xc=0.0, yc=0.0)
        Wb = mesh.vortex_fields(m.boundary_face_centres(), xc=0.0, yc=0.0)
    else:
        m = mesh.forward_step_triangles(points, seed=seed, renumber=order)
        W, Wb = mesh.uniform_fields(m, 1.0, 3.0, 0.0, 1.0)
    cfg = CaseConfig(stencilType="edgeNeighbour", CFL=cfl)
    hf = precompute(m, cfg, W, Wb, want_rbf64=True)
    return m, hf, cfg, time.time() - t0


def algorithmic_bytes_per_step(hf, policy: str) -> float:
    """Compulsory HBM bytes of one RK3 step (three stages + the CFL step), counting each compulsory
    array once per stage and no intermediate (gradients, limiters, flags, face values, fluxes):
      B_stage = sum_cells [8 wW + 96 + 24 + 2 m wO + 4 S + 4 m + 2]
              + sum_internal_faces [40 + 8 + (S_own + 1 + S_nei + 1) wO]
              + sum_boundary_faces [40 + 4 + 1 + 4 wW]
      B_step  = 3 B_stage + Nc (4 wW + 16) + 48 Nf
    wW = bytes per primitive word (8 ref/fp64, 4 mixed); wO = operator word (4 ref/mixed, 8 fp64)."""
    wW = 4 if policy == "mixed" else 8
    wO = 8 if policy == "fp64" else 4
    S = hf.stencilSize.astype(np.float64)
    m = hf.compactStencilSize.astype(np.float64)
    nb = hf.neighbour.reshape(-1, 2)
    cells = np.sum(8 * wW + 96 + 24 + 2 * m * wO + 4 * S + 4 * m + 2)
    faces = np.sum(40 + 8 + (S[nb[:, 0]] + 1 + S[nb[:, 1]] + 1) * wO)
    bfaces = hf.nb * (40 + 4 + 1 + 4 * wW)
    return 3.0 * (cells + faces + bfaces) + hf.nc * (4 * wW + 16) + 48.0 * hf.nf


def reconstruct_bytes_per_launch(hf, policy: str) -> float:
    """Compulsory bytes of one reconstruct launch: its inputs read once and its outputs written once.
      per cell: W (4 wW), LS rows (2 m wO), stencil ids (4 S), face ids (4 m), counts (2), face
                geometry (2 x 2 words per face slot, 4 m wG), gradient out (8 wG), limiter out
                (4 wS), troubled flag out (1)
      per internal face: O3 weights of both sides ((S_own+1 + S_nei+1) wO; mixed, whose sums run in
                         difference form, reads no own-cell weight: (S_own + S_nei) wO), face values out (8 wG)
    wG = gradient/face-value word, wS = limiter word (4 for mixed, else 8 and 4/8)."""
    wW = 4 if policy == "mixed" else 8
    wO = 8 if policy == "fp64" else 4
    wG = 4 if policy == "mixed" else 8
    wS = 8 if policy == "fp64" else 4
    S = hf.stencilSize.astype(np.float64)
    m = hf.compactStencilSize.astype(np.float64)
    nb = hf.neighbour.reshape(-1, 2)
    cells = np.sum(4 * wW + 2 * m * wO + 4 * S + 4 * m + 2 + 4 * m * wG + 8 * wG + 4 * wS + 1)
    own_w = 0 if policy == "mixed" else 2
    faces = np.sum((S[nb[:, 0]] + S[nb[:, 1]] + own_w) * wO + 8 * wG)
    return float(cells + faces)


def peaks():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ------------------------------------------------------------------------------------ CPU legs
# The CPU baseline and the reference arm time the oracle (the reference's algorithm restated in C,
# OpenMP) in a process of its own: threads pinned (OMP_PROC_BIND=close, OMP_PLACES=cores) and counted,
# on the workload's mesh saved by another helper process.  So the timing process maps the oracle's
# library only, and both legs measure the same thing the same way.
CPU_SAMPLE_RK3 = 5  # RK3 steps of the full mesh per timed CPU "step" (a bounded sample)


def cpu_samples(steps: int, warmup: int):
    """Timed and warm-up CPU samples for a run of `steps` timed / `warmup` warm-up steps: the same
    counts, capped at 20 and 3 so the whole CPU leg stays within ~25 s and its 115 RK3 steps stay
    inside the ~180 this impulsive start runs before breaking down at the step corner."""
    return max(1, min(steps, 20)), max(1, min(warmup, 3))


def save_workload(hf, cfg, path: str):
    hf.save(path)
    with open(path + ".json", "w") as f:
        json.dump({"R": cfg.R, "Cv": cfg.Cv, "CFL": cfg.CFL}, f)


def cached_workload_subprocess(args, path: str):
    """Builds the workload's mesh and precompute in a helper process (it maps libafar) and saves it."""
    cmd = [sys.executable, os.path.abspath(__file__), "--cache-mesh", path, "--points", str(args.points),
           "--seed", str(args.seed), "--cfl", str(args.cfl), "--mesh", args.mesh, "--mixed-n", str(args.mixed_n),
           "--order", args.order]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("workload helper failed: " + r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def run_cache_mesh(args):
    m, hf, cfg, setup_s = make_workload(args.points, args.seed, args.cfl, args.mesh, args.mixed_n, args.order)
    save_workload(hf, cfg, args.cache_mesh)
    print(json.dumps({"cells": hf.nc, "internal_faces": hf.nf, "boundary_faces": hf.nb, "setup_s": setup_s}))


def cpu_rate_subprocess(path: str, threads: int, policy: str, samples: int, warmup: int,
                        sample_steps: int = CPU_SAMPLE_RK3):
    """The oracle timed in a pinned process of its own (see run_cpu_sample)."""
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PROC_BIND="close", OMP_PLACES="cores")
    cmd = [sys.executable, os.path.abspath(__file__), "--cpu-sample", path, "--cpu-threads", str(threads),
           "--cpu-policy", policy, "--steps", str(samples), "--warmup", str(warmup), "--sample-steps",
           str(sample_steps)]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("CPU sample failed: " + r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def run_cpu_sample(args):
    """Times the oracle on a saved mesh: `warmup` untimed then `steps` timed samples of sample_steps
    whole RK3 steps each (Courant step from the state each step); prints cell-steps/s."""
    from afar_cudaeuler2dmixo3rk3solver_gb300.solver import HostFields
    from oracle.oracle import Oracle, max_threads, set_threads

    hf = HostFields.load(args.cpu_sample)
    with open(args.cpu_sample + ".json") as f:
        gas = json.load(f)
    if args.cpu_threads > 0:
        set_threads(args.cpu_threads)
    o = Oracle(hf, gas["R"], gas["Cv"], args.cpu_policy)
    st = o.new_state()
    n = args.sample_steps

    def sample():
        for _ in range(n):
            o.evolve(st, o.delta_t(st["FD"], gas["CFL"]))

    for _ in range(args.warmup):
        sample()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sample()
    el = time.perf_counter() - t0
    W_ = st["FD"][:hf.nc]
    print(json.dumps({"value": hf.nc * n * args.steps / el, "unit": "cell-steps/s", "seconds": el,
                      "samples": args.steps, "warmup_samples": args.warmup, "rk3_steps_per_sample": n,
                      "threads": max_threads(), "policy": args.cpu_policy, "cells": hf.nc,
                      "pinning": "OMP_PROC_BIND=close OMP_PLACES=cores",
                      "affinity_cores": len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else None,
                      "finite": bool(np.isfinite(st["cFD"]).all() and (W_[:, 0] > 0).all())}))


def cpu_leg(path: str, samples: int, warmup: int, policy: str = "ref"):
    """The CPU baseline of a saved workload on all host cores, pinned (the reference arm's measure)."""
    nproc = os.cpu_count() or 1
    r = cpu_rate_subprocess(path, nproc, policy, samples, warmup)
    r["sample"] = (f"{r['samples']} samples of {r['rk3_steps_per_sample']} full RK3 steps (after "
                   f"{r['warmup_samples']} warm-up samples) of the {r['cells']}-cell mesh, CPU oracle ({policy} "
                   f"policy), {r['threads']} threads pinned, {r['seconds']:.1f} s")
    return r


def cpu_baseline_grid(path: str, workload: str, vortex_path: str, steps: int = 10):
    """The CPU oracle in its FP64 policy for a fixed number of RK3 steps, on all host cores and on
    one (pinned), on the benchmark mesh and on the 256 x 256 periodic isentropic vortex (the
    plain-FP64 small case): cell-steps/s of each."""
    nproc = os.cpu_count() or 1
    out = []
    for name, p in (("vortex_256x256_periodic", vortex_path), (workload, path)):
        for threads in sorted({nproc, 1}, reverse=True):
            r = cpu_rate_subprocess(p, threads, "fp64", 1, 1, sample_steps=steps)
            out.append({"mesh": name, "cells": r["cells"], "policy": "fp64", "threads": r["threads"], "steps": steps,
                        "seconds": round(r["seconds"], 3), "value": r["value"], "unit": "cell-steps/s",
                        "pinning": r["pinning"], "finite": r["finite"]})
    return out


def run_reference_arm(args, dist: Dist):
    """The reference arm: the reference has no CPU implementation of this path, so this times its
    algorithm restated in C (the oracle, ref policy) on all host cores, pinned.  The mesh comes from
    a helper process; this process maps neither libafar nor the oracle."""
    if dist.rank != 0:
        return
    import shutil
    import tempfile

    tmp = tempfile.mkdtemp(prefix="afar_bench_")
    try:
        path = os.path.join(tmp, "workload.npz")
        info = cached_workload_subprocess(args, path)
        K, W = cpu_samples(args.steps, args.warmup)
        r = cpu_leg(path, K, W)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    rate = r["value"]
    line = {
        "metric": METRIC, "value": rate, "unit": "cell-steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["seconds"] / r["samples"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": WORKLOADS[args.mesh][1],
        "impl": "reference",
        "config": {"workload": WORKLOADS[args.mesh][0], "cells": info["cells"], "internal_faces": info["internal_faces"],
                   "boundary_faces": info["boundary_faces"], "points": args.points, "cfl": args.cfl,
                   "stencil": "edgeNeighbour", "cell_order": args.order, "parallelism": "replicas",
                   "step": f"one step = a sample of {CPU_SAMPLE_RK3} full RK3 steps of the mesh; "
                           f"{r['samples']} timed after {r['warmup_samples']} warm-up samples"},
        "cpu_baseline": {"value": rate, "unit": "cell-steps/s", "cores": r["threads"], "kind": "port",
                         "sample": r["sample"], "pinning": r["pinning"]},
        "e2e": {"value": rate, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference has no CPU implementation of the path; this is its algorithm restated in C "
                "(oracle/afar_oracle.c), OpenMP over all host threads, pinned",
    }
    print(json.dumps(line), flush=True)


def reference_gpu_rate(hf, cfg, steps: int):
    """The reference's own kernels (cubin compiled from its sources) on the same inputs: its time
    loop (adjustTimeStep with the host round trip, then GPUevolve) and the kernels alone."""
    from oracle import ref_harness

    ref_harness.build()
    if not ref_harness.available():
        return None
    r = ref_harness.RefKernels(hf)
    dt = r.adjust_dt(cfg.R, cfg.Cv, cfg.CFL)
    r.evolve(2, cfg.R, cfg.Cv, dt)
    t0 = time.perf_counter()
    for _ in range(steps):
        dt = r.adjust_dt(cfg.R, cfg.Cv, cfg.CFL)
        r.evolve(1, cfg.R, cfg.Cv, dt)
    loop_s = time.perf_counter() - t0
    ms = r.evolve(steps, cfg.R, cfg.Cv, dt)
    r.close()
    return {"value": hf.nc * steps / loop_s, "unit": "cell-steps/s", "kernels_only": hf.nc * steps / (ms * 1e-3),
            "sample": f"{steps} steps of the same mesh", "cubin": os.path.basename(ref_harness.cubin_path()),
            "note": "reference kernels compiled from its sources for Blackwell; time loop with adjustTimeStep"}


def run_ours(args, dist: Dist):
    import ctypes as C

    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver, _ffi
    from afar_cudaeuler2dmixo3rk3solver_gb300 import build as b

    b.build_all()
    device = dist.local
    m, hf, cfg, setup_s = make_workload(args.points, args.seed, args.cfl, args.mesh, args.mixed_n, args.order)
    K, Wm = args.steps, max(3, args.warmup)
    hbm, peak_kind = peaks()
    policies = [p for p in args.policies.split(",") if p]
    results = {}
    sampler = ClockSampler(device)
    solvers = {}
    chunks = [min(args.chunk, K - i) for i in range(0, K, args.chunk)]
    for pol in policies:
        s = CudaSolver(hf, cfg, policy=pol, device=device)
        if pol == "mixed" and args.recon != "auto":
            s.set_tuning(0 if args.recon == "tile" else 1)
        s.run(Wm)  # warm-up steps (graph capture, first touch)
        s.save()   # every timed chunk restarts here, so every timed step is a physical one
        solvers[pol] = s
    dist.barrier()
    sampler.start()
    for pol in policies:
        s = solvers[pol]
        ms = 0.0
        finite = True
        for n in chunks:
            s.restore()
            s.synchronize()
            dist.barrier()
            ms += dist.max(s.run_timed(n))
            st = s.state()
            W_ = st["FD"][:hf.nc]
            finite &= bool(np.isfinite(st["cFD"]).all() and (W_[:, 0] > 0).all() and (W_[:, 3] > 0).all())
        results[pol] = {"ms": ms, "finite": finite, "launches": s.launches_per_step()}
    clocks = sampler.stop()
    for pol in policies:
        s = solvers[pol]
        s.restore()
        # per-kernel device time: CUDA events between the stage kernels on the solver's stream,
        # averaged over PROFILE_STEPS steps from the post-warm-up state
        acc = {}
        for _ in range(PROFILE_STEPS):
            for k, v in s.profile_step().items():
                acc[k] = acc.get(k, 0.0) + v / PROFILE_STEPS
        results[pol]["kernels_ms"] = acc
        results[pol]["device_bytes"] = s.device_bytes()
        if pol == "mixed":
            results[pol]["tuning"] = s.tuning()
        results[pol]["switch_counts"] = s.switch_counts()  # the last profiled stage's decisions

    # e2e through the reference-shaped C ABI with host buffers (mixed policy)
    pol0 = policies[0]
    import torch

    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    FD_h, cFD_h = pin(hf.FD), pin(hf.cFD)
    out_FD = pin(np.zeros_like(hf.FD))
    out_si = pin(np.zeros(2 * (hf.nc + hf.nb), dtype=np.int8))
    s = solvers[pol0]
    s.synchronize()
    dist.barrier()
    check = _ffi.check
    L = _ffi.lib()
    sz = hf.sizes
    dtv = C.c_double()
    fp = _ffi.FieldPointer()
    fp.FD = out_FD.ctypes.data
    fp.shockIndicator = out_si.ctypes.data
    t0 = time.perf_counter()
    for n in chunks:  # per chunk: state in from pinned host memory, n reference-shaped steps, fields out
        check(L.afar_upload_state(s.h, FD_h.ctypes.data, cFD_h.ctypes.data, cFD_h.ctypes.data))
        for _ in range(n):
            check(L.afar_adjustTimeStep(s.h, hf.nf, cfg.R, cfg.Cv, cfg.CFL, C.byref(dtv)))
            check(L.afar_GPUevolve(s.h, cfg.R, cfg.Cv, dtv.value, sz["cellsNum"], sz["facesNum"],
                                   sz["totalBoundaryFacesNum"], sz["maxStencilSize"], sz["maxCompactStencilSize"],
                                   sz["maxLocalBlockStencilSize"], sz["maxCompactLocalBlockStencilSize"]))
        check(L.afar_copyFieldDataDeviceToHost(C.byref(fp), s.h, hf.nc, hf.nb))
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_finite = bool(np.isfinite(out_FD).all() and (out_FD[:hf.nc, 0] > 0).all())
    h2d = (FD_h.nbytes + cFD_h.nbytes) * len(chunks) / K + 24  # cFDold is cFD: copied on the device
    d2h = (out_FD.nbytes + out_si.nbytes) * len(chunks) / K + 8

    # accuracy of the timed (first) policy against the FP64 policy on this mesh, over the steps a timed
    # chunk covers from the start (warm-up + chunk), stepped side by side with the FP64 Courant step
    accuracy = None
    if pol0 == "mixed" and not args.no_accuracy:
        nacc = Wm + max(chunks)
        accuracy, _, _ = accuracy_pair(hf, cfg, device, n_steps=nacc, every=max(1, nacc // 5))
        accuracy["what"] = (f"mixed against the FP64 policy after {nacc} RK3 steps from the workload's start (the "
                            f"{Wm} warm-up steps and a timed chunk), same step sizes; area-weighted L1 and L-inf of "
                            f"density, cells whose final switch differs")
        if args.floor_in_bench:
            accuracy["fp64_floor_perturbed_start"] = fp64_perturbation_floor(hf, cfg, device, n_steps=nacc)
    fp64_peak = None
    if "fp64" in policies:
        try:
            gf, pms = C.c_double(), C.c_float()
            _ffi.check(L.afar_measure_fp64_peak(device, C.byref(gf), C.byref(pms)))
            fp64_peak = {"gflops": gf.value, "launch_ms": pms.value,
                         "method": "independent DFMA chains on every SM, CUDA events, best of 5 (afar_measure_fp64_peak)"}
        except Exception as e:  # report, do not fail the bench
            fp64_peak = {"unavailable": str(e)[:200]}

    cpu = None
    refgpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        import shutil
        import tempfile

        from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh, precompute

        tmp = tempfile.mkdtemp(prefix="afar_bench_")
        try:
            path = os.path.join(tmp, "workload.npz")
            save_workload(hf, cfg, path)
            vm = mesh.periodic_quad_grid(256, 256, 0.0, 10.0, 0.0, 10.0)
            vcfg = CaseConfig(stencilType="edgeNeighbour", CFL=0.5)
            vpath = os.path.join(tmp, "vortex.npz")
            save_workload(precompute(vm, vcfg, mesh.vortex_fields(vm.cell_centres()), None, want_rbf64=True), vcfg,
                          vpath)
            Kc, Wc = cpu_samples(K, args.warmup)
            r = cpu_leg(path, Kc, Wc)
            cpu = {"value": r["value"], "unit": "cell-steps/s", "cores": r["threads"], "kind": "port",
                   "sample": r["sample"], "pinning": r["pinning"], "nproc": os.cpu_count(),
                   "fp64_fixed_steps": cpu_baseline_grid(path, WORKLOADS[args.mesh][0], vpath)}
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
    if dist.rank == 0 and not args.no_reference_gpu:
        try:
            refgpu = reference_gpu_rate(hf, cfg, min(K, 50))
        except Exception as e:  # the harness is test infrastructure; report, do not fail the bench
            refgpu = {"unavailable": str(e)[:200]}

    for s in solvers.values():
        s.close()
    if dist.rank != 0:
        return
    n = dist.world
    head = results[pol0]
    ms_step = head["ms"] / K
    value = n * hf.nc * K / (head["ms"] * 1e-3)
    bstep = algorithmic_bytes_per_step(hf, pol0)
    step_gbps = bstep / (ms_step * 1e-3) / 1e9
    prof = head["kernels_ms"]
    tot = sum(prof.values())
    dom = max(prof, key=prof.get)
    # the dominant kernel (reconstruct, three launches per step)
    b_launch = reconstruct_bytes_per_launch(hf, pol0)
    t_launch = prof["reconstruct"] / 3.0
    achieved = b_launch / (t_launch * 1e-3) / 1e9
    tuning = head.get("tuning")
    tile = tuning is not None and tuning["recon_variant"] == 0
    per_cell = (RECON_TRAFFIC_BYTES_PER_CELL or {}).get(args.order) if args.mesh == "step" else None
    traffic = per_cell * hf.nc if per_cell is not None and pol0 == "mixed" and tile else None
    recon_kind = ("reconstruct (mixed, tile-staged)" if tile else "reconstruct (mixed, register pass)"
                  if pol0 == "mixed" else f"reconstruct ({pol0}, staged)")
    by_policy = {}
    for pol in policies:
        r = results[pol]
        b_s = algorithmic_bytes_per_step(hf, pol)
        by_policy[pol] = {
            "value": hf.nc * K / (r["ms"] * 1e-3), "ms_per_step": r["ms"] / K, "finite": r["finite"],
            "algorithmic_GBps": b_s / (r["ms"] / K * 1e-3) / 1e9, "bytes_per_cell_step": b_s / hf.nc,
            "hbm_frac": b_s / (r["ms"] / K * 1e-3) / 1e9 / hbm,
            "kernels_ms_per_step": r["kernels_ms"], "launches_per_step": r["launches"],
            "device_bytes": r["device_bytes"], "switch_counts": r["switch_counts"],
        }
    if "fp64" in by_policy and fp64_peak and "gflops" in fp64_peak:
        # the fp64 policy's flux is bound by the FP64 pipe: its FP64 instructions per launch (the ncu
        # counts per face above) over its CUDA-event launch time, against the measured DFMA issue rate
        flux_ms = results["fp64"]["kernels_ms"]["flux"] / 3.0
        inst = FP64_FLUX_INST_PER_FACE * hf.nf
        flops = FP64_FLUX_FLOPS_PER_FACE * hf.nf
        peak_inst = fp64_peak["gflops"] / 2.0  # DFMA instructions per second (G)
        by_policy["fp64"]["fp64_roofline"] = {
            "bound": "fp64 pipe", "kernel": "flux (fp64)", "peak_gflops": fp64_peak["gflops"],
            "peak_method": fp64_peak["method"], "launch_ms": flux_ms,
            "fp64_inst_per_face": FP64_FLUX_INST_PER_FACE, "fp64_flops_per_face": FP64_FLUX_FLOPS_PER_FACE,
            "achieved_ginst_per_s": inst / (flux_ms * 1e-3) / 1e9,
            "frac": inst / (flux_ms * 1e-3) / 1e9 / peak_inst,
            "achieved_gflops": flops / (flux_ms * 1e-3) / 1e9,
            "flops_frac": flops / (flux_ms * 1e-3) / 1e9 / fp64_peak["gflops"],
            "frac_is": "FP64 instructions issued per second over the peak DFMA issue rate (the pipe's occupancy); "
                       "flops_frac counts DADD and DMUL as one operation against the DFMA's two",
            "note": "hbm_frac is the whole fp64 step's algorithmic bytes over the HBM peak; its flux and update "
                    "are bound by the FP64 pipe, not by memory"}
    line = {
        "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": n, "steps": K, "warmup": Wm,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if pol0 == "mixed" else "f64",
        "data": WORKLOADS[args.mesh][1],
        "config": {"workload": WORKLOADS[args.mesh][0], "policy": pol0, "cells": hf.nc, "internal_faces": hf.nf,
                   "boundary_faces": hf.nb, "points": args.points, "cfl": args.cfl, "stencil": "edgeNeighbour",
                   "max_stencil": hf.sizes["maxStencilSize"], "cell_order": args.order,
                   "dt": "device CFL step every step",
                   "l2": ("working set > L2 (no flush needed)" if hf.nc >= 1_000_000 else
                          "working set fits in L2: steps run back to back, as a solve does"),
                   "parallelism": "replicas" if n > 1 else "single",
                   "timed_chunks": chunks, "chunk_start": f"state after {Wm} warm-up steps (device snapshot)",
                   "setup_s": round(setup_s, 1)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "peak_kind": peak_kind, "kernel": recon_kind, "autotune": tuning,
                     "algorithmic_bytes_per_launch": b_launch, "launch_ms": t_launch,
                     "dominant_kernel": dom, "dominant_share": prof[dom] / tot if tot else None,
                     "step": {"algorithmic_bytes": bstep, "achieved_GBps": step_gbps, "frac": step_gbps / hbm}},
        "clocks": clocks,
        "gpu_launches": K * head["launches"] + 1,
        "e2e": {"value": n * hf.nc * K / e2e_s, "unit": "cell-steps/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "finite": e2e_finite,
                "path": "per chunk: afar_upload_state (pinned host), n x (afar_adjustTimeStep + afar_GPUevolve), "
                        "afar_copyFieldDataDeviceToHost"},
        "accuracy": accuracy,
        "policies": by_policy,
        "cpu_baseline": cpu,
        "reference_gpu": refgpu,
    }
    print(json.dumps(line), flush=True)


def run_serve(args, dist: Dist):
    """Serving workload: requests arrive as a Poisson process (rate --serve-rate); each takes a mesh
    drawn log-uniformly from a pool of quad Riemann problems of 10k-2M cells and a step count
    uniform in [100, 2000], stopped earlier at t = 0.3 (the four-quadrant problem's usual end; the
    coarsest mesh breaks down near t = 0.75), solved in the mixed policy; a 5% sample is also
    re-solved in the fp64 policy on a second server, both to the same end time, and compared.  Each
    server has a 180 GB budget and 50-step chunks; a request's latency runs from submit to its
    fields being back in its host buffers.  The pool's precompute is outside the timed region
    (request inputs are resident host arrays).  Prints served cell-steps/s of the mixed requests,
    the latency percentiles and the sample's accuracy."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, CudaSolver, Server, mesh, precompute
    from afar_cudaeuler2dmixo3rk3solver_gb300 import build as b

    b.build_all()  # with several ranks, each serves its own queue on its own GPU (replicas)
    rng = np.random.default_rng(args.seed + 17 * dist.rank)
    pool = []
    for n in (100, 224, 500, 1000, 1414):
        m = mesh.quad_grid(n, n, 0.0, 1.2, 0.0, 1.0)
        W, Wb = mesh.riemann_fields(m)
        cfg = CaseConfig(stencilType="faceNeighbour", CFL=0.3)
        pool.append((precompute(m, cfg, W, Wb, want_rbf64=True), cfg))
    sizes = np.array([hf.nc for hf, _ in pool], dtype=np.float64)
    logp = np.log(sizes)
    nreq = args.serve_requests
    pick = [int(np.argmin(np.abs(logp - rng.uniform(logp[0], logp[-1])))) for _ in range(nreq)]
    steps = rng.integers(100, 2001, nreq)
    fp64 = rng.uniform(size=nreq) < 0.05  # the sample re-solved in FP64
    gaps = rng.exponential(1.0 / args.serve_rate, nreq)
    # A sampled request and its FP64 re-solve end at the same time: t_s = min(0.3, 0.8 x its steps x
    # the mesh's initial Courant step), with room for three times its steps (both land on t_s).
    dt0 = []
    for hf, cfg in pool:
        s_ = CudaSolver(hf, cfg, policy="mixed", device=dist.local)
        dt0.append(s_.set_delta_t())
        s_.close()
    t_sample = {i: min(0.3, 0.8 * int(steps[i]) * dt0[pick[i]]) for i in range(nreq) if fp64[i]}
    servers = {p: Server(p, device=dist.local, hbm_budget_bytes=180 << 30, chunk_steps=50) for p in ("mixed", "fp64")}
    for srv in servers.values():
        srv.wait(srv.submit(*pool[0], n_steps=5))
    dist.barrier()
    t0 = time.perf_counter()
    ids = []
    resolve = {}
    accuracy = []
    t_next = t0
    for i in range(nreq):
        t_next += gaps[i]
        while time.perf_counter() < t_next:
            time.sleep(min(1e-3, max(0.0, t_next - time.perf_counter())))
        if fp64[i]:
            kw = {"t_end": t_sample[i], "n_steps": 3 * int(steps[i])}
            resolve[i] = servers["fp64"].submit(*pool[pick[i]], **kw)
        else:
            kw = {"t_end": 0.3, "n_steps": int(steps[i])}
        ids.append((servers["mixed"], servers["mixed"].submit(*pool[pick[i]], **kw)))
    lat = []
    done_steps = []
    results = {}
    ok = True
    for i, (srv, rid) in enumerate(ids):
        FD, si, ms, n = srv.wait(rid, with_steps=True)
        lat.append(ms)
        done_steps.append(n)
        ok = ok and bool(np.isfinite(FD).all())
        if fp64[i]:
            results[i] = (FD, si, n)
    wall = dist.max(time.perf_counter() - t0)  # the served (mixed) requests; the re-solves may run on
    fp64_work = 0.0
    for i, rid in resolve.items():
        FD, si, ms, n = servers["fp64"].wait(rid, with_steps=True)
        fp64_work += sizes[pick[i]] * n
        hf, cfg = pool[pick[i]]
        FDm, sim, nm = results[i]
        rho = lambda F: F[:hf.nc, 0] / (cfg.R * F[:hf.nc, 3])
        V = hf.cellVolume
        d = np.abs(rho(FDm) - rho(FD))
        accuracy.append({"request": i, "cells": hf.nc, "t": t_sample[i], "steps_mixed": nm, "steps_fp64": n,
                         "landed": bool(nm < 3 * int(steps[i]) and n < 3 * int(steps[i])),
                         "L1_rho": float(np.sum(d * V) / np.sum(V)), "Linf_rho": float(d.max()),
                         "switch_flips": int(np.count_nonzero(si[1:2 * hf.nc:2] != sim[1:2 * hf.nc:2]))})
    st = {p: srv.stats() for p, srv in servers.items()}
    for srv in servers.values():
        srv.close()
    work = dist.sum(float(sum(sizes[pick[i]] * done_steps[i] for i in range(nreq))))
    if dist.rank != 0:
        return
    lat = np.array(lat)
    print(json.dumps({
        "metric": "served cell-RK3-steps/s", "value": work / wall, "unit": "cell-steps/s", "n_gpus": dist.world,
        "higher_is_better": True, "data": "synthetic (quad Riemann meshes 10k-2M cells, seeded)",
        "config": {"workload": "serve_poisson", "requests": nreq, "rate_per_s": args.serve_rate,
                   "steps": "U[100,2000], at most to t = 0.3", "policy": "mixed; a 5% sample re-solved in fp64",
                   "chunk_steps": 50, "budget_bytes": 180 << 30, "fp64_resolves": int(fp64.sum())},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "max": float(lat.max())},
        "wall_s": wall, "peak_running": {p: v["peakRunning"] for p, v in st.items()},
        "peak_bytes": {p: v["peakBytes"] for p, v in st.items()}, "finite": ok,
        "fp64_resolve_cell_steps": fp64_work,
        "accuracy": {"what": "per sampled request: the mixed result against its FP64 re-solve at the same "
                             "end time (area-weighted L1 and L-inf of density, cells whose final switch differs)",
                     "requests": accuracy},
    }), flush=True)


def compare_policies(hf, a, b):
    """Mixed state b against FP64 state a on the cells: area-weighted L1 and the L-inf of the
    density, and the cells whose troubled-cell flag (si[2c]) or final switch (si[2c+1]) differ."""
    V = hf.cellVolume
    ra, rb = a["cFD"][:, 0], b["cFD"][:, 0]
    d = np.abs(ra - rb)
    nc = hf.nc
    sa, sb = a["shockIndicator"][:2 * nc], b["shockIndicator"][:2 * nc]
    l1 = float(np.sum(d * V) / np.sum(V))
    return {"L1_rho": l1, "Linf_rho": float(d.max()), "rel_L1_rho": l1 / float(np.sum(np.abs(ra) * V) / np.sum(V)),
            "switch_flips": int(np.count_nonzero(sa[1::2] != sb[1::2])),
            "troubled_flips": int(np.count_nonzero(sa[0::2] != sb[0::2])),
            "finite": bool(np.isfinite(ra).all() and np.isfinite(rb).all())}


def accuracy_pair(hf, cfg, device, t_end=0.0, n_steps=0, every=10, init=None):
    """The FP64 policy (checked against the CPU oracle at 1e-10 on small meshes, the FP64 oracle at
    this scale) and the mixed policy stepped side by side with the same step sizes -- the FP64
    policy's Courant step, clipped to t_end -- from the same initial state.  Every `every` steps the
    states and switch decisions are compared; returns the final comparison, the largest L1 seen and
    the flips summed over the compared steps."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver

    f = CudaSolver(hf, cfg, policy="fp64", device=device)
    m = CudaSolver(hf, cfg, policy="mixed", device=device)
    if init is not None:
        for s in (f, m):
            s.upload_state(FD=init[0], cFD=init[1], cFDold=init[1])
    t, k = 0.0, 0
    worst, sw_sum, tr_sum, samples = 0.0, 0, 0, 0
    while (n_steps and k < n_steps) or (not n_steps and t < t_end * (1.0 - 1e-12)):
        dt = f.set_delta_t()
        if t_end > 0.0:
            dt = min(dt, t_end - t)
        f.evolve(dt)
        m.evolve(dt)
        t += dt
        k += 1
        if k % every == 0:
            c = compare_policies(hf, f.state(), m.state())
            worst = max(worst, c["L1_rho"])
            sw_sum += c["switch_flips"]
            tr_sum += c["troubled_flips"]
            samples += 1
    a, b = f.state(), m.state()
    out = compare_policies(hf, a, b)
    out.update({"steps": k, "t": f.time()[0], "max_L1_rho_over_run": max(worst, out["L1_rho"]),
                "compared_steps": samples, "switch_flips_summed": sw_sum, "troubled_flips_summed": tr_sum})
    f.close()
    m.close()
    return out, a, b


def fp64_perturbation_floor(hf, cfg, device, n_steps=0, t_end=0.0, every=10, init=None, seed=1, kind="ulp"):
    """The FP64 policy against itself from a perturbed start, with the same step sizes.  kind "ulp":
    each stored double moved up or down one unit in the last place at random -- how far rounding
    alone carries two FP64 solves apart on this configuration (the floor under any mixed-precision
    form's difference from FP64).  kind "float": every stored value rounded to the nearest float --
    a one-time perturbation of the size FP32 storage makes (2^-24 relative), showing how much of a
    mixed-precision form's difference the configuration's sensitivity to a perturbation of that
    size explains, however precisely its switches are then evaluated."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver

    a = CudaSolver(hf, cfg, policy="fp64", device=device)
    b = CudaSolver(hf, cfg, policy="fp64", device=device)
    FD0, U0 = (hf.FD, hf.cFD) if init is None else (np.concatenate([init[0], hf.FD[hf.nc:]]), init[1])
    rng = np.random.default_rng(seed)

    def ulp_nudge(x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if kind == "float":
            return x.astype(np.float32).astype(np.float64)
        return np.where(rng.integers(0, 2, x.shape) == 1, np.nextafter(x, np.inf), np.nextafter(x, -np.inf))

    a.upload_state(FD=FD0, cFD=U0, cFDold=U0)
    Up = ulp_nudge(U0)
    FDp = np.array(FD0, dtype=np.float64, copy=True)
    FDp[:hf.nc] = ulp_nudge(FDp[:hf.nc])
    b.upload_state(FD=FDp, cFD=Up, cFDold=Up)
    t, k, worst = 0.0, 0, 0.0
    while (n_steps and k < n_steps) or (not n_steps and t < t_end * (1.0 - 1e-12)):
        dt = a.set_delta_t()
        if t_end > 0.0:
            dt = min(dt, t_end - t)
        a.evolve(dt)
        b.evolve(dt)
        t += dt
        k += 1
        if k % every == 0:
            worst = max(worst, compare_policies(hf, a.state(), b.state())["L1_rho"])
    out = compare_policies(hf, a.state(), b.state())
    out.update({"steps": k, "max_L1_rho_over_run": max(worst, out["L1_rho"]),
                "what": ("FP64 policy vs itself from a start perturbed by 1 ulp per stored value, same step sizes"
                         if kind == "ulp" else
                         "FP64 policy vs itself from the start rounded to float (2^-24 relative), same step sizes")})
    a.close()
    b.close()
    return out


def fp64_reorder_floor(make_mesh, make_fields, cfg, device, n_steps=0, t_end=0.0, every=10):
    """The FP64 policy against itself on the same mesh with its cells in another order (reverse
    Cuthill-McKee as generated, and along a Hilbert curve): the face and stencil lists, and so every
    summation, follow the numbering, and the O3 weights are solved with the stencil rows permuted.
    Both solves take the first one's step sizes; the states are compared cell for cell (matched by
    centroid).  make_mesh(order) builds the mesh in "rcm" or "hilbert" order; make_fields(mesh) ->
    (W, Wb, U or None)."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver, precompute

    m, m2 = make_mesh("rcm"), make_mesh("hilbert")
    c1, c2 = m.cell_centres(), m2.cell_centres()
    o1, o2 = np.lexsort((c1[:, 1], c1[:, 0])), np.lexsort((c2[:, 1], c2[:, 0]))
    to2 = np.empty(m.n_cells, dtype=np.int64)
    to2[o1] = o2  # cell i of m is cell to2[i] of m2
    assert np.array_equal(c1, c2[to2]), "cell centroids do not match between the two orders"
    solvers, hfs = [], []
    for mm in (m, m2):
        W, Wb, U = make_fields(mm)
        hf = precompute(mm, cfg, W, Wb, want_rbf64=True, device=device)
        s = CudaSolver(hf, cfg, policy="fp64", device=device)
        if U is not None:
            s.upload_state(FD=np.concatenate([W, hf.FD[hf.nc:]]), cFD=U, cFDold=U)
        solvers.append(s)
        hfs.append(hf)
    a, b = solvers

    def cmp():
        sa, sb = a.state(), b.state()
        si = sb["shockIndicator"]
        sb = {"cFD": sb["cFD"][to2],
              "shockIndicator": np.stack([si[0:2 * hfs[1].nc:2][to2], si[1:2 * hfs[1].nc:2][to2]], axis=1).reshape(-1)}
        return compare_policies(hfs[0], sa, sb)

    t, k, worst = 0.0, 0, 0.0
    while (n_steps and k < n_steps) or (not n_steps and t < t_end * (1.0 - 1e-12)):
        dt = a.set_delta_t()
        if t_end > 0.0:
            dt = min(dt, t_end - t)
        a.evolve(dt)
        b.evolve(dt)
        t += dt
        k += 1
        if k % every == 0:
            worst = max(worst, cmp()["L1_rho"])
    out = cmp()
    out.update({"steps": k, "t": t, "max_L1_rho_over_run": max(worst, out["L1_rho"]),
                "what": "FP64 policy vs itself, cells in RCM vs Hilbert-curve order (other summation orders), "
                        "same step sizes"})
    a.close()
    b.close()
    return out


def run_accuracy(args, dist: Dist):
    """Accuracy of the mixed policy against the FP64 policy, per config: the periodic isentropic
    vortex (256^2 quads on [0,10]^2, CFL 0.5, to t = 2; also against the exact solution), the
    Mach 3 step (--acc-steps RK3 steps at CFL 0.2 from the impulsive start: the scheme has no
    positivity fix and the start breaks down at the step corner after ~180 steps, so t = 4 is out
    of reach in every policy), the 4M-cell mixed quad/triangle Riemann problem to t = 0.3, and a
    sample of the batched ramps (500 steps each).  One JSON line per config."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, gauss_quadrature, mesh, precompute
    from afar_cudaeuler2dmixo3rk3solver_gb300 import build as b

    b.build_all()
    dev = dist.local
    out = []
    for name in [x.strip() for x in args.accuracy.split(",") if x.strip()]:
        t0 = time.time()
        line = {"metric": "mixed vs FP64 policy", "config": name,
                "steps_dt": "shared: the FP64 policy's Courant step each step"}
        if name == "vortex":
            m = mesh.periodic_quad_grid(256, 256, 0.0, 10.0, 0.0, 10.0)
            cfg = CaseConfig(stencilType="edgeNeighbour", CFL=0.5)
            q = gauss_quadrature(m, cfg)
            U0 = mesh.vortex_cell_averages(m, q, 0.0, centre=(5.0, 5.0))
            W0 = mesh.primitive_from_conserved(U0)
            hf = precompute(m, cfg, W0, None, want_rbf64=True, device=dev)
            r, a, bb = accuracy_pair(hf, cfg, dev, t_end=2.0, every=25, init=(W0, U0))
            exact = mesh.vortex_cell_averages(m, q, 2.0, centre=(5.0, 5.0))[:, 0]
            area = m.cell_areas()
            r["L1_rho_vs_exact"] = {p: float(np.sum(np.abs(s_["cFD"][:, 0] - exact) * area) / area.sum())
                                    for p, s_ in (("fp64", a), ("mixed", bb))}

            def fields(mm):
                U = mesh.vortex_cell_averages(mm, gauss_quadrature(mm, cfg), 0.0, centre=(5.0, 5.0))
                return mesh.primitive_from_conserved(U), None, U

            run, init = {"t_end": 2.0, "every": 25}, (W0, U0)
            make_mesh = lambda o: mesh.periodic_quad_grid(256, 256, 0.0, 10.0, 0.0, 10.0, renumber=o)
        elif name == "step":
            m = mesh.forward_step_triangles(args.points, seed=args.seed)
            W, Wb = mesh.uniform_fields(m, 1.0, 3.0, 0.0, 1.0)
            cfg = CaseConfig(stencilType="edgeNeighbour", CFL=args.cfl)
            hf = precompute(m, cfg, W, Wb, want_rbf64=True, device=dev)
            r, _, _ = accuracy_pair(hf, cfg, dev, n_steps=args.acc_steps, every=10)

            def fields(mm):
                return (*mesh.uniform_fields(mm, 1.0, 3.0, 0.0, 1.0), None)

            run, init = {"n_steps": args.acc_steps, "every": 10}, None
            make_mesh = lambda o: mesh.forward_step_triangles(args.points, seed=args.seed, renumber=o)
        elif name == "riemann_mixed":
            m = mesh.riemann_mixed(args.mixed_n, seed=args.seed)
            W, Wb = mesh.riemann_fields(m)
            cfg = CaseConfig(stencilType="edgeNeighbour", CFL=0.3)
            hf = precompute(m, cfg, W, Wb, want_rbf64=True, device=dev)
            r, _, _ = accuracy_pair(hf, cfg, dev, t_end=0.3, every=100)

            def fields(mm):
                return (*mesh.riemann_fields(mm), None)

            run, init = {"t_end": 0.3, "every": 100}, None
            make_mesh = lambda o: mesh.riemann_mixed(args.mixed_n, seed=args.seed, renumber=o)
        elif name == "batch":
            rng = np.random.default_rng(args.seed)
            params = [batch_member_params(rng) for _ in range(args.batch_solves)]
            pick = np.linspace(0, args.batch_solves - 1, args.acc_sample).round().astype(int)
            members = []
            for k in pick:
                mm, W, Wb, cfg = batch_member(params[k])
                hf = precompute(mm, cfg, W, Wb, want_rbf64=True, device=dev)
                rk, _, _ = accuracy_pair(hf, cfg, dev, n_steps=args.batch_steps, every=50)
                rk.update({"member": int(k), "cells": mm.n_cells})
                if args.floor:
                    brun = {"n_steps": args.batch_steps, "every": 50}
                    rk["fp64_floor_reorder"] = fp64_reorder_floor(
                        lambda o, p_=params[k]: batch_member_mesh(p_, renumber=o),
                        lambda m_, p_=params[k]: (*batch_member_fields(m_, p_), None), cfg, dev, **brun)
                    rk["fp64_floor_perturbed_start"] = fp64_perturbation_floor(hf, cfg, dev, **brun)
                    rk["fp64_float_start"] = fp64_perturbation_floor(hf, cfg, dev, kind="float", **brun)
                members.append(rk)
            r = {"members": members, "L1_rho_max": max(x["L1_rho"] for x in members),
                 "Linf_rho_max": max(x["Linf_rho"] for x in members),
                 "switch_flips_total": sum(x["switch_flips"] for x in members)}
            hf = None
        else:
            raise SystemExit(f"--accuracy: unknown config {name}")
        if hf is not None:
            line["cells"] = hf.nc
            if args.floor:
                r["fp64_floor_reorder"] = fp64_reorder_floor(make_mesh, fields, cfg, dev, **run)
                r["fp64_floor_perturbed_start"] = fp64_perturbation_floor(hf, cfg, dev, init=init, **run)
                r["fp64_float_start"] = fp64_perturbation_floor(hf, cfg, dev, init=init, kind="float", **run)
        line.update(r)
        line["wall_s"] = round(time.time() - t0, 1)
        if dist.rank == 0:
            print(json.dumps(line), flush=True)
        out.append(line)


def run_setup(args, dist: Dist):
    """Set-up time of the workload's mesh: the native precompute with every stage on the host (all
    host threads) against the same with its RBF stage (P matrices, inverses, O3 weights) on the GPU;
    the two bundles are compared bit for bit."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh, precompute
    from afar_cudaeuler2dmixo3rk3solver_gb300 import build as b

    b.build_all()
    t0 = time.perf_counter()
    if args.mesh == "riemann_mixed":
        m = mesh.riemann_mixed(args.mixed_n, seed=args.seed)
        W, Wb = mesh.riemann_fields(m)
    else:
        m = mesh.forward_step_triangles(args.points, seed=args.seed)
        W, Wb = mesh.uniform_fields(m, 1.0, 3.0, 0.0, 1.0)
    t_mesh = time.perf_counter() - t0
    cfg = CaseConfig(stencilType="edgeNeighbour", CFL=args.cfl)
    precompute(mesh.quad_grid(8, 8), cfg, *mesh.uniform_fields(mesh.quad_grid(8, 8), 1.0, 0.0, 0.0, 1.0),
               device=dist.local)  # context creation outside the timing
    times = {}
    out = {}
    for where, dev in (("host", None), ("device", dist.local)):
        t = time.perf_counter()
        out[where] = precompute(m, cfg, W, Wb, want_rbf64=True, device=dev)
        times[where] = time.perf_counter() - t
    same = all(np.array_equal(out["host"].a[k].view(np.uint8), out["device"].a[k].view(np.uint8))
               for k in out["host"].a)
    if dist.rank != 0:
        return
    print(json.dumps({
        "metric": "precompute seconds", "workload": args.mesh, "cells": m.n_cells,
        "internal_faces": m.n_internal_faces, "mesh_generation_s": round(t_mesh, 3),
        "host_s": round(times["host"], 3), "rbf_stage_on_gpu_s": round(times["device"], 3),
        "host_threads": os.cpu_count(), "bit_identical": bool(same),
    }), flush=True)


def batch_member_params(rng):
    """One solve of the batched workload: cells log-uniform in [5k, 200k], ramp angle U[5, 20]
    degrees, inflow Mach U[1.5, 4], vortex strength U[0, 5] (drawn in this order)."""
    nc = float(np.exp(rng.uniform(np.log(5e3), np.log(2e5))))
    angle = rng.uniform(5.0, 20.0)
    u0 = rng.uniform(1.5, 4.0) * np.sqrt(1.4)  # rho = p = 1: sound speed sqrt(1.4)
    strength = rng.uniform(0.0, 5.0)
    return nc, angle, u0, strength


def batch_member(params):
    """The compression ramp of batch_member_params: quads in a 2:1 channel, label-6 inflow, an
    isentropic vortex carried in the stream; face-neighbour stencils, CFL 0.3."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh

    m = batch_member_mesh(params)
    W, Wb = batch_member_fields(m, params)
    return m, W, Wb, CaseConfig(stencilType="faceNeighbour", CFL=0.3)


def batch_member_mesh(params, renumber="rcm"):
    """The compression-ramp mesh of a batched solve (quads in a 2:1 channel)."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import mesh

    nc, angle, _, _ = params
    ny = max(8, int(round(np.sqrt(nc / 2.0))))
    return mesh.wedge_quads(2 * ny, ny, angle, renumber=renumber)


def batch_member_fields(m, params):
    """Initial cells and inflow ghosts of a batched solve: the vortex carried in the stream."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import mesh

    _, _, u0, strength = params
    W = mesh.vortex_fields(m.cell_centres(), strength=strength, xc=0.5, yc=0.6, u0=u0, v0=0.0)
    Wb = mesh.vortex_fields(m.boundary_face_centres(), strength=0.0, xc=0.5, yc=0.6, u0=u0, v0=0.0)
    return W, Wb


def run_batch(args, dist: Dist):
    """Batched workload (the shape of the batched config): --batch-solves independent supersonic
    compression ramps, cells log-uniform in [5k, 200k] (quads, 2:1 channel), inflow Mach U[1.5, 4]
    through a label-6 inflow patch, ramp angle U[5, 20] degrees, an isentropic vortex of strength
    U[0, 5] carried in the stream; mixed policy, CFL 0.3; all stepped together --batch-steps RK3
    steps by one afar_batch (13 launches per step for the whole batch).  Compared with stepping
    the same solves one after another (afar_run_timed, 40 steps each)."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Batch, CaseConfig, CudaSolver, mesh, precompute
    from afar_cudaeuler2dmixo3rk3solver_gb300 import build as b

    b.build_all()
    rng = np.random.default_rng(args.seed + 31 * dist.rank)
    t0 = time.time()
    solvers, cells = [], []
    for k in range(args.batch_solves):
        m, W, Wb, cfg = batch_member(batch_member_params(rng))
        s = CudaSolver(precompute(m, cfg, W, Wb), cfg, policy="mixed", device=dist.local)
        solvers.append(s)
        cells.append(m.n_cells)
    setup_s = time.time() - t0
    cells = np.array(cells, dtype=np.float64)
    # one after another: device time of 40 graph-replayed steps each, from the initial state
    solo_ms = 0.0
    for s in solvers:
        s.save()
        if args.batch_no_solo:
            continue
        s.run_timed(3)
        s.restore()
        solo_ms += s.run_timed(40) / 40.0
        s.restore()
    batch = Batch("mixed", device=dist.local)
    for s in solvers:
        s.set_step_params()
        batch.add(s)
    batch.run(3)
    for s in solvers:  # restore the initial states before the timed run
        s.restore()
    dist.barrier()
    ms = dist.max(batch.run(args.batch_steps))
    schedule = batch.schedule()
    finite = all(bool(np.isfinite(s.state()["FD"]).all()) for s in solvers)
    batch.close()
    for s in solvers:
        s.close()
    total = dist.sum(float(cells.sum()))
    if dist.rank != 0:
        return
    print(json.dumps({
        "metric": "batched cell-RK3-steps/s", "value": total * args.batch_steps / (ms * 1e-3), "unit": "cell-steps/s",
        "n_gpus": dist.world, "higher_is_better": True, "ms_per_step": ms / args.batch_steps,
        "data": "synthetic (compression ramps 5k-200k quads, Mach 1.5-4, 5-20 deg, vortex 0-5, seeded)",
        "config": {"workload": "batch_wedges", "solves": args.batch_solves, "cells": int(cells.sum()),
                   "steps": args.batch_steps, "policy": "mixed", "launches_per_step": 13, "setup_s": round(setup_s, 1)},
        "schedule": schedule,
        "one_after_another": None if args.batch_no_solo else {
            "value": float(cells.sum()) / (solo_ms * 1e-3), "ms_per_step": solo_ms,
            "launches_per_step": 13 * args.batch_solves},
        "finite": finite,
    }), flush=True)


def main():
    args = parse()
    dist = Dist()
    if args.cache_mesh:
        return run_cache_mesh(args)
    if args.cpu_sample:
        return run_cpu_sample(args)
    try:
        if args.accuracy:
            run_accuracy(args, dist)
        elif args.setup:
            run_setup(args, dist)
        elif args.serve:
            run_serve(args, dist)
        elif args.batch:
            run_batch(args, dist)
        elif args.impl == "reference":
            run_reference_arm(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
