"""Throughput benchmark of the GB300 flux path: face-flux updates per second.

Default workload: the 2D shear-layer instability with 1,048,576 generators (1024x1024
jittered lattice, seeded) on a periodic unit box, gamma = 5/3, p = 2.5, a dense band
|y - 0.5| < 0.25 (rho = 2, v_x = 0.5) in rho = 1, v_x = -0.5 surroundings, v_y =
0.01 sin(4 pi x) + seeded noise of amplitude 1e-3; piecewise-linear MUSCL-Hancock,
HLLC, CFL 0.5, FP32 reconstruction / Riemann with FP64 accumulation.  A step is one
pass of the flux path over the mesh (moving-mesh stage order: generator and face
velocities, gradients, states + Riemann + deboost, segmented conserved update,
primitives, CFL time step); the host re-tessellation is outside the path and the mesh
is held fixed across steps.

Prints one JSON line (rank 0).  ``--impl reference`` times the CPU implementation of
the same path on this machine's host cores instead.
"""
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

METRIC = "face-flux updates/s FP32 vs FP64 at stated L1 err; adjoint/forward time ratio"
UNIT = "faces/s"
# steps per captured CUDA graph in the timed loop (even: see run_ours)
GRAPH_CHUNK = 10


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--solver", default="hllc", choices=["hll", "hllc", "exact"])
    ap.add_argument("--n-side", type=int, default=1024)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--workload", default="shear", choices=["shear", "ensemble", "adjoint", "explosion", "moving"])
    ap.add_argument("--adj-steps", type=int, default=200, help="adjoint workload: recorded steps")
    ap.add_argument("--adj-dirs", type=int, default=16, help="adjoint workload: finite-difference directions")
    ap.add_argument("--runs", type=int, default=256)
    ap.add_argument("--no-tune", action="store_true", help="FP32: default launch shapes instead of autotuned")
    ap.add_argument("--no-extra", action="store_true",
                    help="leave out the explosion and ensemble summaries of the default line")
    return ap.parse_args()


def shear_layer(n_side, seed=0):
    """Generators and primitives (all cells, ghosts included) of the shear layer."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    mesh, _ = pkg.meshgen.build_mesh(pkg.meshgen.jittered_lattice(n_side, seed=seed), "periodic")
    rng = np.random.default_rng(seed + 1)
    x = mesh.x
    band = np.abs(x[1] - 0.5) < 0.25
    prim = np.stack([np.where(band, 2.0, 1.0), np.where(band, 0.5, -0.5),
                     0.01 * np.sin(4 * np.pi * x[0]) + 1e-3 * rng.uniform(-1.0, 1.0, x.shape[1]),
                     np.full(x.shape[1], 2.5)])
    return mesh, pkg.meshgen.fill_ghosts(mesh, prim)


# --------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0, period_ms=20):
        self.index, self.period_ms = index, period_ms
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", str(self.period_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.05)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(np.max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def job_rate(units_local, ms_local, device=None):
    """Whole-job throughput over the ranks of the current process group: the units all
    ranks processed divided by the slowest rank's time (MAX over ranks).  Returns
    (units per second, max ms).  One rank (or no process group): local values."""
    import torch
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        t = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
        u = torch.tensor([float(units_local)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        ms_max, units = float(t.item()), float(u.item())
    else:
        ms_max, units = float(ms_local), float(units_local)
    return units / (ms_max * 1e-3), ms_max


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of each kernel from the committed ncu summary, scaled to
    this workload's face count (profiles/ncu_traffic.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return None


# Compulsory ("algorithmic") bytes per launch of each FP32 step kernel in this
# layout: every array touched by the kernel counted once, no re-reads.
#   k_grad32:   per cell tag 1, list bounds 4, prim4 16 (the neighbours' rows are the
#               same array), cell_geo 16, flip 1, cellrec written 64, w2 written 8; per
#               list entry entry_rec 16 + csr_nbr 4
#   k_face32:   per face pair ids 8, face_geo 16, face_ar 8, flux4 written 16; per cell
#               its cellrec 64 (gathered from both sides; each row counted once)
#   k_update32: per cell tag 1, list bounds 4, cell_geo 16, FP64 totals 32 read + 32
#               written, prim4 written 16; per entry csr_face 4; per face flux4 16
def algorithmic_bytes(n, F, n_real):
    e = 2 * F
    grad = n * (1 + 4 + 16 + 16 + 1 + 64 + 8) + e * (16 + 4)
    face = F * (8 + 16 + 8 + 16) + n * 64
    update = n * (1 + 4 + 16 + 32 + 32 + 16) + e * 4 + F * 16
    return {"k_grad32": grad, "k_face32": face, "k_update32": update}


# The layout-independent count of the flux step (compulsory traffic with each array
# read or written once: 64 B of face record and 8 B of list per face, 204 B per cell),
# about 140 B per face at F/N = 3.
def step_bytes_layout_free(n, F):
    return F * (64 + 8) + n * 204


def algorithmic_bytes_f64(n, F, n_real):
    e = 2 * F
    grad = n * (16 + 16 + 8 + 1 + 32 + 64 + 4) + e * 4 + F * (8 + 8 + 16)
    face = F * (8 + 16 + 16 + 16 + 32) + n * (32 + 64 + 16 + 16)
    update = n * (4 + 1 + 32 + 32 + 8 + 32) + e * 4 + F * (8 + 8 + 32)
    return {"k_gradients": grad, "k_face_flux": face, "k_update_step": update}


# --------------------------------------------------------------------------------------
def cpu_baseline(n_side_sample, seconds, solver, prefer_reference=True, steps=None, warmup=0):
    """CPU throughput of the same path, one host thread, on a bounded sample of the same
    workload (a smaller lattice of the same problem): the reference's own Cython modules
    when they are built on this machine (kind "reference"), else the C restatement
    (oracle/phd_oracle.c, kind "port").  With `steps`, `warmup` untimed steps are run and
    then `steps` timed ones (stopping early once `seconds` have passed); otherwise steps
    are timed until `seconds` have passed."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    mesh, prim = shear_layer(n_side_sample)
    gamma = 5.0 / 3.0
    kind = "port"
    if prefer_reference:
        import ref_harness as rh
        if rh.available():
            kind = "reference"
    if kind == "reference":
        s = rh.RefStep(mesh, prim, gamma=gamma, riemann=solver)

        def one():
            s.moving_step_fixed_mesh(s.time_step())
    else:
        import oracle as O
        O.build()
        p = prim.copy()
        c = O.cons_from_prim(mesh, p, gamma)
        stp = O.OracleStepper(mesh, gamma=gamma, solver=solver, moving=True)

        def one():
            stp.step(O.time_step(mesh, p, gamma, 0.5, True), p, c)
    for _ in range(warmup):
        one()
    limit = steps if steps is not None else 10000
    done, t0 = 0, time.perf_counter()
    while True:
        one()
        done += 1
        el = time.perf_counter() - t0
        if done >= limit or el >= seconds:
            break
    what = "the reference's Cython flux path" if kind == "reference" else "the C restatement"
    return {"value": mesh.n_faces * done / el, "unit": UNIT, "cores": 1, "kind": kind, "steps": done,
            "ms_per_step": 1e3 * el / done, "faces": mesh.n_faces,
            "sample": "%d moving-mesh %s steps (FP64) of %s on the %dx%d shear layer (%d faces), 1 host thread"
                      % (done, solver.upper(), what, n_side_sample, n_side_sample, mesh.n_faces)}


def _cpu_worker(args):
    n_side, seconds, solver, steps, warmup = args
    return cpu_baseline(n_side, seconds, solver, steps=steps, warmup=warmup)


def run_reference(args, rank, world):
    """Reference arm: the CPU implementation of the path on the host cores -- one
    independent replica of the bounded sample per host core (the reference scales
    across cores by MPI domain decomposition; replicas are its upper bound)."""
    if rank != 0:
        return
    import multiprocessing as mp
    n_side = 256
    cores = max(1, os.cpu_count() or 1)
    ctx = mp.get_context("spawn")
    # each replica: `warmup` untimed steps, then `steps` timed steps of its 256x256
    # sample (about 0.17 s per step per core), capped at 150 s
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(n_side, 150.0, args.solver, args.steps, args.warmup)] * cores)
    value = float(sum(r["value"] for r in res))
    sample = ("each host core steps its own %dx%d sample of the same problem (%d faces): %s; %d concurrent "
              "replicas" % (n_side, n_side, res[0]["faces"], res[0]["sample"].replace(", 1 host thread", ""), cores))
    kind = res[0]["kind"]
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": min(r["steps"] for r in res),
           "warmup": args.warmup, "ms_per_step": float(np.median([r["ms_per_step"] for r in res])),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": "shear layer 1024x1024 jittered lattice, periodic, gamma 5/3",
                      "solver": args.solver, "precision": "fp64 (the reference computes in FP64)",
                      "sample": "bounded: a %dx%d lattice of the same problem per host core" % (n_side, n_side),
                      "parallelism": "%d host cores, one replica each" % cores},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# --------------------------------------------------------------------------------------
def run_ours(args, rank, world):
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from phd_code_gb300 import _lib as L
    from phd_code_gb300.device import DeviceMesh
    from phd_code_gb300.step import FluxStepper

    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    mesh, prim = shear_layer(args.n_side, seed=rank)
    n, F = mesh.n_cells, mesh.n_faces
    st = FluxStepper(mesh, prim, gamma=5.0 / 3.0, cfl=0.5, solver=args.solver, moving=True,
                     precision=args.precision, device=dev)
    lib = L.lib()
    import ctypes
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(4 * args.steps)]
    for e in marks:
        e.record()
    torch.cuda.synchronize()
    launch_cfg = "default (256 threads, one per item)"
    if st.precision == "fp32" and not args.no_tune:
        from phd_code_gb300.autotune import tune
        lch, _ = tune(st)
        st.launch = lch
        launch_cfg = {"blocks": [lch.block_grad, lch.block_face, lch.block_update],
                      "grid_caps": [lch.grid_cap_grad, lch.grid_cap_face, lch.grid_cap_update],
                      "items_per_thread": [lch.items_grad, lch.items_face, lch.items_update]}
    # the timed steps replay a CUDA graph of GRAPH_CHUNK steps (an even count, so the
    # double-buffered conserved state returns to the buffer the graph was recorded
    # on); a remainder of steps % GRAPH_CHUNK runs as direct launches after the replays
    chunk = GRAPH_CHUNK
    st.step(max(3, args.warmup))
    torch.cuda.synchronize()
    st.check_status()
    st.capture(chunk)
    st.replay()                                  # untimed: uploads the graph
    torch.cuda.synchronize()
    st.check_status()
    untimed = max(3, args.warmup) + chunk

    def marked_step(k):
        st._launch_step(marks=(ctypes.c_void_p * 4)(*(marks[4 * k + q].cuda_event for q in range(4))))

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.1)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps // chunk):
        st.replay()
    st.step(args.steps % chunk)
    e1.record()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms_total = e0.elapsed_time(e1)
    st.check_status()
    # per-kernel durations: the same number of steps again, launched directly with CUDA
    # events recorded between the kernels on the launching stream
    for k in range(args.steps):
        marked_step(k)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    st.check_status()
    names = (["k_grad32", "k_face32", "k_update32"] if st.precision == "fp32"
             else ["k_gradients", "k_face_flux", "k_update_step"])
    per = {nm: 0.0 for nm in names}
    for k in range(args.steps):
        for q, nm in enumerate(names):
            per[nm] += marks[4 * k + q].elapsed_time(marks[4 * k + q + 1])
    per = {nm: v / args.steps for nm, v in per.items()}
    value, ms_max = job_rate(F * args.steps, ms_total, device=dev)

    # roofline of the dominant kernel
    peak, peak_src = measured_peaks()
    algo = (algorithmic_bytes if st.precision == "fp32" else algorithmic_bytes_f64)(n, F, mesh.n_real)
    dom = max(per, key=per.get)
    achieved = algo[dom] / (per[dom] * 1e-3) / 1e9
    tr = ncu_traffic()
    traffic = None
    if tr and dom in tr.get("kernels", {}):
        k = tr["kernels"][dom]
        traffic = k["dram_bytes_per_face"] * F if "dram_bytes_per_face" in k else None
    step_ms = ms_max / args.steps
    free = step_bytes_layout_free(n, F)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "kernel": dom,
                "peak_source": peak_src, "algorithmic_bytes": algo[dom],
                "kernel_ms": {k: round(v, 5) for k, v in per.items()},
                "kernel_frac": {k: round(algo[k] / (per[k] * 1e-3) / 1e9 / peak, 4) for k in per},
                "step": {"bytes_per_face_layout_free": round(free / F, 1), "bytes_layout_free": free,
                         "bytes_this_layout": sum(algo.values()), "ms": round(step_ms, 5),
                         "frac_layout_free": round(free / (step_ms * 1e-3) / 1e9 / peak, 4),
                         "frac_this_layout": round(sum(algo.values()) / (step_ms * 1e-3) / 1e9 / peak, 4)}}

    # end to end through the public API with host buffers: the host mesh hands over
    # its face list and cell geometry each step (pinned host -> device), the step runs,
    # and the generator velocities (what the host re-mesh needs) plus the clock come back
    accuracy = None
    if st.precision == "fp32" and not args.no_accuracy:
        accuracy = fp32_accuracy(st, mesh, prim, untimed + 2 * args.steps, dev, args.solver)
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, st, mesh, prim, dev)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(256, args.cpu_seconds, args.solver)

    adjoint = None
    if not args.no_adjoint and rank == 0:
        adjoint = adjoint_cost(dev)

    explosion = ensemble = None
    if rank == 0 and not args.no_extra:
        explosion = explosion_summary(dev)
        ensemble = ensemble_summary(dev)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": untimed, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32" if st.precision == "fp32" else "f64",
               "data": "synthetic",
               "config": {"workload": "shear layer 1024x1024 jittered lattice, periodic, gamma 5/3"
                          if args.n_side == 1024 else "shear layer %dx%d" % (args.n_side, args.n_side),
                          "cells": mesh.n_real, "ghosts": mesh.n_ghost, "faces": F, "solver": args.solver,
                          "reconstruction": "piecewise linear, AREPO limiter + GIZMO pair limiter",
                          "precision": st.precision + ("+fp64-accumulate" if st.precision == "fp32" else ""),
                          "mesh": "fixed across steps (host re-mesh outside the path)",
                          "l2": (("inputs larger than L2 (per-step working set %.0f MB > 129 MB)"
                                  if sum(algo.values()) > 129e6 else
                                  "per-step working set %.0f MB fits the 129 MB L2: not an HBM figure")
                                 % (sum(algo.values()) / 1e6)),
                          "parallelism": "replicas" if world > 1 else "single GPU", "launch": launch_cfg,
                          "timing": "CUDA graph of %d steps replayed %d times, %d direct steps after; per-kernel "
                                    "times from a second pass of %d directly launched steps with CUDA events "
                                    "between the kernels" % (chunk, args.steps // chunk, args.steps % chunk,
                                                             args.steps)},
               "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "accuracy": accuracy,
               "adjoint": adjoint,
               "fp64_value": accuracy["fp64_faces_per_s"] if accuracy else None,
               "fp32_over_fp64": (value / accuracy["fp64_faces_per_s"]) if accuracy else None,
               "explosion": explosion, "ensemble": ensemble,
               # per step: FP32 k_grad32 (with the generator velocities), k_face32, k_update32;
               # FP64 k_gen_vel, k_face_vel, k_gradients, k_face_flux, k_update_step
               "gpu_launches": (3 if st.precision == "fp32" else 5) * args.steps, "clocks": clocks}
        print(json.dumps(out), flush=True)


def fp32_accuracy(st, mesh, prim, n_steps, dev, solver):
    """L1 density error of the FP32 run against an FP64 run of the same steps from the
    same state (mean |rho32 - rho64| over real cells) and the FP32 run's relative
    mass / energy drift |sum U(t) - sum U(0)| / sum U(0)."""
    import torch
    from phd_code_gb300.step import FluxStepper
    ref = FluxStepper(st.dmesh, prim, gamma=5.0 / 3.0, cfl=0.5, solver=solver, moving=True, precision="fp64",
                      device=dev)
    ref.step(2)                                   # warm-up (timed below: the FP64 path's own throughput)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    ev[0].record()
    ref.step(n_steps - 2)
    ev[1].record()
    torch.cuda.synchronize()
    fp64_ms = ev[0].elapsed_time(ev[1]) / (n_steps - 2)
    nr = mesh.n_real
    r32 = st.prim4[:nr, 0].double()
    r64 = ref.prim[0, :nr]
    l1 = float((r32 - r64).abs().mean())
    u0 = torch.as_tensor(prim[:, :nr]).to(dev)
    vol = st.dmesh.vol[:nr]
    m0 = float((u0[0] * vol).sum())
    e0 = float(((0.5 * u0[0] * (u0[1] ** 2 + u0[2] ** 2) + u0[3] / (5.0 / 3.0 - 1.0)) * vol).sum())
    c = st.cons[:, :nr]
    c64 = ref.cons[:, :nr]
    return {"steps": n_steps, "l1_density_vs_fp64": l1, "mass_drift": abs(float(c[0].sum()) - m0) / m0,
            "energy_drift": abs(float(c[3].sum()) - e0) / e0,
            "fp64_mass_drift": abs(float(c64[0].sum()) - m0) / m0,
            "fp64_energy_drift": abs(float(c64[3].sum()) - e0) / e0,
            "t_fp32": st.read_clock().t, "t_fp64": ref.read_clock().t,
            "fp64_ms_per_step": fp64_ms, "fp64_faces_per_s": mesh.n_faces / (fp64_ms * 1e-3),
            "fp64_timing": "CUDA events around %d directly launched FP64 steps (the reference-parity path), after "
                           "2 warm-up steps" % (n_steps - 2)}


def adjoint_cost(dev, n_side=128, n_steps=200, checkpoint=20, n_dirs=16, h=1e-6, h_small=1e-10, noise=1e-3):
    """The differentiation workload: 128x128 periodic box, gamma 1.4, HLLC, CFL 0.4,
    static mesh.  The target density is a Gaussian bump (amplitude 0.1, width 0.05) on
    rho = p = 1 evolved for n_steps in FP64; the differentiated run starts from the
    background with seeded noise of amplitude `noise` on rho, v and p (an exactly uniform
    state sits on the limiters' non-differentiable point, where no derivative is
    unique); loss = sum (rho_T - rho_target)^2.  Timed with CUDA events: forward, backward
    (recompute from checkpoints every `checkpoint` steps), and the adjoint step alone
    against the forward step.  The gradient is checked against central differences
    along n_dirs seeded random directions at step h and at h_small: the limited scheme is
    piecewise smooth, and over 200 steps a perturbation of 1e-6 crosses limiter branch
    switches in most directions (seen in the one-sided slopes), so only the smaller step
    measures the local derivative."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from phd_code_gb300.adjoint import FluxRun, FluxRunRecord, StepRecord
    from phd_code_gb300.device import DeviceMesh
    from phd_code_gb300.step import FluxStepper
    mesh, prim_bump, info = pkg.problems.gaussian_bump(n_side, background=False)
    _, prim_bg, _ = pkg.problems.gaussian_bump(n_side, background=True)
    nr = mesh.n_real
    dm = DeviceMesh(mesh, device=dev)
    st_t = FluxStepper(dm, prim_bump, gamma=1.4, cfl=0.4, solver="hllc", moving=False, device=dev)
    st_t.step(n_steps)
    st_t.check_status()
    target = st_t.prim[0, :nr].clone()
    rng = np.random.default_rng(3)
    p_init = prim_bg.copy()
    p_init[:, :nr] += noise * rng.uniform(-1.0, 1.0, (4, nr))
    p_init = pkg.meshgen.fill_ghosts(mesh, p_init)
    st = FluxStepper(dm, p_init, gamma=1.4, cfl=0.4, solver="hllc", moving=False, device=dev)
    fw = torch.zeros((2, mesh.n_faces), dtype=torch.float64, device=dev)
    recs = []
    for _ in range(n_steps):
        recs.append(StepRecord(dm, fw, st.read_clock().dt))
        st.step(1)
    run = FluxRunRecord(recs, gamma=1.4, solver="hllc", checkpoint=checkpoint)
    p0 = torch.as_tensor(p_init[:, :nr]).to(dev).requires_grad_(True)

    def loss_of(p):
        return ((FluxRun.apply(p, run) - target) ** 2).sum()

    for _ in range(2):                                   # warm-up
        loss_of(p0).backward()
    p0.grad = None
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    e[0].record()
    loss = loss_of(p0)
    e[1].record()
    loss.backward()
    e[2].record()
    torch.cuda.synchronize()
    fwd, bwd = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
    g = p0.grad.detach().clone()
    # the adjoint step alone (reverse kernels at recorded states) against the forward step
    states = run._replay_segment(0, n_steps)
    lam = torch.zeros((4, nr), dtype=torch.float64, device=dev)
    lam[0] = 1.0
    torch.cuda.synchronize()
    e[0].record()
    for k in range(n_steps - 1, -1, -1):
        lam = run._adjoint(recs[k], states[k], lam)
    e[1].record()
    torch.cuda.synchronize()
    adj_step = e[0].elapsed_time(e[1]) / n_steps
    del states
    # central differences along seeded directions, at the configured step and at a step
    # small enough to stay between the limiters' branch switches; the one-sided slopes'
    # spread shows whether [-h, h] crossed a switch (a kink of the piecewise-smooth map)
    drng = np.random.default_rng(11)
    fd_rows = []
    with torch.no_grad():
        L0 = float(loss_of(p0.detach()))
        # the same differences through the branch-frozen forward (every limiter
        # selection, GIZMO clamp, positivity revert, wave-speed estimate and Riemann
        # region of the run from p0 replayed): the derivative on the branch the run takes
        L0f = float(((run.final_density_frozen(p0.detach(), record=True) - target) ** 2).sum())

        def frozen(pp):
            return float(((run.final_density_frozen(pp) - target) ** 2).sum())
        for _ in range(n_dirs):
            d = torch.as_tensor(drng.standard_normal((4, nr))).to(dev)
            d = d / torch.linalg.norm(d)               # unit direction: the step is h
            gd = float((g * d).sum())
            row = {"gd": gd}
            for tag, hh in (("h", h), ("h_small", h_small)):
                Lp, Lm = float(loss_of(p0.detach() + hh * d)), float(loss_of(p0.detach() - hh * d))
                fd = (Lp - Lm) / (2 * hh)
                row[tag] = {"rel_err": abs(fd - gd) / max(abs(gd), 1e-300),
                            "one_sided_spread": abs((Lp - L0) - (L0 - Lm)) / hh / max(abs(gd), 1e-300)}
            for tag, hh in (("frozen_h", h), ("frozen_h10", 10 * h), ("frozen_h100", 100 * h)):
                Lp, Lm = frozen(p0.detach() + hh * d), frozen(p0.detach() - hh * d)
                fd = (Lp - Lm) / (2 * hh)
                row[tag] = {"rel_err": abs(fd - gd) / max(abs(gd), 1e-300), "fd": fd}
            fd_rows.append(row)
    return {"config": "gaussian bump %dx%d periodic, HLLC, FP64, CFL 0.4, %d steps, checkpoint every %d; start = "
                      "background + %g noise" % (n_side, n_side, n_steps, checkpoint, noise),
            "forward_ms": fwd, "backward_ms": bwd, "ratio": bwd / fwd,
            "forward_step_ms": fwd / n_steps, "adjoint_step_ms": adj_step, "step_ratio": adj_step * n_steps / fwd,
            "fd_check": {"directions": n_dirs, "h": h, "h_small": h_small,
                         "max_rel_err_frozen_h": max((r["frozen_h"]["rel_err"] for r in fd_rows), default=None),
                         "median_rel_err_frozen_h": float(np.median([r["frozen_h"]["rel_err"] for r in fd_rows]))
                         if fd_rows else None,
                         "frozen_loss_vs_forward_loss": abs(L0f - L0) / max(abs(L0), 1e-300),
                         "normwise_rel_err_frozen_h": float(np.sqrt(sum((r["frozen_h"]["fd"] - r["gd"]) ** 2
                                                                        for r in fd_rows) /
                                                                    max(sum(r["gd"] ** 2 for r in fd_rows), 1e-300)))
                         if fd_rows else None,
                         "max_abs_err_frozen_h": max((abs(r["frozen_h"]["fd"] - r["gd"]) for r in fd_rows),
                                                     default=None),
                         "max_abs_directional_derivative": max((abs(r["gd"]) for r in fd_rows), default=None),
                         "max_rel_err_frozen_10h": max((r["frozen_h10"]["rel_err"] for r in fd_rows), default=None),
                         "max_rel_err_frozen_100h": max((r["frozen_h100"]["rel_err"] for r in fd_rows), default=None),
                         "directions_are": "unit vectors (seeded normal draws divided by their norm)",
                         "frozen": "central differences through phd_step_f64_frozen replaying the decisions "
                                   "(limiter selections, GIZMO clamps, positivity reverts, wave-speed estimate, "
                                   "Riemann region) recorded on the run from p0",
                         "max_rel_err_h": max((r["h"]["rel_err"] for r in fd_rows), default=None),
                         "max_rel_err_h_small": max((r["h_small"]["rel_err"] for r in fd_rows), default=None),
                         "median_rel_err_h_small": float(np.median([r["h_small"]["rel_err"] for r in fd_rows]))
                         if fd_rows else None,
                         "directions_crossing_a_switch_at_h": sum(r["h"]["one_sided_spread"] > 1e-3 for r in fd_rows),
                         "max_one_sided_spread_h_small": max((r["h_small"]["one_sided_spread"] for r in fd_rows),
                                                             default=None)}}


def run_e2e(args, st, mesh, prim, dev):
    """The same step through the public API with host buffers: every step the host
    hands over its tessellation from pinned memory with FluxStepper.load_mesh -- for
    FP32 the compact hand-over (per-cell face ranges, pair-j, FP32 area and centroid
    offset along the face: 12 B per face, plus the ghost map and ghost codes; the real cells' positions
    are the device's own, as after its generator move), for FP64 the full one (pair-i/j,
    FP64 area and centroid, x, dcom, vol, map) -- which forms the neighbour lists, ghost
    positions, flip bits, periodic twins and FP32 geometry on the device, re-creates the
    ghosts and recovers the primitives; the step runs; the generator velocities (what the
    host re-mesh needs) and the clock come back."""
    import torch
    from phd_code_gb300 import _lib as L
    dm = st.dmesh
    fp32 = st.precision == "fp32"
    pinned = dm.pinned_host_compact(mesh, resident=True) if fp32 else dm.pinned_host(mesh)
    w_host = torch.empty_like(st.w2 if st.precision == "fp32" else st.w, device="cpu").pin_memory()
    clk_host = torch.empty(L.CLOCK_BYTES, dtype=torch.uint8).pin_memory()
    d2h = w_host.numel() * w_host.element_size() + clk_host.numel()
    h2d = [0]

    def one():
        h2d[0] = st.load_mesh(pinned)
        st.step_and_fetch(w_host)                # velocities leave while the step finishes
        clk_host.copy_(st.clock.buf, non_blocking=True)

    for _ in range(2):
        one()
    torch.cuda.synchronize()
    if dm.upload_errors():
        raise RuntimeError("mesh upload reported faces with out-of-range cells")
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    import torch.distributed as tdist
    if tdist.is_available() and tdist.is_initialized():
        tdist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0.record()
    for _ in range(args.e2e_steps):
        one()
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    st.check_status()
    # the larger of device and host time (the host issues the copies), slowest rank
    ms_run = max(e0.elapsed_time(e1), 1e3 * wall)
    rate, ms_max = job_rate(mesh.n_faces * args.e2e_steps, ms_run, device=dev)
    return {"value": rate, "unit": UNIT,
            "h2d_bytes_per_step": int(h2d[0]), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": ms_max / args.e2e_steps, "steps": args.e2e_steps,
            "what": "per step: host tessellation H2D from pinned memory (%s); neighbour lists, flip bits, "
                    "periodic twins, FP32 geometry, ghost refresh and primitives formed on the device; flux step, "
                    "its generator velocities D2H as soon as its first kernel has formed them; clock D2H" % ("compact FP32 face list: per-cell face ranges, pair-j, "
                                                           "FP32 area and centroid offset; ghost map and codes (real "
                                                           "positions stay on the device)"
                                                           if fp32 else "face list + cell geometry, FP64")}


def ensemble_summary(dev, n_runs=256, steps=20, warmup=3, seed=0, seq_steps=10):
    """The batching workload: n_runs independent two-state Riemann runs (N log-uniform in
    [1000, 65536]) advanced together, one launch per stage, a CUDA graph of two steps,
    autotuned launch shapes; against the same runs as separate single-run steppers
    launched one after another.  Returns the aggregate faces/s of both."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from phd_code_gb300.autotune import tune
    from phd_code_gb300.ensemble import EnsembleStepper, SequentialEnsemble
    runs, info = pkg.problems.riemann_ensemble(n_runs=n_runs, seed=seed)
    ens = EnsembleStepper(runs, device=dev)
    launch, table = tune(ens)
    ens.launch = launch
    ens.capture(2)
    for _ in range(max(3, warmup)):
        ens.replay()
    steps = steps if steps % 2 == 0 else steps + 1
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps // 2):
        ens.replay()
    e1.record()
    torch.cuda.synchronize()
    ens.check_status()
    ms = e0.elapsed_time(e1)
    seq = SequentialEnsemble(runs, device=dev)
    seq.step(2)
    torch.cuda.synchronize()
    e0.record()
    seq.step(seq_steps)
    e1.record()
    torch.cuda.synchronize()
    seq_rate = seq.faces * seq_steps / (e0.elapsed_time(e1) * 1e-3)
    batched = ens.faces * steps / (ms * 1e-3)
    return {"runs": n_runs, "cells": int(ens.dmesh.n_real), "faces": int(ens.faces), "steps": steps,
            "faces_per_s": batched, "ms_per_step": ms / steps, "sequential_faces_per_s": seq_rate,
            "sequential_steps": seq_steps, "speedup_vs_sequential": batched / seq_rate,
            "launch": {"block": [launch.block_grad, launch.block_face, launch.block_update],
                       "grid_cap": [launch.grid_cap_grad, launch.grid_cap_face, launch.grid_cap_update],
                       "items_per_thread": [launch.items_grad, launch.items_face, launch.items_update]}}


def run_ensemble(args, rank, world):
    """Batched two-state Riemann ensemble as its own line (one replica per rank)."""
    import torch
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    r = ensemble_summary(dev, n_runs=args.runs, steps=args.steps, warmup=args.warmup, seed=rank,
                         seq_steps=min(args.steps, 20))
    clocks = sampler.stop()
    batched, ms = job_rate(r["faces"] * r["steps"], r["ms_per_step"] * r["steps"], device=dev)
    if rank == 0:
        out = {"metric": METRIC, "value": batched, "unit": UNIT, "n_gpus": world, "steps": r["steps"],
               "warmup": max(3, args.warmup), "ms_per_step": ms / r["steps"], "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": {"workload": "ensemble of %d two-state Riemann runs, N log-uniform in [1000, 65536], "
                                      "reflective unit boxes, gamma 1.4, FP32+FP64-accumulate HLLC" % args.runs,
                          "cells": r["cells"], "faces": r["faces"], "launch": r["launch"]},
               "sequential": {"value": r["sequential_faces_per_s"], "unit": UNIT, "steps": r["sequential_steps"],
                              "what": "the same runs as separate single-run steppers launched in turn"},
               "speedup_vs_sequential": r["speedup_vs_sequential"], "gpu_launches": 3 * r["steps"],
               "clocks": clocks}
        print(json.dumps(out), flush=True)


def explosion_summary(dev, n_side=256, seed=0, solvers=("hllc", "exact")):
    """The point-explosion workload: n_side^2 jittered periodic box, rho = 1, p = 1e-5,
    E = 1 deposited within two lattice spacings of the centre, gamma 1.4, run to
    t = 0.05 (the clock clips the last step onto t_end) with each solver in FP64 and in
    FP32 + FP64 accumulation (moving-mesh stage order, mesh held fixed).  Reports each
    run's faces/s, the FP32 run's L1 density error against the FP64 run (the FP64 path
    matches the reference to 1e-12, tests/) and both runs' total-energy drift."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from phd_code_gb300.step import FluxStepper
    mesh, prim, info = pkg.problems.point_explosion(n_side, seed=seed)
    nr, F = mesh.n_real, mesh.n_faces
    t_end, gamma = info["t_end"], info["gamma"]

    def run(solver, precision, chunk):
        st = FluxStepper(mesh, prim, gamma=gamma, cfl=0.5, solver=solver, moving=True, precision=precision,
                         t_end=t_end, device=dev)
        e0 = st.cons_host()[3, :nr].sum()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        steps, ms = 0, 0.0
        while True:
            ev[0].record()
            st.step(chunk)
            ev[1].record()
            c = st.read_clock()                       # synchronises
            ms += ev[0].elapsed_time(ev[1])
            steps += chunk
            if c.t >= t_end * (1.0 - 1e-12) or steps > 200000:
                break
        st.check_status()
        cons = st.cons_host()[:, :nr]
        return {"steps": steps, "t": c.t, "faces_per_s": F * steps / (ms * 1e-3),
                "energy_drift": abs(cons[3].sum() - e0) / abs(e0), "rho": cons[0] / mesh.vol[:nr]}

    out = {"workload": "point explosion %dx%d jittered periodic, E = 1, gamma 1.4, to t = 0.05" % (n_side, n_side),
           "cells": nr, "faces": F}
    for solver in solvers:
        r64 = run(solver, "fp64", 10)
        r32 = run(solver, "fp32", 25)
        out[solver] = {"fp64": {k: v for k, v in r64.items() if k != "rho"},
                       "fp32": {k: v for k, v in r32.items() if k != "rho"},
                       "l1_density_fp32_vs_fp64": float(np.mean(np.abs(r32["rho"] - r64["rho"]))),
                       "fp32_over_fp64_faces_per_s": r32["faces_per_s"] / r64["faces_per_s"]}
    return out


def run_explosion(args, rank, world):
    """The point-explosion workload as its own line."""
    import torch
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    out = explosion_summary(dev, seed=rank)
    clocks = sampler.stop()
    if rank == 0:
        print(json.dumps({"metric": METRIC, "value": out["hllc"]["fp32"]["faces_per_s"], "unit": UNIT,
                          "n_gpus": world, "steps": out["hllc"]["fp32"]["steps"], "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                          "config": {"workload": out["workload"], "cells": out["cells"], "faces": out["faces"],
                                     "mesh": "fixed across steps (face velocities from the moving-mesh stage)"},
                          "runs": {k: v for k, v in out.items() if k in ("hllc", "exact")}, "clocks": clocks}),
              flush=True)


def run_moving(args, rank, world):
    """The whole moving-mesh loop (integrate.py:385-428) on the shear layer: every step
    the device takes the flux step and moves the real generators by dt*w (wrapped into
    the periodic box; real cells keep their order), the positions come back, the host
    re-tessellates them (C++ Tess2d, strips on the host threads) straight into the
    compact FP32 hand-over and the device continues on it (FluxStepper.load_mesh).
    Reports faces/s of the whole loop, the time of each phase, and the mass / energy
    exchanged across the re-meshes."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from phd_code_gb300.step import FluxStepper
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    mesh, prim = shear_layer(args.n_side, seed=rank)
    nr = mesh.n_real
    st = FluxStepper(mesh, prim, gamma=5.0 / 3.0, cfl=0.5, solver=args.solver, moving=True, precision="fp32",
                     device=dev)
    c0 = st.cons_host()[:, :nr].sum(axis=1)
    x = np.ascontiguousarray(mesh.x[:, :nr])
    mesher = pkg.tess.CompactMesher("periodic", resident=True)
    phases = {"device_step_and_move": 0.0, "positions_d2h": 0.0, "tessellation_to_hand_over": 0.0, "load_mesh": 0.0}
    faces = 0
    n_steps = max(1, min(args.steps, 20))
    t_all = time.perf_counter()
    for k in range(n_steps + 1):                  # the first step is a warm-up
        if k == 1:
            t_all = time.perf_counter()
            faces = 0
            phases = {p: 0.0 for p in phases}
        t = time.perf_counter()
        st.step(1)
        xd = st.move_generators()                 # x + dt*w, periodic wrap, on the device
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        x = xd.cpu().numpy()
        t2 = time.perf_counter()
        faces += st.dmesh.n_faces
        pinned = mesher(x)
        t3 = time.perf_counter()
        st.load_mesh(pinned)
        torch.cuda.synchronize()
        t4 = time.perf_counter()
        for name, a, b in (("device_step_and_move", t, t1), ("positions_d2h", t1, t2),
                           ("tessellation_to_hand_over", t2, t3), ("load_mesh", t3, t4)):
            phases[name] += b - a
    wall = time.perf_counter() - t_all
    st.check_status()
    c1 = st.cons_host()[:, :nr].sum(axis=1)
    if rank == 0:
        print(json.dumps({"metric": METRIC, "value": faces / wall, "unit": UNIT, "n_gpus": world, "steps": n_steps,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                          "data": "synthetic",
                          "config": {"workload": "shear layer %dx%d, moving mesh re-tessellated every step" %
                                                 (args.n_side, args.n_side), "cells": nr, "solver": args.solver,
                                     "mesh": "host C++ Tess2d every step straight into the pinned compact FP32 "
                                             "hand-over (tess.CompactMesher)",
                                     "host_threads": os.cpu_count()},
                          "ms_per_step": 1e3 * wall / n_steps,
                          "phases_ms_per_step": {k: round(1e3 * v / n_steps, 3) for k, v in phases.items()},
                          "mass_drift": float(abs(c1[0] - c0[0]) / abs(c0[0])),
                          "energy_drift": float(abs(c1[3] - c0[3]) / abs(c0[3]))}), flush=True)


def run_adjoint(args, rank, world):
    """The differentiation workload alone (one replica per rank): adjoint_cost's line
    with the backward/forward time ratio as the value."""
    import torch
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    adj = adjoint_cost(dev, n_steps=args.adj_steps, n_dirs=args.adj_dirs)
    clocks = sampler.stop()
    if rank == 0:
        print(json.dumps({"metric": "adjoint / forward time ratio (backward with recompute)", "value": adj["ratio"],
                          "unit": "x", "n_gpus": world, "steps": args.adj_steps, "higher_is_better": False,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                          "config": {"workload": adj["config"]}, "adjoint": adj, "clocks": clocks}), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group(backend=backend)
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        elif args.workload == "ensemble":
            run_ensemble(args, rank, world)
        elif args.workload == "adjoint":
            run_adjoint(args, rank, world)
        elif args.workload == "explosion":
            run_explosion(args, rank, world)
        elif args.workload == "moving":
            run_moving(args, rank, world)
        else:
            run_ours(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
