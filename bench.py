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
def algorithmic_bytes(n, F, n_real):
    e = 2 * F
    grad = n * (16 + 16 + 4 + 1 + 32 + 8) + e * 8 + F * (16 + 8)
    face = F * (8 + 16 + 8 + 16) + n * (16 + 32 + 16 + 8)
    update = n * (4 + 1 + 32 + 32 + 8 + 16) + e * 4 + F * (8 + 16)
    return {"k_grad32": grad, "k_face32": face, "k_update32": update}


def algorithmic_bytes_f64(n, F, n_real):
    e = 2 * F
    grad = n * (16 + 16 + 8 + 1 + 32 + 64 + 4) + e * 4 + F * (8 + 8 + 16)
    face = F * (8 + 16 + 16 + 16 + 32) + n * (32 + 64 + 16 + 16)
    update = n * (4 + 1 + 32 + 32 + 8 + 32) + e * 4 + F * (8 + 8 + 32)
    return {"k_gradients": grad, "k_face_flux": face, "k_update_step": update}


# --------------------------------------------------------------------------------------
def cpu_baseline(n_side_sample, seconds, solver, prefer_reference=True):
    """CPU throughput of the same path, one host thread, on a bounded sample of the same
    workload (a smaller lattice of the same problem): the reference's own Cython modules
    when they are built on this machine (kind "reference"), else the C restatement
    (oracle/phd_oracle.c, kind "port")."""
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
    steps, t0 = 0, time.perf_counter()
    while True:
        one()
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 10000:
            break
    what = "the reference's Cython flux path" if kind == "reference" else "the C restatement"
    return {"value": mesh.n_faces * steps / el, "unit": UNIT, "cores": 1, "kind": kind,
            "sample": "%d moving-mesh %s steps (FP64) of %s on the %dx%d shear layer (%d faces), 1 host thread"
                      % (steps, solver.upper(), what, n_side_sample, n_side_sample, mesh.n_faces)}


def _cpu_worker(args):
    n_side, seconds, solver = args
    return cpu_baseline(n_side, seconds, solver)


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
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(n_side, max(5.0, args.cpu_seconds), args.solver)] * cores)
    value = float(sum(r["value"] for r in res))
    sample = "%s; %d concurrent replicas" % (res[0]["sample"].replace(", 1 host thread", ""), cores)
    kind = res[0]["kind"]
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": "shear layer %dx%d periodic (bounded CPU sample of the 1024x1024 run)"
                                  % (n_side, n_side), "solver": args.solver, "precision": "fp64"},
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
    st.step(max(3, args.warmup))
    torch.cuda.synchronize()
    st.check_status()

    def marked_step(k):
        arr = (ctypes.c_void_p * 4)(*(marks[4 * k + q].cuda_event for q in range(4)))
        s = L.stream_handle()
        if st.precision == "fp32":
            rc = lib.phd_step_f32_marked(st.dmesh.ref, ctypes.byref(st.geo), ctypes.byref(st.params),
                                         int(st.moving), L.ptr(st.prim4), L.ptr(st.cons), L.ptr(st.cons_next),
                                         L.ptr(st.grad8), L.ptr(st.w2), L.ptr(st.flux4), st.clock.ptr, s, arr)
        else:
            rc = lib.phd_step_f64_marked(st.dmesh.ref, ctypes.byref(st.params), int(st.moving), L.ptr(st.prim),
                                         L.ptr(st.cons), L.ptr(st.cons_next), L.ptr(st.grad), L.ptr(st.w),
                                         L.ptr(st.face_w), L.ptr(st.flux), st.clock.ptr, s, arr)
        L.check(rc, "step")
        st.cons, st.cons_next = st.cons_next, st.cons

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.1)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(args.steps):
        marked_step(k)
    e1.record()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    if world > 1:
        torch.distributed.barrier()
    ms_total = e0.elapsed_time(e1)
    st.check_status()
    names = (["k_grad32", "k_face32", "k_update32"] if st.precision == "fp32"
             else ["k_gradients", "k_face_flux", "k_update_step"])
    per = {nm: 0.0 for nm in names}
    for k in range(args.steps):
        for q, nm in enumerate(names):
            per[nm] += marks[4 * k + q].elapsed_time(marks[4 * k + q + 1])
    per = {nm: v / args.steps for nm, v in per.items()}
    t = torch.tensor([ms_total], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(t.item())
    value = world * F * args.steps / (ms_max * 1e-3)

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
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "kernel": dom,
                "peak_source": peak_src, "algorithmic_bytes": algo[dom],
                "kernel_ms": {k: round(v, 5) for k, v in per.items()}}

    # end to end through the public API with host buffers: the host mesh hands over
    # its face list and cell geometry each step (pinned host -> device), the step runs,
    # and the generator velocities (what the host re-mesh needs) plus the clock come back
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, st, mesh, prim, dev)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(256, args.cpu_seconds, args.solver)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": max(3, args.warmup), "ms_per_step": ms_max / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32" if st.precision == "fp32" else "f64",
               "data": "synthetic",
               "config": {"workload": "shear layer 1024x1024 jittered lattice, periodic, gamma 5/3"
                          if args.n_side == 1024 else "shear layer %dx%d" % (args.n_side, args.n_side),
                          "cells": mesh.n_real, "ghosts": mesh.n_ghost, "faces": F, "solver": args.solver,
                          "reconstruction": "piecewise linear, AREPO limiter + GIZMO pair limiter",
                          "precision": st.precision + ("+fp64-accumulate" if st.precision == "fp32" else ""),
                          "mesh": "fixed across steps (host re-mesh outside the path)",
                          "l2": "inputs larger than L2 (per-step working set %.0f MB > 129 MB)"
                                % (sum(algo.values()) / 1e6),
                          "parallelism": "replicas" if world > 1 else "single GPU"},
               "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
               "gpu_launches": 3 * args.steps, "clocks": clocks}
        print(json.dumps(out), flush=True)


def run_e2e(args, st, mesh, prim, dev):
    import torch
    from phd_code_gb300 import _lib as L
    import ctypes
    dm = st.dmesh
    names = ("tag", "type", "map", "x", "dcom", "vol", "pair_i", "pair_j", "area", "com", "normal",
             "nbr_ptr", "nbr_idx")
    host = {nm: getattr(dm, nm).cpu().pin_memory() for nm in names}
    w_host = torch.empty_like(st.w2 if st.precision == "fp32" else st.w, device="cpu").pin_memory()
    clk_host = torch.empty(L.CLOCK_BYTES, dtype=torch.uint8).pin_memory()
    lib = L.lib()
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    d2h = w_host.numel() * w_host.element_size() + clk_host.numel()

    def one():
        s = L.stream_handle()
        for nm in names:
            getattr(dm, nm).copy_(host[nm], non_blocking=True)
        if st.precision == "fp32":
            out = L.PhdGeom32Out(*(t.data_ptr() for t in (st.face_geo, st.face_ar, st.csr_face, st.csr_nbr,
                                                           st.cell_geo)))
            L.check(lib.phd_prepare_f32(dm.ref, L.ptr(st.twin), ctypes.byref(out), s), "prepare")
        st.step(1)
        w_host.copy_(st.w2 if st.precision == "fp32" else st.w, non_blocking=True)
        clk_host.copy_(st.clock.buf, non_blocking=True)

    for _ in range(2):
        one()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record()
    for _ in range(args.e2e_steps):
        one()
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms = e0.elapsed_time(e1) / args.e2e_steps
    return {"value": mesh.n_faces / (max(ms * 1e-3, wall / args.e2e_steps)), "unit": UNIT,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": max(ms, 1e3 * wall / args.e2e_steps), "steps": args.e2e_steps,
            "what": "per step: host mesh (face list + cell geometry) H2D from pinned memory, FP32 geometry "
                    "prepare, flux step, generator velocities + clock D2H"}


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
        else:
            run_ours(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
