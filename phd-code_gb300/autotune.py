"""Autotuner for the launch shape of the FP32 step kernels.

For each of the three kernels (gradients, face fluxes, update) it times candidate
(threads per block, grid cap, items per thread) shapes with CUDA events recorded
between the kernels of real steps (``phd_step_f32_batched`` with stage marks), and
keeps the fastest shape of each kernel independently -- the kernels do not share
launch state.  Items per thread sets how many cells or faces one thread handles in a
block's tile (a warp then covers 32 * items faces); every shape gives the same bits.  The state is
saved before tuning and restored afterwards, so tuning does not advance the run.
A grid cap of k * SMs turns a kernel into a persistent launch whose blocks loop over
the work.
"""
import ctypes

import torch

from . import _lib as L

BLOCKS = (128, 256, 384, 512)
FACE_MAX_BLOCK = 256           # k_face32's launch bound (48 registers per thread)
CAP_WAVES = (0, 2, 4, 8)       # 0: one thread per item; k: k blocks per SM
ITEMS = (1, 2, 4)              # cells / faces per thread


def _sm_count(device):
    return torch.cuda.get_device_properties(device).multi_processor_count


def tune(stepper, blocks=BLOCKS, cap_waves=CAP_WAVES, items=ITEMS, reps=9):
    """Pick a PhdLaunch for an EnsembleStepper or an fp32 FluxStepper; returns
    (launch, table) where table maps (block, waves, items) to per-kernel milliseconds
    (the median over ``reps`` timed steps, which keeps a noisy step from deciding)."""
    dev = stepper.device
    sms = _sm_count(dev)
    saved = {k: getattr(stepper, k).clone() for k in ("cons", "cons_next", "prim4", "cellrec", "w2", "flux4")}
    clock_attr = "clocks" if hasattr(stepper, "clocks") else "clock"
    clk_buf = stepper.clocks if clock_attr == "clocks" else stepper.clock.buf
    clk_saved = clk_buf.clone()
    n_runs = getattr(stepper, "n_runs", 1)
    cell_run = getattr(stepper, "cell_run", None)
    lib = L.lib()
    table = {}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4 * reps)]
    for e in ev:
        e.record()
    torch.cuda.synchronize(dev)
    shapes = [(b, w, k) for b in blocks for w in cap_waves for k in items]
    for b, w, it in shapes:
            cap = w * sms
            lch = L.PhdLaunch(b, min(b, FACE_MAX_BLOCK), b, cap, cap, cap, it, it, it)
            for k in range(reps + 1):
                arr = None
                if k > 0:
                    arr = (ctypes.c_void_p * 4)(*(ev[4 * (k - 1) + q].cuda_event for q in range(4)))
                rc = lib.phd_step_f32_batched(stepper.dmesh.ref, ctypes.byref(stepper.geo),
                                              ctypes.byref(stepper.params), int(stepper.moving), ctypes.byref(lch),
                                              L.ptr(stepper.prim4), L.ptr(stepper.cons), L.ptr(stepper.cons_next),
                                              L.ptr(stepper.cellrec), L.ptr(stepper.w2), L.ptr(stepper.flux4),
                                              L.ptr(clk_buf), n_runs, L.ptr(cell_run), L.stream_handle(), arr)
                L.check(rc, "tune step")
            torch.cuda.synchronize(dev)
            samples = [[ev[4 * k + q].elapsed_time(ev[4 * k + q + 1]) for k in range(reps)] for q in range(3)]
            table[(b, w, it)] = [sorted(v)[len(v) // 2] for v in samples]
    for k, v in saved.items():
        getattr(stepper, k).copy_(v)
    clk_buf.copy_(clk_saved)
    best = [min(table, key=lambda key: table[key][q]) for q in range(3)]

    def cap_of(key):
        return key[1] * sms

    launch = L.PhdLaunch(best[0][0], min(best[1][0], FACE_MAX_BLOCK), best[2][0], cap_of(best[0]), cap_of(best[1]),
                         cap_of(best[2]), best[0][2], best[1][2], best[2][2])
    return launch, table
