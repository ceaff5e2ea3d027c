"""Generate the golden fixtures from the reference's own compiled flux path.

Needs the reference build made by ``oracle/build_ref.py`` (development container
only).  For two small seeded meshes (periodic and reflective 12x12 jittered
lattices) it records the mesh, an initial state and the reference's outputs for every
stage and solver, plus a three-step moving-mesh run, and the reference's Hilbert keys
of random integer points.  The fixtures travel with the repository; the GPU tests
compare against them where the reference itself is not available.

Usage:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__ as ge  # noqa: E402

pkg = ge.load_package()
import ref_harness as rh  # noqa: E402

MESH_KEYS = ("x", "tag", "type", "map", "vol", "dcom", "pair_i", "pair_j", "area", "com", "normal",
             "nbr_ptr", "nbr_idx")


def initial_state(m):
    x = m.x
    prim = np.stack([1.0 + 0.5 * np.sin(6 * x[0]) * np.cos(3 * x[1]),
                     0.3 * np.cos(5 * x[1]),
                     0.2 * np.sin(4 * x[0]),
                     1.0 + 0.3 * np.cos(3 * x[1]) + 0.2 * (x[0] > 0.5)])
    return pkg.meshgen.fill_ghosts(m, prim)


def case(boundary, seed, n_side=12):
    m, _ = pkg.meshgen.build_mesh(pkg.meshgen.jittered_lattice(n_side, seed=seed), boundary)
    prim = initial_state(m)
    out = {k: getattr(m, k) for k in MESH_KEYS}
    out["xmin"] = np.array(m.xmin)
    out["xmax"] = np.array(m.xmax)
    out["n_real"] = np.array(m.n_real)
    out["boundary"] = np.array(boundary)
    out["prim0"] = prim
    configs = [("hll", "arepo", True), ("hllc", "arepo", True), ("hllc", "tess", True),
               ("hllc", "arepo", False), ("exact", "arepo", True)]
    for solver, limiter, boost in configs:
        tag = "%s_%s_%s" % (solver, limiter, "boost" if boost else "lab")
        s = rh.RefStep(m, prim, riemann=solver, limiter=limiter, boost=boost)
        dt = s.time_step()
        s.generator_velocities()
        s.face_velocities()
        s.gradients()
        s.states(0.5 * dt)
        L, R = s.left_right()
        s.fluxes()
        c0 = s.cons()
        s.update(dt)
        out[tag + "/dt"] = np.array(dt)
        out[tag + "/w"] = s.w()
        out[tag + "/face_w"] = s.face_w()
        out[tag + "/grad"] = s.grad()
        out[tag + "/left"] = L
        out[tag + "/right"] = R
        out[tag + "/flux"] = s.flux()
        out[tag + "/cons0"] = c0
        out[tag + "/cons1"] = s.cons()
    # piecewise-constant states + HLLC
    s = rh.RefStep(m, prim, riemann="hllc", reconstruction="constant")
    dt = s.time_step()
    s.states(0.5 * dt)
    L, R = s.left_right()
    s.fluxes()
    out["pwc_hllc/dt"] = np.array(dt)
    out["pwc_hllc/left"] = L
    out["pwc_hllc/right"] = R
    out["pwc_hllc/flux"] = s.flux()
    # three whole moving-mesh steps on the fixed mesh
    for solver in ("hllc", "exact"):
        s = rh.RefStep(m, prim, riemann=solver)
        dts = []
        for _ in range(3):
            dt = s.time_step()
            dts.append(dt)
            s.moving_step_fixed_mesh(dt)
        out["run3_%s/dts" % solver] = np.array(dts)
        out["run3_%s/prim" % solver] = s.prim()
        out["run3_%s/cons" % solver] = s.cons()
    return out


def main():
    if not rh.available():
        raise SystemExit("reference build missing: run python oracle/build_ref.py first")
    for boundary, seed in (("periodic", 11), ("reflective", 12)):
        d = case(boundary, seed)
        np.savez_compressed(os.path.join(HERE, "step_%s_12.npz" % boundary), **d)
    R = rh._import()
    rng = np.random.default_rng(5)
    xh = rng.integers(0, 2 ** 18, 256).astype(np.int32)
    yh = rng.integers(0, 2 ** 18, 256).astype(np.int32)
    keys = np.array([R["py_hilbert_key_2d"](np.array([a, b], dtype=np.int32), 18) for a, b in zip(xh, yh)],
                    dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "hilbert_2d.npz"), xh=xh, yh=yh, keys=keys)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
