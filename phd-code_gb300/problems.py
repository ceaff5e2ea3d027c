"""Seeded synthetic initial conditions for the flux path's workloads.

Each function returns ``(mesh, prim, info)``: a host mesh (cells real-then-ghost,
Hilbert-ordered), primitives for all cells (ghosts filled from their images with the
reflective velocity flip) and a dict of run parameters.  They stand in for the
reference's own problem scripts (``test_suite/``), which have no public dataset: the
shapes, sizes and value ranges are those of the workloads this package is measured on.
"""
import numpy as np

from . import meshgen


def _finish(mesh, rho, vx, vy, p):
    prim = np.stack([rho, vx, vy, p]).astype(np.float64)
    return meshgen.fill_ghosts(mesh, prim)


def shock_tube(n_side=100, seed=0, jitter=0.1):
    """Two-state shock tube: reflective unit box, x < 0.5: rho = 1, p = 1; else
    rho = 0.125, p = 0.1; u = 0; gamma = 1.4 (cf. test_suite/sod/2d/random)."""
    mesh, _ = meshgen.build_mesh(meshgen.jittered_lattice(n_side, jitter=jitter, seed=seed), "reflective")
    x = mesh.x
    left = x[0] < 0.5
    z = np.zeros(x.shape[1])
    return mesh, _finish(mesh, np.where(left, 1.0, 0.125), z, z, np.where(left, 1.0, 0.1)), \
        {"gamma": 1.4, "t_end": 0.1, "cfl": 0.5, "solver": "hllc"}


def point_explosion(n_side=256, seed=0, jitter=0.1, energy=1.0, gamma=1.4):
    """Periodic unit box, rho = 1, p = 1e-5, u = 0; total energy E deposited as a
    uniform energy density in the cells whose generators lie within two lattice
    spacings of the centre (cf. test_suite/sedov)."""
    mesh, _ = meshgen.build_mesh(meshgen.jittered_lattice(n_side, jitter=jitter, seed=seed), "periodic")
    x = mesh.x
    n = mesh.n_real
    dx = 1.0 / n_side
    r = np.hypot(x[0, :n] - 0.5, x[1, :n] - 0.5)
    dep = r <= 2.0 * dx
    p = np.full(mesh.n_cells, 1e-5)
    p[:n][dep] = (gamma - 1.0) * energy / mesh.vol[:n][dep].sum()
    z = np.zeros(mesh.n_cells)
    return mesh, _finish(mesh, np.ones(mesh.n_cells), z, z, p), \
        {"gamma": gamma, "t_end": 0.05, "cfl": 0.5, "deposit_cells": int(dep.sum())}


def shear_layer(n_side=1024, seed=0, jitter=0.1):
    """Periodic unit box, gamma = 5/3, p = 2.5; |y - 0.5| < 0.25: rho = 2, v_x = 0.5;
    else rho = 1, v_x = -0.5; v_y = 0.01 sin(4 pi x) + uniform noise of amplitude
    1e-3 (cf. test_suite/kelvin_helmholtz)."""
    mesh, _ = meshgen.build_mesh(meshgen.jittered_lattice(n_side, jitter=jitter, seed=seed), "periodic")
    rng = np.random.default_rng(seed + 1)
    x = mesh.x
    band = np.abs(x[1] - 0.5) < 0.25
    vy = 0.01 * np.sin(4 * np.pi * x[0]) + 1e-3 * rng.uniform(-1.0, 1.0, x.shape[1])
    return mesh, _finish(mesh, np.where(band, 2.0, 1.0), np.where(band, 0.5, -0.5), vy,
                         np.full(x.shape[1], 2.5)), {"gamma": 5.0 / 3.0, "steps": 200, "cfl": 0.5}


def gaussian_bump(n_side=128, seed=0, jitter=0.1, amplitude=0.1, width=0.05, background=True):
    """Periodic unit box, gamma = 1.4, rho = 1, p = 1, u = 0, plus (unless
    ``background`` only) a density bump amplitude * exp(-r^2 / (2 width^2)) at a seeded
    centre -- width is the Gaussian standard deviation."""
    mesh, _ = meshgen.build_mesh(meshgen.jittered_lattice(n_side, jitter=jitter, seed=seed), "periodic")
    rng = np.random.default_rng(seed + 7)
    c = rng.uniform(0.25, 0.75, 2)
    x = mesh.x
    # distance on the periodic box
    d = np.abs(x - c[:, None])
    d = np.minimum(d, 1.0 - d)
    bump = amplitude * np.exp(-(d[0] ** 2 + d[1] ** 2) / (2.0 * width ** 2))
    rho = 1.0 + (0.0 if background else bump)
    z = np.zeros(x.shape[1])
    return mesh, _finish(mesh, np.broadcast_to(rho, z.shape).copy(), z, z, np.ones_like(z)), \
        {"gamma": 1.4, "steps": 200, "cfl": 0.4, "checkpoint": 20, "centre": c.tolist()}


def riemann_ensemble(n_runs=256, n_min=1000, n_max=65536, seed=0, jitter=0.1):
    """Independent two-state Riemann problems: generator counts log-uniform in
    [n_min, n_max] (jittered lattice of ceil(sqrt(N))^2 points on the unit box,
    reflective walls); an interface through the centre at a random angle; on each
    side rho, p ~ U[0.1, 1] and v ~ U[-0.5, 0.5]^2; gamma = 1.4.  Returns a list of
    (mesh, prim) and the parameters."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(n_min), np.log(n_max), n_runs))
    runs = []
    for r, N in enumerate(counts):
        side = int(np.ceil(np.sqrt(N)))
        mesh, _ = meshgen.build_mesh(meshgen.jittered_lattice(side, jitter=jitter, seed=seed * 1000 + r),
                                     "reflective")
        ang = rng.uniform(0.0, np.pi)
        nrm = np.array([np.cos(ang), np.sin(ang)])
        st = rng.uniform(0.1, 1.0, (2, 2))          # [side][rho, p]
        vel = rng.uniform(-0.5, 0.5, (2, 2))        # [side][vx, vy]
        x = mesh.x
        s = ((x[0] - 0.5) * nrm[0] + (x[1] - 0.5) * nrm[1]) > 0
        rho = np.where(s, st[1, 0], st[0, 0])
        p = np.where(s, st[1, 1], st[0, 1])
        vx = np.where(s, vel[1, 0], vel[0, 0])
        vy = np.where(s, vel[1, 1], vel[0, 1])
        runs.append((mesh, _finish(mesh, rho, vx, vy, p)))
    return runs, {"gamma": 1.4, "steps": 100, "cfl": 0.5}
