"""The C restatement against the reference's own compiled Cython path on fresh seeded
meshes (development container only: skipped where the reference build is absent)."""
import numpy as np
import pytest

import oracle as O
import ref_harness as rh
from _util import lattice_mesh, smooth_state

pytestmark = pytest.mark.skipif(not rh.available(), reason="reference build (oracle/_ref) not present")


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
@pytest.mark.parametrize("solver", ["hll", "hllc", "exact"])
@pytest.mark.parametrize("seed", [21, 22])
def test_moving_steps_bit_exact(boundary, solver, seed):
    m = lattice_mesh(20, boundary, seed=seed)
    prim = smooth_state(m, "sod" if seed % 2 else "wave")
    s = rh.RefStep(m, prim, riemann=solver)
    stp = O.OracleStepper(m, solver=solver, moving=True)
    p = prim.copy()
    c = O.cons_from_prim(m, p, 1.4)
    for _ in range(4):
        dt = s.time_step()
        assert dt == O.time_step(m, p, 1.4, 0.5, True)
        s.moving_step_fixed_mesh(dt)
        assert stp.step(dt, p, c) == 0
    assert np.array_equal(p, s.prim())
    assert np.array_equal(c, s.cons())


@pytest.mark.parametrize("limiter", ["arepo", "tess"])
@pytest.mark.parametrize("boost", [True, False])
def test_static_steps_bit_exact(limiter, boost):
    m = lattice_mesh(18, "reflective", seed=5)
    prim = smooth_state(m)
    s = rh.RefStep(m, prim, riemann="hllc", limiter=limiter, boost=boost)
    stp = O.OracleStepper(m, solver="hllc", moving=False, limiter=0 if limiter == "arepo" else 1, boost=boost)
    p = prim.copy()
    c = O.cons_from_prim(m, p, 1.4)
    for _ in range(3):
        dt = s.time_step()
        s.static_step(dt)
        stp.step(dt, p, c)
    assert np.array_equal(p, s.prim())


def test_hilbert_random_points():
    R = rh._import()
    rng = np.random.default_rng(99)
    xh = rng.integers(-2 ** 20, 2 ** 20, 3000).astype(np.int32)
    yh = rng.integers(-2 ** 20, 2 ** 20, 3000).astype(np.int32)
    ref = np.array([R["py_hilbert_key_2d"](np.array([a, b], dtype=np.int32), 18) for a, b in zip(xh, yh)])
    assert np.array_equal(ref, O.hilbert_key_2d(xh, yh))
