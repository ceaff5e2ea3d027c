"""Fused FP64 device step against the oracle on larger meshes, CUDA-graph replay,
determinism and device time-step control."""
import numpy as np
import pytest
import torch

import oracle as O
import phd_code_gb300 as pkg
from _util import FP64_TOL, lattice_mesh, assert_parity, rel_rows, smooth_state

pytestmark = pytest.mark.gpu


def run_oracle(m, prim, solver, n_steps, moving=True, limiter=0, boost=True, reconstruction="linear"):
    p = prim.copy()
    c = O.cons_from_prim(m, p, 1.4)
    stp = O.OracleStepper(m, solver=solver, moving=moving, limiter=limiter, boost=boost,
                          linear=reconstruction == "linear")
    dts = []
    for _ in range(n_steps):
        dt = O.time_step(m, p, 1.4, 0.5, boost or solver == "exact")
        dts.append(dt)
        assert stp.step(dt, p, c) == 0
    return p, c, np.array(dts)


@pytest.mark.parametrize("boundary,n_side", [("periodic", 64), ("reflective", 48)])
@pytest.mark.parametrize("solver", ["hll", "hllc", "exact"])
@pytest.mark.parametrize("moving", [True, False])
def test_fused_step_matches_oracle(boundary, n_side, solver, moving):
    m = lattice_mesh(n_side, boundary, seed=n_side)
    prim = smooth_state(m)
    p_ref, c_ref, dts = run_oracle(m, prim, solver, 4, moving=moving)
    st = pkg.FluxStepper(m, prim, solver=solver, moving=moving)
    got = []
    for _ in range(4):
        got.append(st.read_clock().dt)
        st.step(1)
    st.check_status()
    assert_parity(np.array(got), dts)
    assert_parity(st.prim_host(), p_ref)
    assert_parity(st.cons_host(), c_ref)


@pytest.mark.parametrize("limiter", ["arepo", "tess"])
@pytest.mark.parametrize("boost", [True, False])
def test_fused_step_options(limiter, boost):
    m = lattice_mesh(40, "periodic", seed=3)
    prim = smooth_state(m)
    p_ref, c_ref, _ = run_oracle(m, prim, "hllc", 3, limiter=0 if limiter == "arepo" else 1, boost=boost)
    st = pkg.FluxStepper(m, prim, solver="hllc", limiter=limiter, boost=boost)
    st.step(3)
    assert_parity(st.prim_host(), p_ref)


def test_constant_reconstruction_step():
    m = lattice_mesh(40, "reflective", seed=9)
    prim = smooth_state(m, "sod")
    p_ref, _, _ = run_oracle(m, prim, "hllc", 3, reconstruction="constant")
    st = pkg.FluxStepper(m, prim, solver="hllc", reconstruction="constant")
    st.step(3)
    assert_parity(st.prim_host(), p_ref)


def test_sod_reflective_many_steps():
    m = lattice_mesh(50, "reflective", seed=1)
    prim = smooth_state(m, "sod")
    p_ref, c_ref, _ = run_oracle(m, prim, "hllc", 20)
    st = pkg.FluxStepper(m, prim, solver="hllc")
    st.step(20)
    st.check_status()
    assert_parity(st.prim_host(), p_ref)


def test_graph_replay_equals_eager_and_is_deterministic():
    m = lattice_mesh(64, "periodic", seed=2)
    prim = smooth_state(m)
    a = pkg.FluxStepper(m, prim, solver="hllc")
    a.step(6)
    b = pkg.FluxStepper(m, prim, solver="hllc")
    b.capture(2)
    for _ in range(3):
        b.replay()
    torch.cuda.synchronize()
    assert np.array_equal(a.prim_host(), b.prim_host())       # bitwise: no atomics in sums
    assert a.read_clock().step == b.read_clock().step == 6
    assert a.read_clock().dt == b.read_clock().dt


def test_t_end_clipping():
    m = lattice_mesh(32, "periodic", seed=4)
    prim = smooth_state(m)
    st = pkg.FluxStepper(m, prim, solver="hllc", t_end=1e-3)
    for _ in range(200):
        c = st.read_clock()
        if c.t >= 1e-3:
            break
        st.step(1)
    c = st.read_clock()
    assert c.t == 1e-3
