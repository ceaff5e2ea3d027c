"""The C restatement (oracle) reproduces the reference's own outputs recorded in the
golden fixtures, stage by stage and over three whole steps (CPU only)."""
import platform

import numpy as np
import pytest

import oracle as O
from _util import CONFIGS, load_golden, rel_rows, split

# same glibc and no FMA contraction on x86: bit-identical; elsewhere libm pow may
# round differently in the last place
EXACT = platform.machine() in ("x86_64", "AMD64")
TOL = 0.0 if EXACT else 1e-13


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
@pytest.mark.parametrize("cfg", CONFIGS)
def test_stages_match_reference(boundary, cfg):
    m, d = load_golden(boundary)
    om = O.OracleMesh(m)
    solver, limiter, boost = split(cfg)
    prim = d["prim0"]
    dt = O.time_step(om, prim, 1.4, 0.5, boost or solver == "exact")
    assert dt == float(d[cfg + "/dt"]) or abs(dt - float(d[cfg + "/dt"])) <= TOL * dt
    w = O.generator_velocities(om, prim, 1.4)
    assert rel_rows(w, d[cfg + "/w"]) <= TOL
    fw = O.face_velocities(om, w)
    assert rel_rows(fw, d[cfg + "/face_w"]) <= TOL
    g, st = O.gradients(om, prim, 0 if limiter == "arepo" else 1)
    assert st == 0
    assert rel_rows(g, d[cfg + "/grad"]) <= TOL
    bst = boost or solver == "exact"
    Lf, Rf = O.states(om, prim, g, fw, 1.4, 0.5 * dt, boost=bst)
    assert rel_rows(Lf, d[cfg + "/left"]) <= TOL
    assert rel_rows(Rf, d[cfg + "/right"]) <= TOL
    fl, st = O.riemann(om, solver, 1.4, bst, Lf, Rf, fw)
    assert st == 0
    assert rel_rows(fl, d[cfg + "/flux"]) <= TOL
    c0 = O.cons_from_prim(om, prim, 1.4)
    assert rel_rows(c0, d[cfg + "/cons0"]) <= TOL
    c1, st = O.update(om, fl, dt, c0)
    assert st == 0
    n = m.n_real
    assert rel_rows(c1[:, :n], d[cfg + "/cons1"][:, :n]) <= TOL


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_constant_reconstruction(boundary):
    m, d = load_golden(boundary)
    prim = d["prim0"]
    Lf, Rf = O.states(m, prim, None, np.zeros((2, m.n_faces)), 1.4, 0.0, boost=True, linear=False)
    assert rel_rows(Lf, d["pwc_hllc/left"]) <= TOL
    assert rel_rows(Rf, d["pwc_hllc/right"]) <= TOL
    fl, _ = O.riemann(m, "hllc", 1.4, True, Lf, Rf, np.zeros((2, m.n_faces)))
    assert rel_rows(fl, d["pwc_hllc/flux"]) <= TOL


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
@pytest.mark.parametrize("solver", ["hllc", "exact"])
def test_three_steps_match_reference(boundary, solver):
    m, d = load_golden(boundary)
    prim = d["prim0"].copy()
    cons = O.cons_from_prim(m, prim, 1.4)
    stp = O.OracleStepper(m, solver=solver, moving=True)
    dts = []
    for _ in range(3):
        dt = O.time_step(m, prim, 1.4, 0.5, True)
        dts.append(dt)
        assert stp.step(dt, prim, cons) == 0
    assert rel_rows(np.array(dts), d["run3_%s/dts" % solver]) <= TOL
    assert rel_rows(prim, d["run3_%s/prim" % solver]) <= TOL
    assert rel_rows(cons, d["run3_%s/cons" % solver]) <= TOL


def test_hilbert_keys_match_reference():
    d = np.load(__import__("_util").GOLDEN + "/hilbert_2d.npz")
    assert np.array_equal(O.hilbert_key_2d(d["xh"], d["yh"]), d["keys"])
    import phd_code_gb300 as pkg
    assert np.array_equal(pkg.hilbert.hilbert_key_2d(d["xh"], d["yh"]), d["keys"])


def test_hll_known_answer():
    """HLL/HLLC/Exact on the reference's own known-answer vector
    (phd/riemann/test/test_riemann.py:88-122): rho=1, u=+-2, p=0.4, gamma=1.4,
    n = x, w = 0 gives (mass, mom-x, mom-y, energy) = (+-2, 4.4, 0, +-6.8)."""
    from phd_code_gb300.meshgen import HostMesh
    m = HostMesh(dim=2, n_real=2, x=np.zeros((2, 2)), tag=np.zeros(2, np.int8), type=np.zeros(2, np.int8),
                 map=np.arange(2, dtype=np.int32), vol=np.ones(2), dcom=np.zeros((2, 2)),
                 pair_i=np.array([0], np.int32), pair_j=np.array([1], np.int32), area=np.ones(1),
                 com=np.zeros((2, 1)), normal=np.array([[1.0], [0.0]]),
                 nbr_ptr=np.array([0, 1, 2], np.int32), nbr_idx=np.array([0, 0], np.int32))
    for u, ans in ((2.0, (2.0, 4.4, 0.0, 6.8)), (-2.0, (-2.0, 4.4, 0.0, -6.8))):
        st = np.array([[1.0], [u], [0.0], [0.4]])
        for solver, boost in (("hll", False), ("hllc", False), ("hllc", True), ("exact", True)):
            f, s = O.riemann(m, solver, 1.4, boost, st, st, np.zeros((2, 1)))
            assert s == 0
            np.testing.assert_allclose(f[:, 0], ans, rtol=0, atol=1e-12)
