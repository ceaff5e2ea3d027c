"""The exact Riemann solver against samples of the reference's own Toro exact solver
(test_suite/sod/riemann.py; fixture tests/golden/exact_riemann.npz, made by
tests/golden/make_exact_riemann.py): Toro's tests 1-5 (near-vacuum double rarefaction,
strong shocks, shock collision) and 400 seeded random problems.  The C oracle (the
restatement of riemann.pyx Exact that the GPU's FP64 path matches bit for bit) must give
the flux of the exact solution at the face to the accuracy of its Newton tolerance
(2|dp|/(p_new + p_old) <= 1e-6, quadratic convergence): bound 1e-8 of each field's
largest flux (measured 1.3e-13).  The GPU's exact solver is checked against the same
samples in tests/test_gpu_exact_riemann_golden.py."""
import numpy as np
import pytest

import oracle as O
from _exact_golden import face_mesh, load, rel_err, sample_flux, states

TOL = 1e-8


@pytest.mark.parametrize("gamma", [1.4, 5.0 / 3.0])
def test_oracle_exact_solver_matches_the_exact_solution(gamma):
    d = load()
    sel = np.flatnonzero(np.isclose(d["gamma"], gamma))
    m = face_mesh(len(sel))
    left, right = states(d, sel)
    flux, st = O.riemann(m, "exact", gamma, True, left, right, np.zeros((2, len(sel))))
    assert st == 0
    err = rel_err(flux, sample_flux(d, sel))
    assert np.all(err <= TOL), err


def test_toro_tests_pstar():
    d = load()
    # Toro, table 4.2: p* of tests 1-5, to the digits printed there (within one unit of
    # the last printed digit: the table truncates 1691.647 to 1691.64)
    printed = np.array([0.30313, 0.00189, 460.894, 46.0950, 1691.64])
    last_digit = np.array([1e-5, 1e-5, 1e-3, 1e-4, 1e-2])
    assert np.all(np.abs(d["pstar"][:5] - printed) <= last_digit)
