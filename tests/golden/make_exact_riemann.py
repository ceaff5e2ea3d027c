"""Golden samples of the exact Riemann solution at x/t = 0 from the reference's own
Toro exact solver, test_suite/sod/riemann.py (Derivative, State).

That file is Python 2 (print statements) and writes HDF5, so it cannot be imported here.
This script parses it and runs only its two arithmetic functions, Derivative (the
pressure functions f_K and f_K' of Toro section 4.3) and State (the sampling of the
wave pattern, Toro section 4.5), which are valid Python 3.  The Newton iteration of the
file's riemann() is restated around Derivative, started from the PVRS estimate and run
until the relative change is below 1e-14 instead of the file's 1e-6, so each sample is
the exact solution to FP64 rounding.  Problems: Toro's tests 1-5 (Riemann Solvers and
Numerical Methods for Fluid Dynamics, 3rd ed., table 4.1) and seeded random states.

Run where the reference tree is mounted (the fixture is committed; the GPU machine never
reads the reference):
    python tests/golden/make_exact_riemann.py [REFERENCE_DIR]
"""
import ast
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "exact_riemann.npz")


def reference_functions(reference):
    path = os.path.join(reference, "test_suite", "sod", "riemann.py")
    tree = ast.parse(open(path).read().replace("print ", "pass #"), filename=path)
    keep = [node for node in tree.body if isinstance(node, ast.FunctionDef) and node.name in ("Derivative", "State")]
    if len(keep) != 2:
        raise RuntimeError("Derivative / State not found in %s" % path)
    scope = {"sqrt": __import__("math").sqrt}
    exec(compile(ast.Module(body=keep, type_ignores=[]), path, "exec"), scope)
    return scope["Derivative"], scope["State"]


def solve(derivative, state, dl, ul, pl, dr, ur, pr, g):
    cl, cr = np.sqrt(g * pl / dl), np.sqrt(g * pr / dr)
    p = max(1e-14, 0.5 * (pl + pr) + 0.125 * (ul - ur) * (dl + dr) * (cl + cr))
    for _ in range(200):
        fl, dfl = derivative(p, dl, pl, cl, g)
        fr, dfr = derivative(p, dr, pr, cr, g)
        p_new = p - (fl + fr + ur - ul) / (dfl + dfr)
        if p_new <= 0.0:
            p_new = 1e-14
        done = 2.0 * abs(p_new - p) <= 1e-14 * (p_new + p)
        p = p_new
        if done:
            break
    else:
        raise RuntimeError("no convergence")
    fl, _ = derivative(p, dl, pl, cl, g)
    fr, _ = derivative(p, dr, pr, cr, g)
    u = 0.5 * (ul + ur + fr - fl)
    d, us, ps = state(p, u, 0.0, dl, ul, pl, cl, dr, ur, pr, cr, g)
    return p, u, d, us, ps


def main():
    reference = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PHD_REFERENCE_DIR", "/root/reference")
    derivative, state = reference_functions(reference)
    toro = [(1.0, 0.0, 1.0, 0.125, 0.0, 0.1), (1.0, -2.0, 0.4, 1.0, 2.0, 0.4), (1.0, 0.0, 1000.0, 1.0, 0.0, 0.01),
            (1.0, 0.0, 0.01, 1.0, 0.0, 100.0), (5.99924, 19.5975, 460.894, 5.99242, -6.19633, 46.0950)]
    rows = [t + (1.4,) for t in toro]
    rng = np.random.default_rng(7)
    for _ in range(400):
        dl, dr, pl, pr = rng.uniform(0.1, 2.0, 4)
        ul, ur = rng.uniform(-1.5, 1.5, 2)
        rows.append((dl, ul, pl, dr, ur, pr, float(rng.choice([1.4, 5.0 / 3.0]))))
    inp = np.array(rows)
    out = np.array([solve(derivative, state, *r) for r in rows])
    np.savez_compressed(OUT, left=inp[:, 0:3], right=inp[:, 3:6], gamma=inp[:, 6], pstar=out[:, 0],
                        ustar=out[:, 1], sample=out[:, 2:5])
    print("wrote %s: %d problems, Toro test 1 p* = %.6f u* = %.6f" % (OUT, len(rows), out[0, 0], out[0, 1]))


if __name__ == "__main__":
    main()
