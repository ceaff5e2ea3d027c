"""ctypes front end of the C restatement in ``oracle/phd_oracle.c``.

TEST INFRASTRUCTURE ONLY: used by tests/, ``__graft_entry__.smoke()`` and the CPU
baseline of ``bench.py`` as the checker.  The product path never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "phd_oracle.c")
LIB = os.path.join(HERE, "libphd_oracle.so")

HLL, HLLC, EXACT = 0, 1, 2
SOLVERS = {"hll": HLL, "hllc": HLLC, "exact": EXACT}


def build(force=False):
    """Compile the restatement with the reference's FP semantics (no FMA contraction).
    C-level ``pow(x, 2.0)`` folds into ``x*x`` here as it does in the reference's
    compiled Cython; the one square the reference evaluates through Python's float
    power at run time calls libm through a pointer (phd_oracle.c)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "phd_oracle.h")),
            os.path.getmtime(os.path.abspath(__file__))):
        return LIB
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                           "-fno-fast-math", "-o", LIB + ".tmp", SRC, "-lm"])
    os.replace(LIB + ".tmp", LIB)
    return LIB


class _Mesh(C.Structure):
    _fields_ = [("dim", C.c_int), ("n_cells", C.c_int), ("n_faces", C.c_int),
                ("reflective", C.c_int),
                ("tag", C.c_void_p), ("type", C.c_void_p), ("map", C.c_void_p),
                ("x", C.c_void_p), ("dcom", C.c_void_p), ("vol", C.c_void_p),
                ("pair_i", C.c_void_p), ("pair_j", C.c_void_p),
                ("area", C.c_void_p), ("com", C.c_void_p), ("normal", C.c_void_p),
                ("nbr_ptr", C.c_void_p), ("nbr_idx", C.c_void_p),
                ("xmin", C.c_double * 3), ("xmax", C.c_double * 3)]


class _Params(C.Structure):
    _fields_ = [("gamma", C.c_double), ("eta", C.c_double),
                ("reconstruction", C.c_int), ("limiter", C.c_int), ("gizmo", C.c_int),
                ("solver", C.c_int), ("boost", C.c_int), ("moving", C.c_int),
                ("regularize", C.c_int), ("exact_max_iter", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, i, d = C.c_void_p, C.c_int, C.c_double
        P = C.POINTER(_Mesh)
        L.orc_compute_gradients.argtypes = [P, vp, i, vp]
        L.orc_pwc_states.argtypes = [P, vp, vp, i, vp, vp]
        L.orc_add_spatial.argtypes = [P, vp, vp, vp, i, i, vp, vp]
        L.orc_add_temporal.argtypes = [P, vp, vp, vp, d, d, i, vp, vp]
        L.orc_riemann.argtypes = [P, i, d, i, vp, vp, vp, vp, i]
        L.orc_update_from_fluxes.argtypes = [P, vp, d, vp]
        L.orc_ghost_refresh_cons.argtypes = [P, vp]
        L.orc_prim_from_cons.argtypes = [i, i, d, vp, vp, vp]
        L.orc_cons_from_prim.argtypes = [i, i, d, vp, vp, vp]
        L.orc_time_step.argtypes = [P, vp, d, d, i]
        L.orc_time_step.restype = d
        L.orc_generator_velocities.argtypes = [P, vp, d, d, i, vp]
        L.orc_face_velocities.argtypes = [P, vp, vp]
        L.orc_hilbert_key_2d.argtypes = [i, vp, vp, i, vp]
        L.orc_step.argtypes = [P, C.POINTER(_Params), d, vp, vp, vp, vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class OracleMesh:
    """Keeps contiguous copies of a HostMesh alive for the C structure."""

    def __init__(self, m):
        self.m = m
        self.arrs = dict(
            tag=_c(m.tag, np.int8), type=_c(m.type, np.int8), map=_c(m.map, np.int32),
            x=_c(m.x, np.float64), dcom=_c(m.dcom, np.float64), vol=_c(m.vol, np.float64),
            pair_i=_c(m.pair_i, np.int32), pair_j=_c(m.pair_j, np.int32),
            area=_c(m.area, np.float64), com=_c(m.com, np.float64),
            normal=_c(m.normal, np.float64), nbr_ptr=_c(m.nbr_ptr, np.int32),
            nbr_idx=_c(m.nbr_idx, np.int32))
        s = _Mesh()
        s.dim, s.n_cells, s.n_faces = m.dim, m.n_cells, m.n_faces
        s.reflective = 1 if m.boundary == "reflective" else 0
        for k, a in self.arrs.items():
            setattr(s, k, a.ctypes.data)
        for k in range(m.dim):
            s.xmin[k] = m.xmin[k]
            s.xmax[k] = m.xmax[k]
        self.s = s
        self.ref = C.byref(s)

    @property
    def n(self):
        return self.m.n_cells

    @property
    def F(self):
        return self.m.n_faces


def _om(mesh):
    return mesh if isinstance(mesh, OracleMesh) else OracleMesh(mesh)


def gradients(mesh, prim, limiter=0):
    om = _om(mesh)
    prim = _c(prim, np.float64)
    g = np.zeros((4 * om.m.dim, om.n))
    st = lib().orc_compute_gradients(om.ref, _p(prim), limiter, _p(g))
    return g, st


def states(mesh, prim, grad, face_w, gamma, dt_half, boost=True, gizmo=True, linear=True):
    om = _om(mesh)
    prim = _c(prim, np.float64)
    face_w = _c(face_w, np.float64)
    L = np.zeros((4, om.F))
    R = np.zeros((4, om.F))
    if linear:
        grad = _c(grad, np.float64)
        lib().orc_add_spatial(om.ref, _p(prim), _p(grad), _p(face_w), int(boost), int(gizmo), _p(L), _p(R))
        lib().orc_add_temporal(om.ref, _p(prim), _p(grad), _p(face_w), gamma, dt_half, int(boost), _p(L), _p(R))
    else:
        lib().orc_pwc_states(om.ref, _p(prim), _p(face_w), int(boost), _p(L), _p(R))
    return L, R


def riemann(mesh, solver, gamma, boost, left, right, face_w, exact_max_iter=1000):
    om = _om(mesh)
    left, right, face_w = (_c(a, np.float64) for a in (left, right, face_w))
    flux = np.zeros((4, om.F))
    st = lib().orc_riemann(om.ref, SOLVERS.get(solver, solver), gamma, int(boost),
                           _p(left), _p(right), _p(face_w), _p(flux), exact_max_iter)
    return flux, st


def update(mesh, flux, dt, cons):
    om = _om(mesh)
    cons = _c(cons, np.float64).copy()
    flux = _c(flux, np.float64)
    st = lib().orc_update_from_fluxes(om.ref, _p(flux), dt, _p(cons))
    return cons, st


def ghost_refresh_cons(mesh, cons):
    om = _om(mesh)
    cons = _c(cons, np.float64).copy()
    lib().orc_ghost_refresh_cons(om.ref, _p(cons))
    return cons


def prim_from_cons(mesh, cons, gamma):
    m = mesh.m if isinstance(mesh, OracleMesh) else mesh
    cons = _c(cons, np.float64)
    vol = _c(m.vol, np.float64)
    prim = np.zeros_like(cons)
    lib().orc_prim_from_cons(m.dim, m.n_cells, gamma, _p(vol), _p(cons), _p(prim))
    return prim


def cons_from_prim(mesh, prim, gamma):
    m = mesh.m if isinstance(mesh, OracleMesh) else mesh
    prim = _c(prim, np.float64)
    vol = _c(m.vol, np.float64)
    cons = np.zeros_like(prim)
    lib().orc_cons_from_prim(m.dim, m.n_cells, gamma, _p(vol), _p(prim), _p(cons))
    return cons


def time_step(mesh, prim, gamma, cfl, boost=True):
    om = _om(mesh)
    prim = _c(prim, np.float64)
    return lib().orc_time_step(om.ref, _p(prim), gamma, cfl, int(boost))


def generator_velocities(mesh, prim, gamma, eta=0.25, regularize=True):
    om = _om(mesh)
    prim = _c(prim, np.float64)
    w = np.zeros((om.m.dim, om.n))
    lib().orc_generator_velocities(om.ref, _p(prim), gamma, eta, int(regularize), _p(w))
    return w


def face_velocities(mesh, w):
    om = _om(mesh)
    w = _c(w, np.float64)
    fw = np.zeros((om.m.dim, om.F))
    lib().orc_face_velocities(om.ref, _p(w), _p(fw))
    return fw


def hilbert_key_2d(xh, yh, order=18):
    xh = _c(xh, np.int32)
    yh = _c(yh, np.int32)
    keys = np.zeros(xh.size, dtype=np.int64)
    lib().orc_hilbert_key_2d(xh.size, _p(xh), _p(yh), order, _p(keys))
    return keys


class OracleStepper:
    """Advance (prim, cons) by whole steps on a fixed mesh (see orc_step)."""

    def __init__(self, mesh, gamma=1.4, solver="hllc", linear=True, limiter=0, gizmo=True,
                 boost=True, moving=True, regularize=True, eta=0.25, face_w=None,
                 exact_max_iter=1000):
        self.om = _om(mesh)
        m = self.om.m
        P = _Params()
        P.gamma, P.eta = gamma, eta
        P.reconstruction = 1 if linear else 0
        P.limiter, P.gizmo = limiter, int(gizmo)
        P.solver = SOLVERS.get(solver, solver)
        P.boost = int(boost if P.solver != EXACT else True)
        P.moving, P.regularize, P.exact_max_iter = int(moving), int(regularize), exact_max_iter
        self.P = P
        n, F, d = m.n_cells, m.n_faces, m.dim
        self.w = np.zeros((d, n))
        self.face_w = np.zeros((d, F)) if face_w is None else _c(face_w, np.float64).copy()
        self.grad = np.zeros((4 * d, n))
        self.left = np.zeros((4, F))
        self.right = np.zeros((4, F))
        self.flux = np.zeros((4, F))

    def step(self, dt, prim, cons):
        st = lib().orc_step(self.om.ref, C.byref(self.P), dt, _p(prim), _p(cons), _p(self.w),
                            _p(self.face_w), _p(self.grad), _p(self.left), _p(self.right),
                            _p(self.flux))
        return st
