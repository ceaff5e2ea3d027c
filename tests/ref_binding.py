"""Reference-side binding of the GB300 flux path: what a maintainer adds to
rickyfernandez/phd-code to run its flux step on the GPU behind its own plugin classes.

TEST HELPER: this is the binding that INTEGRATION.md prints, kept as code so that it is
exercised (tests/test_gpu_ref_dropin.py drives the reference's own integrator with it)
and so that its structures are checked against include/phdflux.h on every CPU run
(tests/test_ref_binding_abi.py).  It uses ctypes only and allocates device memory
through the CUDA runtime, so the reference needs no new dependency.

The drop-in classes are Python subclasses of the reference's cdef classes
(PieceWiseLinear, HLLC, Mesh).  Their cpdef methods -- compute_gradients,
compute_states (reconstruction.pyx:563, 1074), compute_fluxes (riemann.pyx:74) and
update_from_fluxes (mesh.pyx:479) -- are overridable from Python, and a subclass passes
the integrator's check_class guard (integrate.py:148-161, tools.py:19-33).  Each call
copies the state it needs to the device, runs one library entry, and copies the result
back into the reference's own containers: per-stage copies, not the resident path (that
is phd_step_f64 / phd_step_f32 driven by phd_code_gb300.FluxStepper).

The reference keeps Mesh.neighbors as a C++ attribute (mesh.pxd:34) that Python cannot
read; a production binding copies it into CSR from a small .pyx that cimports Mesh.
Here the caller hands the same CSR lists it injected into the reference mesh.
"""
import ctypes as C
import os

import numpy as np

PRIM = ["density", "velocity-x", "velocity-y", "pressure"]
CONS = ["mass", "momentum-x", "momentum-y", "energy"]
GRAD = ["density_x", "density_y", "velocity-x_x", "velocity-x_y",
        "velocity-y_x", "velocity-y_y", "pressure_x", "pressure_y"]
PHD_HLLC = 1                                  # solver selector of phd_riemann_f64
LIMITERS = {"arepo": 0, "tess": 1}


class PhdMesh(C.Structure):
    """phd_mesh (include/phdflux.h)."""
    _fields_ = [("dim", C.c_int32), ("n_cells", C.c_int32), ("n_real", C.c_int32),
                ("n_faces", C.c_int32), ("tag", C.c_void_p), ("map", C.c_void_p),
                ("flip", C.c_void_p), ("x", C.c_void_p), ("dcom", C.c_void_p),
                ("vol", C.c_void_p), ("pair_i", C.c_void_p), ("pair_j", C.c_void_p),
                ("area", C.c_void_p), ("com", C.c_void_p), ("normal", C.c_void_p),
                ("nbr_ptr", C.c_void_p), ("nbr_idx", C.c_void_p)]


class PhdClock(C.Structure):
    """phd_clock (include/phdflux.h): 9 fields, 64 bytes."""
    _fields_ = [("dt", C.c_double), ("t", C.c_double), ("t_end", C.c_double),
                ("dt_hydro", C.c_double), ("dtmin_bits", C.c_uint64),
                ("arrive", C.c_uint32), ("status", C.c_int32), ("step", C.c_int64),
                ("dt_last", C.c_double)]


class PhdParams(C.Structure):
    """phd_params (include/phdflux.h)."""
    _fields_ = [("gamma", C.c_double), ("cfl", C.c_double), ("eta", C.c_double),
                ("reconstruction", C.c_int32), ("limiter", C.c_int32), ("gizmo", C.c_int32),
                ("solver", C.c_int32), ("boost", C.c_int32), ("regularize", C.c_int32),
                ("exact_max_iter", C.c_int32), ("pad_", C.c_int32)]


def load_cudart():
    for name in ("libcudart.so.13", "libcudart.so", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    raise OSError("the CUDA runtime library was not found")


class Device(object):
    """Device buffers through the CUDA runtime (cudaMalloc / cudaMemcpy / cudaFree)."""

    H2D, D2H = 1, 2

    def __init__(self, cudart):
        self.rt = cudart
        self.rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        self.rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        self.rt.cudaFree.argtypes = [C.c_void_p]
        self.live = []

    def upload(self, a):
        a = np.ascontiguousarray(a)
        p = C.c_void_p()
        if self.rt.cudaMalloc(C.byref(p), C.c_size_t(max(a.nbytes, 16))) != 0:
            raise RuntimeError("cudaMalloc failed")
        if a.nbytes and self.rt.cudaMemcpy(p, a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes), self.H2D) != 0:
            raise RuntimeError("cudaMemcpy to the device failed")
        self.live.append(p)
        return p

    def zeros(self, shape, dtype):
        return self.upload(np.zeros(shape, dtype))

    def download(self, p, shape, dtype):
        out = np.empty(shape, dtype)
        if out.nbytes and self.rt.cudaMemcpy(out.ctypes.data_as(C.c_void_p), p, C.c_size_t(out.nbytes),
                                             self.D2H) != 0:
            raise RuntimeError("cudaMemcpy to the host failed")
        return out

    def free_all(self):
        for p in self.live:
            self.rt.cudaFree(p)
        self.live = []


def load_library(lib_path):
    lib = C.CDLL(lib_path)
    vp, i32, f64 = C.c_void_p, C.c_int32, C.c_double
    pm = C.POINTER(PhdMesh)
    sig = {
        "phd_gradients_f64": [pm, vp, i32, vp, vp, vp],
        "phd_states_f64": [pm, vp, vp, vp, f64, f64, i32, i32, i32, i32, vp, vp, vp],
        "phd_riemann_f64": [pm, i32, f64, i32, i32, vp, vp, vp, vp, vp, vp],
        "phd_update_from_fluxes_f64": [pm, vp, f64, vp, vp, vp],
        "phd_flip_mask": [i32, i32, vp, vp, vp, vp, i32, vp, vp],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    return lib


def _stack(container, names):
    return np.stack([np.asarray(container[f], dtype=np.float64) for f in names])


class _DeviceView(object):
    """The reference state of one call on the device: cells, faces and lists."""

    def __init__(self, dev, lib, particles, mesh, domain_manager, csr):
        n = particles.get_carray_size()
        faces = mesh.faces
        F = faces.get_carray_size()
        self.n, self.F = n, F
        m = PhdMesh()
        m.dim, m.n_cells, m.n_faces = 2, n, F
        tag = np.asarray(particles["tag"]).astype(np.int8)
        m.n_real = int(np.count_nonzero(tag == 0))
        m.tag = dev.upload(tag)
        m.map = dev.upload(np.asarray(particles["map"]).astype(np.int32))
        x = _stack(particles, ["position-x", "position-y"])
        m.x = dev.upload(x)
        m.dcom = dev.upload(_stack(particles, ["dcom-x", "dcom-y"]))
        m.vol = dev.upload(np.asarray(particles["volume"], dtype=np.float64))
        m.pair_i = dev.upload(np.asarray(faces["pair-i"]).astype(np.int32))
        m.pair_j = dev.upload(np.asarray(faces["pair-j"]).astype(np.int32))
        m.area = dev.upload(np.asarray(faces["area"], dtype=np.float64))
        m.com = dev.upload(_stack(faces, ["com-x", "com-y"]))
        m.normal = dev.upload(_stack(faces, ["normal-x", "normal-y"]))
        m.nbr_ptr = dev.upload(np.asarray(csr[0], dtype=np.int32))
        m.nbr_idx = dev.upload(np.asarray(csr[1], dtype=np.int32))
        # reflective ghosts flip the normal-velocity gradient (boundary.pyx:287-307)
        flip = dev.zeros(n, np.int8)
        reflective = type(domain_manager.boundary_condition).__name__ == "Reflective"
        lo = (C.c_double * 3)(*(list(domain_manager.xmin) + [0.0])[:3])
        hi = (C.c_double * 3)(*(list(domain_manager.xmax) + [0.0])[:3])
        ty = dev.upload(np.asarray(particles["type"]).astype(np.int8))
        check(lib.phd_flip_mask(2, n, ty, m.x, lo, hi, int(reflective), flip, None), "phd_flip_mask")
        m.flip = flip
        self.mesh = m
        self.prim = dev.upload(_stack(particles, PRIM))
        self.clock = dev.upload(np.frombuffer(bytes(PhdClock()), np.uint8).copy())


def check(rc, what):
    if rc != 0:
        raise RuntimeError("%s returned %d" % (what, rc))


def gpu_plugins(PieceWiseLinear, HLLC, Mesh, lib_path):
    """GPU subclasses of the reference's PieceWiseLinear, HLLC and Mesh classes (pass the
    classes from phd.reconstruction.reconstruction, phd.riemann.riemann, phd.mesh.mesh).
    Set `csr = (nbr_ptr, nbr_idx)` on the reconstruction instance before stepping."""
    lib = load_library(lib_path)
    dev = Device(load_cudart())

    class GpuPieceWiseLinear(PieceWiseLinear):
        csr = None

        def compute_gradients(self, particles, mesh, domain_manager):
            v = _DeviceView(dev, lib, particles, mesh, domain_manager, self.csr)
            grad = dev.zeros((8, v.n), np.float64)
            check(lib.phd_gradients_f64(C.byref(v.mesh), v.prim, LIMITERS[self.limiter], grad, v.clock, None),
                  "phd_gradients_f64")
            g = dev.download(grad, (8, v.n), np.float64)
            st = dev.download(v.clock, (C.sizeof(PhdClock),), np.uint8)
            dev.free_all()
            status = PhdClock.from_buffer_copy(st.tobytes()).status
            if status:
                raise RuntimeError("ERROR: incorrect neighbors!")
            self.grad.resize(v.n)
            for k, f in enumerate(GRAD):
                self.grad[f][:] = g[k]

        def compute_states(self, particles, mesh, gamma, domain_manager, dt, boost):
            v = _DeviceView(dev, lib, particles, mesh, domain_manager, self.csr)
            grad = dev.upload(_stack(self.grad, GRAD))
            fw = dev.upload(_stack(mesh.faces, ["velocity-x", "velocity-y"]))
            left, right = dev.zeros((4, v.F), np.float64), dev.zeros((4, v.F), np.float64)
            # dt is the half step the integrator hands over (integrate.py:398-400)
            check(lib.phd_states_f64(C.byref(v.mesh), v.prim, grad, fw, float(gamma), float(dt), int(boost), 1,
                                     int(self.gizmo_limiter), 3, left, right, None), "phd_states_f64")
            lh = dev.download(left, (4, v.F), np.float64)
            rh = dev.download(right, (4, v.F), np.float64)
            dev.free_all()
            self.left_states.resize(v.F)
            self.right_states.resize(v.F)
            for k, f in enumerate(PRIM):
                self.left_states[f][:] = lh[k]
                self.right_states[f][:] = rh[k]

    class GpuHLLC(HLLC):
        def compute_fluxes(self, particles, mesh, reconstruction, eos):
            faces = mesh.faces
            F = faces.get_carray_size()
            m = PhdMesh()
            m.dim, m.n_cells, m.n_faces = 2, particles.get_carray_size(), F
            m.normal = dev.upload(_stack(faces, ["normal-x", "normal-y"]))
            left = dev.upload(_stack(reconstruction.left_states, PRIM))
            right = dev.upload(_stack(reconstruction.right_states, PRIM))
            fw = dev.upload(_stack(faces, ["velocity-x", "velocity-y"]))
            out = dev.zeros((4, F), np.float64)
            clk = dev.upload(np.frombuffer(bytes(PhdClock()), np.uint8).copy())
            check(lib.phd_riemann_f64(C.byref(m), PHD_HLLC, float(eos.get_gamma()), int(self.boost), 1000, left,
                                      right, fw, out, clk, None), "phd_riemann_f64")
            flux = dev.download(out, (4, F), np.float64)
            dev.free_all()
            self.fluxes.resize(F)
            for k, f in enumerate(CONS):
                self.fluxes[f][:] = flux[k]

    class GpuMesh(Mesh):
        csr = None
        domain_manager = None

        def update_from_fluxes(self, particles, riemann, dt):
            v = _DeviceView(dev, lib, particles, self, self.domain_manager, self.csr)
            flux = dev.upload(_stack(riemann.fluxes, CONS))
            cons = dev.upload(_stack(particles, CONS))
            check(lib.phd_update_from_fluxes_f64(C.byref(v.mesh), flux, float(dt), cons, v.clock, None),
                  "phd_update_from_fluxes_f64")
            u = dev.download(cons, (4, v.n), np.float64)
            st = dev.download(v.clock, (C.sizeof(PhdClock),), np.uint8)
            dev.free_all()
            status = PhdClock.from_buffer_copy(st.tobytes()).status
            if status & 1:
                raise RuntimeError("Mass less than zero in flux update")
            if status & 2:
                raise RuntimeError("Energy less than zero in flux update")
            for k, f in enumerate(CONS):
                particles[f][:] = u[k]

    return GpuPieceWiseLinear, GpuHLLC, GpuMesh

