"""The C-ABI libraries build (libphdflux.so for sm_103a, libphdtess.so for the host),
load, and export every entry point that include/phdflux.h and include/phdtess.h
declare (no kernel is launched: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

import phd_code_gb300 as pkg
from phd_code_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


HEADERS = {"phdflux.h": "libphdflux.so", "phdtess.h": "libphdtess.so"}


def declared(header="phdflux.h"):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(phd_[a-z0-9_]+)\s*\(", text)))


def test_every_header_has_a_library():
    assert sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")) == sorted(HEADERS)


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("phd_build", os.path.join(ROOT, "phd-code_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    return ctypes.CDLL(b.LIB)


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_tessellation_library_exports(lib):
    from phd_code_gb300 import tess
    names = declared("phdtess.h")
    assert len(names) >= 10
    t = ctypes.CDLL(tess.LIB_PATH)
    missing = [n for n in names if not hasattr(t, n)]
    assert not missing, missing
    assert set(names) <= set(tess._SIGNATURES), set(names) - set(tess._SIGNATURES)


def test_binding_covers_declarations(lib):
    assert set(declared()) <= set(_lib.SIGNATURES), set(declared()) - set(_lib.SIGNATURES)


def test_host_only_calls(lib):
    lib.phd_abi_version.restype = ctypes.c_int
    assert lib.phd_abi_version() == 1
    lib.phd_status_string.restype = ctypes.c_char_p
    lib.phd_status_string.argtypes = [ctypes.c_int]
    assert lib.phd_status_string(1) == b"Mass less than zero in flux update"


def test_argument_errors_are_rejected_on_the_host(lib):
    """Entry points validate their arguments before touching the device: missing
    pointers and malformed sizes return PHD_ERR_ARG (no GPU is needed to see that)."""
    L = _lib
    f = L.lib()                      # argtypes / restypes from the ctypes table
    assert f.phd_step_f64(None, None, 0, None, None, None, None, None, None, None, None, None) == L.PHD_ERR_ARG
    assert f.phd_gradients_f64(None, None, 0, None, None, None) == L.PHD_ERR_ARG
    assert f.phd_build_csr(None, None, None, None, None, None) == L.PHD_ERR_ARG
    assert f.phd_face_normals_f64(None, None, None, None) == L.PHD_ERR_ARG
    assert f.phd_prepare_f32(None, None, None, None) == L.PHD_ERR_ARG
    m = L.PhdMesh()
    m.dim, m.n_cells, m.n_real, m.n_faces = 2, 10, 10, 5
    # a mesh with faces but no normals is refused by the FP64 entries that read normals
    one = ctypes.c_void_p(1)
    assert f.phd_riemann_f64(ctypes.byref(m), L.HLLC, 1.4, 1, 100, one, one, None, one, one, None) == L.PHD_ERR_ARG
    # launch shapes out of range, and several runs without a cell-to-run table
    par = L.PhdParams()
    geo = L.PhdGeom32()
    for lch in (L.PhdLaunch(48, 128, 128, 0, 0, 0),       # not a multiple of 32
                L.PhdLaunch(128, 512, 128, 0, 0, 0),      # face kernel above its 256-thread bound
                L.PhdLaunch(128, 128, 128, 0, 0, 0, 3, 1, 1)):   # items per thread other than 1, 2, 4
        rc = f.phd_step_f32_batched(ctypes.byref(m), ctypes.byref(geo), ctypes.byref(par), 0, ctypes.byref(lch),
                                    one, one, one, one, one, one, one, 1, None, None, None)
        assert rc == L.PHD_ERR_ARG
    assert f.phd_prim_f32_batched(ctypes.byref(m), ctypes.byref(par), one, one, one, 3, None, None) == L.PHD_ERR_ARG
    # compact hand-over: missing ranges / outputs, and faces without their FP32 geometry
    assert f.phd_pair_i_from_face_ptr(ctypes.byref(m), None, one, one, None) == L.PHD_ERR_ARG
    out = L.PhdGeom32Out(1, 1, 1, 1, 1)
    assert f.phd_prepare_f32_faces_compact(ctypes.byref(m), None, None, ctypes.byref(out), None) == L.PHD_ERR_ARG
    assert f.phd_prepare_f32_faces_compact(None, one, one, ctypes.byref(out), None) == L.PHD_ERR_ARG
    # generator move: exactly one velocity array, and a real box
    m.x = 1
    assert f.phd_move_generators(ctypes.byref(m), None, None, one, 1, 0.0, 0.0, 1.0, 1.0, one, None) == L.PHD_ERR_ARG
    assert f.phd_move_generators(ctypes.byref(m), one, one, one, 1, 0.0, 0.0, 1.0, 1.0, one, None) == L.PHD_ERR_ARG
    # one-call compact hand-over: incomplete hand-over, a mesh that still carries FP64
    # normals, an empty box, ghosts without their codes
    h = L.PhdHandover32(face_ptr=1, pair_j=1, area32=1, ct32=1, type=1, d_face_ptr=1, d_area32=1, d_ct32=1,
                        twin=1, csr_work=1, bad=1, periodic=1, dedup_periodic=1,
                        xmin=(ctypes.c_double * 2)(0.0, 0.0), xmax=(ctypes.c_double * 2)(1.0, 1.0))
    ev = (ctypes.c_void_p * 8)(1, 1, 1, 1, 1, 1, 1, 1)
    sides = (ctypes.c_void_p * 2)(None, None)
    m.x, m.normal, m.n_real = 1, None, 8
    m.pair_i = m.pair_j = m.map = m.flip = m.nbr_ptr = m.nbr_idx = 1

    def load(mesh, hh):
        return f.phd_load_mesh_f32(ctypes.byref(mesh), ctypes.byref(hh), ctypes.byref(par), ctypes.byref(out), one,
                                   one, one, None, sides, ev)

    assert load(m, h) == L.PHD_ERR_ARG                    # 2 ghosts, neither positions nor ghost codes
    h.ghost_code, h.d_ghost_code = 1, 1
    m.normal = 1
    assert load(m, h) == L.PHD_ERR_ARG                    # FP64 normals still attached
    m.normal = None
    h.xmax = (ctypes.c_double * 2)(0.0, 1.0)
    assert load(m, h) == L.PHD_ERR_ARG                    # empty box
    h.xmax = (ctypes.c_double * 2)(1.0, 1.0)
    h.twin = None
    assert load(m, h) == L.PHD_ERR_ARG                    # no twin table
    assert f.phd_load_mesh_f32(None, ctypes.byref(h), ctypes.byref(par), ctypes.byref(out), one, one, one, None,
                               sides, ev) == L.PHD_ERR_ARG
