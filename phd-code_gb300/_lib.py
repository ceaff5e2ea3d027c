"""ctypes binding of ``libphdflux.so`` (the C ABI declared in ``include/phdflux.h``).

The product path has no CPU fallback: if the library is missing or fails to load,
every device operation raises ``RuntimeError``.  Torch tensors only provide device
memory and streams; the C ABI takes raw pointers.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libphdflux.so")

# host return codes / device status bits / selectors (phdflux.h)
PHD_OK, PHD_ERR_ARG, PHD_ERR_LAUNCH, PHD_ERR_UNSUPPORTED, PHD_ERR_SCRATCH_TOO_SMALL = 0, 1, 2, 3, 4
ADJ_NOALLOC_MAX_DOUBLES = 4194304
GRAD_TAPE_F64_ROWS, GRAD_TAPE_I32_ROWS = 12, 13
STATUS_NEG_MASS, STATUS_NEG_ENERGY, STATUS_RIEMANN_NONCONVERGED, STATUS_BAD_INDEX = 1, 2, 4, 8
STATUS_LEFT_DOMAIN = 16
STATUS_NONFINITE = 32
HLL, HLLC, EXACT = 0, 1, 2
PREP_FACES, PREP_CELLS, PREP_LISTS, PREP_ALL, PREP_CELLS_FROM_FACES, PREP_RECORDS = 1, 2, 4, 7, 8, 16
CONSTANT, LINEAR = 0, 1
LIMITER_AREPO, LIMITER_TESS = 0, 1
STAGE_SPATIAL, STAGE_TEMPORAL = 1, 2
FROZEN_RECORD, FROZEN_REPLAY = 0, 1

STATUS_MESSAGES = {
    STATUS_NEG_MASS: "Mass less than zero in flux update",
    STATUS_NEG_ENERGY: "Energy less than zero in flux update",
    STATUS_RIEMANN_NONCONVERGED: "No convergence in Exact Riemann Solver",
    STATUS_BAD_INDEX: "ERROR: incorrect neighbors!",
    STATUS_LEFT_DOMAIN: "particle left domain in reflective boundary condition!!",
    STATUS_NONFINITE: "Non-finite primitive state after flux update",
}


class PhdMesh(C.Structure):
    _fields_ = [("dim", C.c_int32), ("n_cells", C.c_int32), ("n_real", C.c_int32),
                ("n_faces", C.c_int32),
                ("tag", C.c_void_p), ("map", C.c_void_p), ("flip", C.c_void_p),
                ("x", C.c_void_p), ("dcom", C.c_void_p), ("vol", C.c_void_p),
                ("pair_i", C.c_void_p), ("pair_j", C.c_void_p), ("area", C.c_void_p),
                ("com", C.c_void_p), ("normal", C.c_void_p),
                ("nbr_ptr", C.c_void_p), ("nbr_idx", C.c_void_p)]


class PhdClock(C.Structure):
    _fields_ = [("dt", C.c_double), ("t", C.c_double), ("t_end", C.c_double),
                ("dt_hydro", C.c_double), ("dtmin_bits", C.c_uint64), ("arrive", C.c_uint32),
                ("status", C.c_int32), ("step", C.c_int64), ("dt_last", C.c_double)]


class PhdParams(C.Structure):
    _fields_ = [("gamma", C.c_double), ("cfl", C.c_double), ("eta", C.c_double),
                ("reconstruction", C.c_int32), ("limiter", C.c_int32), ("gizmo", C.c_int32),
                ("solver", C.c_int32), ("boost", C.c_int32), ("regularize", C.c_int32),
                ("exact_max_iter", C.c_int32), ("pad_", C.c_int32)]


class PhdGeom32(C.Structure):
    _fields_ = [("face_geo", C.c_void_p), ("face_ar", C.c_void_p), ("csr_face", C.c_void_p),
                ("csr_nbr", C.c_void_p), ("cell_geo", C.c_void_p), ("entry_rec", C.c_void_p)]


class PhdLaunch(C.Structure):
    _fields_ = [("block_grad", C.c_int32), ("block_face", C.c_int32), ("block_update", C.c_int32),
                ("grid_cap_grad", C.c_int32), ("grid_cap_face", C.c_int32), ("grid_cap_update", C.c_int32),
                ("items_grad", C.c_int32), ("items_face", C.c_int32), ("items_update", C.c_int32)]


class PhdAdjIndex(C.Structure):
    _fields_ = [("partner", C.c_void_p), ("ghost_ptr", C.c_void_p), ("ghost_idx", C.c_void_p)]


class PhdGeom32Out(C.Structure):
    _fields_ = PhdGeom32._fields_


class PhdHandover32(C.Structure):
    """phd_handover32: one compact re-mesh hand-over to an FP32 stepper (phd_load_mesh_f32)."""
    _fields_ = [(nm, C.c_void_p) for nm in ("face_ptr", "pair_j", "area32", "ct32", "ghost_map", "ghost_code", "x",
                                            "x_real", "type", "d_face_ptr", "d_area32", "d_ct32", "d_ghost_code",
                                            "twin", "csr_work", "bad")] + \
        [("periodic", C.c_int32), ("dedup_periodic", C.c_int32), ("xmin", C.c_double * 2), ("xmax", C.c_double * 2),
         ("pair_dj", C.c_void_p), ("pair_x", C.c_void_p), ("n_pair_x", C.c_int32), ("d_pair_dj", C.c_void_p),
         ("d_pair_x", C.c_void_p), ("list_len", C.c_void_p), ("d_list_len", C.c_void_p), ("face32", C.c_void_p),
         ("d_face32", C.c_void_p)]


CLOCK_BYTES = C.sizeof(PhdClock)

_lib = None
_load_error = None

_vp, _i32, _f64 = C.c_void_p, C.c_int32, C.c_double
_PM = C.POINTER(PhdMesh)
_PP = C.POINTER(PhdParams)
_PG = C.POINTER(PhdGeom32)

SIGNATURES = {
    "phd_abi_version": ([], C.c_int),
    "phd_status_string": ([C.c_int], C.c_char_p),
    "phd_gradients_f64": ([_PM, _vp, _i32, _vp, _vp, _vp], C.c_int),
    "phd_states_f64": ([_PM, _vp, _vp, _vp, _f64, _f64, _i32, _i32, _i32, _i32, _vp, _vp, _vp], C.c_int),
    "phd_riemann_f64": ([_PM, _i32, _f64, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp], C.c_int),
    "phd_update_from_fluxes_f64": ([_PM, _vp, _f64, _vp, _vp, _vp], C.c_int),
    "phd_ghost_cons_f64": ([_PM, _vp, _vp], C.c_int),
    "phd_prim_from_cons_f64": ([_i32, _i32, _f64, _vp, _vp, _vp, _vp], C.c_int),
    "phd_cons_from_prim_f64": ([_i32, _i32, _f64, _vp, _vp, _vp, _vp], C.c_int),
    "phd_time_step_f64": ([_PM, _vp, _f64, _f64, _i32, _i32, _vp, _vp], C.c_int),
    "phd_generator_velocities_f64": ([_PM, _vp, _f64, _f64, _i32, _vp, _vp], C.c_int),
    "phd_face_velocities_f64": ([_PM, _vp, _vp, _vp], C.c_int),
    "phd_step_f64": ([_PM, _PP, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], C.c_int),
    "phd_step_f64_marked": ([_PM, _PP, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], C.c_int),
    "phd_step_f64_taped": ([_PM, _PP, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], C.c_int),
    "phd_gradients_f64_taped": ([_PM, _vp, _i32, _vp, _vp, _vp, _vp, _vp], C.c_int),
    "phd_step_f32_marked": ([_PM, _PG, _PP, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], C.c_int),
    "phd_step_f32_batched": ([_PM, _PG, _PP, _i32, C.POINTER(PhdLaunch), _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32,
                              _vp, _vp, _vp], C.c_int),
    "phd_prepare_f32": ([_PM, _vp, C.POINTER(PhdGeom32Out), _vp], C.c_int),
    "phd_prepare_f32_parts": ([_PM, _vp, C.POINTER(PhdGeom32Out), _i32, _vp], C.c_int),
    "phd_prim_f32": ([_PM, _PP, _vp, _vp, _vp, _vp], C.c_int),
    "phd_prim_f32_cells": ([_PM, _vp, _PP, _vp, _vp, _vp, _vp], C.c_int),
    "phd_prim_f32_batched": ([_PM, _PP, _vp, _vp, _vp, _i32, _vp, _vp], C.c_int),
    "phd_step_f32": ([_PM, _PG, _PP, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], C.c_int),
    "phd_adjoint_work_doubles": ([_i32, _i32], C.c_size_t),
    "phd_adjoint_step_f64": ([_PM, C.POINTER(PhdAdjIndex), _PP, _f64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
                             C.c_int),
    "phd_adjoint_step_f64_taped": ([_PM, C.POINTER(PhdAdjIndex), _PP, _f64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                    _vp, _vp], C.c_int),
    "phd_adjoint_step_f64_noalloc": ([_PM, C.POINTER(PhdAdjIndex), _PP, _f64, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
                                     C.c_int),
    "phd_flip_mask": ([_i32, _i32, _vp, _vp, _vp, _vp, _i32, _vp, _vp], C.c_int),
    "phd_hilbert_keys_2d": ([_i32, _vp, _f64, _f64, _f64, _i32, _vp, _vp], C.c_int),
    "phd_face_normals_f64": ([_PM, _vp, _vp, _vp], C.c_int),
    "phd_csr_work_ints": ([_i32], C.c_size_t),
    "phd_build_csr": ([_PM, _vp, _vp, _vp, _vp, _vp], C.c_int),
    "phd_pair_i_from_face_ptr": ([_PM, _vp, _vp, _vp, _vp], C.c_int),
    "phd_move_generators": ([_PM, _vp, _vp, _vp, _i32, _f64, _f64, _f64, _f64, _vp, _vp], C.c_int),
    "phd_ghost_positions": ([_PM, _vp, _f64, _f64, _f64, _f64, _vp, _vp], C.c_int),
    "phd_prepare_f32_faces_compact": ([_PM, _vp, _vp, C.POINTER(PhdGeom32Out), _vp], C.c_int),
    "phd_load_mesh_f32": ([_PM, C.POINTER(PhdHandover32), C.POINTER(PhdParams), C.POINTER(PhdGeom32Out), _vp, _vp,
                           _vp, _vp, _vp, _vp], C.c_int),
    "phd_periodic_twins": ([_PM, _i32, _f64, _f64, _vp, _vp], C.c_int),
    "phd_step_f64_frozen": ([_PM, _PP, _i32, _f64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], C.c_int),
}


def lib():
    """The loaded library; raises if it was not built (no CPU fallback exists)."""
    global _lib, _load_error
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("phd_code_gb300: CUDA extension %s is missing; run "
                           "__graft_entry__.build() first" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def exported_symbols():
    """Names of the SIGNATURES entries the loaded library actually exports."""
    L = lib()
    return sorted(n for n in SIGNATURES if getattr(L, n, None) is not None)


def check(rc, what):
    if rc != PHD_OK:
        raise RuntimeError("%s failed with host code %d" % (what, rc))


def raise_status(status):
    """Map device status bits to the reference's RuntimeError messages."""
    if status:
        msgs = [m for b, m in STATUS_MESSAGES.items() if status & b]
        raise RuntimeError("; ".join(msgs) or ("status %d" % status))


def geom32(tensors, out=False):
    """PhdGeom32 (or PhdGeom32Out) over the FP32 geometry tensors (face_geo, face_ar,
    csr_face, csr_nbr, cell_geo, entry_rec); None gives a NULL pointer."""
    cls = PhdGeom32Out if out else PhdGeom32
    return cls(*(None if t is None else t.data_ptr() for t in tensors))


def ptr(t):
    """Raw device pointer of a tensor (None -> NULL)."""
    return None if t is None else C.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return C.c_void_p(s.cuda_stream)
