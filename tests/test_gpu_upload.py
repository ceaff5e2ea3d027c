"""The per-step mesh hand-over: what the device derives from an uploaded face list
(neighbour lists, FP64 normals, periodic twins) against the host's own, and steps that
continue on a re-numbered tessellation through FluxStepper.load_mesh.

Neighbour lists are the reference's Mesh.neighbors order (tess.cpp:378-379: ascending
face ids per cell) and must match exactly; FP64 normals (tess.cpp:320-327, 367-369) must
be bit-identical to the host's IEEE evaluation; the twin table must equal the host's
periodic_twins.  Faces are shuffled before upload so nothing can rely on the
tessellation's own face order.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O
import phd_code_gb300 as pkg
from phd_code_gb300 import _lib as L
from phd_code_gb300.device import DeviceMesh
from phd_code_gb300.meshgen import HostMesh
from phd_code_gb300.step import FluxStepper
from phd_code_gb300.twins import periodic_twins
from _util import FP64_TOL, lattice_mesh, rel_rows, smooth_state

pytestmark = pytest.mark.gpu


def shuffle_faces(m, seed):
    """The same tessellation with its faces re-numbered by a seeded permutation."""
    F = m.n_faces
    perm = np.random.default_rng(seed).permutation(F)      # new face f = old face perm[f]
    pair_i, pair_j = m.pair_i[perm], m.pair_j[perm]
    cells = np.concatenate([pair_i, pair_j]).astype(np.int64)
    fids = np.concatenate([np.arange(F), np.arange(F)])
    o = np.lexsort((fids, cells))
    nbr_idx = fids[o].astype(np.int32)
    nbr_ptr = np.concatenate([[0], np.cumsum(np.bincount(cells, minlength=m.n_cells))]).astype(np.int32)
    return HostMesh(dim=2, n_real=m.n_real, x=m.x, tag=m.tag, type=m.type, map=m.map, vol=m.vol, dcom=m.dcom,
                    pair_i=pair_i, pair_j=pair_j, area=m.area[perm], com=m.com[:, perm].copy(),
                    normal=m.normal[:, perm].copy(), nbr_ptr=nbr_ptr, nbr_idx=nbr_idx, xmin=m.xmin, xmax=m.xmax,
                    boundary=m.boundary)


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
@pytest.mark.parametrize("shuffled", [False, True])
def test_device_derived_mesh_data_matches_host(boundary, shuffled):
    m = lattice_mesh(24, boundary, seed=3)
    if shuffled:
        m = shuffle_faces(m, 11)
    dm = DeviceMesh(m)
    lib = L.lib()
    s = L.stream_handle()
    n, F = dm.n_cells, dm.n_faces
    ptr = torch.full((n + 1,), -7, dtype=torch.int32, device="cuda")
    idx = torch.full((2 * F,), -7, dtype=torch.int32, device="cuda")
    work = torch.empty(int(lib.phd_csr_work_ints(n)), dtype=torch.int32, device="cuda")
    bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    for _ in range(2):                                     # the work array is reusable
        L.check(lib.phd_build_csr(dm.ref, L.ptr(ptr), L.ptr(idx), L.ptr(work), L.ptr(bad), s), "csr")
    nrm = torch.zeros((2, F), dtype=torch.float64, device="cuda")
    L.check(lib.phd_face_normals_f64(dm.ref, L.ptr(nrm), L.ptr(bad), s), "normals")
    twin = torch.full((F,), 5, dtype=torch.int32, device="cuda")
    L.check(lib.phd_periodic_twins(dm.ref, int(boundary == "periodic"), 1.0, 1.0, L.ptr(twin), s), "twins")
    torch.cuda.synchronize()
    assert int(bad.item()) == 0
    assert np.array_equal(ptr.cpu().numpy(), m.nbr_ptr)
    assert np.array_equal(idx.cpu().numpy(), m.nbr_idx)
    assert np.array_equal(nrm.cpu().numpy(), m.normal)     # bit-identical
    assert np.array_equal(twin.cpu().numpy(), periodic_twins(m))


def test_device_csr_counts_and_skips_broken_faces():
    m = lattice_mesh(12, "periodic", seed=1)
    pj = m.pair_j.copy()
    pj[5] = m.n_cells + 3                                  # out of range
    pj[9] = m.pair_i[9]                                    # a cell paired with itself
    broken = HostMesh(**{**m.__dict__, "pair_j": pj})
    dm = DeviceMesh(broken)
    lib = L.lib()
    n, F = dm.n_cells, dm.n_faces
    ptr = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    idx = torch.full((2 * F,), -1, dtype=torch.int32, device="cuda")
    work = torch.empty(int(lib.phd_csr_work_ints(n)), dtype=torch.int32, device="cuda")
    bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    L.check(lib.phd_build_csr(dm.ref, L.ptr(ptr), L.ptr(idx), L.ptr(work), L.ptr(bad), L.stream_handle()), "csr")
    torch.cuda.synchronize()
    assert int(bad.item()) == 2
    p = ptr.cpu().numpy()
    assert p[-1] == 2 * (F - 2)
    got = idx.cpu().numpy()[:p[-1]]
    assert 5 not in got and 9 not in got


def _oracle_replay(meshes, prim, gamma):
    """Step on mesh k, carry the real totals to mesh k+1, refresh ghosts, recover prims."""
    p = prim.copy()
    c = O.cons_from_prim(meshes[0], p, gamma)
    for k in range(len(meshes) - 1):
        mk = meshes[k]
        dt = O.time_step(mk, p, gamma, 0.5, True)
        O.OracleStepper(mk, gamma=gamma, solver="hllc", moving=True).step(dt, p, c)
        nxt = meshes[k + 1]
        c_new = np.zeros((4, nxt.n_cells))
        c_new[:, :nxt.n_real] = c[:, :mk.n_real]
        c = O.ghost_refresh_cons(nxt, c_new)
        p = O.prim_from_cons(nxt, c, gamma)
    return c, p


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_load_mesh_fp64_continues_like_the_oracle(boundary):
    m = lattice_mesh(20, boundary, seed=5)
    prim = smooth_state(m)
    meshes = [m, shuffle_faces(m, 1), shuffle_faces(m, 2), shuffle_faces(m, 3)]
    st = FluxStepper(m, prim, gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp64")
    for k in range(1, len(meshes)):
        st.step(1)
        h2d = st.load_mesh(st.dmesh.pinned_host(meshes[k]))
        assert h2d > 0
    st.check_status()
    assert st.dmesh.upload_errors() == 0
    c, p = _oracle_replay(meshes, prim, 1.4)
    nr = m.n_real
    assert rel_rows(st.cons_host()[:, :nr], c[:, :nr]) <= FP64_TOL
    assert rel_rows(st.prim_host(), p) <= FP64_TOL


def test_load_mesh_fp32_conserves_and_tracks_fp64():
    m = lattice_mesh(24, "periodic", seed=6)
    prim = smooth_state(m)
    meshes = [m, shuffle_faces(m, 4), shuffle_faces(m, 5), shuffle_faces(m, 6)]
    st = FluxStepper(m, prim, gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp32")
    c0 = st.cons_host()[:, :m.n_real].sum(axis=1)
    for k in range(1, len(meshes)):
        st.step(1)
        st.load_mesh(st.dmesh.pinned_host(meshes[k]))
    st.check_status()
    cons = st.cons_host()[:, :m.n_real]
    c1 = cons.sum(axis=1)
    for q in (0, 3):                                       # mass and energy exchanged exactly
        assert abs(c1[q] - c0[q]) <= 1e-12 * abs(c0[q])
    c, _ = _oracle_replay(meshes, prim, 1.4)
    rho32 = cons[0] / m.vol[:m.n_real]
    rho64 = c[0, :m.n_real] / m.vol[:m.n_real]
    assert np.mean(np.abs(rho32 - rho64)) <= 1e-5


def _geom32_buffers(n, F):
    f32 = torch.float32
    return [torch.zeros((F, 4), dtype=f32, device="cuda"), torch.zeros((F, 2), dtype=f32, device="cuda"),
            torch.zeros(2 * F, dtype=torch.int32, device="cuda"), torch.zeros(2 * F, dtype=torch.int32, device="cuda"),
            torch.zeros((n, 4), dtype=f32, device="cuda")]


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_cell_geometry_from_faces_matches_host_volumes(boundary):
    """PHD_PREP_CELLS_FROM_FACES (volume and centre-of-mass sums of tess.cpp:330-393 in
    FP32 from the prepared faces) against the FP32 rounding of the host's FP64 volumes
    and centroids."""
    m = lattice_mesh(24, boundary, seed=4)
    dm = DeviceMesh(m)
    n, F = dm.n_cells, dm.n_faces
    lib = L.lib()
    twin = torch.as_tensor(periodic_twins(m)).cuda()
    a, b = _geom32_buffers(n, F), _geom32_buffers(n, F)
    oa = L.PhdGeom32Out(*(t.data_ptr() for t in a))
    ob = L.PhdGeom32Out(*(t.data_ptr() for t in b))
    s = L.stream_handle()
    L.check(lib.phd_prepare_f32(dm.ref, L.ptr(twin), ctypes.byref(oa), s), "prepare")
    L.check(lib.phd_prepare_f32_parts(dm.ref, L.ptr(twin), ctypes.byref(ob),
                                      L.PREP_FACES | L.PREP_LISTS | L.PREP_CELLS_FROM_FACES, s), "prepare parts")
    torch.cuda.synchronize()
    ga, gb = a[4].double().cpu().numpy(), b[4].double().cpu().numpy()
    dx = 1.0 / 24
    assert np.max(np.abs(gb[:, 2] / ga[:, 2] - 1.0)) <= 2e-6          # 1/V
    assert np.max(np.abs(gb[:, 3] / ga[:, 3] - 1.0)) <= 2e-6          # sqrt(V/pi)
    assert np.max(np.abs(gb[:, :2] - ga[:, :2])) <= 1e-6 * dx          # dcom
    for k in range(4):                                                 # faces and lists unchanged
        assert torch.equal(a[k], b[k])
