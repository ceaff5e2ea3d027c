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
from _util import FP64_TOL, lattice_mesh, assert_parity, rel_rows, smooth_state

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
    assert_parity(st.cons_host()[:, :nr], c[:, :nr])
    assert_parity(st.prim_host(), p)


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


def _moved_meshes(n, boundary, seed, count):
    """Tessellations of the same real cells (same count and order) at new generator
    positions -- a lattice jittered by up to 0.4 spacings, drawn afresh per re-mesh --
    so the ghost and face counts change from one mesh to the next."""
    out = []
    for k in range(count):
        x = pkg.meshgen.jittered_lattice(n, jitter=0.4, seed=seed + k)
        m, _ = pkg.meshgen.build_mesh(x, boundary, hilbert=False)
        out.append(m)
    return out


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_load_mesh_with_changing_counts_fp64_follows_the_oracle(boundary):
    meshes = _moved_meshes(18, boundary, 7, 5)
    assert len({(m.n_cells, m.n_faces) for m in meshes}) > 1
    prim = smooth_state(meshes[0])
    st = FluxStepper(meshes[0], prim, gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp64")
    for k in range(1, len(meshes)):
        st.step(1)
        st.load_mesh(st.dmesh.pinned_host(meshes[k]))
        assert (st.dmesh.n_cells, st.dmesh.n_faces) == (meshes[k].n_cells, meshes[k].n_faces)
    st.check_status()
    assert st.dmesh.upload_errors() == 0
    c, p = _oracle_replay(meshes, prim, 1.4)
    nr = meshes[0].n_real
    assert_parity(st.cons_host()[:, :nr], c[:, :nr])
    assert_parity(st.prim_host(), p)


def test_load_mesh_with_changing_counts_fp32_conserves_and_replays():
    """FP32 through re-meshes with changing counts: exact exchange of mass and energy,
    density close to the FP64 oracle, and a CUDA graph captured after the last
    re-shape replays the same steps as direct launches."""
    meshes = _moved_meshes(24, "periodic", 8, 5)
    assert len({(m.n_cells, m.n_faces) for m in meshes}) > 1
    prim = smooth_state(meshes[0])
    st = FluxStepper(meshes[0], prim, gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp32")
    nr = meshes[0].n_real
    c0 = st.cons_host()[:, :nr].sum(axis=1)
    for k in range(1, len(meshes)):
        st.step(1)
        st.load_mesh(st.dmesh.pinned_host(meshes[k]))
    st.check_status()
    cons = st.cons_host()[:, :nr]
    c1 = cons.sum(axis=1)
    for q in (0, 3):
        assert abs(c1[q] - c0[q]) <= 1e-12 * abs(c0[q])
    c, _ = _oracle_replay(meshes, prim, 1.4)
    vol = meshes[-1].vol[:nr]
    assert np.mean(np.abs(cons[0] / vol - c[0, :nr] / vol)) <= 1e-5
    # graph after the re-shape: 4 captured steps == 4 direct steps
    clock0 = st.clock.buf.clone()
    cons0, prim0 = st.cons.clone(), st.prim4.clone()
    st.step(4)
    torch.cuda.synchronize()
    direct = st.cons_host()
    st.clock.buf.copy_(clock0)
    st.cons.copy_(cons0)
    st.prim4.copy_(prim0)
    st.capture(4)
    st.clock.buf.copy_(clock0)
    st.cons.copy_(cons0)
    st.prim4.copy_(prim0)
    st.replay()
    torch.cuda.synchronize()
    assert np.array_equal(st.cons_host(), direct)


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_compact_hand_over_equals_the_full_one(boundary):
    """The compact FP32 hand-over (pair-i from per-cell face ranges, FP32 area and
    centroid offset rounded on the host) forms the same FP32 geometry bit for bit, so
    the steps that follow are identical; it moves about half the bytes."""
    meshes = _moved_meshes(20, boundary, 3, 4)
    prim = smooth_state(meshes[0])
    kw = dict(gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp32", handover_records=True)
    a = FluxStepper(meshes[0], prim, **kw)
    b = FluxStepper(meshes[0], prim, **kw)
    for k in range(1, len(meshes)):
        a.step(1)
        b.step(1)
        na = a.load_mesh(a.dmesh.pinned_host(meshes[k]))
        nb = b.load_mesh(b.dmesh.pinned_host_compact(meshes[k]))
        assert nb < 0.7 * na
        torch.cuda.synchronize()
        assert b.dmesh.upload_errors() == 0
        for name in ("face_geo", "face_ar", "csr_face", "csr_nbr", "cell_geo", "twin", "prim4"):
            assert torch.equal(getattr(a, name), getattr(b, name)), name
        e = int(a.dmesh.nbr_ptr[a.dmesh.n_real].item())
        assert torch.equal(a.entry_rec[:e], b.entry_rec[:e])
        assert torch.equal(a.dmesh.pair_i, b.dmesh.pair_i)
    a.step(3)
    b.step(3)
    a.check_status()
    b.check_status()
    assert np.array_equal(a.cons_host(), b.cons_host())


def test_compact_hand_over_rejects_broken_face_ranges():
    """Face ranges that do not tile the face list are counted as upload errors (and
    never written); the stepper refuses the compact hand-over in FP64."""
    meshes = _moved_meshes(12, "periodic", 5, 2)
    prim = smooth_state(meshes[0])
    st = FluxStepper(meshes[0], prim, gamma=1.4, precision="fp32")
    pinned = st.dmesh.pinned_host_compact(meshes[1])
    pinned["face_ptr"][5] = pinned["face_ptr"][6] + 1           # cell 5's range runs backwards
    st.load_mesh(pinned)
    torch.cuda.synchronize()
    assert st.dmesh.upload_errors() >= 1
    st64 = FluxStepper(meshes[0], prim, gamma=1.4, precision="fp64")
    with pytest.raises(ValueError, match="FP32"):
        st64.load_mesh(st64.dmesh.pinned_host_compact(meshes[1]))


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_compact_mesher_equals_the_host_mesh_path(boundary):
    """tess.CompactMesher writes the compact hand-over straight from the C++
    tessellation into reused pinned buffers: the same arrays, bit for bit, as building
    the host mesh and rounding it in DeviceMesh.pinned_host_compact."""
    meshes = _moved_meshes(22, boundary, 9, 3)
    st = FluxStepper(meshes[0], smooth_state(meshes[0]), gamma=1.4, precision="fp32")
    mesher = pkg.tess.CompactMesher(boundary)
    for m in meshes[1:]:
        a = st.dmesh.pinned_host_compact(m)
        b = mesher(m.x[:, :m.n_real])
        assert sorted(a) == sorted(b)
        for k in a:
            assert torch.equal(a[k], b[k]), k
        st.load_mesh(b)
        torch.cuda.synchronize()
        assert st.dmesh.upload_errors() == 0


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_device_generator_move_follows_the_reference(precision):
    """move_generators (domain_manager.pyx:566-590 + the periodic wrap of
    boundary.pyx:502-538) on the device equals the host evaluation with the step's dt and
    generator velocities, bit for bit."""
    m = lattice_mesh(24, "periodic", seed=4)
    prim = smooth_state(m)
    prim[1] += 0.8                                   # drift right so generators cross x = 1
    st = FluxStepper(m, prim, gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision=precision)
    st.step(1)
    c = st.read_clock()
    c.dt_last = 0.05                                 # a long move, so that generators cross the box
    dt = c.dt_last
    st.clock.buf.copy_(torch.frombuffer(bytearray(bytes(c)), dtype=torch.uint8))
    xd = st.move_generators().cpu().numpy()
    st.check_status()
    nr = m.n_real
    w = (st.w2[:nr].double().t() if precision == "fp32" else st.w[:, :nr]).cpu().numpy()
    xs = m.x[:, :nr] + dt * w
    out = (xs < 0.0) | (xs > 1.0)
    outside = out[0] | out[1]
    expect = xs.copy()
    for k in range(2):
        expect[k] = np.where(outside & (xs[k] <= 0.0), expect[k] + 1.0, expect[k])
        expect[k] = np.where(outside & (xs[k] >= 1.0), expect[k] - 1.0, expect[k])
    assert outside.any()
    assert np.array_equal(xd, expect)


def test_generator_leaving_a_reflective_box_is_flagged():
    m = lattice_mesh(16, "reflective", seed=2)
    prim = smooth_state(m)
    prim[1] -= 3.0                                   # everything rushes to the x = 0 wall: with
    st = FluxStepper(m, prim, gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp32")
    st.step(1)                                       # boost the CFL step ignores |v|, so the
    st.move_generators()                             # cells at the wall cross it in one step
    with pytest.raises(RuntimeError, match="particle left domain in reflective boundary condition"):
        st.check_status()


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_resident_positions_hand_over_equals_the_full_one(boundary):
    """A compact hand-over without positions: the real positions stay on the device and
    the ghosts' come from their codes (phd_ghost_positions) -- equal to the host's bit
    for bit, so the steps are identical to the full hand-over's; with the device's own
    generator move in the loop, positions never cross the link to the device."""
    meshes = _moved_meshes(20, boundary, 11, 3)
    prim = smooth_state(meshes[0])
    a = FluxStepper(meshes[0], prim, gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp32")
    b = FluxStepper(meshes[0], prim, gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp32")
    nb_full = a.load_mesh(a.dmesh.pinned_host(meshes[0]))
    nb = b.load_mesh(b.dmesh.pinned_host_compact(meshes[0], resident=True))
    assert nb < 0.55 * nb_full
    torch.cuda.synchronize()
    assert b.dmesh.upload_errors() == 0
    assert torch.equal(a.dmesh.x, b.dmesh.x)                    # ghosts formed on the device
    a.step(2)
    b.step(2)
    assert np.array_equal(a.cons_host(), b.cons_host())
    # the whole loop: device move, host tessellation of the moved generators, resident hand-over
    mesher = pkg.tess.CompactMesher(boundary, resident=True)
    full = pkg.tess.CompactMesher(boundary)
    for _ in range(3):
        a.step(1)
        b.step(1)
        xa = a.move_generators()
        xb = b.move_generators()
        a.check_status()
        x_host = xa.cpu().numpy()
        assert np.array_equal(x_host, xb.cpu().numpy())
        a.load_mesh(full(x_host))
        b.load_mesh(mesher(x_host))
        torch.cuda.synchronize()
        assert b.dmesh.upload_errors() == 0
        assert torch.equal(a.dmesh.x, b.dmesh.x)
    a.step(2)
    b.step(2)
    a.check_status()
    assert np.array_equal(a.cons_host(), b.cons_host())


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_step_and_fetch_returns_the_step_velocities_early(precision):
    """step_and_fetch copies the generator velocities to pinned host memory on a copy
    stream as soon as the step's first stage has formed them: the same velocities and
    the same state as a plain step followed by a copy, several steps in a row."""
    m = lattice_mesh(24, "periodic", seed=4)
    prim = smooth_state(m)
    a = FluxStepper(m, prim, gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision=precision)
    b = FluxStepper(m, prim, gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision=precision)
    wa = a.w2 if precision == "fp32" else a.w
    host = torch.empty_like(wa, device="cpu").pin_memory()
    for _ in range(3):
        a.step(1)
        ev = b.step_and_fetch(host)
        ev.synchronize()
        assert torch.equal(host, wa.cpu())
    a.check_status()
    b.check_status()
    assert np.array_equal(a.cons_host(), b.cons_host())
    fixed = FluxStepper(m, prim, gamma=1.4, cfl=0.5, solver="hllc", moving=False, precision=precision)
    with pytest.raises(RuntimeError, match="moving-mesh"):
        fixed.step_and_fetch(host)


def test_compact_hand_over_without_periodic_dedup():
    """With periodic twin de-duplication off, the one-call compact hand-over leaves the
    twin table empty (every entry -1) and forms the same lists, geometry and state as
    the full hand-over with de-duplication off."""
    meshes = _moved_meshes(20, "periodic", 5, 3)
    prim = smooth_state(meshes[0])
    kw = dict(gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp32", dedup_periodic=False,
              handover_records=True)
    a = FluxStepper(meshes[0], prim, **kw)
    b = FluxStepper(meshes[0], prim, **kw)
    for k in range(1, len(meshes)):
        a.step(1)
        b.step(1)
        a.load_mesh(a.dmesh.pinned_host(meshes[k]))
        b.load_mesh(b.dmesh.pinned_host_compact(meshes[k]))
        torch.cuda.synchronize()
        assert b.dmesh.upload_errors() == 0
        assert bool((b.twin == -1).all())
        for name in ("face_geo", "face_ar", "csr_face", "csr_nbr", "cell_geo", "twin", "prim4"):
            assert torch.equal(getattr(a, name), getattr(b, name)), name
        e = int(a.dmesh.nbr_ptr[a.dmesh.n_real].item())
        assert torch.equal(a.entry_rec[:e], b.entry_rec[:e])
    a.step(2)
    b.step(2)
    assert np.array_equal(a.cons_host(), b.cons_host())


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
@pytest.mark.parametrize("limiter", ["arepo", "tess"])
def test_steps_without_entry_records_equal_steps_with_them(boundary, limiter):
    """A hand-over without the per-entry gradient records: the gradient kernel forms
    each entry's record from its face with the same roundings, so cell records,
    velocities and conserved totals equal those of a stepper whose hand-over wrote the
    records, bit for bit, through the device generator move and compact re-meshes; the
    records built afterwards equal the hand-over's, and a captured graph uses them."""
    meshes = _moved_meshes(20, boundary, 13, 2)
    prim = smooth_state(meshes[0])
    kw = dict(gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp32", limiter=limiter)
    a = FluxStepper(meshes[0], prim, handover_records=True, **kw)
    b = FluxStepper(meshes[0], prim, **kw)
    mesher = pkg.tess.CompactMesher(boundary, resident=True)
    for _ in range(3):
        a.step(1)
        b.step(1)
        xa = a.move_generators()
        xb = b.move_generators()
        a.check_status()
        b.check_status()
        x_host = xa.cpu().numpy()
        assert np.array_equal(x_host, xb.cpu().numpy())
        a.load_mesh(mesher(x_host))
        b.load_mesh(mesher(x_host))
        assert a.records and not b.records and b.geo.entry_rec is None
        a.step(1)
        b.step(1)
        torch.cuda.synchronize()
        assert torch.equal(a.cellrec, b.cellrec)
        assert torch.equal(a.w2, b.w2)
        assert np.array_equal(a.cons_host(), b.cons_host())
    e = int(a.dmesh.nbr_ptr[a.dmesh.n_real].item())
    b.capture(2)                                  # builds the records first
    assert b.records and b.geo.entry_rec is not None
    torch.cuda.synchronize()
    assert torch.equal(a.entry_rec[:e], b.entry_rec[:e])
    a.step(2)
    b.replay()
    torch.cuda.synchronize()
    assert np.array_equal(a.cons_host(), b.cons_host())


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_packed_pair_j_hand_over_equals_the_int32_one(boundary):
    """pair-j handed over as 16-bit differences to the owner cell plus the escaped faces
    (pair_dj, pair_x) decodes on the device to the int32 hand-over's pair-j: every derived
    array and the steps that follow are the same, bit for bit.  67,600 real cells, so
    faces to far ghosts escape; the C++ mesher's packed hand-over equals numpy's."""
    meshes = _moved_meshes(260, boundary, 23, 2)
    prim = smooth_state(meshes[0])
    kw = dict(gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp32")
    a = FluxStepper(meshes[0], prim, **kw)
    b = FluxStepper(meshes[0], prim, **kw)
    pa = a.dmesh.pinned_host_compact(meshes[1], pair16=False)
    pb = b.dmesh.pinned_host_compact(meshes[1])
    assert pb["pair_x"].numel() > 0
    na = a.load_mesh(pa)
    nb = b.load_mesh(pb)
    assert nb < na
    torch.cuda.synchronize()
    assert a.dmesh.upload_errors() == 0 and b.dmesh.upload_errors() == 0
    for name in ("pair_i", "pair_j", "nbr_ptr", "nbr_idx", "x", "flip"):
        assert torch.equal(getattr(a.dmesh, name), getattr(b.dmesh, name)), name
    for name in ("face_geo", "face_ar", "csr_face", "csr_nbr", "cell_geo", "twin", "prim4"):
        assert torch.equal(getattr(a, name), getattr(b, name)), name
    a.step(2)
    b.step(2)
    a.check_status()
    assert np.array_equal(a.cons_host(), b.cons_host())
    c = pkg.tess.CompactMesher(boundary)(meshes[1].x[:, :meshes[1].n_real])
    assert sorted(c) == sorted(pb)
    for k in pb:
        assert torch.equal(c[k], pb[k]), k


@pytest.mark.parametrize("delta", [1, -1])
def test_wrong_list_lengths_are_upload_errors(delta):
    """List lengths handed over with the packed pair-j that do not match the faces (one
    cell's length off by one, so the lists either overrun their storage by one entry or
    leave one unfilled) are counted as upload errors; the lists stay inside their storage
    and a correct hand-over afterwards is clean again."""
    meshes = _moved_meshes(16, "periodic", 29, 2)
    prim = smooth_state(meshes[0])
    st = FluxStepper(meshes[0], prim, gamma=1.4, precision="fp32")
    bad = st.dmesh.pinned_host_compact(meshes[1])
    assert "list_len" in bad
    bad["list_len"][7] += delta
    st.load_mesh(bad)
    torch.cuda.synchronize()
    assert st.dmesh.upload_errors() >= 1
    e = st.dmesh.nbr_ptr.cpu().numpy()
    assert np.all(np.diff(e) >= 0) and e[-1] <= 2 * meshes[1].n_faces
    st.load_mesh(st.dmesh.pinned_host_compact(meshes[1]))
    torch.cuda.synchronize()
    assert st.dmesh.upload_errors() == 0
    assert np.array_equal(st.dmesh.nbr_idx.cpu().numpy(), meshes[1].nbr_idx)
