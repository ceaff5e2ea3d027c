"""Host C++ tessellation (include/phdtess.h, phd-code_gb300/tess.py) against the
independent scipy/Qhull builder, the reference's Tess2d method semantics
(phd/mesh/tess.cpp) and the reference's mesh identities (phd/mesh/test/test_mesh.py).
CPU only."""
import numpy as np
import pytest

import phd_code_gb300 as pkg
from phd_code_gb300 import meshgen, tess

BOX = ((0.0, 0.0), (1.0, 1.0))


def _pair(n, boundary, seed, jitter=0.1):
    x = meshgen.jittered_lattice(n, jitter=jitter, seed=seed)
    a, _ = meshgen.build_mesh(x, boundary, hilbert=False, backend="scipy")
    b, _ = meshgen.build_mesh(x, boundary, hilbert=False, backend="native")
    return a, b


def _face_keys(m):
    """Faces keyed by (real cell, image of the other cell, other cell's position)."""
    return {(int(i), int(m.map[j]), float(m.x[0, j]), float(m.x[1, j])): f
            for f, (i, j) in enumerate(zip(m.pair_i, m.pair_j))}


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
@pytest.mark.parametrize("n", [16, 48])
def test_periodic_mesh_equals_scipy_builder(n, seed):
    a, b = _pair(n, "periodic", seed)
    dx = 1.0 / n
    assert (a.n_cells, a.n_faces) == (b.n_cells, b.n_faces)
    for k in ("pair_i", "pair_j", "nbr_ptr", "nbr_idx", "map", "tag", "type"):
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)
    np.testing.assert_array_equal(a.x, b.x)
    np.testing.assert_array_equal(a.normal, b.normal)          # same formula on the same generators
    assert np.max(np.abs(a.area - b.area)) <= 1e-12 * dx        # circumcentres agree to rounding
    assert np.max(np.abs(a.com - b.com)) <= 1e-12 * dx
    assert np.max(np.abs(a.vol / b.vol - 1.0)) <= 1e-12
    assert np.max(np.abs(a.dcom - b.dcom)) <= 1e-11 * dx


@pytest.mark.parametrize("seed", [0, 1])
def test_reflective_mesh_differs_only_by_zero_area_faces(seed):
    """A generator, its neighbour and their mirror images across a wall are exactly
    cocircular: either diagonal is Delaunay, so the two builders may emit different
    zero-area faces there (their two circumcentres coincide to rounding) and nowhere
    else."""
    a, b = _pair(24, "reflective", seed)
    dx = 1.0 / 24
    ka, kb = _face_keys(a), _face_keys(b)
    only_a, only_b = set(ka) - set(kb), set(kb) - set(ka)
    assert all(a.area[ka[k]] <= 1e-12 * dx for k in only_a)
    assert all(b.area[kb[k]] <= 1e-12 * dx for k in only_b)
    for k in set(ka) & set(kb):
        assert abs(a.area[ka[k]] - b.area[kb[k]]) <= 1e-12 * dx
    n = a.n_real
    assert np.max(np.abs(a.vol[:n] / b.vol[:n] - 1.0)) <= 1e-12
    assert np.max(np.abs(a.dcom[:, :n] - b.dcom[:, :n])) <= 1e-11 * dx


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_unjittered_lattice_is_all_squares(boundary):
    """test_mesh.py:206-251 on a lattice, where every four neighbours are cocircular:
    the exact predicates still give a valid tessellation."""
    n = 12
    m, _ = meshgen.build_mesh(meshgen.jittered_lattice(n, jitter=0.0), boundary, backend="native")
    np.testing.assert_allclose(m.vol[:m.n_real], 1.0 / n ** 2, rtol=1e-12)
    assert np.max(np.abs(m.dcom[:, :m.n_real])) < 1e-13
    assert abs(m.vol[:m.n_real].sum() - 1.0) < 1e-12


def test_random_points_and_cocircular_rings_cover_the_box():
    """Uniform random generators plus rings of exactly cocircular points (a regular
    polygon around a centre): total volume is the box (test_mesh.py:132-145)."""
    rng = np.random.default_rng(4)
    pts = [rng.uniform(0.0, 1.0, (2, 400))]
    for cx, cy, r in ((0.3, 0.3, 0.05), (0.7, 0.6, 0.08)):
        ang = np.arange(8) * (np.pi / 4)
        pts.append(np.stack([cx + r * np.cos(ang), cy + r * np.sin(ang)]))
        pts.append(np.array([[cx], [cy]]))
    x = np.concatenate(pts, axis=1)
    for boundary in ("periodic", "reflective"):
        m, _ = meshgen.build_mesh(x, boundary, backend="native")
        assert abs(m.vol[:m.n_real].sum() - 1.0) < 1e-12
        assert np.all(m.vol[:m.n_real] > 0.0)


def test_duplicate_generator_is_an_error():
    x = meshgen.jittered_lattice(8, seed=1)
    x[:, 5] = x[:, 9]
    with pytest.raises(RuntimeError, match="duplicate"):
        tess.build_mesh_native(x, "periodic", *BOX, pad=3.0 / 8)


def test_tess2d_methods_follow_the_reference():
    """build_initial_tess -> radius -1 on the hull, 2*max Voronoi-vertex distance inside
    (tess.cpp:35-142); count_number_of_faces -1 until ghosts close the hull cells
    (tess.cpp:189-236); update_initial_tess / update_radius / extract_geometry then give
    the mesh the whole-box builder gives (before its ghost pruning)."""
    n = 10
    x = meshgen.jittered_lattice(n, seed=2)
    t = tess.Tess2d()
    radius = np.zeros(n * n)
    assert t.build_initial_tess(x, radius, n * n) == 0
    from scipy.spatial import Delaunay                           # the independent triangulation
    tri = Delaunay(x.T)
    on_hull = np.zeros(n * n, dtype=bool)
    on_hull[np.unique(tri.convex_hull)] = True
    np.testing.assert_array_equal(radius < 0, on_hull)
    cc = meshgen._circumcenters(x.T.copy(), tri.simplices)
    expect = np.zeros(n * n)
    for k in range(3):
        v = tri.simplices[:, k]
        np.maximum.at(expect, v, np.sum((cc - x.T[v]) ** 2, axis=1))
    inner = ~on_hull
    np.testing.assert_allclose(radius[inner], 2.0 * np.sqrt(expect[inner]), rtol=1e-9)
    assert t.count_number_of_faces() == -1

    gx, gmap = meshgen._ghosts(x, "periodic", BOX[0], BOX[1], 3.0 / n)
    allx = np.concatenate([x, gx], axis=1)
    assert t.update_initial_tess(allx, n * n, allx.shape[1]) == 0
    assert t.update_radius(radius, np.arange(n * n)) == 0
    assert np.all(radius > 0.0)
    geo = t.extract_geometry()
    ref, _ = meshgen.build_mesh(x, "periodic", hilbert=False, backend="native")
    assert geo["pair_i"].size == ref.n_faces
    np.testing.assert_array_equal(geo["pair_i"], ref.pair_i)
    np.testing.assert_array_equal(gmap[geo["pair_j"][geo["pair_j"] >= n * n] - n * n],
                                  ref.map[ref.pair_j[ref.pair_j >= n * n]])
    np.testing.assert_array_equal(geo["area"], ref.area)
    np.testing.assert_array_equal(geo["volume"], ref.vol[:n * n])
    np.testing.assert_array_equal(geo["dcom"], ref.dcom[:, :n * n])
    for c in range(n * n):                                       # ascending face lists
        lst = geo["nbr_idx"][geo["nbr_ptr"][c]:geo["nbr_ptr"][c + 1]]
        assert np.all(np.diff(lst) > 0)


def test_hilbert_keys_native_equal_reference_vectors():
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "hilbert_2d.npz"))
    np.testing.assert_array_equal(tess.hilbert_keys_2d(d["xh"], d["yh"], 18), d["keys"])
    rng = np.random.default_rng(0)
    xh = rng.integers(0, 2 ** 18, 5000).astype(np.int32)
    yh = rng.integers(0, 2 ** 18, 5000).astype(np.int32)
    np.testing.assert_array_equal(tess.hilbert_keys_2d(xh, yh, 18), pkg.hilbert.hilbert_key_2d(xh, yh))


def test_hilbert_order_same_for_both_backends():
    x = meshgen.jittered_lattice(40, seed=3)
    _, oa = meshgen.build_mesh(x, "periodic", backend="scipy")
    _, ob = meshgen.build_mesh(x, "periodic", backend="native")
    np.testing.assert_array_equal(oa, ob)


@pytest.mark.parametrize("jitter", [0.1, 0.0])
@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_strip_parallel_build_equals_the_serial_one(boundary, jitter):
    """Strips tessellated on parallel threads give the whole box's tessellation bit for
    bit -- also with exactly cocircular generators (a lattice, mirror images at walls),
    which the symbolic perturbation of the lift decides the same way in every strip."""
    x = meshgen.jittered_lattice(80, jitter=jitter, seed=6)
    ref, _ = tess.build_mesh_native(x, boundary, *BOX, pad=3.0 / 80, n_strips=1)
    for k in (2, 5):
        o, _ = tess.build_mesh_native(x, boundary, *BOX, pad=3.0 / 80, n_strips=k)
        for name in o:
            np.testing.assert_array_equal(o[name], ref[name], err_msg="%s, %d strips" % (name, k))


def test_insertion_order_does_not_change_the_mesh():
    """With the perturbed lift the Delaunay triangulation is unique: the same generators
    in another order give the same neighbour pairs and volumes, even on an exact lattice
    with mirror images at the walls."""
    n = 24
    nr = n * n
    x = meshgen.jittered_lattice(n, jitter=0.0)
    perm = np.random.default_rng(1).permutation(nr)        # b's real cell k is a's cell perm[k]
    a, _ = tess.build_mesh_native(x, "reflective", *BOX, pad=3.0 / n)
    b, _ = tess.build_mesh_native(x[:, perm], "reflective", *BOX, pad=3.0 / n)

    def pairs(m, label):
        out = set()
        for i, j in zip(m["pair_i"], m["pair_j"]):
            if j < nr:
                out.add(("real",) + tuple(sorted((int(label[i]), int(label[j])))))
            else:
                out.add(("ghost", int(label[i]), int(label[m["map"][j]]), float(m["x"][0, j]), float(m["x"][1, j])))
        return out

    assert a["pair_i"].size == b["pair_i"].size
    assert pairs(a, np.arange(nr)) == pairs(b, perm)
    np.testing.assert_allclose(b["vol"][:nr], a["vol"][perm], rtol=1e-13)


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_compact_pair_j_packing_round_trips(boundary):
    """phd_mesh2d_copy_compact16: pair-j as the 16-bit difference to the owner cell with
    the faces that do not fit listed as (face id, pair-j) in ascending face id -- decoded,
    the int32 pair-j of phd_mesh2d_copy_compact; every other array is the same (area and
    offset interleaved in face32); a list buffer that is too small gives -5 and the number
    needed; the list lengths are each cell's face count."""
    import ctypes as C
    L = tess.lib()
    x = meshgen.jittered_lattice(260, jitter=0.4, seed=3)         # 67,600 real cells: escapes
    h = L.phd_tess2d_create()
    try:
        pad = 3.0 / 260
        assert L.phd_mesh2d_build_strips(h, x[0].ctypes.data_as(C.c_void_p), x[1].ctypes.data_as(C.c_void_p),
                                         x.shape[1], {"periodic": 0, "reflective": 1}[boundary], 0.0, 0.0, 1.0,
                                         1.0, pad, 0) >= 0
        nc, nf, pu = C.c_int32(), C.c_int32(), C.c_double()
        L.phd_mesh2d_sizes(h, C.byref(nc), C.byref(nf), C.byref(pu))
        n, F, nr = nc.value, nf.value, x.shape[1]

        def bufs():
            return {"face_ptr": np.zeros(nr + 1, np.int32), "area32": np.zeros(F, np.float32),
                    "ct32": np.zeros(F, np.float32), "x": np.zeros((2, n)), "map": np.zeros(n, np.int32),
                    "tag": np.zeros(n, np.int8), "type": np.zeros(n, np.int8),
                    "ghost_code": np.zeros(max(n - nr, 1), np.int8)}

        p = lambda a: a.ctypes.data_as(C.c_void_p)
        rest = ("x", "map", "tag", "type", "ghost_code")
        a = bufs()
        pair_j = np.zeros(F, np.int32)
        assert L.phd_mesh2d_copy_compact(h, p(a["face_ptr"]), p(pair_j), p(a["area32"]), p(a["ct32"]),
                                         *(p(a[k]) for k in rest)) == 0
        b = bufs()
        dj = np.zeros(F, np.uint16)
        face32 = np.zeros((F, 2), np.float32)
        k = C.c_int32()
        small = np.zeros(2 * 4, np.int32)
        assert L.phd_mesh2d_copy_compact16(h, p(b["face_ptr"]), p(dj), p(small), 4, C.byref(k), None, p(face32),
                                           *(p(b[nm]) for nm in rest)) == -5
        K = k.value
        assert K > 4
        px = np.zeros(2 * K, np.int32)
        ln = np.zeros(n, np.uint8)
        assert L.phd_mesh2d_copy_compact16(h, p(b["face_ptr"]), p(dj), p(px), K, C.byref(k), p(ln), p(face32),
                                           *(p(b[nm]) for nm in rest)) == 0
        assert k.value == K
    finally:
        L.phd_tess2d_destroy(h)
    b["area32"], b["ct32"] = face32[:, 0].copy(), face32[:, 1].copy()
    for nm in a:
        np.testing.assert_array_equal(a[nm], b[nm], err_msg=nm)
    owner = np.repeat(np.arange(nr), np.diff(a["face_ptr"]))
    fid, pj = px[0::2], px[1::2]
    assert np.all(np.diff(fid) > 0)
    assert np.array_equal(np.flatnonzero(dj == 0), fid)
    decoded = owner + dj.astype(np.int64)
    decoded[fid] = pj
    np.testing.assert_array_equal(decoded, pair_j)
    d = pair_j.astype(np.int64) - owner
    assert np.array_equal((d >= 1) & (d <= 65534), dj != 0)
    np.testing.assert_array_equal(ln, np.bincount(np.concatenate([owner, pair_j]), minlength=n))
    assert not np.any(dj == 65535)
