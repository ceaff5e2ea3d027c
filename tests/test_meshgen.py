"""Host mesh builder: the reference's extract_geometry conventions and the mesh
identities the reference's own mesh tests check (phd/mesh/test/test_mesh.py)."""
import numpy as np
import pytest

import phd_code_gb300 as pkg
from _util import lattice_mesh


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_total_volume_is_box(boundary):
    m = lattice_mesh(20, boundary, seed=3)
    assert abs(m.vol[:m.n_real].sum() - 1.0) < 1e-12      # test_mesh.py:132-145


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_unjittered_lattice_identities(boundary):
    """test_mesh.py:206-251: on a Cartesian lattice every cell is a dx^2 square with
    its generator at the centroid."""
    n = 10
    m = lattice_mesh(n, boundary, jitter=0.0)
    dx = 1.0 / n
    np.testing.assert_allclose(m.vol[:m.n_real], dx * dx, rtol=1e-10)
    assert np.max(np.abs(m.dcom[:, :m.n_real])) < 1e-12


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_face_conventions(boundary):
    m = lattice_mesh(16, boundary, seed=4)
    n = m.n_real
    assert np.all(m.pair_i < n)                                  # pair-i always real
    assert np.all(m.pair_i < m.pair_j)                           # tess.cpp:363
    d = m.x[:, m.pair_j] - m.x[:, m.pair_i]
    np.testing.assert_allclose(m.normal, d / np.linalg.norm(d, axis=0), atol=1e-14)
    assert np.all(np.diff(m.pair_i) >= 0)                        # emitted per real cell
    for c in range(m.n_cells):                                   # ascending face ids
        lst = m.nbr_idx[m.nbr_ptr[c]:m.nbr_ptr[c + 1]]
        assert np.all(np.diff(lst) > 0)
        assert np.all((m.pair_i[lst] == c) | (m.pair_j[lst] == c))
    g = np.arange(n, m.n_cells)
    assert np.all(m.tag[g] == 1) and np.all(m.tag[:n] == 0)
    np.testing.assert_array_equal(m.vol[g], m.vol[m.map[g]])
    np.testing.assert_array_equal(m.dcom[:, g], m.dcom[:, m.map[g]])


def test_periodic_ghost_shifts():
    m = lattice_mesh(16, "periodic", seed=5)
    g = np.arange(m.n_real, m.n_cells)
    d = m.x[:, g] - m.x[:, m.map[g]]
    assert np.all(np.isclose(np.abs(d), 0.0) | np.isclose(np.abs(d), 1.0))
    assert np.all(m.flip_mask() == 0)


def test_reflective_ghost_mirrors():
    m = lattice_mesh(16, "reflective", seed=6)
    g = np.arange(m.n_real, m.n_cells)
    fm = m.flip_mask()[g]
    assert np.all((fm == 1) | (fm == 2))                         # one mirror axis each
    for k in range(2):
        sel = (fm & (1 << k)) != 0
        xi = m.x[k, m.map[g[sel]]]
        xg = m.x[k, g[sel]]
        edge = np.where(xg < 0.0, 0.0, 1.0)
        np.testing.assert_allclose(xg, 2 * edge - xi, atol=1e-15)


def test_hilbert_order_is_local():
    x = pkg.meshgen.jittered_lattice(32, seed=1)
    m, order = pkg.meshgen.build_mesh(x, "periodic", hilbert=True)
    assert sorted(order.tolist()) == list(range(32 * 32))
    step = np.linalg.norm(np.diff(m.x[:, :m.n_real], axis=1), axis=0)
    assert np.median(step) < 2.0 / 32
