"""Periodic twin-face pairing used by the FP32 path for exact conservation (CPU)."""
import numpy as np

from phd_code_gb300.twins import periodic_twins
from _util import lattice_mesh


def test_twins_pair_each_periodic_face_once():
    m = lattice_mesh(24, "periodic", seed=8)
    tw = periodic_twins(m)
    drop = np.nonzero(tw >= 0)[0]
    keep = tw[drop]
    assert drop.size > 0
    assert np.all(keep < drop)
    assert np.unique(keep).size == keep.size                      # one twin per kept face
    i1, g1 = m.pair_i[keep], m.pair_j[keep]
    i2, g2 = m.pair_i[drop], m.pair_j[drop]
    assert np.all(m.map[g1] == i2) and np.all(m.map[g2] == i1)    # (i, ghost of k) <-> (k, ghost of i)
    np.testing.assert_allclose(m.area[keep], m.area[drop], rtol=0, atol=1e-14)   # circumcentres of shifted points
    np.testing.assert_allclose(m.normal[:, keep], -m.normal[:, drop], atol=1e-12)
    # every ghost face of a periodic mesh has its twin (boundary faces come in pairs)
    ghost_faces = np.nonzero(m.pair_j >= m.n_real)[0]
    assert 2 * drop.size == ghost_faces.size


def test_no_twins_for_reflective():
    m = lattice_mesh(16, "reflective", seed=2)
    assert np.all(periodic_twins(m) == -1)
