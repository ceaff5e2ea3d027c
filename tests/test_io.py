"""Snapshots in the reference's Hdf5 layout (phd/io/read_write.py:52-100, stored as
.npz) and FluxStepper checkpoints that continue bit for bit."""
import types

import numpy as np
import pytest
import torch

import phd_code_gb300 as pkg
from phd_code_gb300.io import SnapshotWriter, load_checkpoint, save_checkpoint
from _util import lattice_mesh, smooth_state


def test_snapshot_round_trip_in_the_reference_layout(tmp_path):
    pc = pkg.HydroParticleCreator(50, dim=2, device="cpu")
    rng = np.random.default_rng(0)
    for name in ("density", "velocity-x", "velocity-y", "pressure", "mass", "position-x"):
        pc[name] = torch.as_tensor(rng.uniform(0.1, 1.0, 50))
    pc["tag"][40:] = 1
    pc["ids"] = torch.arange(50, dtype=torch.int32)
    integ = types.SimpleNamespace(particles=pc, dt=0.01, time=0.25, iteration=7)
    w = SnapshotWriter()
    path = w.write("snap_0007", str(tmp_path), integ)
    with np.load(path) as f:                                  # the reference's HDF5 paths
        assert float(f["dt"]) == 0.01 and float(f["time"]) == 0.25 and int(f["iteration"]) == 7
        assert int(f["particles/number_particles"]) == 50
        assert int(f["particles/Real"]) == 0 and int(f["particles/Ghost"]) == 1
        assert str(f["particles/density/dtype"]) == "double" and str(f["particles/tag/dtype"]) == "int"
    back = w.read(path, device="cpu")
    assert back.get_carray_size() == 50
    for name in pc.carrays:
        assert torch.equal(back[name], pc[name]), name
        assert back.carray_dtypes[name] == pc.carray_dtypes[name]
    assert w.attrs(path) == {"dt": 0.01, "time": 0.25, "iteration": 7}


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_checkpoint_continues_bit_for_bit(tmp_path, precision):
    m = lattice_mesh(20, "periodic", seed=8)
    prim = smooth_state(m)
    kw = dict(gamma=1.4, cfl=0.5, solver="hllc", moving=True)
    a = pkg.FluxStepper(m, prim, precision=precision, **kw)
    a.step(3)
    path = save_checkpoint(a, str(tmp_path / "ckpt.npz"), m)
    a.step(4)
    b, _ = load_checkpoint(path, **kw)
    b.step(4)
    a.check_status()
    b.check_status()
    assert np.array_equal(a.cons_host(), b.cons_host())
    assert np.array_equal(a.prim_host(), b.prim_host())
    ca, cb = a.read_clock(), b.read_clock()
    assert (ca.t, ca.dt, ca.step) == (cb.t, cb.dt, cb.step)
