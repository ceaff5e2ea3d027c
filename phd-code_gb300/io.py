"""Snapshots and checkpoints (host side).

``SnapshotWriter`` mirrors the reference's ``Hdf5`` reader/writer
(``phd/io/read_write.py:52-100``): the attributes ``dt``, ``time`` and ``iteration``,
and a ``particles`` group holding ``Real`` / ``Ghost`` / ``number_particles`` and one
group per particle field with its ``dtype`` and ``data``.  HDF5 libraries are not part
of this build, so the same tree is stored in a NumPy ``.npz`` archive whose keys are the
HDF5 paths (``particles/density/data``, ``particles/density/dtype``, ``dt``, ...).

``save_checkpoint`` / ``load_checkpoint`` write and restore a ``FluxStepper`` -- the
host mesh, the FP64 conserved totals, the primitives the next step starts from and the
device clock -- so that a restored run continues bit for bit.
"""
import os

import numpy as np

from .meshgen import HostMesh, REAL, GHOST

_MESH_FIELDS = ("x", "tag", "type", "map", "vol", "dcom", "pair_i", "pair_j", "area", "com", "normal",
                "nbr_ptr", "nbr_idx")


class SnapshotWriter:
    """``Hdf5.write`` / ``Hdf5.read`` of the reference with an ``.npz`` container."""

    extension = ".npz"

    def write(self, base_name, output_directory, integrator):
        """Every particle field of ``integrator.particles`` plus dt / time / iteration
        (read_write.py:54-80).  Returns the file written."""
        pc = integrator.particles
        tree = {"dt": np.float64(integrator.dt), "time": np.float64(integrator.time),
                "iteration": np.int64(integrator.iteration),
                "particles/Real": np.int64(REAL), "particles/Ghost": np.int64(GHOST),
                "particles/number_particles": np.int64(pc.get_carray_size())}
        for name, data in pc.carrays.items():
            tree["particles/%s/dtype" % name] = np.array(pc.carray_dtypes[name])
            tree["particles/%s/data" % name] = data.detach().cpu().numpy()
        path = os.path.join(output_directory, base_name + self.extension)
        np.savez(path, **tree)
        return path

    def read(self, file_name, device="cuda"):
        """A particle container holding every field of a snapshot (read_write.py:82-100)."""
        from .containers import CarrayContainer
        import torch
        with np.load(file_name) as f:
            n = int(f["particles/number_particles"])
            pc = CarrayContainer(n, device=device)
            names = sorted({k.split("/")[1] for k in f.files if k.startswith("particles/") and k.count("/") == 2})
            for name in names:
                pc.register_carray(n, name, str(f["particles/%s/dtype" % name]))
                pc[name] = torch.as_tensor(f["particles/%s/data" % name]).to(pc.device)
        return pc

    @staticmethod
    def attrs(file_name):
        with np.load(file_name) as f:
            return {"dt": float(f["dt"]), "time": float(f["time"]), "iteration": int(f["iteration"])}


def save_checkpoint(stepper, path, host_mesh):
    """The stepper's mesh (the host mesh it runs on), FP64 conserved totals, primitives
    and clock."""
    from . import _lib as L
    tree = {"mesh/" + k: np.asarray(getattr(host_mesh, k)) for k in _MESH_FIELDS}
    tree.update({"mesh/n_real": np.int64(host_mesh.n_real), "mesh/xmin": np.asarray(host_mesh.xmin),
                 "mesh/xmax": np.asarray(host_mesh.xmax), "mesh/boundary": np.array(host_mesh.boundary),
                 "cons": stepper.cons_host(), "clock": stepper.clock.buf.cpu().numpy(),
                 "prim": (stepper.prim4 if stepper.precision == "fp32" else stepper.prim).cpu().numpy(),
                 "precision": np.array(stepper.precision), "clock_bytes": np.int64(L.CLOCK_BYTES)})
    np.savez(path, **tree)
    return path


def load_checkpoint(path, **stepper_kwargs):
    """A FluxStepper continuing a checkpoint: same mesh, conserved totals, primitives and
    clock.  ``stepper_kwargs`` are the physics options of the original stepper (gamma,
    solver, ...).  Returns (stepper, host mesh)."""
    import torch
    from . import _lib as L
    from .step import FluxStepper
    with np.load(path) as f:
        if int(f["clock_bytes"]) != L.CLOCK_BYTES:
            raise ValueError("checkpoint clock layout differs from this library's")
        mesh = HostMesh(dim=2, n_real=int(f["mesh/n_real"]), xmin=tuple(f["mesh/xmin"]), xmax=tuple(f["mesh/xmax"]),
                        boundary=str(f["mesh/boundary"]), **{k: f["mesh/" + k] for k in _MESH_FIELDS})
        cons, clock, prim = f["cons"], f["clock"], f["prim"]
        precision = str(f["precision"])
    nf = mesh.dim + 2
    st = FluxStepper(mesh, np.ones((nf, mesh.n_cells)), precision=precision, **stepper_kwargs)
    st.cons.copy_(torch.as_tensor(cons))
    (st.prim4 if precision == "fp32" else st.prim).copy_(torch.as_tensor(prim))
    st.clock.buf.copy_(torch.as_tensor(clock))
    return st, mesh
