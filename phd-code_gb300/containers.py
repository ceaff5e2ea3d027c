"""Named structure-of-arrays containers in device memory.

Mirrors the reference's ``CarrayContainer`` (``phd/containers/containers.pyx:13-395``)
and ``HydroParticleCreator`` (``phd/utils/particle_creator.pyx:4-62``): fields are
addressed by name (``pc["density"]``), grouped by ``carray_named_groups``, and sized by
``get_carray_size()``.  Unlike the reference, fields that the kernels read together
live in one contiguous ``[field][index]`` block ("primitive", "conservative",
"position", ...), and each named field is a row view of its block, so the C ABI gets
one pointer per group.  Dtype names follow the reference: "double" = float64,
"long" = int32, "int" = int8, "longlong" = int64 (``carray.pxd:31-103``).
"""
import torch

DTYPES = {"double": torch.float64, "long": torch.int32, "int": torch.int8,
          "longlong": torch.int64, "float": torch.float32}


class CarrayContainer:
    def __init__(self, carray_size=0, carrays_to_register=None, device="cuda"):
        self.device = torch.device(device)
        self._size = int(carray_size)
        self._blocks = {}          # block name -> tensor [rows, size]
        self._index = {}           # field name -> (block name, row)
        self.carray_dtypes = {}
        self.carray_named_groups = {}
        if carrays_to_register:
            for name, dtype in carrays_to_register.items():
                self.register_carray(self._size, name, dtype)

    # -- registration ---------------------------------------------------------
    def register_carray(self, carray_size, carray_name, dtype="double"):
        """One field in a block of its own (containers.pyx:39-72)."""
        if carray_name in self._index:
            return
        self._size = int(carray_size) if not self._blocks else self._size
        self._blocks[carray_name] = torch.zeros((1, self._size), dtype=DTYPES[dtype], device=self.device)
        self._index[carray_name] = (carray_name, 0)
        self.carray_dtypes[carray_name] = dtype

    def register_block(self, block, fields, dtype="double"):
        """Several fields stored as consecutive rows of one contiguous tensor."""
        t = torch.zeros((len(fields), self._size), dtype=DTYPES[dtype], device=self.device)
        self._blocks[block] = t
        for r, f in enumerate(fields):
            self._index[f] = (block, r)
            self.carray_dtypes[f] = dtype

    def attach_block(self, block, tensor):
        """Replace a block's storage by an existing [rows, size] tensor (no copy)."""
        old = self._blocks[block]
        if tensor.dim() != 2 or tensor.shape[0] != old.shape[0]:
            raise ValueError("block %s: shape %s does not match %s" % (block, tuple(tensor.shape), tuple(old.shape)))
        self._blocks[block] = tensor
        self._size = tensor.shape[1]

    # -- access ------------------------------------------------------------------
    @property
    def carrays(self):
        return {f: self[f] for f in self._index}

    def __getitem__(self, carray_name):
        try:
            b, r = self._index[carray_name]
        except KeyError:
            raise AttributeError("Unrecognized field: %s" % carray_name)
        return self._blocks[b][r]

    def __setitem__(self, carray_name, value):
        self[carray_name].copy_(torch.as_tensor(value).to(self[carray_name]))

    def __contains__(self, carray_name):
        return carray_name in self._index

    def block(self, name):
        return self._blocks[name]

    def get_carray_size(self):
        return self._size

    def resize(self, carray_size):
        """Resize every block, keeping the leading entries (containers.pyx:133-146)."""
        n = int(carray_size)
        if n == self._size:
            return
        for b, t in list(self._blocks.items()):
            new = torch.zeros((t.shape[0], n), dtype=t.dtype, device=t.device)
            k = min(n, self._size)
            new[:, :k] = t[:, :k]
            self._blocks[b] = new
        self._size = n


def HydroParticleCreator(num=0, dim=2, device="cuda"):
    """Particle fields of the reference's hydro run (particle_creator.pyx:4-62)."""
    axes = "xyz"[:dim]
    pc = CarrayContainer(num, device=device)
    vel = ["velocity-" + a for a in axes]
    mom = ["momentum-" + a for a in axes]
    pc.register_block("primitive", ["density"] + vel + ["pressure"])
    pc.register_block("conservative", ["mass"] + mom + ["energy"])
    pc.register_block("position", ["position-" + a for a in axes])
    pc.register_carray(num, "tag", "int")
    pc.register_carray(num, "type", "int")
    pc.register_carray(num, "ids", "long")
    pc.carray_named_groups = {
        "position": ["position-" + a for a in axes],
        "velocity": vel,
        "momentum": mom,
        "primitive": ["density"] + vel + ["pressure"],
        "conservative": ["mass"] + mom + ["energy"],
    }
    pc["type"][:] = 4        # ParticleTAGS.Undefined; tag already 0 = Real
    return pc
