"""GB300-native flux path for the AREPO-style moving-mesh code rickyfernandez/phd-code.

The package mirrors the reference's plugin interface for the per-step flux path --
``PieceWiseConstant`` / ``PieceWiseLinear`` reconstruction, ``HLL`` / ``HLLC`` /
``Exact`` Riemann solvers, ``IdealGas``, the ``Mesh`` face-to-cell update and the
MUSCL-Hancock integrators -- and runs every stage as a hand-written sm_103a kernel
behind the C ABI in ``include/phdflux.h``.  ``FluxStepper`` is the fused fast path.

Importable as ``phd_code_gb300`` (the directory name carries a hyphen; see
``__graft_entry__.load_package``).
"""
__version__ = "0.1.0"

from . import meshgen, hilbert, problems, tess, io               # noqa: F401  (host only)
from .containers import CarrayContainer, HydroParticleCreator    # noqa: F401
from .equation_state import EquationStateBase, IdealGas           # noqa: F401
from .domain import DomainManager, Reflective, Periodic           # noqa: F401
from .mesh import Mesh                                            # noqa: F401
from .reconstruction import ReconstructionBase, PieceWiseConstant, PieceWiseLinear  # noqa: F401
from .riemann import RiemannBase, HLL, HLLC, Exact                # noqa: F401
from .integrate import StaticMeshMUSCLHancock, MovingMeshMUSCLHancock  # noqa: F401
from .step import FluxStepper                                     # noqa: F401
from .device import DeviceMesh, DeviceClock, make_params          # noqa: F401
