"""tatva_gb300: the element-level finite-element hot path of tatva on GB300 (sm_103a).

Mirrors the reference's public surface for the hot path::

    from tatva_gb300 import Mesh, Operator, element, sparse
    mesh = Mesh.unit_square(64, 64)
    op = Operator(mesh, element.Tri3())
    E = op.integrate(0.5 * (op.grad(u) ** 2).sum(-1))     # CUDA kernels + torch autograd

plus fused energies (``materials``), device solvers (``solvers``), the batched
multi-mesh solver (``batched``) and the request loop (``serving``).
"""

from . import batched, compound, element, lifter, materials, sparse, solvers  # noqa: F401
from ._build import build  # noqa: F401
from ._lib import BreakdownError, NotConvergedError  # noqa: F401
from .mesh import Mesh  # noqa: F401
from .operator import Operator  # noqa: F401

__version__ = "0.1.0"
__all__ = ["Mesh", "Operator", "element", "sparse", "materials", "lifter", "solvers", "batched",
           "compound", "build"]
