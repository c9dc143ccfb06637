"""brille_gb300 — brille's Brillouin-zone trellis query path on one GB300.

The public surface mirrors the reference's Python module for this path:
``Lattice``, ``Symmetry``, ``Basis``, ``BrillouinZone`` and the
``BZTrellisQdd`` / ``BZTrellisQdc`` / ``BZTrellisQcc`` grids with ``fill``,
``sort``, ``ir_interpolate_at`` and ``interpolate_at``, and the mesh grids
``BZMeshQ*`` and ``BZNestQ*`` on the same query path.  Queries run as CUDA kernels
for sm_103a behind the C ABI declared in include/brx.h.
"""
from .crystal import Basis, Lattice, PointSymmetry, Symmetry, spacegroup  # noqa: F401
from .bz import BrillouinZone  # noqa: F401
from .grid import (BZMeshQcc, BZMeshQdc, BZMeshQdd, BZNestQcc, BZNestQdc, BZNestQdd,  # noqa: F401
                   BZTrellisQcc, BZTrellisQdc, BZTrellisQdd, LengthUnit, NodeType, RotatesLike)
from ._lib import BrxError  # noqa: F401
from .approx import ApproxConfig, real_space_tolerance, reciprocal_space_tolerance  # noqa: F401

__all__ = ["Basis", "Lattice", "PointSymmetry", "Symmetry", "spacegroup", "BrillouinZone",
           "BZTrellisQdd", "BZTrellisQdc", "BZTrellisQcc", "BZMeshQdd", "BZMeshQdc", "BZMeshQcc",
           "BZNestQdd", "BZNestQdc", "BZNestQcc", "BrxError", "ApproxConfig", "real_space_tolerance",
           "reciprocal_space_tolerance", "NodeType", "RotatesLike", "LengthUnit"]
