"""The reference's convenience constructors ``create_bz`` and ``create_grid``
(brille/utils.py:63-356) with the same argument forms, building this
package's BrillouinZone and grids.

Host set-up only: the grids they return answer queries on the GPU.
"""
from __future__ import annotations

import numpy as np

from .bz import BrillouinZone
from .crystal import Lattice


def create_bz(*args, is_reciprocal=False, use_primitive=True, search_length=1, time_reversal_symmetry=False,
              wedge_search=True, snap_to_symmetry=True, **kwargs):
    """A BrillouinZone from lattice parameters and a space group:
    ``create_bz(a, b, c, alpha, beta, gamma, spacegroup)``,
    ``create_bz(lens, angs, spacegroup)`` or
    ``create_bz(lattice_vectors, spacegroup)``, or the same by keyword
    (a, b, c, alpha, beta, gamma, lens, angs, lattice_vectors, spacegroup).
    Angles are radians when none exceeds π, else degrees;
    ``is_reciprocal`` for reciprocal parameters in Å⁻¹.  The space group is
    a name of this package's table (or P1).  ``snap_to_symmetry`` is accepted
    for compatibility."""
    named = {k: kwargs.pop(k, None) for k in ("a", "b", "c", "alpha", "beta", "gamma", "lens", "angs")}
    lattice_vectors = kwargs.pop("lattice_vectors", None)
    spacegroup = kwargs.pop("spacegroup", None)
    if kwargs:
        raise TypeError(f"create_bz() got unexpected keyword arguments {sorted(kwargs)}")
    lens, angs = named["lens"], named["angs"]
    if (lens is None or angs is None) and all(named[k] is not None for k in ("a", "b", "c", "alpha", "beta", "gamma")):
        lens = [named["a"], named["b"], named["c"]]
        angs = [named["alpha"], named["beta"], named["gamma"]]
    sg_pos = 0
    if (lens is None or angs is None) and lattice_vectors is None:
        if not args:
            raise ValueError("No lattice parameters or vectors given")
        first = np.shape(args[0])
        if first == ():
            lens, angs, sg_pos = args[:3], args[3:6], 6
        elif first in ((3,), (3, 1), (1, 3)):
            lens, angs, sg_pos = np.ravel(args[0]), np.ravel(args[1]), 2
        elif first == (3, 3):
            lattice_vectors, sg_pos = args[0], 1
        else:
            raise ValueError("No lattice parameters or vectors given")
    if spacegroup is None:
        if len(args) <= sg_pos:
            raise ValueError("Spacegroup not given")
        spacegroup = args[sg_pos]
    if not isinstance(spacegroup, str):
        raise ValueError("Invalid spacegroup input. It must be a string")
    values = (tuple(np.ravel(lens)), tuple(np.ravel(angs))) if lattice_vectors is None else np.asarray(lattice_vectors)
    lat = Lattice(values, spacegroup=spacegroup, real_space=not is_reciprocal)
    return BrillouinZone(lat, use_primitive=use_primitive, search_length=search_length,
                         time_reversal_symmetry=time_reversal_symmetry, wedge_search=wedge_search)


def create_grid(bz, complex_values=False, complex_vectors=False, mesh=False, nest=False, **kwargs):
    """A BZTrellisQ (default), BZMeshQ (``mesh``) or BZNestQ (``nest``) grid
    over bz, of the dd / dc / cc kind the complex flags select.  Keywords:
    trellis ``node_volume_fraction`` (default 1e-5, Å⁻³) and
    ``always_triangulate``; mesh ``max_size``, ``num_levels``,
    ``max_points``; nest ``max_volume`` or ``number_density`` and
    ``max_branchings``."""
    from . import grid as G

    if not isinstance(bz, BrillouinZone):
        raise ValueError("The `bz` input parameter is not a BrillouinZone object")
    if nest and mesh:
        raise ValueError("Both nest=True and mesh=True is set. Please use one or the other")
    kind = "cc" if (complex_values and complex_vectors) else ("dc" if complex_vectors else "dd")
    trellis_kw = ("node_volume_fraction", "always_triangulate")
    mesh_kw = ("max_size", "num_levels", "max_points")
    nest_kw = ("max_volume", "number_density", "max_branchings")

    def refuse(names, what):
        if any(k in kwargs for k in names):
            raise ValueError(f"Parameters given are consistent with a {what} grid")

    if nest:
        refuse(trellis_kw, "trellis")
        refuse(mesh_kw, "mesh")
        cls = getattr(G, "BZNestQ" + kind)
        branch = int(kwargs.pop("max_branchings", 5))
        if "max_volume" in kwargs:
            return cls(bz, float(kwargs.pop("max_volume")), branch)
        if "number_density" in kwargs:
            return cls(bz, int(kwargs.pop("number_density")), branch)
        raise ValueError("A nest grid needs max_volume or number_density")
    if mesh:
        refuse(trellis_kw, "trellis")
        refuse(nest_kw, "nested")
        return getattr(G, "BZMeshQ" + kind)(bz, float(kwargs.pop("max_size", -1.0)), int(kwargs.pop("num_levels", 3)),
                                            int(kwargs.pop("max_points", -1)))
    refuse(nest_kw, "nested")
    refuse(mesh_kw, "mesh")
    return getattr(G, "BZTrellisQ" + kind)(bz, float(kwargs.pop("node_volume_fraction", 1.0e-5)),
                                           bool(kwargs.pop("always_triangulate", False)))
