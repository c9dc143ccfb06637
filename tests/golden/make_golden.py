"""Regenerate tests/golden/nacl_gamma.npz from the reference's fixture.

The reference's Γ-rotation test data (wrap/tests/test_5_gamma.npz, NaCl,
8-atom conventional cell, 192 space-group operations, 29 grid points,
24 modes, 48 symmetry-equivalent q) is the only golden data for the rotation
stage of the query path.  This script copies the arrays the tests use into a
fixture that travels with the repository.

Usage: python tests/golden/make_golden.py <path to the reference's wrap/tests/test_5_gamma.npz>
"""
import os
import sys

import numpy as np

KEYS = ["basis_vectors", "atom_positions", "atom_index", "spacegroup_mat", "spacegroup_vec",
        "grid_max_volume", "grid_rlu", "grid_values", "grid_vectors", "q_nu",
        "euphonic_values", "euphonic_vectors", "brille_values", "brille_vectors"]


def main(src):
    d = np.load(src)
    out = {k: d[k] for k in KEYS}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "nacl_gamma.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    main(sys.argv[1])
