"""Permutation tables written by save_permutations and read back by
load_permutations answer every key and every query as before."""
import numpy as np
import pytest

from brille_gb300 import BZTrellisQdc
from tests._cases import crystal_case
from tests.test_sort_oracle import shuffled

pytestmark = pytest.mark.gpu


def _grid(case):
    return BZTrellisQdc(case["bz"], trellis=case["tr"], device=0)


def test_save_and_load_permutations(tmp_path):
    case = crystal_case("diamond2", 1 / 300)
    ws, vs, sigma = shuffled(case)
    g = _grid(case)
    g.fill(ws, [1, 0, 0, 0, 3], vs, [0, 6, 0, 2, 1], sort=True)
    keys, perms = g.permutation_table()
    path = tmp_path / "perms.npz"
    g.save_permutations(path)
    g2 = _grid(case)
    g2.fill(ws, [1, 0, 0, 0, 3], vs, [0, 6, 0, 2, 1])
    g2.load_permutations(path)
    k2, p2 = g2.permutation_table()
    assert np.array_equal(k2, keys) and np.array_equal(p2, perms)
    Q = np.random.default_rng(2).uniform(-1, 1, (2000, 3))
    a, b = g.ir_interpolate_at(Q), g2.ir_interpolate_at(Q)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
