"""sort() on the GPU (brx_sort) against the oracle and against known answers.

brx_sort replaces DualInterpolator::sort (src/interpolatordual.hpp:398-434):
one warp per vertex pair forms the FP64 cost matrix and solves the
assignment exactly.  Bars:
- shuffled modes with a unique optimum: every permutation equals the known
  answer, for FP64, FP32 and BF16 storage and every vector cost function;
- Born–von Kármán data: permutations equal the oracle's; where they differ
  (exact or near ties) the GPU's assignment costs, under the oracle's cost
  matrix, no more than 1e-9 relative above the optimum;
- queries after sort() use the table: values bit-exact and vectors within
  1e-12 of the oracle run on the same table.
"""
import ctypes as C

import numpy as np
import pytest

from brille_gb300 import BZTrellisQdc, _abi
from brille_gb300._lib import BrxError, check, load
from oracle import oracle as O
from oracle.oracle import Oracle
from tests._cases import crystal_case, values_vectors
from tests.test_sort_oracle import expected_perms, shuffled

pytestmark = pytest.mark.gpu


def _grid(case):
    return BZTrellisQdc(case["bz"], trellis=case["tr"], device=0)


@pytest.mark.parametrize("storage", ["f64", "f32", "bf16"])
@pytest.mark.parametrize("vf", [0, 1, 2, 3, 4])
def test_sort_recovers_shuffles(storage, vf):
    case = crystal_case("diamond2", 1 / 300)
    ws, vs, sigma = shuffled(case)
    g = _grid(case)
    g.fill(ws, [1, 0, 0, 0, 3, 0, 0], vs, [0, 6, 0, 2, 1, 0, vf], sort=True, storage=storage)
    keys, perms = g.permutation_table()
    assert np.array_equal(keys, case["tr"].permutation_keys())
    assert np.array_equal(perms, expected_perms(keys, sigma))


def _check_against_oracle(case, vf=0, weights=(1.0, 1.0, 1.0)):
    vals, vecs = values_vectors(case)
    g = _grid(case)
    g.fill(case["w"], [1, 0, 0, 0, 3, 0, 0], (1.0, 1.0, 1.0), case["v"], [0, vecs[1][1], 0, 2, 1, 0, vf],
           weights, True)
    keys, perms = g.permutation_table()
    ref, costs = O.sort_permutations((vals[0], vals[1], 0, (1, 1, 1)), (vecs[0], vecs[1], vf, weights), keys,
                                     return_costs=True)
    diff = np.nonzero((perms != ref).any(axis=1))[0]
    V = len(case["tr"].vertices)
    for k in diff:
        i, j = keys[k] // V, keys[k] % V
        kk = k if i < j else np.searchsorted(keys, j * V + i)
        row = perms[kk]
        c = costs[kk]
        opt = c[np.arange(len(row)), ref[kk]].sum()
        got = c[np.arange(len(row)), row].sum()
        assert got <= opt + 1e-9 * (1 + abs(opt)), (k, got, opt)
    assert len(diff) <= max(2, len(keys) // 100), f"{len(diff)} of {len(keys)} permutations differ"
    return g, keys, perms


@pytest.mark.parametrize("vf", [0, 1, 2])
def test_sort_bvk_diamond2(vf):
    _check_against_oracle(crystal_case("diamond2"), vf=vf)


def test_sort_bvk_diamond8_weights():
    _check_against_oracle(crystal_case("diamond8"), vf=0, weights=(1.0, 2.0, 1.0))


def test_query_after_sort():
    case = crystal_case("diamond2", 1 / 300)
    ws, vs, sigma = shuffled(case, seed=4)
    g = _grid(case)
    g.fill(ws, [1, 0, 0, 0, 3, 0, 0], vs, [0, 6, 0, 2, 1, 0, 0], sort=True)
    keys, perms = g.permutation_table()
    assert (perms != np.arange(perms.shape[1])).any(axis=1).mean() > 0.5
    rng = np.random.default_rng(7)
    Q = rng.uniform(-1, 1, (4000, 3))
    gv, gc = g.ir_interpolate_at(Q)
    V, B = ws.shape
    o = Oracle(case["tables"])
    ov, oc, rc, st = o.interpolate_at(Q, (ws[:, :, None], [1, 0, 0], 0, 3), (vs.reshape(V, B, 6), [0, 6, 0], 2, 1),
                                      perm=(keys, np.arange(len(keys), dtype=np.int32), perms))
    assert rc == 0 and (st == 0).all()
    assert np.array_equal(gv, ov[:, :, 0])
    assert np.abs(gc.reshape(oc.shape) - oc).max() < 1e-12
    # the sorted interpolation follows the true modes: the pivot's own order
    # of the smooth values stays within the spread of one mode
    spread = np.abs(gv - np.round(gv / 3.0) * 3.0).max()
    assert spread < 0.25


def test_sort_errors_and_refill():
    case = crystal_case("diamond2", 1 / 300)
    ws, vs, _ = shuffled(case)
    g = _grid(case)
    with pytest.raises(RuntimeError, match="filled before sorting"):
        g.sort()
    g.fill(ws, [1, 0, 0, 0, 3], vs, [0, 6, 0, 2, 1])
    lib, h = load(), g._handle()
    V = len(case["tr"].vertices)
    one_way = np.array([0 * V + 1], np.int64)
    st = lib.brx_sort(h, 1, one_way.ctypes.data, None, None, None)
    assert st == 1 and b"non-existant key" in lib.brx_last_error(h)
    bad = _abi.SortCost()
    bad.scalar_fn, bad.vector_fn = 1, 0
    bad.weight[:] = [1, 1, 1]
    keys = g.permutation_keys()
    st = lib.brx_sort(h, keys.size, keys.ctypes.data, C.byref(bad), None, None)
    assert st == 8  # BRX_ERR_UNSUPPORTED
    g.sort()
    assert load().brx_permutation_count(h) == keys.size
    g.fill(ws, [1, 0, 0, 0, 3], vs, [0, 6, 0, 2, 1])  # new data drops the table
    assert load().brx_permutation_count(h) == 0
    g.set_flags_weights([0, 3, 0, 0], [1, 1, 1], [2, 1, 0, 4], [1, 1, 1], sort=True)
    assert load().brx_permutation_count(h) == keys.size
    with pytest.raises(BrxError, match="strictly increasing"):
        unsorted = np.array([5, 3], np.int64)
        check(lib.brx_sort(h, 2, unsorted.ctypes.data, None, None, None), h)

