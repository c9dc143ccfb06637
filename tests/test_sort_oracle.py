"""sort() on the CPU: the oracle's assignment, cost matrices and keys.

The oracle restates DualInterpolator::sort (src/interpolatordual.hpp:385-434)
with the reference's cost functions (src/interpolator.hpp:246-300,
src/utilities.tpp:249-431, 567-598).  Its assignment solver is pinned against
scipy's linear_sum_assignment (an independent exact solver), its cost
matrices against a numpy restatement of the reference's formulas and against
the phase-free reformulation the GPU kernel uses, and its permutations
against shuffles whose answer is known.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests._cases import crystal_case


def test_assignment_matches_scipy():
    lsa = pytest.importorskip("scipy.optimize").linear_sum_assignment
    rng = np.random.default_rng(0)
    for n in list(range(1, 13)) + [24, 47, 48, 96]:
        for _ in range(20):
            c = rng.standard_normal((n, n))
            _, col = lsa(c)
            assert np.array_equal(O.assign(c), col), n


def test_assignment_optimal_with_ties():
    """Integer costs have many optimal assignments; every one found must
    reach the optimum."""
    lsa = pytest.importorskip("scipy.optimize").linear_sum_assignment
    rng = np.random.default_rng(1)
    for n in (2, 5, 17, 40):
        for _ in range(20):
            c = rng.integers(0, 3, (n, n)).astype(float)
            r, col = lsa(c)
            a = O.assign(c)
            assert np.array_equal(np.sort(a), np.arange(n))
            assert c[np.arange(n), a].sum() == c[r, col].sum()


def _ref_vec_cost(vf, a, b):
    """The reference's vector cost functions (utilities.tpp) in numpy."""
    cplx = np.iscomplexobj(a) or np.iscomplexobj(b)
    if vf == 1:
        return np.sqrt(np.sum(np.abs(a - b) ** 2))
    if cplx:
        h = np.sum(np.conj(a) * b)
        if vf == 2:
            return 1 - abs(h) ** 2
        na, nb = np.linalg.norm(a), np.linalg.norm(b)
        if vf == 3:
            c = np.sum(a.real * b.real + a.imag * b.imag) / (na * nb)
        else:
            c = abs(h) / (na * nb)
    else:
        if vf == 2:
            return 1 - np.sum(a * b)
        c = np.sum(a * b) / (np.linalg.norm(a) * np.linalg.norm(b))
    c = float(np.clip(c, -1, 1))
    th = np.arccos(c)
    return th if vf in (3, 4) else np.sin(th) ** 2


def _ref_cost(sides, i, j):
    """cost_matrix(i, j) in numpy (interpolator_cost.tpp:19-61)."""
    B = sides[0][0].shape[1]
    C = np.zeros((B, B))
    for k, (arr, el, vf, w) in enumerate(sides):
        e0, e1, e2 = el
        for a in range(B):
            for b in range(B):
                x, y = arr[i, a], arr[j, b]
                if k == 1 and np.iscomplexobj(arr):
                    h = np.sum(np.conj(x) * y)
                    y = y * np.exp(-1j * np.angle(h))
                s = np.sum(np.abs(x[:e0] - y[:e0]))
                v = _ref_vec_cost(vf, x[e0:e0 + e1], y[e0:e0 + e1]) if e1 else 0.0
                m = sum(np.sqrt(np.sum(np.abs(x[e0 + e1 + 9 * q:e0 + e1 + 9 * q + 9] -
                                              y[e0 + e1 + 9 * q:e0 + e1 + 9 * q + 9]) ** 2)) for q in range(e2 // 9))
                C[a, b] += w[0] * s + w[1] * v + w[2] * m
    return C


def _gpu_form_cost(sides, i, j):
    """The GPU kernel's phase-free form: vector costs from ⟨x, y⟩ over the
    vector part and e = conj(h)/|h| of the whole branch; scalars and matrices
    against e·y."""
    B = sides[0][0].shape[1]
    C = np.zeros((B, B))
    for k, (arr, el, vf, w) in enumerate(sides):
        e0, e1, e2 = el
        cplx = np.iscomplexobj(arr)
        for a in range(B):
            for b in range(B):
                x, y = arr[i, a], arr[j, b]
                e = 1.0
                if k == 1 and cplx:
                    h = np.sum(np.conj(x) * y)
                    e = np.conj(h) / abs(h) if abs(h) > 0 else 1.0
                xv, yv = x[e0:e0 + e1], y[e0:e0 + e1]
                s = np.sum(np.abs(x[:e0] - e * y[:e0]))
                v = 0.0
                if e1:
                    g = np.sum(np.conj(xv) * yv) if cplx else np.sum(xv * yv)
                    na, nb = np.linalg.norm(xv), np.linalg.norm(yv)
                    if vf == 1:
                        v = np.sqrt(np.sum(np.abs(xv - e * yv) ** 2))
                    elif vf == 2:
                        v = 1 - (abs(g) ** 2 if cplx else g)
                    else:
                        c = (np.real(e * g) if vf == 3 else abs(g)) if cplx else g
                        th = np.arccos(np.clip(c / (na * nb), -1, 1))
                        v = th if vf in (3, 4) else np.sin(th) ** 2
                m = sum(np.sqrt(np.sum(np.abs(x[e0 + e1 + 9 * q:e0 + e1 + 9 * q + 9] -
                                              e * y[e0 + e1 + 9 * q:e0 + e1 + 9 * q + 9]) ** 2)) for q in range(e2 // 9))
                C[a, b] += w[0] * s + w[1] * v + w[2] * m
    return C


@pytest.mark.parametrize("vf", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("cplx", [True, False])
def test_cost_matrices(vf, cplx):
    rng = np.random.default_rng(vf + 10 * cplx)
    V, B = 5, 4
    vals = rng.standard_normal((V, B, 2))
    el_c = (1, 6, 9)  # a scalar, two 3-vectors, one matrix per mode
    vecs = rng.standard_normal((V, B, 16))
    if cplx:
        vecs = vecs + 1j * rng.standard_normal((V, B, 16))
    sides = [(vals, (1, 0, 0), 0, (1.0, 0.5, 1.0)), (vecs, el_c, vf, (0.3, 1.0, 0.7))]
    sides[0] = (np.ascontiguousarray(vals[:, :, :1]), (1, 0, 0), 0, (1.0, 0.5, 1.0))
    keys = np.array([0 * V + 3, 1 * V + 2, 2 * V + 1, 3 * V + 0], np.int64)
    perm, costs = O.sort_permutations(sides[0], sides[1], keys, return_costs=True)
    for k, (i, j) in enumerate([(0, 3), (1, 2)]):
        kk = np.searchsorted(keys, i * V + j)
        ref = _ref_cost(sides, i, j)
        np.testing.assert_allclose(costs[kk], ref, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(_gpu_form_cost(sides, i, j), ref, rtol=1e-10, atol=1e-12)
        col = O.assign(ref)
        assert np.array_equal(perm[kk], col)
        kr = np.searchsorted(keys, j * V + i)
        assert np.array_equal(perm[kr][col], np.arange(B))


def test_keys_brute_force():
    tr = crystal_case("diamond2", 1 / 300)["tr"]
    keys = tr.permutation_keys()
    n = len(tr.vertices)
    want = set()
    for grp in list(tr.cube_vertices) + list(tr.tet_vertices):
        for a in grp:
            for b in grp:
                if a != b:
                    want.add(int(a) * n + int(b))
    assert np.array_equal(keys, np.array(sorted(want), np.int64))
    i, j = keys // n, keys % n
    assert np.isin(j * n + i, keys).all()


def shuffled(case, seed=0):
    """Vertex data whose modes are shuffled per vertex by sigma (stored mode m
    at vertex i holds true mode sigma[i, m]); the true modes are well apart in
    value and orthogonal as vectors, so the optimal assignment is unique."""
    rng = np.random.default_rng(seed)
    xyz = case["tr"].vertices
    V = len(xyz)
    B, nat = 6, 2
    base = np.linalg.qr(rng.standard_normal((3 * nat, 3 * nat)) + 1j * rng.standard_normal((3 * nat, 3 * nat)))[0]
    w = np.arange(B, dtype=float)[None, :] * 3.0 + 0.2 * np.sin(xyz[:, :1] * 5)
    v = base.T[None, :, :] * np.exp(1j * rng.uniform(0, 2 * np.pi, (V, B, 1)))
    v = v + 0.02 * np.sin(xyz[:, None, :1] * 3 + np.arange(3 * nat)[None, None, :])
    sigma = np.array([rng.permutation(B) for _ in range(V)])
    ws = np.take_along_axis(w, sigma, axis=1)
    vs = np.take_along_axis(v, sigma[:, :, None], axis=1)
    return ws, vs, sigma


def expected_perms(keys, sigma):
    V = len(sigma)
    inv = np.argsort(sigma, axis=1)
    i, j = keys // V, keys % V
    return np.take_along_axis(inv[j], sigma[i], axis=1)


def test_oracle_recovers_shuffles():
    case = crystal_case("diamond2", 1 / 300)
    ws, vs, sigma = shuffled(case)
    keys = case["tr"].permutation_keys()
    perm = O.sort_permutations((ws[:, :, None], (1, 0, 0), 0, (1, 1, 1)), (vs, (0, 6, 0), 0, (1, 1, 1)), keys)
    assert np.array_equal(perm, expected_perms(keys, sigma))


def test_munkres_known_answer():
    """src/tests/munkres_test.cpp: the cost matrix
    [[1, 2, 3], [2, 4, 6], [3, 6, 9]] is assigned rows → columns [2, 1, 0]."""
    c = np.array([[1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [3.0, 6.0, 9.0]])
    assert O.assign(c).tolist() == [2, 1, 0]


def test_table_from_moved_round_trip():
    """save_permutations keeps only the permutations that move a mode;
    table_from_moved rebuilds a table that answers every key as before."""
    from brille_gb300.grid import table_from_moved

    rng = np.random.default_rng(9)
    B, n = 7, 50
    keys = np.sort(rng.choice(10_000, n, replace=False)).astype(np.int64)
    perms = np.tile(np.arange(B, dtype=np.int32), (n, 1))
    moved = rng.uniform(size=n) < 0.4
    for k in np.nonzero(moved)[0]:
        while (perms[k] == np.arange(B)).all():
            perms[k] = rng.permutation(B)
    k2, ids, table = table_from_moved(keys, moved, perms[moved], B)
    assert np.array_equal(k2, keys)
    assert np.array_equal(table[ids], perms)
    assert (table[0] == np.arange(B)).all()
    with pytest.raises(ValueError):
        table_from_moved(keys, moved, perms[moved][:-1], B)
