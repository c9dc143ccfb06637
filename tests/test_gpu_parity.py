"""Parity of the CUDA query path with the oracle, through the C ABI.

Bar: bit-exact for every index the locate stages choose (q_ir, τ, R, R⁻¹,
node, tetrahedron, vertex list) and for the FP64 weights; FP64
interpolated eigenvalues bit-exact (same operation order); FP64 vectors
within 1e-12 (the GPU forms e^{-iθ} algebraically instead of through atan2);
FP32 storage within 2e-5 relative on eigenvalues and 1e-4 on eigenvector
overlap; BF16 eigenvector storage within 2e-2 overlap.  Reduced-precision
eigenvectors are compared on (q, mode) pairs whose antiphase is well
conditioned (conditioned_modes): elsewhere the reference's own algorithm
takes its phase from rounding noise.
"""
import numpy as np
import pytest

from _cases import boundary_q, conditioned_modes, crystal_case, nacl, values_vectors
from brille_gb300 import BZTrellisQdc
from brille_gb300.grid import BZTrellisQdd
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

NAMES = ["diamond2", "diamond8", "hex16", "P-1", "R-3m", "Im-3m"]


def _grid(case, cls=BZTrellisQdc):
    return cls(case["bz"], trellis=case["tr"])


def _queries(case, n=4000, seed=0):
    Q = np.random.default_rng(seed).uniform(-2, 2, size=(n, 3))
    return np.concatenate([Q, boundary_q(case, n // 2, seed=seed + 1)])


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("ir", [True, False])
def test_locate_bit_exact(name, ir):
    c = crystal_case(name)
    g = _grid(c)
    Q = _queries(c)
    if not ir:
        # the trellis covers the irreducible polyhedron only; fold Q first
        Q = Oracle(c["tables"]).move(Q, ir=True)[0]
    got = g.locate(Q, ir=ir, do_not_move_points=not ir)
    ref = Oracle(c["tables"]).move_locate(Q, ir=ir, no_move=not ir)
    for k in ("status", "q_ir", "tau", "rot", "node", "n_weights", "vertex", "weight"):
        assert np.array_equal(got[k], ref[k]), k
    assert not got["status"].any()


def _overlap(a, b):
    """|<a,b>| per (q, mode) for unit eigenvectors (N, B, n, 3)."""
    return np.abs(np.einsum("qmij,qmij->qm", np.conj(a), b))


@pytest.mark.parametrize("name", NAMES[:4])
def test_ir_interpolate_fp64(name):
    c = crystal_case(name)
    g = _grid(c)
    vals, vecs = values_vectors(c)
    nv, B = c["w"].shape
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * c["model"].n_atoms, 0, 2, 1])
    Q = _queries(c, 3000)
    gv, gc = g.ir_interpolate_at(Q)
    ov, oc, rc, st = Oracle(c["tables"]).interpolate_at(Q, vals, vecs)
    assert rc == 0
    assert gv.shape == (len(Q), B) and gc.shape == (len(Q),) + c["v"].shape[1:]
    assert np.array_equal(gv, ov[:, :, 0])
    err = np.abs(gc.reshape(oc.shape) - oc).max()
    assert err < 1e-12, err


# P-1 (3 atoms) and R-3m (21 atoms): eigenvector rows of 72 and 504 bytes,
# not a multiple of 16, staged from below their start by the FP32 gather
@pytest.mark.parametrize("name", ["diamond8", "hex16", "P-1", "R-3m"])
@pytest.mark.parametrize("storage,vtol,otol", [("f32", 2e-5, 1e-4), ("bf16", 2e-5, 2e-2)])
def test_ir_interpolate_reduced_precision(name, storage, vtol, otol):
    c = crystal_case(name)
    g = _grid(c)
    vals, vecs = values_vectors(c)
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * c["model"].n_atoms, 0, 2, 1], storage=storage)
    Q = _queries(c, 3000)
    for out_f32 in (False, True):
        gv, gc = g.ir_interpolate_at(Q, out_f32=out_f32)
        ov, oc, rc, st = Oracle(c["tables"]).interpolate_at(Q, vals, vecs)
        scale = np.abs(ov).max()
        assert np.abs(gv - ov[:, :, 0]).max() <= vtol * scale
        a = oc.reshape(gc.shape)
        na = np.linalg.norm(a.reshape(len(Q), a.shape[1], -1), axis=-1)
        nb = np.linalg.norm(gc.reshape(len(Q), a.shape[1], -1), axis=-1)
        ov_ = _overlap(a, gc) / np.maximum(na * nb, 1e-300)
        ok = (na > 1e-6) & conditioned_modes(c, Q)
        assert ok.mean() > 0.2
        assert (1 - ov_[ok]).max() < otol


def test_nacl_golden_gpu():
    d, lat, bz, tr, t = nacl()
    g = BZTrellisQdc(bz, trellis=tr)
    vec_els = np.array([0, 24, 0, 2, 3, 0, 0])
    g.fill(d["grid_values"], np.array([1.0]).astype(int), np.array([13605.693, 0, 0]), d["grid_vectors"], vec_els,
           np.array([0.0, 1.0, 0.0]), False)
    br_val, br_vec = g.ir_interpolate_at(d["q_nu"])
    br_val = np.squeeze(br_val)
    assert np.allclose(br_val, d["euphonic_values"])
    br_vec = np.einsum("ba,ijkb->ijka", d["basis_vectors"], br_vec)
    eu = d["euphonic_vectors"]
    ph = np.exp(-1j * np.angle(np.einsum("qmij,qmij->qm", np.conj(eu), br_vec)))
    assert np.abs(np.einsum("ab,abij->abij", ph, br_vec) - eu).max() < 1e-12


@pytest.mark.parametrize("combo", [(0, 1), (1, 0), (2, 2), (2, 4)])
def test_unsupported_combinations_raise(combo):
    d, lat, bz, tr, t = nacl()
    g = BZTrellisQdc(bz, trellis=tr)
    g.fill(d["grid_values"], [1], [13605.693, 0, 0], d["grid_vectors"], np.array([0, 24, 0, *combo, 0, 0]),
           [0, 1, 0])
    with pytest.raises(RuntimeError):
        g.ir_interpolate_at(d["q_nu"])


def test_interpolate_at_first_zone_only():
    c = crystal_case("diamond8")
    g = _grid(c)
    vals, vecs = values_vectors(c)
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 24, 0, 2, 1])
    # points strictly inside trellis cells, shifted by the reciprocal lattice
    # vector (1,1,1) of the F-centred cell: the first-zone move brings them back
    tr, lat = c["tr"], c["lat"]
    rng = np.random.default_rng(9)
    t = tr.tet_vertices[rng.integers(0, len(tr.tet_vertices), 1500)]
    bc = rng.dirichlet([4, 4, 4, 4], size=len(t))
    x = np.einsum("nk,nkd->nd", bc, tr.vertices[t])
    Q = x @ np.linalg.inv(lat.B) + np.array([1.0, 1.0, 1.0])
    gv, gc = g.interpolate_at(Q)
    ov, oc, rc, st = Oracle(c["tables"]).interpolate_at(Q, vals, vecs, ir=False)
    assert rc == 0
    assert np.array_equal(gv, ov[:, :, 0])
    assert np.abs(gc.reshape(oc.shape) - oc).max() < 1e-12


def test_errors_and_edge_cases():
    c = crystal_case("diamond2")
    g = _grid(c)
    with pytest.raises(RuntimeError, match="filled"):
        g.ir_interpolate_at(np.zeros((3, 3)))
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 6, 0, 2, 1])
    v, e = g.ir_interpolate_at(np.zeros((0, 3)))
    assert v.shape == (0, 6)
    with pytest.raises(RuntimeError):
        g.ir_interpolate_at(np.array([[np.nan, 0, 0]]))
    # a point outside the trellis with do_not_move_points
    with pytest.raises(RuntimeError):
        g.ir_interpolate_at(np.array([[7.5, 7.5, 7.5]]), do_not_move_points=True)
    # Γ, zone-face and far-away points
    Q = np.array([[0, 0, 0], [0.5, 0.5, 0.5], [1, 0, 0], [37.25, -11.5, 3.0], [-1e3, 2e3, 0.125]])
    gv, gc = g.ir_interpolate_at(Q)
    vals, vecs = values_vectors(c)
    ov, oc, rc, st = Oracle(c["tables"]).interpolate_at(Q, vals, vecs)
    assert rc == 0 and np.array_equal(gv, ov[:, :, 0])


def test_host_device_and_chunking():
    """Host numpy buffers (chunked, two streams) and device torch buffers give
    identical results."""
    torch = pytest.importorskip("torch")
    c = crystal_case("diamond8")
    g = _grid(c)
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 24, 0, 2, 1], storage="f32")
    Q = np.random.default_rng(7).uniform(-3, 3, size=(250_000, 3))
    hv, hc = g.ir_interpolate_at(Q, out_f32=True)
    Qd = torch.from_numpy(Q).cuda()
    dv = torch.empty(hv.shape, dtype=torch.float32, device="cuda")
    dc = torch.empty(hc.shape, dtype=torch.complex64, device="cuda")
    g.query_into(Qd, len(Q), dv, dc, out_f32=True)
    torch.cuda.synchronize()
    assert np.array_equal(dv.cpu().numpy(), hv)
    assert np.array_equal(dc.cpu().numpy(), hc)


def test_values_only_real_grid():
    c = crystal_case("hex16")
    g = BZTrellisQdd(c["bz"], trellis=c["tr"])
    g.fill(c["w"][:, :, None], [1, 0, 0, 0, 3])
    Q = _queries(c, 2000)
    gv, gc = g.ir_interpolate_at(Q)
    assert gc is None
    ov, _, rc, st = Oracle(c["tables"]).interpolate_at(Q, (c["w"][:, :, None], [1, 0, 0], 0, 3))
    assert np.array_equal(gv, ov)


def test_permutation_table():
    """sort()-style mode permutations between vertex pairs
    (PermutationTable::safe_get) are applied as the oracle applies them."""
    c = crystal_case("diamond8")
    g = _grid(c)
    vals, vecs = values_vectors(c)
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 24, 0, 2, 1])
    nv, B = c["w"].shape
    rng = np.random.default_rng(5)
    perms = np.array([np.arange(B)] + [rng.permutation(B) for _ in range(5)], np.int32)
    pairs = {}
    tr = c["tr"]
    sets = [list(cv) for cv in tr.cube_vertices] + [list(tv) for tv in tr.tet_vertices]
    for vs in sets:
        for i in vs:
            for j in vs:
                if i != j and rng.uniform() < 0.5:
                    pairs[int(i) * nv + int(j)] = int(rng.integers(0, len(perms)))
    keys = np.array(sorted(pairs), np.int64)
    ids = np.array([pairs[k] for k in keys], np.int32)
    g.set_permutations(keys, ids, perms)
    Q = _queries(c, 3000)
    gv, gc = g.ir_interpolate_at(Q)
    ov, oc, rc, st = Oracle(c["tables"]).interpolate_at(Q, vals, vecs, perm=(keys, ids, perms))
    assert rc == 0
    assert np.array_equal(gv, ov[:, :, 0])
    assert np.abs(gc.reshape(oc.shape) - oc).max() < 1e-12


@pytest.mark.parametrize("name", ["hex16", "diamond2"])
def test_fp32_screens_match_exact_predicates(name):
    """The shortcuts of the locate stage change no decision and no bit: a
    handle created with BRX_EXACT_PREDICATES=1 (all predicates in FP64, knot
    comparisons in FP64, per-corner cube weights) returns the same records on
    points within 1e-9 r.l.u. of every kind of boundary."""
    import os
    c = crystal_case(name)
    Q = np.concatenate([_queries(c, 4000, seed=21), boundary_q(c, 6000, seed=22, delta=1e-9)])
    a = _grid(c).locate(Q)
    os.environ["BRX_EXACT_PREDICATES"] = "1"
    try:
        b = _grid(c).locate(Q)
    finally:
        del os.environ["BRX_EXACT_PREDICATES"]
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_tune_keeps_results():
    """brx_tune changes launch shapes only: outputs are bit-identical unless
    it switches the FP32 gather kernel, which changes rounding order only."""
    c = crystal_case("hex16")
    g = _grid(c)
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * c["model"].n_atoms, 0, 2, 1], storage="f32")
    Q = _queries(c, 20000, seed=11)
    v0, c0 = g.ir_interpolate_at(Q, out_f32=True)
    kb = g.tune(Q, out_f32=True, reps=1)
    assert kb[1] in (24, 32, 40, 56, 72, 96, 128, 160) and kb[2] in (16, 32, 64, 128) and kb[3] in (1, 2, 4)
    v1, c1 = g.ir_interpolate_at(Q, out_f32=True)
    assert np.array_equal(v0, v1)
    if kb[4] == 0:
        assert np.array_equal(c0, c1)
    else:
        # the other kernel sums in another order: the same vectors to
        # rounding where the antiphase is well conditioned (elsewhere the
        # reference's own phase comes from rounding noise)
        a = c0.reshape(len(Q), c0.shape[1], -1)
        b = c1.reshape(len(Q), c1.shape[1], -1)
        ok = conditioned_modes(c, Q)
        assert ok.mean() > 0.2
        assert np.abs(a - b).max(axis=2)[ok].max() < 1e-5


def test_warp_gather_shape_independent():
    """The FP32 warp-independent gather's outputs do not depend on its launch
    shape (shared-memory budget, hence warps and modes per block; q per
    descriptor) nor on host-staged chunking: bit-identical."""
    c = crystal_case("hex16")
    g = _grid(c)
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * c["model"].n_atoms, 0, 2, 1], storage="f32")
    Q = _queries(c, 6000, seed=13)
    g.set_tuning((56, 56, 32, 2, 0))
    v0, c0 = g.ir_interpolate_at(Q, out_f32=True)
    for kb, gq in ((24, 16), (96, 128), (160, 16), (40, 64)):
        g.set_tuning((56, kb, gq, 2, 0))
        v1, c1 = g.ir_interpolate_at(Q, out_f32=True)
        assert np.array_equal(v0, v1) and np.array_equal(c0, c1), (kb, gq)
