"""Batched queries (brx_batch_*): many grids of different space groups,
trellises, mode counts and ragged q counts in one launch per stage must give
each grid what its own ir_interpolate_at gives (FP64 bit for bit; FP32 to
rounding order), through a plain run, a captured graph replayed on new
inputs, and after autotuning; failures name the item.  Every item's FP64
outputs are also held against the oracle on a sample of its q (eigenvalues
bit-exact, eigenvectors within 1e-12).
"""
import numpy as np
import pytest

from _cases import conditioned_modes, crystal_case, values_vectors
from brille_gb300 import BZTrellisQdc
from brille_gb300.batch import BatchQuery
from brille_gb300.grid import BZTrellisQdd
from brille_gb300._lib import BrxError
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

NAMES = ["diamond2", "hex16", "P-1", "R-3m", "Im-3m", "diamond8"]
COUNTS = [1000, 3001, 0, 1, 2500, 777]


CASES = {}


def _case(name):
    if name not in CASES:
        CASES[name] = crystal_case(name)
    return CASES[name]


def _grids(storage="f64", values_only=False):
    out = []
    for name in NAMES:
        c = _case(name)
        if values_only:
            g = BZTrellisQdd(c["bz"], trellis=c["tr"])
            g.fill(c["w"][:, :, None], [1, 0, 0, 0, 3], storage=storage)
        else:
            g = BZTrellisQdc(c["bz"], trellis=c["tr"])
            g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * c["model"].n_atoms, 0, 2, 1], storage=storage)
        out.append(g)
    return out


def _Q(seed, counts=COUNTS, scale=1.0):
    rng = np.random.default_rng(seed)
    return [rng.uniform(-scale, scale, (n, 3)) for n in counts]


def _check(grids, Qs, vals, vecs, out_f32):
    """FP64: bit-identical.  FP32: the single query may take the
    warp-independent gather, which sums in another order: eigenvalues to
    1e-5, eigenvectors to 1e-4 in overlap on the (q, mode) pairs whose
    antiphase is well conditioned (elsewhere the phase is rounding noise)."""
    for i, (g, Q) in enumerate(zip(grids, Qs)):
        if len(Q) == 0:
            continue
        v, c = g.ir_interpolate_at(Q, out_f32=out_f32)
        bv = vals[i].cpu().numpy()
        if not out_f32:
            assert np.array_equal(bv, v), i
            if c is not None:
                assert np.array_equal(vecs[i].cpu().numpy(), c), i
            # the item against the oracle on a sample of its q
            case = _case(NAMES[i])
            k = min(len(Q), 300)
            ov, oc, rc, _ = Oracle(case["tables"]).interpolate_at(
                Q[:k], *(values_vectors(case) if c is not None else values_vectors(case)[:1]))
            assert rc == 0, i
            assert np.array_equal(bv[:k].reshape(ov.shape), ov), i
            if c is not None:
                assert np.abs(vecs[i].cpu().numpy()[:k].reshape(oc.shape) - oc).max() < 1e-12, i
            continue
        assert np.allclose(bv, v, rtol=1e-5, atol=1e-5 * np.abs(v).max()), i
        if c is None:
            continue
        bc = vecs[i].cpu().numpy().reshape(len(Q), c.shape[1], -1)
        cc = c.reshape(len(Q), c.shape[1], -1)
        ov = np.abs(np.einsum("nbe,nbe->nb", np.conj(bc), cc))
        nrm = np.linalg.norm(bc, axis=-1) * np.linalg.norm(cc, axis=-1)
        ok = (nrm > 1e-12) & conditioned_modes(_case(NAMES[i]), Q)
        if len(Q) >= 100:
            assert ok.mean() > 0.2, i
        if ok.any():
            assert (1 - ov[ok] / nrm[ok]).max() < 1e-4, i


@pytest.mark.parametrize("storage,out_f32", [("f64", False), ("f32", True)])
def test_batch_matches_single_queries(storage, out_f32):
    grids = _grids(storage)
    Qs = _Q(1)
    bq = BatchQuery(grids, COUNTS, out_f32=out_f32)
    # FP32 data: the warp-independent gather takes every item (rows of 6 to
    # 26 atoms, aligned to 16 bytes or not); FP64: the classic gather
    assert (bq.config()["vectors_gather_warps"] > 0) == (storage == "f32")
    vals, vecs = bq.query([torch.from_numpy(q).cuda() for q in Qs])
    _check(grids, Qs, vals, vecs, out_f32)


@pytest.mark.parametrize("storage,out_f32", [("f64", False), ("f32", True)])
def test_values_only_batch_uses_scalar_gather(storage, out_f32):
    """Scalar-only grids need no grouping; FP32 data with FP32 outputs take
    the kernel that reads 4 branches per thread (B = 6, 9, 48, 63, 78, 24:
    float4 rows and element-wise rows)."""
    grids = _grids(storage, values_only=True)
    Qs = _Q(2)
    bq = BatchQuery(grids, COUNTS, out_f32=out_f32)
    vals, vecs = bq.query([torch.from_numpy(q).cuda() for q in Qs])
    assert all(v is None for v in vecs)
    _check(grids, Qs, vals, vecs, out_f32)
    if out_f32:
        # same operation order as the single queries' scalar gather
        for i, (g, Q) in enumerate(zip(grids, Qs)):
            if len(Q):
                assert np.array_equal(vals[i].cpu().numpy(), g.ir_interpolate_at(Q, out_f32=True)[0]), i


def test_graph_replay_on_new_inputs_and_tuning():
    grids = _grids("f32")
    bq = BatchQuery(grids, COUNTS, out_f32=True)
    s = torch.cuda.Stream()
    Q1 = [torch.from_numpy(q).cuda() for q in _Q(3)]
    vals, vecs = bq.outputs()
    bq.set_io(Q1, vals, vecs)
    bq.capture(s.cuda_stream)
    bq.launch(s.cuda_stream)
    bq.sync(s.cuda_stream)
    _check(grids, [q.cpu().numpy() for q in Q1], vals, vecs, True)
    # new Q buffers, same graph
    Q2 = [torch.from_numpy(q).cuda() for q in _Q(4)]
    bq.set_io(Q2, vals, vecs)
    bq.launch(s.cuda_stream)
    bq.sync(s.cuda_stream)
    _check(grids, [q.cpu().numpy() for q in Q2], vals, vecs, True)
    cfg = bq.tune(s.cuda_stream, reps=1)
    assert cfg["locate_threads"] in (64, 128, 256) and cfg["tiles"] > 0
    assert cfg["vectors_ctas_per_sm"] >= 1 and cfg["vectors_gather_warps"] in (0, 4, 8)
    for v in vals:
        v.zero_()
    bq.run(s.cuda_stream)
    bq.sync(s.cuda_stream)
    _check(grids, [q.cpu().numpy() for q in Q2], vals, vecs, True)


@pytest.mark.parametrize("min_groups,small_q", [(-1, 0), (0, 0), (8, 128), (64, 32)])
def test_item_split_between_gathers(min_groups, small_q):
    """Every split of the items between the warp-independent gather and the
    CTA-synchronous one (with its own q per descriptor, a second descriptor
    list) answers as the single queries do."""
    grids = _grids("f32")
    Qs = _Q(6)
    bq = BatchQuery(grids, COUNTS, out_f32=True)
    cfg = bq.config()
    cfg["warp_min_groups"] = min_groups
    cfg["small_q_per_group"] = small_q
    got = bq.set_config(cfg)
    assert got["warp_min_groups"] == min_groups
    if min_groups > 8:
        assert got["small_q_per_group"] == small_q and got["vectors_gather_warps"] == 0
    vals, vecs = bq.outputs()
    bq.set_io([torch.from_numpy(q).cuda() for q in Qs], vals, vecs)
    bq.run()
    bq.sync()
    _check(grids, Qs, vals, vecs, True)


def test_failure_names_the_item():
    grids = _grids("f64")
    counts = [50] * len(grids)
    # points already in each trellis (q_ir of a first locate), except item 3's,
    # moved far outside: with no move, not found
    Qs = [g.locate(q)["q_ir"] for g, q in zip(grids, _Q(5, counts))]
    Qs[3] = Qs[3] + 10.0
    bq = BatchQuery(grids, counts, no_move=True)
    with pytest.raises(BrxError) as e:
        bq.query([torch.from_numpy(q).cuda() for q in Qs])
    assert e.value.item == 3
    assert "item 3" in str(e.value)


def test_mixed_element_kinds_are_rejected():
    c = crystal_case("diamond2")
    a = BZTrellisQdc(c["bz"], trellis=c["tr"])
    a.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 6, 0, 2, 1])
    b = BZTrellisQdd(c["bz"], trellis=c["tr"])
    b.fill(c["w"][:, :, None], [1, 0, 0, 0, 3])
    with pytest.raises(BrxError):
        BatchQuery([a, b], [10, 10])
