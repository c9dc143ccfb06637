"""BrillouinZone.moveinto / ir_moveinto on the GPU against the oracle.

Both run the query path's move and wedge-search kernel through brx_locate on
a stand-in trellis (the irreducible polyhedron alone).  Bar: q, τ and the
operation indices bit-exact with the oracle's restatement of
BrillouinZone::moveinto / ir_moveinto (src/bz_move.cpp:103-163, 257-295);
Q = q + τ and Q = Rᵀ q_ir + τ.
"""
import numpy as np
import pytest

from _cases import crystal_case
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["diamond2", "hex16", "R-3m"])
def test_moveinto_matches_oracle(name):
    c = crystal_case(name)
    bz = c["bz"]
    Q = np.random.default_rng(6).uniform(-4, 4, (3000, 3))
    q, tau = bz.moveinto(Q)
    oq, otau, _, st = Oracle(c["tables"]).move(Q, ir=False)
    assert not st.any()
    assert np.array_equal(q, oq) and np.array_equal(tau, otau)
    assert np.allclose(q + tau, Q, atol=1e-12)


@pytest.mark.parametrize("name", ["diamond2", "hex16", "R-3m"])
def test_ir_moveinto_matches_oracle(name):
    c = crystal_case(name)
    bz = c["bz"]
    Q = np.random.default_rng(7).uniform(-4, 4, (3000, 3)).reshape(30, 100, 3)
    q, tau, R, Rinv = bz.ir_moveinto(Q)
    assert q.shape == Q.shape and R.shape == Q.shape + (3,)
    oq, otau, orot, st = Oracle(c["tables"]).move(Q.reshape(-1, 3), ir=True)
    assert not st.any()
    W = bz.pointgroup.W
    assert np.array_equal(q.reshape(-1, 3), oq) and np.array_equal(tau.reshape(-1, 3), otau)
    assert np.array_equal(R.reshape(-1, 3, 3), W[orot[:, 0]]) and np.array_equal(Rinv.reshape(-1, 3, 3), W[orot[:, 1]])
    back = np.einsum("nji,nj->ni", R.reshape(-1, 3, 3), q.reshape(-1, 3)) + tau.reshape(-1, 3)
    assert np.allclose(back, Q.reshape(-1, 3), atol=1e-12)


def test_move_errors():
    c = crystal_case("diamond2")
    with pytest.raises(RuntimeError, match="last dimension"):
        c["bz"].moveinto(np.zeros((4, 2)))
