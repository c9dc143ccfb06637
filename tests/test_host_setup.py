"""Host-side set-up: space groups, zone, wedge, trellis, Γ table, BvK model."""
import numpy as np
import pytest

from _cases import crystal_case
from brille_gb300 import workloads as W
from brille_gb300.bz import BrillouinZone
from brille_gb300.crystal import SPACEGROUPS, spacegroup

ORDERS = {"P-1": 2, "P2/m": 4, "Pmmm": 8, "P4/mmm": 16, "R-3m": 36, "P6/mmm": 24, "P6_3/mmc": 24,
          "Fm-3m": 192, "Im-3m": 96, "Fd-3m": 192}


@pytest.mark.parametrize("name", sorted(SPACEGROUPS))
def test_spacegroup_orders(name):
    s = spacegroup(name)
    assert s.size == ORDERS[name]
    pg = s.pointgroup()
    inv = pg.inverse_indices()
    for i, j in enumerate(inv):
        assert np.array_equal(pg.W[i] @ pg.W[j], np.eye(3))


@pytest.mark.parametrize("name", ["diamond2", "diamond8", "hex16", "P-1", "P2/m", "Pmmm", "P4/mmm", "R-3m",
                                  "P6/mmm", "Fm-3m", "Im-3m"])
def test_wedge_is_fundamental_domain(name):
    c = crystal_case(name, fraction=1 / 300)
    bz = c["bz"]
    assert abs(bz.volume / bz.ir_volume - bz.pointgroup.size) < 1e-6
    tr = c["tr"]
    v = tr.vertices
    cube = np.prod(np.abs(v[tr.cube_vertices[:, 0]] - v[tr.cube_vertices[:, 7]]), axis=1).sum()
    assert abs(cube + tr.tet_volume.sum() - bz.ir_volume) < 1e-9 * bz.ir_volume


def test_bvk_properties():
    c = crystal_case("diamond8")
    m = c["model"]
    D = m.dynamical_matrix(np.random.default_rng(0).uniform(-1, 1, (5, 3)))
    assert np.allclose(D, np.conj(np.swapaxes(D, 1, 2)))
    w0, _ = m.modes(np.zeros((1, 3)))
    assert np.sum(np.abs(w0) < 1e-4) == 3  # acoustic sum rule: three zero modes at Γ
    q = np.random.default_rng(1).uniform(-1, 1, (3, 3))
    for W_ in c["bz"].pointgroup.W[:8]:
        wq, _ = m.modes(q)
        wr, _ = m.modes(q @ W_)
        assert np.allclose(wq, wr, atol=1e-8)


def test_gamma_table_maps_atoms():
    c = crystal_case("diamond8")
    F0 = c["tables"]["gamma_F0"]
    for r in range(F0.shape[1]):
        assert sorted(F0[:, r]) == list(range(F0.shape[0]))


def test_workload_crystals():
    lat, m = W.hexagonal16()
    assert lat.basis.size == 16 and len(m) == 16
    from brille_gb300.crystal import min_separation
    assert min_separation(lat.A, lat.basis.positions) >= 1.2
    lat2, _ = W.diamond_primitive()
    assert lat2.basis.size == 2 and lat2.pointgroup.size == 48
