"""Trellis tables persist to .npz and come back identical; a file built from
other inputs is not taken for the requested trellis."""
import numpy as np
import pytest

from brille_gb300 import workloads as W
from brille_gb300.bz import BrillouinZone
from brille_gb300.trellis import TrellisBuild


def _bz():
    lat, _ = W.diamond_primitive()
    return BrillouinZone(lat)


def test_save_load_roundtrip(tmp_path):
    bz = _bz()
    t = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume / 500)
    p = tmp_path / "t.npz"
    t.save(p)
    u = TrellisBuild.load(p)
    for k in TrellisBuild._TABLES:
        assert np.array_equal(getattr(t, k), getattr(u, k)), k
    for d in range(3):
        assert np.array_equal(t.knots[d], u.knots[d])
    assert u.shape == t.shape and u.summary() == t.summary()


def test_cache_builds_once_and_checks_inputs(tmp_path):
    bz = _bz()
    p = tmp_path / "c.npz"
    a = TrellisBuild.cached(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume / 300, p)
    mtime = p.stat().st_mtime_ns
    b = TrellisBuild.cached(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume / 300, p)
    assert p.stat().st_mtime_ns == mtime  # loaded, not rebuilt
    assert np.array_equal(a.tet_vertices, b.tet_vertices)
    with pytest.raises(ValueError):
        TrellisBuild.load(p, fingerprint=TrellisBuild.fingerprint(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume / 301))
    TrellisBuild.cached(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume / 301, p)  # other inputs: rebuilt
    fp_new = TrellisBuild.fingerprint(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume / 301)
    fp_old = TrellisBuild.fingerprint(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume / 300)
    TrellisBuild.load(p, fingerprint=fp_new)
    with pytest.raises(ValueError):
        TrellisBuild.load(p, fingerprint=fp_old)
