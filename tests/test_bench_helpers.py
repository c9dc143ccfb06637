"""Host-side helpers of bench.py: output bytes per q and the learned-vs-plain
matching at equal error (no GPU)."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402

CURVE = [dict(trellis="bz/200", vertices=22, max_meV=1.16, rms_meV=0.149, q_per_s=5.7e8),
         dict(trellis="bz/625", vertices=98, max_meV=0.78, rms_meV=0.062, q_per_s=3.4e8),
         dict(trellis="bz/5000", vertices=333, max_meV=0.52, rms_meV=0.022, q_per_s=5.8e8),
         dict(trellis="bz/40000", vertices=1750, max_meV=0.28, rms_meV=0.0070, q_per_s=6.0e8),
         dict(trellis="bz/320000", vertices=8262, max_meV=0.148, rms_meV=0.0020, q_per_s=1.08e9)]


def test_bytes_per_q_matches_the_output_shapes():
    # 48 modes, 16 atoms: float64 values and complex128 (n_atoms, 3) vectors
    assert bench.bytes_per_q(48, 16, False) == (24, 384, 36864)
    assert bench.bytes_per_q(48, 16, True) == (24, 192, 18432)
    assert bench.bytes_per_q(6, 2, False) == (24, 48, 576)


def test_matched_plain_is_the_coarsest_trellis_at_or_below_the_error():
    learned = dict(max_meV=0.227, rms_meV=0.00875, q_per_s=4.83e8)
    m = bench.matched_plain(CURVE, learned, "max_meV")
    assert m["trellis"] == "bz/320000"
    r = bench.matched_plain(CURVE, learned, "rms_meV")
    assert r["trellis"] == "bz/40000"
    assert abs(learned["q_per_s"] / r["q_per_s"] - 0.805) < 1e-9
    # nothing on the curve is that accurate
    assert bench.matched_plain(CURVE, dict(max_meV=1e-3, rms_meV=1e-4), "max_meV") is None
    # an exact tie counts as matched
    assert bench.matched_plain(CURVE, dict(max_meV=0.52), "max_meV")["trellis"] == "bz/5000"
