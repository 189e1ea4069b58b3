"""bench.py's flop accounting (no GPU): the executed GEMM flops of a split CCD sweep that the
roofline divides by the measured GEMM time, against the shapes of the GEMMs ccd_sweep launches.

With nocc <= 64 the split sweep runs X and the ladders folded over occupied pairs (i <= j, np of
them) and virtual pairs (a <= b, nq): X as two GEMMs of o^2 x np x nq, the ladders as two of
np x nq x (np + nq); the ring GEMMs are K-stacked (WmBeJ and the rings K = 2ov, WmBEj and the
third ring K = ov) on ov x ov outputs.
"""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_counts_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def gemm(m, n, k):
    return 2.0 * m * n * k


def test_split_gemm_flops_match_the_launched_shapes():
    b = _bench()
    for o, v in ((40, 160), (20, 80), (5, 20), (64, 300)):
        assert b.folds(o, v)
        np_, nq, ov = o * (o + 1) // 2, v * (v + 1) // 2, o * v
        want = {"ccd_x": 2 * gemm(o * o, np_, nq), "ccd_pp_ladder": 2 * gemm(np_, nq, np_ + nq),
                "ccd_wj": gemm(ov, ov, 2 * ov), "ccd_wk": gemm(ov, ov, ov),
                "ccd_ring": gemm(ov, ov, 2 * ov) + gemm(ov, ov, ov)}
        got = b.ccd_split_gemm_flops(o, v)
        assert got.keys() == want.keys()
        for key in want:
            assert abs(got[key] - want[key]) <= 1e-9 * want[key], (o, v, key)
        assert abs(b.ladder_launch_flops(o, v) - 3 * gemm(np_, nq, np_ + nq)) <= 1e-9 * b.ladder_launch_flops(o, v)


def test_unfolded_form_beyond_64_occupied():
    b = _bench()
    o, v = 65, 100
    assert not b.folds(o, v)
    got = b.ccd_split_gemm_flops(o, v)
    assert got["ccd_pp_ladder"] == gemm(o * o, v * v, o * o + v * v)
    assert got["ccd_x"] == gemm(o * o, o * o, v * v)
    assert not b.folds(40, 362)   # v(v+1)/2 above the finalisation's one-block-per-pair limit


def test_folded_work_at_the_bench_size():
    """At nbf=200 (o = 40, v = 160) the folds cut X and the ladders from 2.36e12 to 0.65e12 flop
    per sweep, and the sweep's GEMMs total 3.79e12 flop (one product)."""
    b = _bench()
    f = b.ccd_split_gemm_flops(40, 160)
    assert abs(f["ccd_x"] + f["ccd_pp_ladder"] - 6.4637e11) < 1e8
    assert abs(sum(f.values()) - 3.7921e12) < 1e8
    o, v = 40.0, 160.0
    assert abs(2 * o**4 * v**2 + 2 * o**2 * v**2 * (o**2 + v**2) - 2.3593e12) < 1e8
