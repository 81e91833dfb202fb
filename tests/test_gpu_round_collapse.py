"""Collapsed search rounds: when almost nothing fits in round 2 or 3 of the
adaptive normal search (scans: points on axis-aligned walls fail the
neighbourhood-box test in every round), one search with the last round's k
stands in for the remaining rounds, which are tested on the prefixes of its
sorted kNN.  kNN(k) is the first k of kNN(32 kn), so the normals, the round
each point is fitted in, the per-round counts and the interpolation must be
bit-identical to searching round by round (lvrgb_debug_round_collapse(0)).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture()
def collapse_toggle(lib):
    yield lambda on: lib.lvrgb_debug_round_collapse(1 if on else 0)
    lib.lvrgb_debug_round_collapse(1)


def walls(n_side=120, sigma=0.001, seed=3):
    """Axis-aligned planes with small noise: their neighbourhood boxes are
    flat in every round."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g = np.stack(np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="ij"), -1).reshape(-1, 2) * 0.1
    floor = np.c_[g[:, 0], rng.normal(0, sigma, len(g)), g[:, 1]]
    wall = np.c_[g[:, 0], g[:, 1], 20.0 + rng.normal(0, sigma, len(g))]
    return np.concatenate([floor, wall]).astype(np.float32)


@pytest.mark.parametrize("cloud", ["scan", "walls"])
@pytest.mark.parametrize("nem", [3, 0, 2])
def test_surface_collapse_is_bit_identical(lib, collapse_toggle, cloud, nem):
    import lvr2_gb300
    from lvr2_gb300 import synthetic
    P = synthetic.scan_scene(60_000, seed=12)[0] if cloud == "scan" else walls()
    out = {}
    for on in (False, True):
        collapse_toggle(on)
        with lvr2_gb300.Surface(P, kn=10, ki=10, nem=nem, flip_point=(0, 0, 0)) as s:
            s.calculate_normals()
            raw, k = s.raw_normals()
            out[on] = (raw, k, s.normals(), s.normal_stats()[:6].copy())
    a, b = out[False], out[True]
    assert np.array_equal(a[0], b[0], equal_nan=True)
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[2], b[2], equal_nan=True)
    assert np.array_equal(a[3], b[3])
    # the case the collapse is for: points still searching after round 2
    assert a[3][2:5].sum() > 0


def test_batch_collapse_is_bit_identical_and_taken(lib, collapse_toggle):
    import lvr2_gb300
    from lvr2_gb300 import synthetic
    scans = synthetic.scan_project(n_scans=4, seed=4, scale=0.02)
    pts = [p for p, _ in scans] + [walls()]
    flips = np.array([f for _, f in scans] + [np.array([5, 5, 5], np.float32)], np.float32)
    res = {}
    for on in (False, True):
        collapse_toggle(on)
        with lvr2_gb300.Batch(pts, flips, kn=10, ki=10, nem=3) as b:
            b.calculate_normals(use_graph=False)   # round by round; chooses the collapse
            b.calculate_normals(use_graph=False)   # with it (when on)
            eager = b.normals()
            rounds = b.round_times()
            b.calculate_normals(use_graph=True)
            graph = b.normals()
            counters, _ = b.stats()
        res[on] = (eager, graph, counters[:6].copy(), rounds)
    a, b = res[False], res[True]
    assert np.array_equal(a[0], b[0], equal_nan=True) and np.array_equal(a[1], b[1], equal_nan=True)
    assert np.array_equal(b[0], b[1], equal_nan=True)
    assert np.array_equal(a[2], b[2])
    # collapsed after round 2: rounds 4 and 5 run inside round 3's launch
    assert a[3][3] > 0 and b[3][2] > 0 and b[3][3] + b[3][4] < 0.05 * b[3][2]
