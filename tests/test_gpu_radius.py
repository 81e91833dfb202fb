"""SearchTree::radiusSearch (lvrgb_radius_search): the k nearest points with
distance below the radius, per-lane (k <= 96) and one-warp-per-query (k > 96)
paths, equal to the k-nearest rows of the oracle cut at float d2 < r * r."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k,radius", [(10, 0.03), (40, 0.06), (200, 0.12), (500, 0.2)])
def test_radius_search_matches_cut_knn(lib, oracle_mod, k, radius):
    import lvr2_gb300
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(100_000, seed=15)
    rng = np.random.Generator(np.random.PCG64(k))
    Q = np.concatenate([P[rng.integers(0, len(P), 3000)],
                        rng.uniform(P.min(0), P.max(0), (1000, 3)).astype(np.float32)])
    with lvr2_gb300.Surface(P, kn=10, ki=10, kd=5, nem=3) as s:
        idx, dist, cnt = s.radius_search(Q, k, radius)
    oi, od, oc = oracle_mod.OracleSurface(P).knn(Q, k)
    r2 = np.float32(radius) * np.float32(radius)
    d2 = np.empty_like(od)
    for j in range(k):  # canonical float d2 of each oracle row entry
        p = P[np.minimum(oi[:, j], len(P) - 1).astype(np.int64)]
        dx, dy, dz = (Q[:, 0] - p[:, 0]), (Q[:, 1] - p[:, 1]), (Q[:, 2] - p[:, 2])
        d2[:, j] = (dx * dx + dy * dy) + dz * dz
    keep = (np.arange(k)[None, :] < oc[:, None]) & (d2 < r2)
    want = keep.sum(1)
    assert np.array_equal(cnt, want)
    assert (want == k).any() and ((want > 0) & (want < k)).any()  # rows cut by k and by the radius
    for i in np.flatnonzero(want):
        n = want[i]
        assert np.array_equal(idx[i, :n], oi[i, :n]) and np.array_equal(dist[i, :n], od[i, :n])
        assert np.all(idx[i, n:] == 0xFFFFFFFF) and np.all(np.isinf(dist[i, n:]))


def test_radius_errors(lib):
    import lvr2_gb300
    P = np.random.default_rng(1).random((1000, 3)).astype(np.float32)
    with lvr2_gb300.Surface(P, kn=10, ki=10, kd=5, nem=3) as s:
        for r in (0.0, -1.0, float("inf")):
            with pytest.raises(lvr2_gb300.LvrgbError):
                s.radius_search(P[:5], 4, r)
