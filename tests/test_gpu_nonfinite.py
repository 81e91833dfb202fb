"""Non-finite inputs: a point with a NaN or infinite coordinate is rejected
with LVRGB_ERR_INVALID_ARGUMENT (surfaces and scan projects); a query with
one has no neighbours, so its kNN rows are padding and its distance is
FLT_MAX, as lvr2's distance() gives for an empty neighbourhood."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLT_MAX = np.float32(3.4028235e38)


@pytest.fixture(scope="module")
def gb(lib):
    import lvr2_gb300
    return lvr2_gb300


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_points_rejected(gb, bad):
    P = np.random.default_rng(0).random((5000, 3)).astype(np.float32)
    P[1234, 1] = bad
    with pytest.raises(gb.LvrgbError) as e:
        gb.Surface(P, kn=10, ki=10, kd=5, nem=3)
    assert e.value.status == 1 and "1234" in str(e.value)
    with pytest.raises(gb.LvrgbError) as e:
        gb.Batch([P[:2000], P[2000:]], np.zeros((2, 3), np.float32), kn=10, ki=10, nem=3)
    assert e.value.status == 1


def test_nonfinite_queries(gb, oracle_mod):
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(50_000, seed=31)
    Q = P[:200].copy()
    Q[::7, 0] = np.nan
    Q[3::7, 2] = np.inf
    bad = ~np.isfinite(Q).all(1)
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3) as s:
        s.calculate_normals()
        for k in (8, 150):  # per-lane and one-warp-per-query kernels
            idx, dist, cnt = s.knn(Q, k)
            assert (cnt[bad] == 0).all() and (idx[bad] == 0xFFFFFFFF).all() and np.isinf(dist[bad]).all()
            oi, od, oc = oracle_mod.OracleSurface(P).knn(Q[~bad], k)
            assert np.array_equal(idx[~bad], oi) and np.array_equal(cnt[~bad], oc)
        proj, eucl = s.distance(Q)
        assert (proj[bad] == FLT_MAX).all() and (eucl[bad] == FLT_MAX).all()
        assert np.isfinite(proj[~bad]).all()
        ridx, rdist, rcnt = s.radius_search(Q, 8, 0.05)
        assert (rcnt[bad] == 0).all()
