"""nem 4: the plane fit of lvr2's LBVH comparator (LBVHIndex::knn_normals,
used by CudaKSearchSurface / --pcm LBVH_CUDA), on the GPU through the C ABI.
One search with k = kn; FP64 sums in the kernel's order over neighbours
1..n-1; equal to the oracle's float64 restatement bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLIP = (1e6, 1e6, 1e6)  # the comparator's fixed flip point


@pytest.fixture(scope="module")
def gb(lib):
    import lvr2_gb300
    return lvr2_gb300


@pytest.mark.parametrize("kn", [10, 20, 50, 96])
def test_lbvh_normals_match_oracle(gb, oracle_mod, kn):
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(120_000, seed=kn)
    with gb.Surface(P, kn=kn, ki=0, kd=5, nem=4, flip_point=FLIP) as s:
        s.calculate_normals()
        n = s.normals()
        raw, k = s.raw_normals()
    assert np.all(k == kn)
    assert np.array_equal(n, raw)
    ref = oracle_mod.lbvh_knn_normals(oracle_mod.OracleSurface(P), kn, flip=FLIP)
    assert np.array_equal(n, ref)


def test_degenerate_neighbourhoods(gb, oracle_mod):
    """Collinear points, duplicates and a cloud smaller than k."""
    rng = np.random.Generator(np.random.PCG64(4))
    line = np.c_[np.linspace(5, 6, 300), np.zeros(300), np.zeros(300)]
    dup = np.repeat(rng.random((50, 3)), 4, axis=0)
    plane = np.c_[rng.random((2000, 2)), np.zeros(2000)]
    P = np.concatenate([line, dup - 5, plane]).astype(np.float32)
    with gb.Surface(P, kn=12, ki=0, kd=5, nem=4, flip_point=FLIP) as s:
        s.calculate_normals()
        n = s.normals()
    ref = oracle_mod.lbvh_knn_normals(oracle_mod.OracleSurface(P), 12, flip=FLIP)
    assert np.array_equal(n, ref)
    assert not n[:300].any()  # collinear on the x axis: every sum but xx is 0, so is the normal
    small = rng.random((7, 3)).astype(np.float32)
    with gb.Surface(small, kn=20, ki=0, kd=5, nem=4, flip_point=FLIP) as s:
        s.calculate_normals()
        n = s.normals()
    assert np.array_equal(n, oracle_mod.lbvh_knn_normals(oracle_mod.OracleSurface(small), 20, flip=FLIP))


def test_interpolation_and_scan_projects(gb, oracle_mod):
    """ki <= kn reuses the search's lists; a scan project fits every scan on
    its own, each flipped toward its own point."""
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(60_000, seed=8)
    with gb.Surface(P, kn=16, ki=8, kd=5, nem=4, flip_point=FLIP) as s:
        s.calculate_normals()
        raw, _ = s.raw_normals()
        n = s.normals()
    o = oracle_mod.OracleSurface(P)
    ref = oracle_mod.lbvh_knn_normals(o, 16, flip=FLIP)
    assert np.array_equal(raw, ref)
    assert np.array_equal(n, o.interpolate(ref, 8))
    scans = [P[:20_000], P[20_000:45_000], P[45_000:]]
    flips = np.array([[1e6, 0, 0], [0, 1e6, 0], [0, 0, -1e6]], np.float32)
    with gb.Batch(scans, flips, kn=16, ki=0, nem=4) as b:
        b.calculate_normals()
        bn = b.normals()
    off = 0
    for sc, f in zip(scans, flips):
        r = oracle_mod.lbvh_knn_normals(oracle_mod.OracleSurface(sc), 16, flip=f)
        assert np.array_equal(bn[off:off + len(sc)], r)
        off += len(sc)


def test_k_limit(gb):
    P = np.random.default_rng(1).random((1000, 3)).astype(np.float32)
    with gb.Surface(P, kn=97, ki=0, kd=5, nem=4) as s:
        with pytest.raises(gb.LvrgbError) as e:
            s.calculate_normals()
        assert e.value.status == 1


def test_normals_from_neighbor_lists(gb, oracle_mod):
    """LBVHIndex::calculate_normals: the fit of given lists, with the rows in
    the given order (the sums follow it), padded rows and counts below k."""
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(50_000, seed=21)
    rng = np.random.Generator(np.random.PCG64(5))
    Q = P[rng.integers(0, len(P), 4000)] + rng.normal(scale=1e-3, size=(4000, 3)).astype(np.float32)
    o = oracle_mod.OracleSurface(P)
    idx, _, cnt = o.knn(Q, 24)
    idx = idx.copy()
    perm = rng.permuted(np.tile(np.arange(1, 24), (len(Q), 1)), axis=1)  # shuffle slots 1..23 per row
    idx[:, 1:] = np.take_along_axis(idx[:, 1:], perm - 1, axis=1)
    cnt = cnt.astype(np.uint32)
    cnt[::7] = rng.integers(0, 24, len(cnt[::7]))  # shorter lists, some below 3
    idx[1::5, 20:] = 0xFFFFFFFF  # padding past the count is never read
    cnt[1::5] = np.minimum(cnt[1::5], 20)
    flip = (0.3, -2.0, 5.0)
    with gb.Surface(P, kn=10, ki=0, kd=5, nem=4, flip_point=flip) as s:
        got = s.normals_from_neighbors(Q, cnt, idx)
        bad = idx.copy()
        bad[3, 2] = len(P)
        with pytest.raises(gb.LvrgbError) as e:
            s.normals_from_neighbors(Q, cnt, bad)
        assert e.value.status == 1
        with pytest.raises(gb.LvrgbError):
            s.normals_from_neighbors(Q, np.full(len(Q), 25, np.uint32), idx)
    ref = oracle_mod.lbvh_fit_lists(P, Q, np.where(idx == 0xFFFFFFFF, 0, idx), cnt, flip=flip)
    assert np.array_equal(got, ref)
    assert not got[cnt < 3].any()
