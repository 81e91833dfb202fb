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
