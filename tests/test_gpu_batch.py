"""Scan projects (lvrgb_batch_*): one segmented LBVH and one normals launch
per search round for all scans must give, bit for bit, the normals of a
separate surface per scan (lvr2_cuda_normals' per-scan CudaSurface runs)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def project():
    from lvr2_gb300 import synthetic
    scans = synthetic.scan_project(n_scans=6, seed=4, scale=0.01)  # log-uniform 500 .. 40k points
    pts = [p for p, _ in scans]
    flips = [f for _, f in scans]
    rng = np.random.Generator(np.random.PCG64(8))
    # a noiseless planar patch forces the adaptive k rounds (flat neighbourhood boxes)
    g = np.stack(np.meshgrid(np.arange(60), np.arange(60), indexing="ij"), -1).reshape(-1, 2).astype(np.float32)
    plane = np.concatenate([g * 0.5, np.zeros((len(g), 1), np.float32)], 1)
    pts.append(plane)
    flips.append(np.array([10, 10, 5], np.float32))
    pts.append(rng.uniform(0, 1, (17, 3)).astype(np.float32))  # one bucket, fewer points than 2kn
    flips.append(np.array([0.5, 0.5, 0.5], np.float32))
    pts.append(rng.uniform(0, 1, (33, 3)).astype(np.float32))  # two buckets
    flips.append(np.array([0.5, 0.5, 3.0], np.float32))
    return pts, np.array(flips, np.float32)


@pytest.mark.parametrize("bucket,nem", [(32, 3), (16, 3), (32, 0), (32, 2)])
def test_batch_equals_per_scan_surfaces(lib, bucket, nem):
    import lvr2_gb300
    scans, flips = project()
    ref = []
    for p, f in zip(scans, flips):
        with lvr2_gb300.Surface(p, kn=10, ki=10, nem=nem, flip_point=f, bucket=bucket) as s:
            s.calculate_normals()
            ref.append(s.normals())
    ref = np.concatenate(ref)
    with lvr2_gb300.Batch(scans, flips, kn=10, ki=10, nem=nem, bucket=bucket) as b:
        b.calculate_normals()
        got = b.normals()
        counters, ms = b.stats()
    assert np.array_equal(got, ref, equal_nan=True)
    assert counters[:5].sum() == sum(len(p) for p in scans)
    assert counters[1] > 0  # the planar patch needed more than one search round


def test_batch_graph_replay_and_autotune(lib):
    import lvr2_gb300
    scans, flips = project()
    with lvr2_gb300.Batch(scans, flips, kn=10, ki=10, nem=3) as b:
        b.calculate_normals(use_graph=False)
        eager = b.normals()
        b.calculate_normals(use_graph=True)   # eager pass + capture + first replay
        g1 = b.normals()
        b.calculate_normals(use_graph=True)   # replay
        g2 = b.normals()
        bucket, radius = b.autotune()
        assert bucket in (16, 32) and radius in (1, 2)
        b.calculate_normals(use_graph=True)
        g3 = b.normals()
    assert np.array_equal(g1, eager) and np.array_equal(g2, eager) and np.array_equal(g3, eager)


def test_batch_argument_checks(lib):
    import lvr2_gb300
    scans, flips = project()
    with pytest.raises(lvr2_gb300.LvrgbError) as e:
        lvr2_gb300.Batch(scans, flips, kn=5, ki=20)
    assert e.value.status == 4
    with pytest.raises(lvr2_gb300.LvrgbError) as e:
        lvr2_gb300.Batch(scans[:2] + [np.zeros((0, 3), np.float32)], flips[:3])
    assert e.value.status == 1


def test_batch_grid_distances_equal_per_chunk_surfaces(lib):
    """The chunk form of LargeScaleReconstruction's GPU block: every chunk's
    grid vertices against that chunk's points and normals, in one call, equal
    lvrgb_grid_distances of one surface per chunk bit for bit."""
    import lvr2_gb300
    scans, flips = project()
    rng = np.random.Generator(np.random.PCG64(12))
    vs = 0.25
    queries = []
    for p in scans:
        lo, hi = p.min(0), p.max(0)
        m = int(rng.integers(0, 3000))
        # grid-like positions in and around the chunk, plus points near its surface
        q = np.concatenate([rng.uniform(lo - vs, hi + vs, (m, 3)), p[rng.choice(len(p), min(len(p), 500))] + 0.01])
        queries.append(q.astype(np.float32))
    queries[1] = np.zeros((0, 3), np.float32)  # a chunk without grid vertices
    ref_d, ref_i = [], []
    for p, f, q in zip(scans, flips, queries):
        with lvr2_gb300.Surface(p, kn=10, ki=10, kd=7, nem=3, flip_point=f) as s:
            s.calculate_normals()
            d, i = s.grid_distances(q, vs) if len(q) else (np.zeros(0, np.float32), np.zeros(0, np.uint8))
        ref_d.append(d)
        ref_i.append(i)
    with lvr2_gb300.Batch(scans, flips, kn=10, ki=10, kd=7, nem=3) as b:
        b.calculate_normals()
        d, i = b.grid_distances(queries, vs)
        d2, i2 = b.grid_distances(queries, vs)
    assert np.array_equal(d, np.concatenate(ref_d)) and np.array_equal(i, np.concatenate(ref_i))
    assert np.array_equal(d, d2) and np.array_equal(i, i2)
    assert 0 < i.mean() < 1
