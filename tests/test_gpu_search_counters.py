"""The search counters behind the bench line's per-warp figures: after a
reconstruct, lvrgb_distance_stats holds the signed-distance searches' sums
and lvrgb_normal_stats the normal searches' (round 1 of kn = 10: k = 20).
Every query fills its heap (k insertions at least) and every warp tile scans
a bucket and expands the root; a warp's insertion rounds are at least its
busiest lane's insertions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_normal_and_distance_counters(lib):
    import lvr2_gb300
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(100_000, seed=33)
    kn, kd = 10, 10
    with lvr2_gb300.Surface(P, kn=kn, ki=10, kd=kd, nem=3) as s:
        s.calculate_normals()
        info = s.reconstruct(voxelsize=0.01, decomposition="PMC")
        ns = s.normal_stats()
        ds = s.distance_stats()
    n, nq = len(P), int(info.grid_vertices)
    warps_n, warps_q = (n + 31) // 32, (nq + 31) // 32
    assert ns[8] >= warps_n and ns[9] >= warps_n and ns[10] >= 2 * kn * n
    assert ds[0] >= warps_q and ds[1] >= warps_q and ds[2] >= kd * nq
    assert ds[3] >= warps_q and ds[4] * 32 >= ds[2]
    assert (ds[5:] == 0).all()
    # a second reconstruct restarts the sums
    with lvr2_gb300.Surface(P, kn=kn, ki=10, kd=kd, nem=3) as s:
        s.calculate_normals()
        s.reconstruct(voxelsize=0.01, decomposition="PMC")
        s.reconstruct(voxelsize=0.01, decomposition="PMC")
        assert np.array_equal(s.distance_stats(), ds)
