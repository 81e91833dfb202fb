"""Scan-pose flip (AdaptiveKSearchSurface with a pose file,
AdaptiveKSearchSurface.tcc:94-139, 252-265): each normal turns toward the
cloud point indexed by its nearest pose (lvr2's own indexing), or toward the
flip point when that index is not a point.  Signs equal the oracle's."""
import numpy as np
import pytest

from tests.helpers import angle_deg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb(lib):
    import lvr2_gb300
    return lvr2_gb300


def test_scan_pose_flip_matches_oracle(gb, oracle_mod):
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(60_000, seed=51)
    flip = np.array([0.5, 0.5, 0.5], np.float32)
    poses = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [0.0, 1.0, 0.5], [1.0, 0.0, 0.2]], np.float32)
    with gb.Surface(P, kn=10, ki=10, kd=5, nem=3, flip_point=flip) as s:
        s.calculate_normals()
        plain, _ = s.raw_normals()
        s.set_scan_poses(poses)
        s.calculate_normals()
        posed, _ = s.raw_normals()
        final = s.normals()
        s.set_scan_poses(None)
        s.calculate_normals()
        again, _ = s.raw_normals()
    assert np.array_equal(again, plain)
    o = oracle_mod.OracleSurface(P)
    targets = oracle_mod.pose_flip_targets(P, poses)
    ref = o.normals(10, nem=3, flip=flip, flip_targets=targets)
    assert np.all(np.sum(posed * ref, axis=1) > 0)  # every sign agrees
    assert np.percentile(angle_deg(posed, ref), 99.9) < 0.5
    flipped = np.sum(posed * plain, axis=1) < 0
    assert flipped.sum() > 100  # the poses change the orientation of many normals
    assert np.isfinite(final).all()


def test_pose_index_beyond_the_cloud(gb, oracle_mod):
    """More poses than points: a point whose nearest pose index is not a point
    keeps the flip point."""
    rng = np.random.Generator(np.random.PCG64(2))
    P = rng.normal(size=(40, 3)).astype(np.float32)
    poses = rng.normal(scale=3.0, size=(200, 3)).astype(np.float32)
    with gb.Surface(P, kn=5, ki=0, kd=5, nem=3, flip_point=(0, 0, 0)) as s:
        s.set_scan_poses(poses)
        s.calculate_normals()
        got, _ = s.raw_normals()
        with pytest.raises(gb.LvrgbError):
            s.set_scan_poses(np.full((3, 3), np.nan, np.float32))
    targets = oracle_mod.pose_flip_targets(P, poses)
    assert np.isnan(targets[:, 0]).any()
    ref = oracle_mod.OracleSurface(P).normals(5, nem=3, flip=np.zeros(3, np.float32), flip_targets=targets)
    assert np.all(np.sum(got * ref, axis=1) > 0)
