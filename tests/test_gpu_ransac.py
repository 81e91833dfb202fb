"""nem 1 (calcPlaneRANSAC, AdaptiveKSearchSurface.tcc:689-781) through the C
ABI against the oracle's restatement.  Bar: bit-exact normals (the same
(d2, index)-ordered neighbour rows, the same libstdc++ draws, IEEE float
arithmetic in the reference's order) and identical adaptive rounds, with k
up to the one-warp-per-query path (k > 96)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb(lib):
    import lvr2_gb300
    return lvr2_gb300


def _clouds():
    from lvr2_gb300 import synthetic
    rng = np.random.Generator(np.random.PCG64(5))
    base = rng.uniform(0, 1, (8000, 3)).astype(np.float32)
    line = rng.uniform(-1, 1, (4000, 3)).astype(np.float32)
    line[:4] = np.float32([[0, 0, 0], [0.5, 0, 0], [-0.25, 0, 0], [0.75, 0, 0]])
    return {
        "spheres": synthetic.spheres_tori(30_000, seed=7),
        "scan": synthetic.scan_scene(20_000, seed=3)[0],
        "duplicates": np.concatenate([base, base[:2000], base[:500]]),
        "line_first": line,
        "tiny": rng.uniform(0, 1, (5, 3)).astype(np.float32),
    }


CLOUDS = None


def cloud(name):
    global CLOUDS
    if CLOUDS is None:
        CLOUDS = _clouds()
    return CLOUDS[name]


def bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a, np.float32).view(np.uint32),
                          np.ascontiguousarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("name", ["spheres", "scan", "duplicates", "line_first", "tiny"])
@pytest.mark.parametrize("kn,adaptive", [(10, True), (3, True), (60, False), (2, False)])
def test_ransac_normals_bit_exact(gb, oracle_mod, name, kn, adaptive):
    P = cloud(name)
    flip = ((P.min(0) + P.max(0)) / 2).astype(np.float32)
    on, ok = oracle_mod.OracleSurface(P).normals(kn, nem=1, adaptive=adaptive, flip=flip, with_k=True)
    with gb.Surface(P, kn=kn, ki=0, nem=1, adaptive=adaptive, flip_point=flip) as s:
        s.calculate_normals()
        gn, gk = s.raw_normals()
    assert (gk == ok).all()
    assert bits_equal(gn, on)
    if name == "line_first" and kn == 2 and not adaptive:
        assert not gn.any()  # every candidate plane degenerate (the cloud's first 4 points)


def test_ransac_wide_rounds_and_interpolation(gb, oracle_mod):
    """Adaptive rounds that escalate past k = 96 (thin structures), then the
    interpolation of the RANSAC normals."""
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(20_000, seed=3)
    P = np.concatenate([P, np.stack([np.linspace(0, 1, 3000), np.zeros(3000), np.zeros(3000)], 1)]).astype(np.float32)
    flip = np.zeros(3, np.float32)
    o = oracle_mod.OracleSurface(P)
    on, ok = o.normals(30, nem=1, adaptive=True, flip=flip, with_k=True)
    assert (ok > 96).any()
    with gb.Surface(P, kn=30, ki=12, nem=1, flip_point=flip) as s:
        s.calculate_normals()
        gn, gk = s.raw_normals()
        final = s.normals()
    assert (gk == ok).all()
    assert bits_equal(gn, on)
    assert bits_equal(final, o.interpolate(gn, 12))


def test_ransac_pose_flip(gb, oracle_mod):
    P = cloud("scan")
    poses = np.float32([[0, 0, 0], [3, 1, 0], [-2, 4, 1]])
    targets = oracle_mod.pose_flip_targets(P, poses)
    flip = np.float32([0.5, 0.5, 0.5])
    on = oracle_mod.OracleSurface(P).normals(10, nem=1, adaptive=True, flip=flip, flip_targets=targets)
    with gb.Surface(P, kn=10, ki=0, nem=1, flip_point=flip) as s:
        s.set_scan_poses(poses)
        s.calculate_normals()
        gn, _ = s.raw_normals()
    assert bits_equal(gn, on)


def test_ransac_errors(gb):
    P = cloud("spheres")
    with gb.Surface(P, kn=1, ki=0, nem=1) as s:  # k = 2: lvr2 reads past its draw set
        with pytest.raises(gb.LvrgbError) as e:
            s.calculate_normals()
        assert e.value.status == 1
    with gb.Surface(P[:2], kn=10, ki=0, nem=1) as s:  # 2 points
        with pytest.raises(gb.LvrgbError) as e:
            s.calculate_normals()
        assert e.value.status == 1
    with pytest.raises(gb.LvrgbError) as e:
        gb.Batch([P[:1000], P[1000:2000]], np.zeros((2, 3), np.float32), kn=10, ki=10, nem=1)
    assert e.value.status == 4


@pytest.mark.parametrize("name", ["sphere", "scan", "lattice"])
def test_ransac_golden(gb, name):
    """The committed frozen oracle outputs (tests/golden/oracle_small.npz,
    kn = 5, adaptive): on the lattice the cloud's first points are collinear,
    so many candidate planes are degenerate and null normals win."""
    from pathlib import Path
    gold = np.load(Path(__file__).resolve().parent / "golden" / "oracle_small.npz")
    P = gold[name + "/points"]
    flip = np.float32([0.5, 0.5, 0.5]) if name == "sphere" else np.zeros(3, np.float32)
    with gb.Surface(P, kn=5, ki=0, nem=1, flip_point=flip) as s:
        s.calculate_normals()
        gn, gk = s.raw_normals()
    assert (gk == gold[name + "/kused_nem1"]).all()
    assert bits_equal(gn, gold[name + "/normals_nem1"])
