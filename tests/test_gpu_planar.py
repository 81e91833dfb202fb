"""BilinearFastBox::optimizePlanarFaces (lvrgb_optimize_planar_faces): the
PMC post-pass that moves the end vertices of border edges in cells with one
or two of them to the centroid of their 5 nearest points.  The GPU mesh after
the post-pass equals the oracle's bit for bit (canonical form: each marked
vertex moves once, from its marching-cubes position)."""
import numpy as np
import pytest

from tests.helpers import canonical_mesh

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb(lib):
    import lvr2_gb300
    return lvr2_gb300


def open_cloud():
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(60_000, seed=3)
    return P[P[:, 0] < 0.55]  # a cut: open surfaces with border contours


@pytest.mark.parametrize("kc", [5, 1, 12])
def test_planar_faces_match_oracle(gb, oracle_mod, kc):
    P = open_cloud()
    flip = ((P.min(0) + P.max(0)) / 2).astype(np.float32)
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3, flip_point=flip) as s:
        s.calculate_normals()
        normals = s.normals()
        s.reconstruct(voxelsize=0.02, decomposition="PMC")
        v0, f0, e0 = s.mesh()
        moved = s.optimize_planar_faces(kc)
        v1, f1, e1 = s.mesh()
        g = s.grid()
    assert np.array_equal(f0, f1) and np.array_equal(e0, e1)  # topology unchanged
    changed = (v0 != v1).any(1)
    assert moved >= changed.sum() > 0.02 * len(v0)
    o = oracle_mod.OracleSurface(P)
    lat, _, dist, inv = g
    r = o.reconstruct(normals, voxelsize=0.02, kd=10, decomposition="PMC", grid_override=(lat, dist, inv),
                      planar_kc=kc)
    assert r["planar_moved"] == moved
    gk, gp, gf = canonical_mesh(e1, v1, f1)
    ok_, op, of = canonical_mesh(r["vkeys"], r["vpos"], r["faces"])
    assert np.array_equal(gk, ok_) and np.array_equal(gf, of)
    assert np.array_equal(gp, op)


def test_closed_surface_is_unchanged(gb):
    """A closed sphere reconstructs without border edges: nothing moves."""
    rng = np.random.Generator(np.random.PCG64(2))
    v = rng.normal(size=(80_000, 3))
    P = (0.3 * v / np.linalg.norm(v, axis=1, keepdims=True) + 0.5).astype(np.float32)
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3, flip_point=(0.5, 0.5, 0.5)) as s:
        s.calculate_normals()
        s.reconstruct(voxelsize=0.02, decomposition="PMC")
        v0, _, _ = s.mesh(with_edges=False)
        moved = s.optimize_planar_faces(5)
        v1, _, _ = s.mesh(with_edges=False)
    assert moved == 0 and np.array_equal(v0, v1)


def test_planar_faces_errors(gb):
    P = open_cloud()[:5000]
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3) as s:
        with pytest.raises(gb.LvrgbError) as e:
            s.optimize_planar_faces(5)
        assert e.value.status == 5  # no mesh yet
        s.calculate_normals()
        s.reconstruct(voxelsize=0.05)
        with pytest.raises(gb.LvrgbError):
            s.optimize_planar_faces(0)
