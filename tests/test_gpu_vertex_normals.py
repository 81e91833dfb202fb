"""calcVertexNormals (lvrgb_mesh_vertex_normals / lvrgb_vertex_normals): the
per-vertex normals lvr2_reconstruct writes with the mesh.  Face normals,
ordered sums and the nearest-point fallback equal the oracle's float32
restatement bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb(lib):
    import lvr2_gb300
    return lvr2_gb300


@pytest.fixture(scope="module")
def scene(gb):
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(60_000, seed=5)
    flip = ((P.min(0) + P.max(0)) / 2).astype(np.float32)
    return P, flip


@pytest.mark.parametrize("decomposition,planar", [("PMC", True), ("MC", False)])
def test_mesh_vertex_normals_match_oracle(gb, oracle_mod, scene, decomposition, planar):
    P, flip = scene
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3, flip_point=flip) as s:
        s.calculate_normals()
        pn = s.normals()
        s.reconstruct(voxelsize=0.02, decomposition=decomposition)
        if planar:
            s.optimize_planar_faces(5)
        v, f, _ = s.mesh(with_edges=False)
        vn = s.vertex_normals()
        vn2, fb = s.vertex_normals(v, f)
    assert len(f) > 10_000
    ref, rfb = oracle_mod.vertex_normals(v, f, pn, oracle_mod.OracleSurface(P))
    assert fb == rfb
    assert np.array_equal(vn, ref) and np.array_equal(vn2, ref)
    ln = np.linalg.norm(vn.astype(np.float64), axis=1)
    assert np.all(np.abs(ln - 1) < 1e-5)


def test_fallbacks(gb, oracle_mod, scene):
    """Vertices without faces, degenerate faces ((0, 0, 1)) and two opposite
    faces whose normals cancel: the nearest point's normal."""
    P, flip = scene
    rng = np.random.Generator(np.random.PCG64(9))
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3, flip_point=flip) as s:
        s.calculate_normals()
        pn = s.normals()
        V = rng.uniform(P.min(0), P.max(0), size=(40, 3)).astype(np.float32)
        F = np.array([[0, 1, 2], [0, 2, 1],      # exactly opposite normals: zero sum at 0, 1, 2
                      [3, 4, 5], [3, 5, 6],      # an ordinary pair
                      [7, 7, 8],                 # degenerate: (0, 0, 1)
                      [9, 10, 11], [12, 13, 14]], np.uint32)
        vn, fb = s.vertex_normals(V, F)
        ref, rfb = oracle_mod.vertex_normals(V, F, pn, oracle_mod.OracleSurface(P))
        assert fb == rfb == 3 + (40 - 15)
        assert np.array_equal(vn, ref)
        assert np.array_equal(vn[7], np.array([0, 0, 1], np.float32))
        # no faces at all: every vertex takes its nearest point's normal
        vn, fb = s.vertex_normals(V, np.zeros((0, 3), np.uint32))
        ref, _ = oracle_mod.vertex_normals(V, np.zeros((0, 3), np.uint32), pn, oracle_mod.OracleSurface(P))
        assert fb == 40 and np.array_equal(vn, ref)
        vn, fb = s.vertex_normals(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
        assert vn.shape == (0, 3) and fb == 0


@pytest.mark.parametrize("width", [3, 4, 1])
def test_vertex_colors_match_oracle(gb, oracle_mod, scene, width):
    """calcColorFromPointCloud: the nearest point's colour per vertex."""
    P, flip = scene
    rng = np.random.Generator(np.random.PCG64(width))
    C = rng.integers(0, 256, size=(len(P), width), dtype=np.uint8)
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3, flip_point=flip) as s:
        s.calculate_normals()
        s.reconstruct(voxelsize=0.02, decomposition="PMC")
        s.optimize_planar_faces(5)
        v, _, _ = s.mesh(with_edges=False)
        vc = s.vertex_colors(C)
        with pytest.raises(ValueError):
            s.vertex_colors(C[:-1])
    ref = oracle_mod.vertex_colors(v, C, oracle_mod.OracleSurface(P))
    assert vc.shape == (len(v), width) and np.array_equal(vc, ref)


def test_errors(gb, scene):
    P, _ = scene
    with gb.Surface(P[:5000], kn=10, ki=10, kd=10, nem=3) as s:
        with pytest.raises(gb.LvrgbError) as e:
            s.vertex_normals()
        assert e.value.status == 5  # no mesh yet
        s.calculate_normals()
        V = np.zeros((4, 3), np.float32)
        with pytest.raises(gb.LvrgbError) as e:
            s.vertex_normals(V, np.array([[0, 1, 4]], np.uint32))  # index out of range
        assert e.value.status == 1
