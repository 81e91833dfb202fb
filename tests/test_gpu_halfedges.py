"""Half-edge connectivity of the mesh (lvrgb_mesh_halfedges), in
pmp::SurfaceMesh's layout, equal to the oracle's canonical restatement for
closed and open marching-cubes meshes (MC, PMC, after the planar pass)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("he_vertex", "he_next", "he_prev", "he_face", "vertex_he", "face_he")


@pytest.fixture(scope="module")
def gb(lib):
    import lvr2_gb300
    return lvr2_gb300


@pytest.mark.parametrize("cut,decomposition,planar", [(None, "MC", False), (0.5, "PMC", True), (0.5, "MC", False)])
def test_halfedges_match_oracle(gb, oracle_mod, cut, decomposition, planar):
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(60_000, seed=41)
    if cut is not None:
        P = P[P[:, 0] < cut]  # open surfaces: boundary loops
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3, flip_point=((P.min(0) + P.max(0)) / 2).astype(np.float32)) as s:
        s.calculate_normals()
        s.reconstruct(voxelsize=0.02, decomposition=decomposition)
        if planar:
            s.optimize_planar_faces(5)
        v, f, _ = s.mesh(with_edges=False)
        H = s.halfedges()
    ref = oracle_mod.halfedges(f, len(v))
    assert H["complex_edges"] == 0 == ref["complex_edges"]
    assert H["edges"] == ref["edges"] and H["boundary_halfedges"] == ref["boundary_halfedges"]
    assert H["boundary_halfedges"] > 0  # culled cells and the cut leave boundary loops
    assert H["complex_vertices"] == ref["complex_vertices"]
    for k in KEYS:
        assert np.array_equal(H[k], ref[k]), k


def test_halfedges_need_a_mesh(gb):
    P = np.random.default_rng(0).random((2000, 3)).astype(np.float32)
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3) as s:
        with pytest.raises(gb.LvrgbError) as e:
            s.halfedges()
        assert e.value.status == 5


def _grid_mesh(n, rng, holes=0.15):
    """Triangulated n x n grid with random faces removed (boundary loops,
    bow-tie vertices where two holes touch) and shuffled face order and
    orientation-preserving corner rotations."""
    ij = np.arange(n * n).reshape(n, n)
    a, b, c, d = ij[:-1, :-1].ravel(), ij[:-1, 1:].ravel(), ij[1:, :-1].ravel(), ij[1:, 1:].ravel()
    F = np.concatenate([np.stack([a, b, d], 1), np.stack([a, d, c], 1)])
    F = F[rng.random(len(F)) >= holes]
    F = F[rng.permutation(len(F))]
    r = rng.integers(0, 3, len(F))
    F = np.stack([F[np.arange(len(F)), (r + j) % 3] for j in range(3)], 1)
    return F.astype(np.uint32), n * n


@pytest.mark.parametrize("n,holes,seed", [(2, 0.0, 0), (7, 0.3, 1), (40, 0.15, 2), (300, 0.05, 3)])
def test_halfedges_of_given_faces_match_oracle(gb, oracle_mod, n, holes, seed):
    rng = np.random.default_rng(seed)
    F, nv = _grid_mesh(n, rng, holes)
    P = rng.random((2000, 3)).astype(np.float32)
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3) as s:
        H = s.halfedges(F, nv + 5)  # trailing isolated vertices
    ref = oracle_mod.halfedges(F, nv + 5)
    assert H["complex_edges"] == 0 == ref["complex_edges"]
    for k in ("edges", "boundary_halfedges", "complex_vertices"):
        assert H[k] == ref[k], k
    assert np.all(H["vertex_he"][nv:] == 0xFFFFFFFF)
    for k in KEYS:
        assert np.array_equal(H[k], ref[k]), k


def test_halfedges_of_given_faces_errors(gb):
    P = np.random.default_rng(0).random((2000, 3)).astype(np.float32)
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3) as s:
        H = s.halfedges(np.zeros((0, 3), np.uint32), 4)  # no faces: isolated vertices
        assert H["edges"] == 0 and np.all(H["vertex_he"] == 0xFFFFFFFF)
        for faces, status in (([[0, 1, 1]], 7),               # repeated vertex
                              ([[0, 1, 2], [0, 1, 3]], 7),    # two faces of one orientation
                              ([[0, 1, 2], [1, 0, 3], [0, 1, 4]], 7),  # three faces on an edge
                              ([[0, 1, 9]], 1)):              # index out of range (nv = 5)
            with pytest.raises(gb.LvrgbError) as e:
                s.halfedges(np.array(faces, np.uint32), 5)
            assert e.value.status == status, faces
