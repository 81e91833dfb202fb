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
