"""HashGrid::toPointBuffer (lvrgb_get_cell_tsdf): the culled cells with their
centres and the distances at their 8 corners.  The cells equal the oracle's
valid cells, the centres follow (index + 0.5) * voxelsize, and every corner
distance is the grid-vertex distance at that corner of the cell."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CORNERS = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]],
                   np.int64)


@pytest.mark.parametrize("extrude", [True, False])
def test_cell_tsdf(lib, oracle_mod, extrude):
    import lvr2_gb300
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(40_000, seed=11)
    flip = ((P.min(0) + P.max(0)) / 2).astype(np.float32)
    with lvr2_gb300.Surface(P, kn=10, ki=10, kd=10, nem=3, flip_point=flip) as s:
        s.calculate_normals()
        normals = s.normals()
        info = s.reconstruct(voxelsize=0.02, extrude=extrude)
        centers, tsdf = s.cell_tsdf()
        _, valid = s.cells()
        lat, _, dist, inv = s.grid()
    assert len(centers) == info.cells_valid > 1000
    vs = np.float32(info.voxelsize)
    assert np.array_equal(centers, (valid.astype(np.float32) + np.float32(0.5)) * vs)
    key = {tuple(v): i for i, v in enumerate(lat.tolist())}
    corner_ids = np.array([[key[tuple(c)] for c in (v + CORNERS).tolist()] for v in valid.astype(np.int64)])
    assert np.array_equal(tsdf, dist[corner_ids])
    assert not inv[corner_ids].any()  # culling kept only cells with valid corners
    r = oracle_mod.OracleSurface(P).reconstruct(normals, voxelsize=0.02, kd=10, extrude=extrude,
                                                grid_override=(lat, dist, inv))
    assert np.array_equal(np.sort(valid.view("i4,i4,i4"), axis=0), np.sort(r["cells_valid"].view("i4,i4,i4"), axis=0))
