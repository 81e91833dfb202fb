"""lvrgb_get_normals_async: the normals copied on a second stream while the
surface's stream goes on with the grid, distances and mesh must equal the
synchronous lvrgb_get_normals read, bit for bit, and leave the mesh as it is
without the copy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_async_normals_equal_sync_and_overlap_reconstruct(lib):
    import torch
    import lvr2_gb300
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(200_000, seed=31)
    with lvr2_gb300.Surface(P, kn=10, ki=10, kd=10, nem=3) as s:
        s.calculate_normals()
        ref = s.normals()
        s.reconstruct(voxelsize=0.02, decomposition="PMC")
        v_ref, f_ref, _ = s.mesh(with_edges=False)
        host = torch.empty((len(P), 3), dtype=torch.float32).pin_memory().numpy()
        host[:] = np.nan
        cs = torch.cuda.Stream()
        for _ in range(2):
            s.calculate_normals()
            out = s.normals_async(host, cs)
            s.reconstruct(voxelsize=0.02, decomposition="PMC")
            v, f, _ = s.mesh(with_edges=False)
            cs.synchronize()
            assert out is host or np.shares_memory(out, host)
            assert np.array_equal(host, ref)
            assert np.array_equal(v, v_ref) and np.array_equal(f, f_ref)


def test_async_normals_rejects_a_wrong_buffer(lib):
    import torch
    import lvr2_gb300
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(20_000, seed=32)
    with lvr2_gb300.Surface(P, kn=10, ki=10) as s:
        s.calculate_normals()
        with pytest.raises(ValueError):
            s.normals_async(np.empty((len(P), 2), np.float32), torch.cuda.Stream())
