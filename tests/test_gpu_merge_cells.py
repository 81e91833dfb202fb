"""lvrgb_reconstruct_cells: the large-scale merge (HashGrid from stored chunk
grids with inner boxes) and marching cubes on the GPU.  Chunk grids come from
lvrgb_get_cell_tsdf of separate surfaces; the merged mesh equals the oracle's
sequential restatement bit for bit (canonical form)."""
import numpy as np
import pytest

from tests.helpers import canonical_mesh

pytestmark = pytest.mark.gpu

BIG = 1e9


@pytest.fixture(scope="module")
def gb(lib):
    import lvr2_gb300
    return lvr2_gb300


def chunk_cells(gb, P, vs, flip):
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3, flip_point=flip) as s:
        s.calculate_normals()
        s.reconstruct(voxelsize=vs, decomposition="MC")
        return s.cell_tsdf()


def same_mesh(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("decomposition", ["MC", "PMC"])
def test_two_chunks_match_oracle(gb, oracle_mod, decomposition):
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(80_000, seed=12)
    flip = ((P.min(0) + P.max(0)) / 2).astype(np.float32)
    vs = 0.02
    ca, ta = chunk_cells(gb, P[P[:, 0] < 0.56], vs, flip)
    cb, tb = chunk_cells(gb, P[P[:, 0] > 0.44], vs, flip)
    C = np.concatenate([ca, cb])
    T = np.concatenate([ta, tb])
    off = np.array([0, len(ca), len(ca) + len(cb)], np.int64)
    boxes = np.array([[-BIG, -BIG, -BIG, 0.5, BIG, BIG], [0.5, -BIG, -BIG, BIG, BIG, BIG]], np.float32)
    with gb.Surface(P[:1000], kn=10, ki=10, kd=10, nem=3) as s:
        info = s.reconstruct_cells(C, T, vs, chunk_offsets=off, inner_boxes=boxes, decomposition=decomposition)
        v, f, e = s.mesh()
        cells, _ = s.cells()
    r = oracle_mod.reconstruct_cells(C, T, vs, chunk_offsets=off, inner_boxes=boxes, decomposition=decomposition)
    assert info.faces == len(r["faces"]) > 10_000
    assert info.cells_valid == len(r["cells_all"])
    assert np.array_equal(np.sort(cells.view("i4,i4,i4"), axis=0), np.sort(r["cells_all"].view("i4,i4,i4"), axis=0))
    assert same_mesh(canonical_mesh(e, v, f), canonical_mesh(r["vkeys"], r["vpos"], r["faces"]))


def test_first_copy_wins(gb, oracle_mod):
    """A cell given twice keeps its first copy; a shared corner keeps the
    distance of the earliest cell holding it."""
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(40_000, seed=13)
    c, t = chunk_cells(gb, P, 0.03, ((P.min(0) + P.max(0)) / 2).astype(np.float32))
    rng = np.random.Generator(np.random.PCG64(1))
    perm = rng.permutation(len(c))
    t2 = t + rng.normal(scale=0.01, size=t.shape).astype(np.float32)
    C = np.concatenate([c[perm], c])
    T = np.concatenate([t2[perm], t])
    with gb.Surface(P[:1000], kn=10, ki=10, kd=10, nem=3) as s:
        info = s.reconstruct_cells(C, T, 0.03)
        v, f, e = s.mesh()
    r = oracle_mod.reconstruct_cells(C, T, 0.03)
    assert info.cells_valid == len(c)
    assert same_mesh(canonical_mesh(e, v, f), canonical_mesh(r["vkeys"], r["vpos"], r["faces"]))
    r1 = oracle_mod.reconstruct_cells(c[perm], t2[perm], 0.03)  # the second copies change nothing
    assert same_mesh(canonical_mesh(r["vkeys"], r["vpos"], r["faces"]),
                     canonical_mesh(r1["vkeys"], r1["vpos"], r1["faces"]))


def test_edge_cases(gb):
    P = np.random.default_rng(2).random((2000, 3)).astype(np.float32)
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3) as s:
        info = s.reconstruct_cells(np.zeros((0, 3), np.float32), np.zeros((0, 8), np.float32), 0.1)
        assert (info.cells_valid, info.faces) == (0, 0)
        c = np.array([[0.05, 0.05, 0.05]], np.float32)
        t = np.array([[1, -1, 1, -1, 1, -1, 1, -1]], np.float32)
        off = np.array([0, 1], np.int64)
        box = np.array([[1, 1, 1, 2, 2, 2]], np.float32)  # the only cell lies outside its box
        info = s.reconstruct_cells(c, t, 0.1, chunk_offsets=off, inner_boxes=box)
        assert (info.cells_valid, info.faces) == (0, 0)
        info = s.reconstruct_cells(c, t, 0.1)
        assert info.cells_valid == 1 and info.faces > 0
        with pytest.raises(gb.LvrgbError) as e:
            s.reconstruct_cells(c, t, 0.1, chunk_offsets=np.array([0, 2], np.int64))
        assert e.value.status == 1
        with pytest.raises(gb.LvrgbError):
            s.reconstruct_cells(c, t, -1.0)
