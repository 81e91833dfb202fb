"""Parity with lvr2's own CUDA LBVH, run unmodified on a GB300.

tests/golden/ref_lbvh.npz holds what lvr2's LBVHIndex (src/liblvr2/
reconstruction/cuda/LBVHIndex.cu) returned for three seeded clouds (made by
tests/golden/make_ref_lbvh.py on a GB300 from the lvr2 sources): kSearch rows
(K = 20, SearchTreeLBVH's leaf size 1) for 1,200 sampled points and 200 random
queries per cloud, and knn_normals (K = 20, its fixed flip point (1e6, 1e6,
1e6)) for every point, on a leaf-size-1 tree (oracle/ref_lbvh.cu says why not
CudaKSearchSurface's 32).

Where the two may legitimately differ, and the bars:
- lvr2's kernels are compiled by NVRTC with FMA contraction on, so its
  squared distances can differ from this library's (each product and sum
  rounded on its own) by an ulp or two: the Euclidean distances agree with
  the square roots of lvr2's squared distances to 2 ulp.
- lvr2's queue admits an equal distance in place of its current maximum
  (last seen wins, static_priorityqueue.cuh:63-70); this library keeps the
  smaller (d2, index).  Neighbour sets are equal except where the k-th and
  (k+1)-th distances tie to within that rounding; every differing neighbour
  must be such a tie (none occur in these clouds).
- nem 4 reproduces knn_normals' FP64 arithmetic: the normals are equal bit
  for bit.
"""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
GOLD = np.load(ROOT / "tests/golden/ref_lbvh.npz")
K = int(GOLD["K"])
NAMES = ["sphere", "scan", "spheres_tori"]
FLIP = (1e6, 1e6, 1e6)


@pytest.fixture(scope="module")
def gb(lib):
    import lvr2_gb300
    return lvr2_gb300


def _d64(P, q, idx):
    d = P[idx].astype(np.float64) - q.astype(np.float64)[None, :]
    return np.sum(d * d, axis=1)


def _ulp_close(a, b, n_ulp=4):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return np.abs(a.astype(np.float64) - b.astype(np.float64)) <= n_ulp * np.spacing(np.maximum(np.abs(a), np.abs(b)))


@pytest.mark.parametrize("name", NAMES)
def test_knn_rows_against_lvr2_lbvh(gb, name):
    P, Q = GOLD[name + "_points"], GOLD[name + "_queries"]
    ridx, rdist, rcnt = GOLD[name + "_idx"], GOLD[name + "_dist"], GOLD[name + "_cnt"]
    with gb.Surface(P) as s:
        gi, gd, gc = s.knn(Q, K)
    assert (rcnt == K).all() and (gc == K).all()
    ties = 0
    for r in range(len(Q)):
        a, b = set(gi[r].tolist()), set(ridx[r].tolist())
        if a != b:
            ties += 1
            only = np.array(sorted(a ^ b), np.int64)
            d = _d64(P, Q[r], only)
            kth = _d64(P, Q[r], gi[r][-1:].astype(np.int64))[0]
            # every differing neighbour lies on the k-th distance, to float32 rounding
            assert np.all(np.abs(d - kth) <= 8 * np.spacing(np.float32(kth))), (r, d, kth)
        # Euclidean distances against the square roots of lvr2's squared ones
        ref_d = np.sqrt(np.sort(rdist[r]).astype(np.float64)).astype(np.float32)
        assert _ulp_close(np.sort(gd[r]), ref_d, 2).all(), r
    assert ties <= len(Q) // 100, ties
    print("%s: %d of %d rows differ only by k-th-distance ties" % (name, ties, len(Q)))


@pytest.mark.parametrize("name", NAMES)
def test_nem4_normals_against_lvr2_knn_normals(gb, name):
    P, ref = GOLD[name + "_points"], GOLD[name + "_normals"]
    with gb.Surface(P, kn=K, ki=0, kd=5, nem=4, flip_point=FLIP) as s:
        s.calculate_normals()
        n = s.normals()
    assert np.array_equal(n, ref)
