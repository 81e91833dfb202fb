"""lvrgb_knn_small_noalloc: the kNN entry point for callers that cannot
allocate device memory during a call (real-time loops and driver callbacks
where an allocation would synchronize the device, hosts with a fixed
device-memory budget).  Its results must equal lvrgb_knn's and the oracle's
kNN rows on the same input, on consecutive calls that reuse the shared static
scratch array, and a call must allocate nothing.

Collected last (file name) so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _cloud(seed, n):
    rng = np.random.Generator(np.random.PCG64(seed))
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return (0.5 + 0.3 * v + rng.normal(scale=1e-3, size=v.shape)).astype(np.float32)


def _noalloc(lib, pts, q, k):
    """One call through the C ABI; returns (status, idx, dist)."""
    import torch
    d_p = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    d_q = torch.from_numpy(np.ascontiguousarray(q).reshape(-1, 3)).cuda()
    nq = len(d_q)
    idx = torch.full((max(nq, 1), k), 7, dtype=torch.int32, device="cuda")
    dist = torch.full((max(nq, 1), k), -1.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = lib.lvrgb_knn_small_noalloc(_ptr(d_p), len(pts), _ptr(d_q), nq, k, _ptr(idx), _ptr(dist), None)
    torch.cuda.synchronize()
    return st, idx.cpu().numpy().view(np.uint32)[:nq], dist.cpu().numpy()[:nq]


def test_noalloc_knn_matches_knn_and_oracle_on_consecutive_calls(lib, oracle_mod):
    import lvr2_gb300
    cases = [(_cloud(1, 60000), 12), (_cloud(2, 20000), 40)]
    for pts, k in cases:
        rng = np.random.Generator(np.random.PCG64(k))
        q = np.concatenate([pts[::5], rng.uniform(0, 1, (3000, 3)).astype(np.float32)])
        with lvr2_gb300.Surface(pts) as s:
            ref_idx, ref_dist, _ = s.knn(q, k)
        o_idx, o_dist, _ = oracle_mod.OracleSurface(pts).knn(q, k)
        st, got_idx, got_dist = _noalloc(lib, pts, q, k)
        assert st == 0, lib.lvrgb_last_error()
        # kNN rows are bit-exact between the two entry points and the oracle
        assert (got_idx == ref_idx).all() and np.array_equal(got_dist, ref_dist)
        assert (got_idx == o_idx).all() and np.array_equal(got_dist, o_dist)


def test_noalloc_knn_allocates_nothing(lib):
    """A warmed-up call leaves the device's free memory unchanged, and an
    injected allocation failure (the n-th next workspace allocation fails)
    is never reached by it."""
    import torch
    pts = _cloud(3, 30000)
    q = pts[::3].copy()
    k = 20
    d_p = torch.from_numpy(pts).cuda()
    d_q = torch.from_numpy(q).cuda()
    idx = torch.empty((len(q), k), dtype=torch.int32, device="cuda")
    dist = torch.empty((len(q), k), dtype=torch.float32, device="cuda")
    args = (_ptr(d_p), len(pts), _ptr(d_q), len(q), k, _ptr(idx), _ptr(dist), None)
    assert lib.lvrgb_knn_small_noalloc(*args) == 0, lib.lvrgb_last_error()  # warm-up: set-up per device
    torch.cuda.synchronize()
    first = (idx.cpu().numpy().copy(), dist.cpu().numpy().copy())
    free_before, _ = torch.cuda.mem_get_info()
    assert lib.lvrgb_debug_fail_allocation(1) == 0
    try:
        for _ in range(3):
            assert lib.lvrgb_knn_small_noalloc(*args) == 0, lib.lvrgb_last_error()
        torch.cuda.synchronize()
    finally:
        assert lib.lvrgb_debug_fail_allocation(0) == 0
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    assert np.array_equal(idx.cpu().numpy(), first[0]) and np.array_equal(dist.cpu().numpy(), first[1])


def test_noalloc_knn_pads_rows_when_fewer_points_than_k(lib, oracle_mod):
    pts = _cloud(4, 7)
    q = np.concatenate([pts, np.array([[0.1, 0.2, 0.3]], np.float32)])
    k = 10
    st, idx, dist = _noalloc(lib, pts, q, k)
    assert st == 0, lib.lvrgb_last_error()
    o_idx, o_dist, _ = oracle_mod.OracleSurface(pts).knn(q, k)
    assert (idx == o_idx).all() and np.array_equal(dist, o_dist)
    assert (idx[:, 7:] == 0xFFFFFFFF).all() and np.isinf(dist[:, 7:]).all() and (dist[:, 7:] > 0).all()
    assert (idx[:, :7] != 0xFFFFFFFF).all()


def test_noalloc_knn_with_no_queries(lib):
    st, idx, dist = _noalloc(lib, _cloud(5, 1000), np.zeros((0, 3), np.float32), 8)
    assert st == 0, lib.lvrgb_last_error()
    assert idx.shape == (0, 8) and dist.shape == (0, 8)


def test_noalloc_knn_rejects_a_nonfinite_point(lib):
    pts = _cloud(6, 5000)
    pts[1234, 1] = np.nan
    st, _, _ = _noalloc(lib, pts, pts[:10], 8)
    assert st == 1
    assert b"point 1234" in lib.lvrgb_last_error()
    # the next call with clean points still works (the marker is reset per call)
    pts[1234, 1] = 0.5
    st, idx, _ = _noalloc(lib, pts, pts[:10], 8)
    assert st == 0, lib.lvrgb_last_error()
    assert (idx[:, 0] == np.arange(10)).all()


def test_noalloc_knn_rejects_sizes_beyond_its_limits(lib):
    import torch
    p = torch.zeros((65537, 3), dtype=torch.float32, device="cuda")
    q = torch.zeros((4, 3), dtype=torch.float32, device="cuda")
    idx = torch.zeros((4, 8), dtype=torch.int32, device="cuda")
    dist = torch.zeros((4, 8), dtype=torch.float32, device="cuda")
    assert lib.lvrgb_knn_small_noalloc(_ptr(p), 65537, _ptr(q), 4, 8, _ptr(idx), _ptr(dist), None) == 1
    assert b"65536" in lib.lvrgb_last_error()
    assert lib.lvrgb_knn_small_noalloc(_ptr(p), 100, _ptr(q), 4, 97, _ptr(idx), _ptr(dist), None) == 1
    assert b"k must be" in lib.lvrgb_last_error()
