"""lvrgb_knn_small_noalloc: the kNN entry point for callers that cannot
allocate device memory during a call (real-time loops and driver callbacks
where an allocation would synchronize the device, hosts with a fixed
device-memory budget).  Its results must equal lvrgb_knn's on the same
input, on consecutive calls that reuse the shared static scratch array.

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


def test_noalloc_knn_matches_knn_on_consecutive_calls(lib):
    import torch

    import lvr2_gb300
    cases = [(_cloud(1, 60000), 12), (_cloud(2, 20000), 40)]
    for pts, k in cases:
        rng = np.random.Generator(np.random.PCG64(k))
        q = np.concatenate([pts[::5], rng.uniform(0, 1, (3000, 3)).astype(np.float32)])
        with lvr2_gb300.Surface(pts) as s:
            ref_idx, ref_dist, _ = s.knn(q, k)
        d_p = torch.from_numpy(pts).cuda()
        d_q = torch.from_numpy(q).cuda()
        idx = torch.full((len(q), k), 7, dtype=torch.int32, device="cuda")
        dist = torch.full((len(q), k), -1.0, dtype=torch.float32, device="cuda")
        st = lib.lvrgb_knn_small_noalloc(_ptr(d_p), len(pts), _ptr(d_q), len(q), k, _ptr(idx), _ptr(dist), None)
        assert st == 0, lib.lvrgb_last_error()
        torch.cuda.synchronize()
        got_idx = idx.cpu().numpy().view(np.uint32)
        got_dist = dist.cpu().numpy()
        # kNN rows are bit-exact between the two entry points
        assert (got_idx == ref_idx).all()
        assert np.array_equal(got_dist, ref_dist)


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
