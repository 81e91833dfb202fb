"""Out-of-memory handling, injected on the host (lvrgb_debug_fail_allocation):
every device allocation of a normal estimation, a reconstruction and a scan
project is made to fail in turn.  Each failure returns
LVRGB_ERR_OUT_OF_MEMORY, and the same handle then gives results identical to
a run without faults (the large-scale tool retries on this status)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OOM = 3


@pytest.fixture(scope="module")
def gb(lib):
    import lvr2_gb300
    return lvr2_gb300


def run_surface(gb, s):
    s.calculate_normals()
    n = s.normals()
    s.reconstruct(voxelsize=0.02, decomposition="PMC")
    s.optimize_planar_faces(5)
    v, f, _ = s.mesh(with_edges=False)
    return n, v, f


def test_every_allocation_of_a_reconstruction(gb):
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(30_000, seed=23)
    L = gb._lib.load()
    with gb.Surface(P, kn=10, ki=10, kd=10, nem=3) as s:
        ref = run_surface(gb, s)
    failures = 0
    for n in range(1, 400):
        with gb.Surface(P, kn=10, ki=10, kd=10, nem=3) as s:
            L.lvrgb_debug_fail_allocation(n)
            try:
                run_surface(gb, s)
                L.lvrgb_debug_fail_allocation(0)
                break  # fewer than n allocations: nothing failed
            except gb.LvrgbError as e:
                L.lvrgb_debug_fail_allocation(0)
                assert e.status == OOM
                failures += 1
            got = run_surface(gb, s)  # the same handle, after the failure
            assert all(np.array_equal(a, b) for a, b in zip(ref, got))
    else:
        pytest.fail("more than 400 allocations")
    assert failures >= 10


def test_scan_project_allocations(gb):
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(40_000, seed=24)
    scans = [P[:15_000], P[15_000:]]
    flips = np.array([[0, 0, 0], [1, 1, 1]], np.float32)
    L = gb._lib.load()
    with gb.Batch(scans, flips, kn=10, ki=10, nem=3) as b:
        b.calculate_normals()
        ref = b.normals()
    failures = 0
    for n in range(1, 200):
        L.lvrgb_debug_fail_allocation(n)
        try:
            with gb.Batch(scans, flips, kn=10, ki=10, nem=3) as b:
                b.calculate_normals()
                L.lvrgb_debug_fail_allocation(0)
                assert np.array_equal(b.normals(), ref)
                break
        except gb.LvrgbError as e:
            L.lvrgb_debug_fail_allocation(0)
            assert e.status == OOM
            failures += 1
    else:
        pytest.fail("more than 200 allocations")
    assert failures >= 5
