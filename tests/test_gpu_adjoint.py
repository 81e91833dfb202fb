"""Adjoint of the signed distance (lvrgb_distance_adjoint) and Newton
projection (lvrgb_project_to_surface).

Checks: the forward values equal lvrgb_distance bit for bit; d/dq against
central finite differences (h = 1e-3, samples whose kd-neighbourhood changes
within +-h are masked and counted); d/dpoints and d/dnormals against a float64
restatement of the analytic gradient over the same neighbourhoods; d/dnormals
against finite differences of the normals; projection lands on the zero level,
bit-exact against a float32 restatement of its operations and within float32
rounding of a float64 projection over the same neighbourhoods.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KD = 10


@pytest.fixture(scope="module")
def gb(lib):
    import lvr2_gb300
    return lvr2_gb300


@pytest.fixture(scope="module")
def scene(gb):
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(40_000, seed=7)
    rng = np.random.Generator(np.random.PCG64(11))
    s = gb.Surface(P, kn=10, ki=10, kd=KD, nem=3, flip_point=None)
    s.calculate_normals()
    N = s.normals()
    # queries near the surface: points displaced along random directions
    base = P[rng.choice(len(P), 3000, replace=False)]
    Q = (base + rng.normal(0, 4e-3, base.shape)).astype(np.float32)
    yield s, P, N, Q
    s.close()


def fp64_gradients(P, N, Q, idx, gd, ge):
    """Analytic gradient of (projected, euclidean) distance in float64 for the
    given neighbourhoods (rows of idx)."""
    P64, N64, Q64 = P.astype(np.float64), N.astype(np.float64), Q.astype(np.float64)
    c = P64[idx].mean(1)
    m = N64[idx].mean(1)
    ml = np.linalg.norm(m, axis=1)
    nh = m / ml[:, None]
    r = Q64 - c
    d = np.sum(r * nh, 1)
    e = np.linalg.norm(r, axis=1)
    gq = gd[:, None] * nh + (ge / np.maximum(e, 1e-300))[:, None] * r
    k = idx.shape[1]
    gp = np.zeros_like(P64)
    gn = np.zeros_like(N64)
    for s in range(k):
        np.add.at(gp, idx[:, s], -gq / k)
        np.add.at(gn, idx[:, s], (gd / (k * ml))[:, None] * (r - d[:, None] * nh))
    return d, e, gq, gp, gn


def test_forward_matches_distance(scene):
    s, P, N, Q = scene
    proj, eucl = s.distance(Q)
    p2, e2, gq, gp, gn = s.distance_adjoint(Q)
    assert np.array_equal(proj, p2) and np.array_equal(eucl, e2)
    # no upstream gradient: all gradients vanish
    assert not gq.any() and not gp.any() and not gn.any()


def test_gradients_against_fp64(scene):
    """Gradients of the projected distance: float32 kernel vs float64."""
    s, P, N, Q = scene
    rng = np.random.Generator(np.random.PCG64(5))
    gd = rng.normal(size=len(Q)).astype(np.float32)
    proj, eucl, gq, gp, gn = s.distance_adjoint(Q, gd, None)
    idx, _, cnt = s.knn(Q, KD)
    assert (cnt == KD).all()
    zero = np.zeros(len(Q))
    d, e, rq, rp, rn = fp64_gradients(P, N, Q, idx.astype(np.int64), gd.astype(np.float64), zero)
    assert np.allclose(proj, d, rtol=0, atol=1e-6) and np.allclose(eucl, e, rtol=0, atol=1e-6)
    assert np.abs(gq - rq).max() <= 1e-5 * max(1.0, np.abs(rq).max())
    # scatter sums: float32 atomics against float64
    assert np.abs(gp - rp).max() <= 1e-5 * max(1.0, np.abs(rp).max())
    assert np.abs(gn - rn).max() <= 1e-4 * max(1.0, np.abs(rn).max())
    assert np.abs(gp).sum() > 0 and np.abs(gn).sum() > 0


def test_euclidean_gradient_against_fp64(scene):
    """d|q - c|/dq = (q - c)/|q - c|: r = q - c carries float32 rounding of
    about 2e-7 absolute, so the unit vector's error scales with 1/|r|."""
    s, P, N, Q = scene
    ge = np.ones(len(Q), np.float32)
    _, eucl, gq, gp, _ = s.distance_adjoint(Q, None, ge, want_normals=False)
    idx, _, _ = s.knn(Q, KD)
    _, e, rq, rp, _ = fp64_gradients(P, N, Q, idx.astype(np.int64), np.zeros(len(Q)), ge.astype(np.float64))
    err = np.abs(gq - rq).max(1)
    assert (err <= 1e-6 + 5e-7 / e).all(), (err / (1e-6 + 5e-7 / e)).max()
    assert np.allclose(np.linalg.norm(gq, axis=1), 1.0, atol=1e-5)


def test_query_gradient_against_finite_differences(scene):
    s, P, N, Q = scene
    h = 1e-3
    _, _, gq, _, _ = s.distance_adjoint(Q, np.ones(len(Q), np.float32), None, want_points=False, want_normals=False)
    idx0, _, _ = s.knn(Q, KD)
    fd = np.zeros_like(gq)
    stable = np.ones(len(Q), bool)
    for a in range(3):
        dq = np.zeros(3, np.float32)
        dq[a] = h
        dp, _ = s.distance(Q + dq)
        dm, _ = s.distance(Q - dq)
        fd[:, a] = (dp.astype(np.float64) - dm) / (2 * h)
        ip, _, _ = s.knn(Q + dq, KD)
        im, _, _ = s.knn(Q - dq, KD)
        stable &= (np.sort(ip, 1) == np.sort(idx0, 1)).all(1) & (np.sort(im, 1) == np.sort(idx0, 1)).all(1)
    # samples whose neighbourhood changes within +-h are masked (and counted)
    assert stable.sum() >= 300, "only %d of %d samples keep their neighbourhood within +-h" % (stable.sum(), len(Q))
    err = np.abs(fd[stable] - gq[stable]).max(1)
    # the distance is linear in q for a fixed neighbourhood: FD error is float32 rounding / h
    assert np.percentile(err, 99) <= 2e-3, np.percentile(err, [50, 99, 100])


def test_normal_gradient_against_finite_differences(scene, gb):
    s, P, N, Q = scene
    rng = np.random.Generator(np.random.PCG64(9))
    gd = rng.normal(size=len(Q)).astype(np.float32)
    _, _, _, _, gn = s.distance_adjoint(Q, gd, None, want_points=False)
    touched = np.flatnonzero(np.abs(gn).sum(1) > 1e-3)
    h = 1e-3
    try:
        for j in rng.choice(touched, 4, replace=False):
            for a in range(3):
                Np, Nm = N.copy(), N.copy()
                Np[j, a] += h
                Nm[j, a] -= h
                s.set_normals(Np)
                lp = np.dot(gd.astype(np.float64), s.distance(Q)[0])
                s.set_normals(Nm)
                lm = np.dot(gd.astype(np.float64), s.distance(Q)[0])
                fd = (lp - lm) / (2 * h)
                assert abs(fd - gn[j, a]) <= 2e-3 * max(1.0, abs(gn[j, a])), (j, a, fd, gn[j, a])
    finally:
        s.set_normals(N)


def test_projection_reaches_zero_level(scene):
    s, P, N, Q = scene
    d0, _ = s.distance(Q)
    pos, nrm = s.project_to_surface(Q, steps=3)
    d1, _ = s.distance(pos)
    # a step lands on the plane of its neighbourhood; where the neighbourhood
    # changes on the way the residual is that of the next plane
    assert np.median(np.abs(d1)) <= 1e-5 < np.median(np.abs(d0))
    assert (np.abs(d1) < np.abs(d0)).mean() > 0.9
    assert np.allclose(np.linalg.norm(nrm, axis=1), 1.0, atol=1e-5)
    # one step from the same point equals x - d(x) n(x) with the adjoint's n = d/dq
    p1, _ = s.project_to_surface(Q, steps=1)
    _, _, gq, _, _ = s.distance_adjoint(Q, np.ones(len(Q), np.float32), None, want_points=False, want_normals=False)
    ref = Q - d0[:, None] * gq
    assert np.abs(p1 - ref).max() <= 1e-6


def project_restatement(oracle_surface, P, N, Q, steps, dtype):
    """Newton projection x <- x - d(x) n(x) restated in numpy: at each step the
    kd nearest points of x (the oracle's kNN rows, ascending (d2, index)), the
    mean point and the normalised mean normal summed in that order, d the
    projected distance.  dtype float32 repeats the kernel's operations one by
    one (each rounded on its own); float64 is the reference projection.
    Also returns, per query, the last step's sum of |n_j| over |sum of n_j|:
    how much the normalisation of the mean normal amplifies rounding."""
    f = np.dtype(dtype).type
    x = Q.astype(dtype)
    nh = np.zeros_like(x)
    amp = np.ones(len(Q))
    for _ in range(steps):
        rows, _, cnt = oracle_surface.knn(x.astype(np.float32), KD)
        assert (cnt == KD).all()
        p = np.zeros_like(x)
        m = np.zeros_like(x)
        mag = np.zeros(len(Q))
        for j in range(KD):
            p = p + P[rows[:, j].astype(np.int64)].astype(dtype)
            m = m + N[rows[:, j].astype(np.int64)].astype(dtype)
            mag += np.linalg.norm(N[rows[:, j].astype(np.int64)].astype(np.float64), axis=1)
        c = f(KD)
        p = p / c
        m = m / c
        ln = np.sqrt((m[:, 0] * m[:, 0] + m[:, 1] * m[:, 1]) + m[:, 2] * m[:, 2])
        n = np.where(ln[:, None] > 0, m / np.where(ln > 0, ln, f(1))[:, None], m)
        r = x - p
        d = (r[:, 0] * n[:, 0] + r[:, 1] * n[:, 1]) + r[:, 2] * n[:, 2]
        x = x - d[:, None] * n
        nh = n
        amp = mag / np.maximum(np.linalg.norm(m.astype(np.float64), axis=1) * KD, 1e-300)
    return x, nh, amp


def test_projection_against_restatements(scene, oracle_mod):
    """Three Newton steps: bit-exact against the float32 restatement of the
    kernel's operations, and within 2e-6 (a few float32 ulps of the unit-cube
    coordinates) of the float64 projection over the same neighbourhoods,
    wherever the float32 and float64 paths meet the same neighbours; the
    normals within float32 rounding amplified by the normalisation of the
    mean normal (1e-6 rad times sum |n_j| / |sum n_j|)."""
    s, P, N, Q = scene
    o = oracle_mod.OracleSurface(P)
    pos, nrm = s.project_to_surface(Q, steps=3)
    x32, n32, _ = project_restatement(o, P, N, Q, 3, np.float32)
    assert np.array_equal(pos, x32) and np.array_equal(nrm, n32)
    x64, n64, amp = project_restatement(o, P, N, Q, 3, np.float64)
    # a float32 rounding can move a position across a kNN tie between steps;
    # compare where the last step's neighbourhoods agree
    r32, _, _ = o.knn(pos, KD)
    r64, _, _ = o.knn(x64.astype(np.float32), KD)
    same = np.all(np.sort(r32, 1) == np.sort(r64, 1), axis=1)
    assert same.mean() > 0.99
    err = np.linalg.norm(pos.astype(np.float64) - x64, axis=1)[same]
    assert np.percentile(err, 99.9) <= 2e-6, np.percentile(err, [50, 99.9, 100])
    # both normalised in float64 first: a float32 unit vector is 1 only to an ulp
    a = nrm.astype(np.float64)
    a /= np.linalg.norm(a, axis=1, keepdims=True)
    b = n64 / np.linalg.norm(n64, axis=1, keepdims=True)
    ang = np.arccos(np.clip(np.abs(np.sum(a * b, axis=1)), -1, 1))[same]
    assert (ang <= 1e-6 * amp[same] + 1e-7).all(), np.percentile(np.degrees(ang), [50, 99.9, 100])


def test_reconstructed_vertices_project(gb):
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(60_000, seed=3)
    with gb.Surface(P, kn=10, ki=10, kd=KD, nem=3, flip_point=None) as s:
        s.calculate_normals()
        s.reconstruct(voxelsize=0.02, decomposition="PMC")
        v, f, _ = s.mesh(with_edges=False)
        d0, _ = s.distance(v)
        pos, nrm = s.project_to_surface(v, steps=3)
        d1, _ = s.distance(pos)
    assert len(v) > 1000
    assert np.median(np.abs(d1)) < 0.05 * np.median(np.abs(d0)) + 1e-7
    # vertices move by a fraction of a voxel (0.02), a few by up to two
    move = np.linalg.norm(pos - v, axis=1)
    assert np.median(move) <= 0.01 and np.percentile(move, 99) <= 0.05


def test_autograd_wrapper(scene):
    torch = pytest.importorskip("torch")
    from lvr2_gb300.autograd import signed_distance
    s, P, N, Q = scene
    q = torch.from_numpy(Q).cuda().requires_grad_(True)
    pts = torch.from_numpy(P).cuda().requires_grad_(True)
    nrm = torch.from_numpy(N).cuda().requires_grad_(True)
    d, e = signed_distance(s, q, pts, nrm)
    w = torch.linspace(-1, 1, len(Q), device="cuda")
    (d * w).sum().backward()
    _, _, gq, gp, gn = s.distance_adjoint(Q, w.cpu().numpy(), None)
    assert np.allclose(q.grad.cpu().numpy(), gq, atol=1e-6)
    assert np.allclose(pts.grad.cpu().numpy(), gp, atol=1e-5)
    assert np.allclose(nrm.grad.cpu().numpy(), gn, atol=1e-4)
    pd, _ = s.distance(Q)
    assert np.array_equal(d.detach().cpu().numpy(), pd)


def test_adjoint_argument_errors(scene, gb):
    s, P, N, Q = scene
    with pytest.raises(gb.LvrgbError):
        s.project_to_surface(Q, steps=0)
    with gb.Surface(P[:100]) as t:
        with pytest.raises(gb.LvrgbError) as e:
            t.distance_adjoint(Q[:4])
        assert e.value.status == 5  # no normals yet
