"""Seeded synthetic point clouds with the shapes of the reconstruction workloads.

The public scan the lvr2 README reconstructs (dat/scan.pts) is not available,
so every workload here is generated from a numpy PCG64 stream:

  scan_scene        289,252-point outdoor scan: ground plane, 6 box buildings,
                    4 cylinders, ray-sampled from a scanner at the origin
                    (density ~ 1/r^2), range noise sigma 0.5, uint8 intensity,
                    inside [-851,-79,1]-[1487,328,808].
  spheres_tori      points uniform (by area) on the surfaces of 200 random
                    spheres (r in [0.02, 0.2]) and 100 tori in the unit cube,
                    isotropic noise sigma 1e-3 (10M points by default).
  folded_sheets     pairs of parallel folded planes (fold angle 1-10 degrees,
                    pair separation 2 * voxel size), noise sigma 1e-4 along the
                    normal only, all coordinates offset by +1e5 (20M points).
  scan_project      64 scans of log-uniform size in [50k, 4M] ray-sampled from
                    their own scanner poses in one box-and-cylinder scene.
  terrain           heightfield of 8 octaves of value noise over 1000 x 1000
                    units, noise sigma 0.2 (30M points).
"""
import math

import numpy as np

SCAN_BOX_LO = np.array([-851.0, -79.0, 1.0])
SCAN_BOX_HI = np.array([1487.0, 328.0, 808.0])
GROUND_Y = -70.0
BOXES = np.array([  # xmin xmax ymin ymax zmin zmax
    [-800, -600, GROUND_Y, 200, 300, 450],
    [-400, -250, GROUND_Y, 150, 500, 700],
    [100, 300, GROUND_Y, 320, 600, 790],
    [500, 700, GROUND_Y, 250, 200, 350],
    [900, 1100, GROUND_Y, 180, 450, 650],
    [1250, 1470, GROUND_Y, 300, 100, 300],
], dtype=np.float64)
CYLINDERS = np.array([  # cx cz radius height
    [-100, 250, 30, 150],
    [400, 450, 40, 200],
    [800, 100, 25, 120],
    [1200, 700, 50, 250],
], dtype=np.float64)


def _raycast(origin, d, boxes=BOXES, cyls=CYLINDERS, ground_y=GROUND_Y):
    """Nearest hit distance along unit rays d from origin (inf = miss)."""
    o = np.asarray(origin, np.float64)
    t = np.full(len(d), np.inf)
    with np.errstate(divide="ignore", invalid="ignore"):
        tp = (ground_y - o[1]) / d[:, 1]
        t = np.where((tp > 1e-6), np.minimum(t, tp), t)
        for b in boxes:
            lo, hi = b[[0, 2, 4]], b[[1, 3, 5]]
            t1 = (lo - o) / d
            t2 = (hi - o) / d
            tn = np.nanmax(np.minimum(t1, t2), axis=1)
            tf = np.nanmin(np.maximum(t1, t2), axis=1)
            hit = (tf >= tn) & (tf > 1e-6)
            th = np.where(tn > 1e-6, tn, tf)
            t = np.where(hit, np.minimum(t, th), t)
        for cx, cz, r, h in cyls:
            ox, oz = o[0] - cx, o[2] - cz
            a = d[:, 0] ** 2 + d[:, 2] ** 2
            bq = 2 * (ox * d[:, 0] + oz * d[:, 2])
            c = ox * ox + oz * oz - r * r
            disc = bq * bq - 4 * a * c
            sq = np.sqrt(np.maximum(disc, 0))
            for tc in ((-bq - sq) / (2 * a), (-bq + sq) / (2 * a)):
                y = o[1] + tc * d[:, 1]
                ok = (disc >= 0) & (tc > 1e-6) & (y >= ground_y) & (y <= ground_y + h)
                t = np.where(ok, np.minimum(t, tc), t)
    return t


def _random_dirs(rng, m, hemisphere_z=False):
    v = rng.normal(size=(m, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    if hemisphere_z:
        v[:, 2] = np.abs(v[:, 2])
    return v


def scan_scene(n=289_252, seed=1, sigma=0.5):
    """(points float32 (n,3), intensity uint8 (n,)) of the outdoor scan scene."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    have = 0
    while have < n:
        d = _random_dirs(rng, max(4 * (n - have), 100_000), hemisphere_z=True)
        t = _raycast(np.zeros(3), d)
        ok = np.isfinite(t)
        p = d[ok] * (t[ok] + rng.normal(scale=sigma, size=ok.sum()))[:, None]
        inb = np.all((p >= SCAN_BOX_LO) & (p <= SCAN_BOX_HI), axis=1)
        p = p[inb]
        out.append(p)
        have += len(p)
    pts = np.concatenate(out)[:n].astype(np.float32)
    rng2 = np.random.Generator(np.random.PCG64(seed + 1000))
    r = np.linalg.norm(pts, axis=1)
    intensity = np.clip(255 * np.exp(-r / 800.0) + rng2.normal(scale=10, size=n), 0, 255).astype(np.uint8)
    return pts, intensity


def spheres_tori(n=10_000_000, seed=2, n_spheres=200, n_tori=100, sigma=1e-3):
    """Points on 200 spheres and 100 tori in [0,1]^3 (float32 (n,3))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sr = rng.uniform(0.02, 0.2, n_spheres)
    sc = rng.uniform(sr[:, None], 1 - sr[:, None], (n_spheres, 3))
    tR = rng.uniform(0.03, 0.15, n_tori)
    tr = rng.uniform(0.005, 0.03, n_tori)
    tc = rng.uniform((tR + tr)[:, None], 1 - (tR + tr)[:, None], (n_tori, 3))
    rot = []
    for _ in range(n_tori):
        q, _r = np.linalg.qr(rng.normal(size=(3, 3)))
        rot.append(q)
    rot = np.array(rot)
    area = np.concatenate([4 * np.pi * sr ** 2, 4 * np.pi ** 2 * tR * tr])
    counts = rng.multinomial(n, area / area.sum())
    pts = np.empty((n, 3), np.float64)
    pos = 0
    for i in range(n_spheres):
        m = counts[i]
        v = rng.normal(size=(m, 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        pts[pos:pos + m] = sc[i] + sr[i] * v
        pos += m
    for j in range(n_tori):
        m = counts[n_spheres + j]
        R, r = tR[j], tr[j]
        u = rng.uniform(0, 2 * np.pi, m)
        v = np.empty(m)
        filled = 0
        while filled < m:  # area-uniform tube angle by rejection
            cand = rng.uniform(0, 2 * np.pi, 2 * (m - filled) + 16)
            acc = cand[rng.uniform(0, 1, len(cand)) < (R + r * np.cos(cand)) / (R + r)]
            take = min(len(acc), m - filled)
            v[filled:filled + take] = acc[:take]
            filled += take
        local = np.stack([(R + r * np.cos(v)) * np.cos(u), (R + r * np.cos(v)) * np.sin(u), r * np.sin(v)], axis=1)
        pts[pos:pos + m] = tc[j] + local @ rot[j].T
        pos += m
    pts += rng.normal(scale=sigma, size=pts.shape)
    perm = rng.permutation(n)
    return pts[perm].astype(np.float32)


def folded_sheets(n=20_000_000, seed=3, tiles=2, tile_size=50.0, sigma_n=1e-4, offset=1e5, voxelsize=None):
    """Pairs of parallel folded planes, offset by +1e5; returns (points, voxelsize)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n_sheets = tiles * tiles * 2
    per = n // n_sheets
    spacing = tile_size / math.sqrt(per)
    vs = 4.0 * spacing if voxelsize is None else voxelsize
    sep = 2.0 * vs
    out = []
    for ty in range(tiles):
        for tx in range(tiles):
            alpha = math.radians(rng.uniform(1.0, 10.0))
            xf = rng.uniform(0.3, 0.7) * tile_size
            for s in range(2):
                m = per if len(out) < n_sheets - 1 else n - per * (n_sheets - 1)
                x = rng.uniform(0, tile_size, m)
                y = rng.uniform(0, tile_size, m)
                beyond = x > xf
                z = np.where(beyond, (x - xf) * math.tan(alpha), 0.0) + s * sep
                nrm = np.zeros((m, 3))
                nrm[:, 2] = 1.0
                nrm[beyond, 0] = -math.sin(alpha)
                nrm[beyond, 2] = math.cos(alpha)
                p = np.stack([x + tx * (tile_size + 5 * vs), y + ty * (tile_size + 5 * vs), z], axis=1)
                p += nrm * rng.normal(scale=sigma_n, size=(m, 1))
                out.append(p)
    pts = np.concatenate(out) + offset
    perm = rng.permutation(len(pts))
    return pts[perm].astype(np.float32), float(vs)


def scan_project(n_scans=64, seed=4, lo=50_000, hi=4_000_000, sigma=0.5, scale=1.0):
    """List of (points float32, scanner position float32) for one scan project."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), n_scans)) * scale
    sizes = np.maximum(sizes.astype(np.int64), 16)
    scans = []
    for i in range(n_scans):
        while True:
            pose = np.array([rng.uniform(-800, 1450), GROUND_Y + 1.5, rng.uniform(20, 790)])
            inside = any((b[0] <= pose[0] <= b[1]) and (b[4] <= pose[2] <= b[5]) for b in BOXES)
            inside |= any((pose[0] - c[0]) ** 2 + (pose[2] - c[1]) ** 2 <= c[2] ** 2 for c in CYLINDERS)
            if not inside:
                break
        m = int(sizes[i])
        pts = []
        have = 0
        while have < m:
            d = _random_dirs(rng, max(2 * (m - have), 50_000))
            t = _raycast(pose, d)
            ok = np.isfinite(t) & (t < 3000)
            p = pose + d[ok] * (t[ok] + rng.normal(scale=sigma, size=ok.sum()))[:, None]
            pts.append(p)
            have += len(p)
        scans.append((np.concatenate(pts)[:m].astype(np.float32), pose.astype(np.float32)))
    return scans


def _value_noise(x, y, rng_seed, freq):
    rng = np.random.Generator(np.random.PCG64(rng_seed))
    gx = int(math.ceil(1000 * freq)) + 2
    lat = rng.uniform(-1, 1, (gx, gx))
    fx, fy = x * freq, y * freq
    ix, iy = np.floor(fx).astype(np.int64), np.floor(fy).astype(np.int64)
    tx, ty = fx - ix, fy - iy
    sx, sy = tx * tx * (3 - 2 * tx), ty * ty * (3 - 2 * ty)
    ix = np.clip(ix, 0, gx - 2)
    iy = np.clip(iy, 0, gx - 2)
    a = lat[ix, iy] * (1 - sx) + lat[ix + 1, iy] * sx
    b = lat[ix, iy + 1] * (1 - sx) + lat[ix + 1, iy + 1] * sx
    return a * (1 - sy) + b * sy


def terrain(n=30_000_000, seed=5, size=1000.0, sigma=0.2, octaves=8):
    """Points on a value-noise heightfield (float32 (n,3))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x = rng.uniform(0, size, n)
    y = rng.uniform(0, size, n)
    h = np.zeros(n)
    amp, freq = 60.0, 1.0 / 200.0
    for o in range(octaves):
        h += amp * _value_noise(x, y, seed * 100 + o, freq)
        amp *= 0.5
        freq *= 2.0
    z = h + rng.normal(scale=sigma, size=n)
    return np.stack([x, y, z], axis=1).astype(np.float32)


def terrain_device(n=30_000_000, seed=5, size=1000.0, sigma=0.2, octaves=8, device="cuda"):
    """terrain()'s heightfield (same value-noise lattices) evaluated with torch
    on a device, positions from a seeded torch generator (a different random
    stream than terrain()).  Returns a contiguous float32 (n, 3) tensor."""
    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    x = torch.rand(n, generator=gen, device=device, dtype=torch.float64) * size
    y = torch.rand(n, generator=gen, device=device, dtype=torch.float64) * size
    h = torch.zeros(n, device=device, dtype=torch.float64)
    amp, freq = 60.0, 1.0 / 200.0
    for o in range(octaves):
        rng = np.random.Generator(np.random.PCG64(seed * 100 + o))
        gx = int(math.ceil(1000 * freq)) + 2
        lat = torch.from_numpy(rng.uniform(-1, 1, (gx, gx))).to(device)
        fx, fy = x * freq, y * freq
        ix, iy = torch.floor(fx), torch.floor(fy)
        tx, ty = fx - ix, fy - iy
        sx, sy = tx * tx * (3 - 2 * tx), ty * ty * (3 - 2 * ty)
        ix = ix.long().clamp(0, gx - 2)
        iy = iy.long().clamp(0, gx - 2)
        a = lat[ix, iy] * (1 - sx) + lat[ix + 1, iy] * sx
        b = lat[ix, iy + 1] * (1 - sx) + lat[ix + 1, iy + 1] * sx
        h += amp * (a * (1 - sy) + b * sy)
        amp *= 0.5
        freq *= 2.0
    z = h + torch.randn(n, generator=gen, device=device, dtype=torch.float64) * sigma
    return torch.stack([x, y, z], dim=1).to(torch.float32).contiguous()


def crop(points, fraction, center=None):
    """Spatial crop keeping about `fraction` of the points at unchanged density."""
    p = np.asarray(points)
    lo, hi = p.min(0), p.max(0)
    c = (lo + hi) / 2 if center is None else np.asarray(center)
    side = (hi - lo) * fraction ** (1 / 3) / 2
    for _ in range(30):
        sel = np.all(np.abs(p - c) <= side, axis=1)
        got = sel.mean()
        if abs(got - fraction) < 0.1 * fraction:
            break
        side *= (fraction / max(got, 1e-9)) ** (1 / 3)
    return p[sel]


def _raycast_torch(origin, d, boxes, cyls, ground_y):
    import torch
    o = origin
    inf = torch.full((d.shape[0],), float("inf"), device=d.device, dtype=d.dtype)
    t = inf.clone()
    tp = (ground_y - o[1]) / d[:, 1]
    t = torch.where(tp > 1e-6, torch.minimum(t, tp), t)
    for b in boxes:
        lo = torch.tensor([b[0], b[2], b[4]], device=d.device, dtype=d.dtype)
        hi = torch.tensor([b[1], b[3], b[5]], device=d.device, dtype=d.dtype)
        t1 = (lo - o) / d
        t2 = (hi - o) / d
        tn = torch.nan_to_num(torch.minimum(t1, t2), nan=-float("inf")).amax(dim=1)
        tf = torch.nan_to_num(torch.maximum(t1, t2), nan=float("inf")).amin(dim=1)
        hit = (tf >= tn) & (tf > 1e-6)
        th = torch.where(tn > 1e-6, tn, tf)
        t = torch.where(hit, torch.minimum(t, th), t)
    for cx, cz, r, h in cyls:
        ox, oz = o[0] - cx, o[2] - cz
        a = d[:, 0] ** 2 + d[:, 2] ** 2
        bq = 2 * (ox * d[:, 0] + oz * d[:, 2])
        c = ox * ox + oz * oz - r * r
        disc = bq * bq - 4 * a * c
        sq = torch.sqrt(torch.clamp(disc, min=0))
        for tc in ((-bq - sq) / (2 * a), (-bq + sq) / (2 * a)):
            y = o[1] + tc * d[:, 1]
            ok = (disc >= 0) & (tc > 1e-6) & (y >= ground_y) & (y <= ground_y + h)
            t = torch.where(ok, torch.minimum(t, tc), t)
    return t


def scan_project_device(n_scans=64, seed=4, lo=50_000, hi=4_000_000, sigma=0.5, scale=1.0, device="cuda"):
    """scan_project's construction evaluated with torch on a device (seeded
    torch generator; a different random stream than scan_project), for
    full-size projects.  Returns (list of device (n_i, 3) float32 tensors,
    flip points (n_scans, 3) float32 numpy)."""
    import torch
    rng = np.random.Generator(np.random.PCG64(seed))
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), n_scans)) * scale
    sizes = np.maximum(sizes.astype(np.int64), 16)
    scans, flips = [], []
    for i in range(n_scans):
        while True:
            pose = np.array([rng.uniform(-800, 1450), GROUND_Y + 1.5, rng.uniform(20, 790)])
            inside = any((b[0] <= pose[0] <= b[1]) and (b[4] <= pose[2] <= b[5]) for b in BOXES)
            inside |= any((pose[0] - c[0]) ** 2 + (pose[2] - c[1]) ** 2 <= c[2] ** 2 for c in CYLINDERS)
            if not inside:
                break
        m = int(sizes[i])
        o = torch.tensor(pose, device=device, dtype=torch.float32)
        parts, have = [], 0
        while have < m:
            k = max(2 * (m - have), 50_000)
            d = torch.randn((k, 3), generator=gen, device=device)
            d = d / d.norm(dim=1, keepdim=True)
            t = _raycast_torch(o, d, BOXES, CYLINDERS, GROUND_Y)
            ok = torch.isfinite(t) & (t < 3000)
            noise = torch.randn((int(ok.sum()),), generator=gen, device=device) * sigma
            p = o + d[ok] * (t[ok] + noise)[:, None]
            parts.append(p)
            have += p.shape[0]
        scans.append(torch.cat(parts)[:m].contiguous())
        flips.append(pose.astype(np.float32))
    return scans, np.array(flips, np.float32)
