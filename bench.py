#!/usr/bin/env python
"""Reconstruction benchmark: 10M-point cloud, normals + signed distance + PMC.

Workload (the lvr2 plain GPU configuration at scale): 10,000,000 float32
points uniform on the surfaces of 200 random spheres (r in [0.02, 0.2]) and
100 tori in the unit cube, noise sigma 1e-3 (seeded, lvr2_gb300.synthetic);
kn = ki = kd = 20, PCA normals (nem 3) with lvr2's adaptive k (2kn .. 32kn),
flip point = bounding-box centroid, voxel size 0.005, PMC decomposition.

One step = the whole hot path on the resident cloud: LBVH build, normal
estimation, normal interpolation, grid build, signed distance at every grid
vertex, culling and marching cubes.  `value` = points / step time (every point
gets its normal and the surface is extracted); the per-stage rates (normals/s,
SDF evals/s, MC cells/s) are reported beside it.  `e2e` runs the same steps
through the C ABI with host buffers (points in, normals and mesh out).

--impl reference times the reference algorithm on the host cores: the CPU
restatement in oracle/ (kd-tree, AdaptiveKSearchSurface, PointsetGrid,
FastReconstruction), on a spatial crop of the same cloud (same density).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "normals/s, SDF evals/s @10M pts; plain vs batched/adjoint form, ≤0.5° error"
KN = KI = KD = 20
VOXELSIZE = 0.005
NEM = 3
PLANAR_KC = 5  # FastReconstruction::getMesh runs optimizePlanarFaces(mesh, 5) for PMC
CPU_SAMPLE_FRACTION = 0.02
# DRAM bytes (read + write) per unit of the two kNN kernels, from one ncu
# capture of the 2M-point spheres-and-tori case; the normal kernel's traffic
# is per-point I/O (the neighbour gathers hit L2), so it scales with the points.
NCU_DRAM_BYTES_PER_NORMAL = (46.772224e6 + 155.092224e6) / 2e6
NCU_DRAM_BYTES_PER_SDF_VERTEX = (150.843648e6 + 28.620544e6) / 4415248


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--points", type=int, default=10_000_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--bucket", type=int, default=32, help="LBVH bucket size (tuning)")
    ap.add_argument("--seed-radius", type=int, default=1, help="seed buckets on each side (tuning)")
    ap.add_argument("--no-batched", action="store_true", help="skip the scan-project (batched) measurement")
    ap.add_argument("--batched-scale", type=float, default=1.0, help="scale of the 64-scan project")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the terrain adjoint measurement")
    ap.add_argument("--adjoint-scale", type=float, default=1.0, help="scale of the 30M-point terrain")
    ap.add_argument("--no-precision", action="store_true", help="skip the folded-sheets precision measurement")
    ap.add_argument("--precision-scale", type=float, default=1.0, help="scale of the 20M-point folded sheets")
    ap.add_argument("--no-scan-scene", action="store_true", help="skip the 289,252-point scan-scene record")
    ap.add_argument("--no-full-form", action="store_true", help="skip the full-form (graph + Newton) record")
    ap.add_argument("--no-reference-gpu", action="store_true", help="skip lvr2's own LBVH on this GPU")
    return ap.parse_args()


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload(n):
    from lvr2_gb300 import synthetic
    return synthetic.spheres_tori(n, seed=2)


def config(n, extra=None):
    c = {"workload": "spheres_tori_%dM" % (n // 1_000_000) if n >= 1_000_000 else "spheres_tori_%d" % n,
         "points": n, "kn": KN, "ki": KI, "kd": KD, "nem": NEM, "adaptive_k": True, "voxelsize": VOXELSIZE,
         "decomposition": "PMC", "planar_post_pass_kc": PLANAR_KC, "flip_point": "bbox centroid",
         "l2": "inputs and per-step working set (>1 GB) larger than L2"}
    if extra:
        c.update(extra)
    return c


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def normal_bytes(stats, kn):
    """Algorithmic bytes of the normal stage (gather model: 16 B per point record
    read, per neighbour per search round, + 16 B query + 12 B normal written)."""
    total = 0
    for r in range(5):
        searched = sum(16 + 16 * kn * (2 ** (j + 1)) for j in range(r + 1))
        total += int(stats[r]) * (searched + 12)
    return total


def sdf_bytes(n_vertices, kd):
    return n_vertices * (12 + 32 * kd + 4 + 1)


def batched_measurement(args, steps):
    """Scan project: 64 scans, log-uniform 50k-4M points (~60M), per-scan flip
    point at the scanner, kn = ki = 10, PCA.  The batched form (one segmented
    LBVH, one launch per search round, CUDA graph replay, autotuned) against
    the plain form (one surface per scan, one after the other) on the same GPU."""
    import torch

    import lvr2_gb300
    from lvr2_gb300 import synthetic
    scans, flips = synthetic.scan_project_device(64, seed=4, scale=args.batched_scale, device="cuda")
    n = sum(int(s.shape[0]) for s in scans)
    # plain: a surface per scan
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for rep in range(2):
        torch.cuda.synchronize()
        ev0.record()
        for sc, f in zip(scans, flips):
            with lvr2_gb300.Surface(sc, kn=10, ki=10, nem=3, flip_point=f) as s:
                s.calculate_normals()
        ev1.record()
        torch.cuda.synchronize()
    plain_ms = ev0.elapsed_time(ev1)
    with lvr2_gb300.Batch(scans, flips, kn=10, ki=10, nem=3) as b:
        bucket, radius = b.autotune()
        tuning = b.tuning()
        b.calculate_normals(use_graph=True)
        times = []
        for _ in range(max(steps, 1)):
            b.calculate_normals(use_graph=True)
            times.append(float(b.stats()[1][3]))
        counters, _ = b.stats()
        b.calculate_normals(use_graph=False)
        _, stage = b.stats()
        round_ms = b.round_times()
    batched_ms = float(np.mean(times))
    return {"workload": "scan_project_64", "scans": 64, "points": n, "kn": 10, "ki": 10, "nem": 3,
            "plain_ms": plain_ms, "plain_normals_per_s": n / (plain_ms / 1000.0),
            "batched_ms": batched_ms, "batched_normals_per_s": n / (batched_ms / 1000.0),
            "speedup_vs_plain": plain_ms / batched_ms,
            "autotuned": dict(zip(["bucket", "seed_radius", "wide_tile", "wide_buffer_slack"], tuning)),
            "batched_stage_ms": {"tree": float(stage[0]), "normals": float(stage[1]), "interpolation": float(stage[2])},
            "fitted_per_round": [int(x) for x in counters[:5]],
            "normals_ms_per_round": [float(x) for x in round_ms],
            "k_per_round": [10 * 2 ** (r + 1) for r in range(5)], "graph": True,
            "note": "round 1 searches every point with k = 20 in both forms; the batched form saves the "
                    "per-scan launches, trees and uncollapsed later rounds, not that search, which bounds "
                    "speedup_vs_plain at plain_ms / (round-1 ms + tree ms)"}


def adjoint_measurement(args, steps):
    """Adjoint form on terrain: 30M points on a value-noise heightfield
    (sigma 0.2), kd = 10, voxel size 0.5.  The grid's vertices go through the
    signed distance (forward, the reconstruct stage) and its adjoint
    (forward + gradients w.r.t. queries, points and normals through
    lvrgb_distance_adjoint, device buffers); the mesh vertices through three
    Newton steps onto the zero level (lvrgb_project_to_surface)."""
    import torch

    import lvr2_gb300
    from lvr2_gb300 import synthetic
    n = int(30_000_000 * args.adjoint_scale)
    pts = synthetic.terrain_device(n, seed=5)
    out = {"workload": "terrain_30M" if args.adjoint_scale == 1.0 else "terrain_%d" % n, "points": n, "kd": 10,
           "voxelsize": 0.5, "kn": 10, "ki": 10, "nem": 3}
    with lvr2_gb300.Surface(pts, kn=10, ki=10, kd=10, nem=3, flip_point=(500.0, 500.0, 500.0)) as s:
        s.calculate_normals()
        info = s.reconstruct(voxelsize=0.5, decomposition="PMC")
        sdf_ms = float(s.timings()[4])
        _, pos, _, _ = s.grid()
        v, _, _ = s.mesh(with_edges=False)
        q = torch.from_numpy(pos).cuda()
        vt = torch.from_numpy(v).cuda()
        nq = q.shape[0]
        gd = torch.ones(nq, device="cuda", dtype=torch.float32)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

        def timed(fn):
            fn()
            torch.cuda.synchronize()
            ev[0].record()
            for _ in range(max(steps, 1)):
                fn()
            ev[1].record()
            torch.cuda.synchronize()
            return ev[0].elapsed_time(ev[1]) / max(steps, 1)

        fwd_ms = timed(lambda: s.distance_adjoint(q, None, None, want_points=False, want_normals=False))
        adj_ms = timed(lambda: s.distance_adjoint(q, gd, None, want_points=True, want_normals=True))
        proj_ms = timed(lambda: s.project_to_surface(vt, steps=3))
    out.update({"grid_vertices": int(nq), "mesh_vertices": int(v.shape[0]), "cells_valid": int(info.cells_valid),
                "sdf_stage_ms": sdf_ms, "sdf_evals_per_s_stage": nq / (sdf_ms / 1000.0),
                "forward_api_ms": fwd_ms, "forward_evals_per_s": nq / (fwd_ms / 1000.0),
                "adjoint_api_ms": adj_ms, "adjoint_evals_per_s": nq / (adj_ms / 1000.0),
                "adjoint_over_forward": adj_ms / fwd_ms,
                "projection_3_steps_ms": proj_ms, "projected_vertices_per_s": v.shape[0] / (proj_ms / 1000.0),
                "note": "API timings include the Morton sort of the queries; device buffers"})
    return out


def precision_measurement(args, steps):
    """Precision stress: folded thin sheets offset by +1e5, 20M points,
    sigma_normal 1e-4, kn = 50, nem 3 (FP32 with FP64 fallback below a
    relative eigengap of 1e-3): normals/s and the angle to float64 PCA of the
    same neighbourhoods on a 2000-point sample (p50, p99.9)."""
    import torch

    import lvr2_gb300
    from lvr2_gb300 import synthetic
    n = int(20_000_000 * args.precision_scale)
    pts, vs = synthetic.folded_sheets(n, seed=3)
    flip = (pts.astype(np.float64).mean(0) + np.array([0.0, 0.0, 1e3])).astype(np.float32)
    d = torch.from_numpy(pts).cuda()
    with lvr2_gb300.Surface(d, kn=50, ki=0, nem=3, flip_point=flip) as s:
        s.calculate_normals()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for _ in range(max(steps, 1)):
            s.calculate_normals()
        ev[1].record()
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / max(steps, 1)
        gn, gk = s.raw_normals()
        stats = s.normal_stats()
        rng = np.random.Generator(np.random.PCG64(4))
        sel = rng.choice(n, 2000, replace=False)
        idx, nbr = [], []
        for k in np.unique(gk[sel]):
            m = sel[gk[sel] == k]
            i, _, _ = s.knn(pts[m], int(k))
            idx.append(m)
            nbr.extend(i)
    idx = np.concatenate(idx)
    P = pts.astype(np.float64)
    ref = np.empty((len(idx), 3))
    for r, (qi, nb) in enumerate(zip(idx, nbr)):
        S = np.concatenate([P[qi:qi + 1], P[nb[nb != 0xFFFFFFFF].astype(np.int64)]])
        w, V = np.linalg.eigh(np.cov(S.T, bias=True))
        ref[r] = V[:, 0] if np.dot(V[:, 0], flip - P[qi]) >= 0 else -V[:, 0]
    a = gn[idx].astype(np.float64)
    a /= np.linalg.norm(a, axis=1, keepdims=True)
    ang = np.degrees(np.arccos(np.clip(np.sum(a * ref, 1), -1, 1)))
    return {"workload": "folded_sheets_offset_1e5_%dM" % round(n / 1e6), "points": n, "kn": 50, "nem": 3,
            "voxelsize": vs, "normals_ms": ms, "normals_per_s": n / (ms / 1000.0),
            "fitted_per_round": [int(x) for x in stats[:5]], "fp64_eigensolves": int(stats[5]),
            "angle_deg_vs_fp64": {"p50": float(np.percentile(ang, 50)), "p99.9": float(np.percentile(ang, 99.9)),
                                  "max": float(ang.max()), "sample": len(idx)},
            "fallback_stress": fallback_stress_measurement()}


def fallback_stress_measurement(n_side=60, jitter=2e-3, kn=10):
    """Where the FP64 eigen fallback runs by default: a cubic lattice (216,000
    points, spacing 1) with 2e-3 jitter, so every neighbourhood is nearly
    isotropic.  Count of FP64 solves under the default relative-eigengap
    threshold 1e-3, and the angle of every normal to float64 PCA of its own
    neighbourhood where that eigenvector is defined (relative gap > 1e-5)."""
    import lvr2_gb300
    rng = np.random.Generator(np.random.PCG64(17))
    g = np.stack(np.meshgrid(*[np.arange(n_side)] * 3, indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
    P = (g + rng.normal(scale=jitter, size=g.shape)).astype(np.float32)
    flip = (P.min(0) + P.max(0)) / 2
    with lvr2_gb300.Surface(P, kn=kn, ki=0, nem=3, flip_point=flip) as s:
        s.calculate_normals()
        gn, gk = s.raw_normals()
        stats = s.normal_stats()
        angs, gaps = [], []
        for k in np.unique(gk):
            m = np.nonzero(gk == k)[0]
            rows, _, _ = s.knn(P[m], int(k))
            S = np.concatenate([P[m][:, None, :], P[rows.astype(np.int64)]], axis=1).astype(np.float64)
            S -= S.mean(axis=1, keepdims=True)
            w, V = np.linalg.eigh(np.einsum("mki,mkj->mij", S, S) / S.shape[1])
            a = gn[m].astype(np.float64)
            a /= np.linalg.norm(a, axis=1, keepdims=True)
            angs.append(np.degrees(np.arccos(np.clip(np.abs(np.sum(a * V[:, :, 0], 1)), 0, 1))))
            gaps.append((w[:, 1] - w[:, 0]) / np.maximum(w[:, 2], 1e-300))
    ang, gap = np.concatenate(angs), np.concatenate(gaps)
    ok = gap > 1e-5
    return {"workload": "jittered_lattice_216k", "points": len(P), "kn": kn, "gap_threshold": 1e-3,
            "fp64_eigensolves": int(stats[5]),
            "angle_deg_vs_fp64_where_defined": {"p50": float(np.percentile(ang[ok], 50)),
                                                "p99.9": float(np.percentile(ang[ok], 99.9)),
                                                "max": float(ang[ok].max()), "defined": int(ok.sum())}}


README_SCAN_MS = {"normals_with_interpolation": 161, "grid_signed_distance_culling": 125, "pmc_with_planar_pass": 47}


def scan_scene_measurement(args, steps):
    """The plain CPU-runnable reconstruction at its full size, both arms on
    the same points: 289,252 points of the seeded scan-shaped scene, kn = ki
    = 10, kd = 5, voxel size 10, PMC with optimizePlanarFaces(5), flip point
    (0, 0, 0), nem 0 (lvr2_reconstruct's default plane fit).  GPU stages
    (device events) beside the oracle's reference-faithful CPU run on all host
    cores and beside the stage times of lvr2's README run (16 threads, its
    scan.pts, which is not in the lvr2 tree)."""
    import torch

    import lvr2_gb300
    from lvr2_gb300 import synthetic
    from oracle import oracle as O
    P, _ = synthetic.scan_scene()
    n = len(P)
    d = torch.from_numpy(P).cuda()
    flip = np.zeros(3, np.float32)
    with lvr2_gb300.Surface(d, kn=10, ki=10, kd=5, nem=0, flip_point=flip) as s:
        def step():
            s.set_points(d)
            s.calculate_normals()
            info = s.reconstruct(voxelsize=10.0, decomposition="PMC")
            return info, s.optimize_planar_faces(PLANAR_KC)

        for _ in range(3):
            step()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        stage = np.zeros(8)
        ev[0].record()
        for _ in range(max(steps, 1)):
            info, moved = step()
            stage += s.timings()
        ev[1].record()
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / max(steps, 1)
        stage /= max(steps, 1)
    O.build()
    best = None
    for _ in range(2):
        t = {}
        t0 = time.perf_counter()
        o = O.OracleSurface(P, leaf_size=20)
        t["tree"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        nr = o.normals(10, nem=0, adaptive=True, flip=flip, canonical=False)
        t["normals"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        nr = o.interpolate(nr, 10, canonical=False)
        t["interpolation"] = time.perf_counter() - t0
        r = o.reconstruct(nr, voxelsize=10.0, kd=5, decomposition="PMC", canonical=False, planar_kc=PLANAR_KC)
        t["grid_signed_distance_culling_mc"] = r["seconds_reconstruct"]
        t["planar_pass"] = r["seconds_planar"]
        if best is None or sum(t.values()) < sum(best.values()):
            best = t
        del o
    cpu_ms = 1000 * sum(best.values())
    gs = {"lbvh_build": stage[0], "normals": stage[1], "interpolation": stage[2], "grid_build": stage[3],
          "signed_distance": stage[4], "culling": stage[5], "marching_cubes": stage[6], "planar_pass": stage[7]}
    return {"workload": "scan_scene_289k", "points": n, "same_config": True, "kn": 10, "ki": 10, "kd": 5,
            "voxelsize": 10.0, "nem": 0, "decomposition": "PMC", "planar_post_pass_kc": PLANAR_KC,
            "flip_point": [0.0, 0.0, 0.0],
            "gpu_ms_per_step": ms, "gpu_normals_per_s": n / (ms / 1000.0),
            "gpu_stages_ms": {k: float(v) for k, v in gs.items()},
            "cpu_ms_per_step": cpu_ms, "cpu_normals_per_s": n / (cpu_ms / 1000.0), "cpu_cores": os.cpu_count(),
            "cpu_kind": "port", "cpu_stages_ms": {k: 1000 * v for k, v in best.items()},
            "gpu_over_cpu": cpu_ms / ms,
            "readme_stages_ms": dict(README_SCAN_MS, note="lvr2 README.md:113-124, 16 threads, CPU unstated, "
                                                          "its own scan.pts (289,252 points), not this scene"),
            "counts": {"cells_valid": int(info.cells_valid), "vertices": int(info.vertices),
                       "faces": int(info.faces), "planar_moved": int(moved),
                       "readme_counts": {"cells": 30040, "vertices": 20157, "faces": 36416}}}


def full_form_measurement(d_pts, flip, plain_ms, steps):
    """The spec form on the same 10M-point cloud as the plain step: the
    normals through the scan-project path (one segmented LBVH, CUDA graph
    replay, FP32 PCA with the FP64 eigen fallback), then grid, signed
    distance, culling, PMC and its planar pass, then three Newton steps of
    every mesh vertex onto the zero level with analytic normals.  Device
    buffers throughout; timed with CUDA events."""
    import ctypes

    import torch

    import lvr2_gb300
    from lvr2_gb300 import _lib
    L = _lib.load()
    n = int(d_pts.shape[0])
    nrm = torch.empty((n, 3), dtype=torch.float32, device=d_pts.device)
    with lvr2_gb300.Batch([d_pts], [flip], kn=KN, ki=KI, nem=NEM) as b, \
            lvr2_gb300.Surface(d_pts, kn=KN, ki=KI, kd=KD, nem=NEM, flip_point=flip) as s:
        def step():
            b.calculate_normals(use_graph=True)
            _lib.check(L.lvrgb_batch_get_normals(b._h, ctypes.c_void_p(nrm.data_ptr()), 1, None))
            s.set_normals(nrm)
            info = s.reconstruct(voxelsize=VOXELSIZE, decomposition="PMC")
            s.optimize_planar_faces(PLANAR_KC)
            v = torch.empty((int(info.vertices), 3), dtype=torch.float32, device=d_pts.device)
            f = torch.empty((int(info.faces), 3), dtype=torch.int32, device=d_pts.device)
            _lib.check(L.lvrgb_get_mesh(s._h, ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(f.data_ptr()), None,
                                        1, None))
            pos, vn = s.project_to_surface(v, steps=3)
            return info

        for _ in range(3):
            step()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for _ in range(max(steps, 1)):
            info = step()
        ev[1].record()
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / max(steps, 1)
        counters, _ = b.stats()
    return {"workload": "spheres_tori_10M", "points": n, "ms_per_step": ms, "normals_per_s": n / (ms / 1000.0),
            "plain_ms_per_step": plain_ms, "full_over_plain_time": ms / plain_ms,
            "mesh_vertices_projected": int(info.vertices), "newton_steps": 3,
            "fp64_eigensolves": int(counters[5]), "graph": True,
            "note": "does the plain step's work plus the Newton projection, with the same kernels; the speed-up "
                    "against a plain GPU implementation is reference_gpu (lvr2's own LBVH on this GPU)"}


def ours_lbvh_calls(P, k=20, reps=3):
    """This library on the calls lvr2's LBVH comparator makes: tree build,
    kNN of every point (lvrgb_knn) and the comparator's normals (nem 4, one
    search with k = kn, flip point (1e6, 1e6, 1e6)).  Wall-clock per call
    with host arrays in and out (as LBVHIndex::kSearch / knn_normals take
    them), and device time with the points resident."""
    import torch

    import lvr2_gb300
    n = len(P)
    d = torch.from_numpy(P).cuda()
    out = {}
    with lvr2_gb300.Surface(d, kn=k, ki=0, kd=5, nem=4, adaptive=False, flip_point=(1e6, 1e6, 1e6)) as s:
        for _ in range(2):
            s.set_points(d)
            s.knn(d, k)
            s.calculate_normals()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        torch.cuda.synchronize()
        ev[0].record()
        for _ in range(reps):
            s.set_points(d)
        ev[1].record()
        for _ in range(reps):
            s.knn(d, k)
        ev[2].record()
        for _ in range(reps):
            s.calculate_normals()
        ev[3].record()
        torch.cuda.synchronize()
        out["device_build_ms"] = ev[0].elapsed_time(ev[1]) / reps
        out["device_knn_ms"] = ev[1].elapsed_time(ev[2]) / reps
        out["device_normals_ms"] = ev[2].elapsed_time(ev[3]) / reps
        # host arrays in and out, as the comparator's calls take them
        t0 = time.perf_counter()
        s.set_points(P)
        out["host_build_ms"] = 1000 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        s.knn(P, k)
        out["host_knn_ms"] = 1000 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        s.calculate_normals()
        s.normals()
        out["host_normals_ms"] = 1000 * (time.perf_counter() - t0)
    return out


def reference_gpu_measurement(sizes=(2_000_000, 10_000_000)):
    """lvr2's own CUDA LBVH (LBVHIndex::build, kSearch, knn_normals; K = 20;
    leaf size 1), unmodified, built from the lvr2 sources by oracle/Makefile
    when they are present: wall-clock times per call, NVRTC compilation
    included; beside it this library on the same calls (ours_lbvh_calls)."""
    exe = ROOT / "oracle" / "_ref" / "ref_lbvh"
    if not exe.exists():
        return {"unavailable": "oracle/_ref/ref_lbvh not built (needs the lvr2 LBVH sources copied by "
                               "`make -C oracle ref-lbvh-src`)"}
    import tempfile

    from lvr2_gb300 import synthetic
    out = {"kind": "lvr2 LBVHIndex (src/liblvr2/reconstruction/cuda/LBVHIndex.cu), sm_103a, NVRTC kernels",
           "K": 20, "runs": []}
    for n in sizes:
        P = synthetic.spheres_tori(int(n), seed=2)
        ours = ours_lbvh_calls(P)
        with tempfile.TemporaryDirectory() as tmp:
            pf = Path(tmp) / "pts.bin"
            with open(pf, "wb") as f:
                f.write(np.int64(len(P)).tobytes())
                f.write(np.ascontiguousarray(P, np.float32).tobytes())
            try:
                r = subprocess.run([str(exe), "run", str(pf), "-", "20"], capture_output=True, text=True,
                                   timeout=600)
            except subprocess.TimeoutExpired:
                out["runs"].append({"points": int(n), "unavailable": "timed out", "ours": ours})
                continue
        if r.returncode != 0:
            out["runs"].append({"points": int(n), "unavailable": "exit %d" % r.returncode, "ours": ours})
            continue
        ref = json.loads(r.stdout.strip().splitlines()[-1])
        ref["ours"] = ours
        ref["knn_speedup_host_calls"] = ref["ksearch_ms"] / ours["host_knn_ms"]
        ref["normals_speedup_host_calls"] = (ref["normals_build_ms"] + ref["knn_normals_ms"]) / (
            ours["host_build_ms"] + ours["host_normals_ms"])
        out["runs"].append(ref)
    return out


def cpu_reference_step(points, threads=0, canonical=False):
    """One pass of the reference algorithm on the host (oracle/)."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    s = O.OracleSurface(points, leaf_size=20, threads=threads)
    lo, hi, c = s.bbox()
    n = s.normals(KN, nem=NEM, adaptive=True, flip=c, canonical=canonical)
    n = s.interpolate(n, KI, canonical=canonical)
    r = s.reconstruct(n, voxelsize=VOXELSIZE, kd=KD, decomposition="PMC", canonical=canonical,
                      planar_kc=PLANAR_KC)
    dt = time.perf_counter() - t0
    return dt, r


def cpu_sample(points):
    from lvr2_gb300 import synthetic
    return np.ascontiguousarray(synthetic.crop(points, CPU_SAMPLE_FRACTION, center=np.array([0.5, 0.5, 0.5])))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    pts = workload(args.points)
    sample = cpu_sample(pts)
    for _ in range(args.warmup):
        cpu_reference_step(sample)
    times = []
    for _ in range(args.steps):
        dt, r = cpu_reference_step(sample)
        times.append(dt)
    value = len(sample) * len(times) / sum(times)
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "normals/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": config(args.points, {"sample_points": len(sample)}),
        "cpu_baseline": {"value": value, "unit": "normals/s", "cores": cores, "kind": "port",
                         "sample": "spatial crop of the %d-point cloud (%d points, same density); full pipeline: "
                                   "kd-tree (leaf 20), adaptive-k PCA normals, ki interpolation, grid + "
                                   "signed distance + culling, PMC marching cubes + optimizePlanarFaces(5)"
                                   % (len(pts), len(sample))},
        "e2e": {"value": value, "unit": "normals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_gpu(args):
    import torch

    import lvr2_gb300
    from lvr2_gb300 import build as B
    from lvr2_gb300.surface import kernel_launches

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    B.build()
    pts = workload(args.points)
    n = len(pts)
    d_pts = torch.from_numpy(pts).to(f"cuda:{local}")
    # the surface works on a stream of its own, as a caller of the C ABI would
    # give it (the legacy default stream serialises with every other stream)
    work = torch.cuda.Stream(device=local)
    torch.cuda.synchronize()  # d_pts was written on the default stream
    s = lvr2_gb300.Surface(d_pts, kn=KN, ki=KI, kd=KD, nem=NEM, adaptive=True, flip_point=None, device=local,
                           bucket=args.bucket, seed_radius=args.seed_radius, stream=work)

    def step():
        s.set_points(d_pts)
        s.calculate_normals()
        info = s.reconstruct(voxelsize=VOXELSIZE, decomposition="PMC")
        s.optimize_planar_faces(PLANAR_KC)
        return info

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    l0 = kernel_launches()
    stage = np.zeros(8)
    stats_acc = np.zeros(16)
    sdf_acc = np.zeros(5)
    infos = []
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(work)
        for _ in range(args.steps):
            info = step()
            stage += s.timings()
            stats_acc += s.normal_stats()
            sdf_acc += s.distance_stats()[:5].astype(np.float64)
            infos.append((info.grid_vertices, info.cells_valid, info.faces, info.vertices))
        t_end.record(work)
        torch.cuda.synchronize()
    launches = (kernel_launches() - l0) // max(args.steps, 1)
    ms = t_start.elapsed_time(t_end) / args.steps
    if dist:
        t = torch.tensor([ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    stage /= args.steps
    stats = stats_acc / args.steps
    sdf_stats = sdf_acc / args.steps
    nq, ncv, nf, nv = infos[-1]
    value = world * n / (ms / 1000.0)

    # ---- end to end through the C ABI with host buffers -----------------------
    e2e = None
    if not args.no_e2e:
        # host buffers in pinned memory, as a caller streaming clouds would use
        h_pts = torch.from_numpy(pts).pin_memory()
        pts_h = h_pts.numpy()
        h_norm = torch.empty((n, 3), dtype=torch.float32).pin_memory().numpy()
        s.set_points(pts_h)
        s.calculate_normals()
        info = s.reconstruct(voxelsize=VOXELSIZE, decomposition="PMC")
        s.optimize_planar_faces(PLANAR_KC)
        cap_v, cap_f = 2 * int(info.vertices) + 1024, 2 * int(info.faces) + 1024
        h_v = torch.empty((cap_v, 3), dtype=torch.float32).pin_memory().numpy()
        h_f = torch.empty((cap_f, 3), dtype=torch.int32).pin_memory().numpy().view(np.uint32)
        # the normals are read back on a second stream while the grid, the
        # distances and the mesh are computed
        copy_stream = torch.cuda.Stream()
        for _ in range(1):
            s.set_points(pts_h)
            s.calculate_normals()
            s.normals_async(h_norm, copy_stream)
            s.reconstruct(voxelsize=VOXELSIZE, decomposition="PMC")
            s.optimize_planar_faces(PLANAR_KC)
            s.mesh(with_edges=False, out_vertices=h_v, out_faces=h_f)
            copy_stream.synchronize()
        torch.cuda.synchronize()
        # host-timed, so at least 20 steps (about a second) against host jitter
        e2e_steps = max(args.steps, 20)
        t0 = time.perf_counter()
        d2h = 0
        for _ in range(e2e_steps):
            s.set_points(pts_h)
            s.calculate_normals()
            out_n = s.normals_async(h_norm, copy_stream)
            info = s.reconstruct(voxelsize=VOXELSIZE, decomposition="PMC")
            s.optimize_planar_faces(PLANAR_KC)
            v, f, _ = s.mesh(with_edges=False, out_vertices=h_v, out_faces=h_f)
            copy_stream.synchronize()
            d2h = out_n.nbytes + v.nbytes + f.nbytes
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        e2e = {"value": world * n / e2e_s, "unit": "normals/s", "h2d_bytes_per_step": int(pts_h.nbytes),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": 1000 * e2e_s, "host_buffers": "pinned",
               "steps": e2e_steps}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    peak, peak_kind = peaks()
    nb = normal_bytes(stats, KN)
    sb = sdf_bytes(nq, KD)
    normals_ms, sdf_ms = float(stage[1]), float(stage[4])
    if normals_ms >= sdf_ms:
        dom = {"kernel": "normals_kernel<3> (fused kNN + PCA + flip, all adaptive rounds)",
               "bytes": nb, "ms": normals_ms, "traffic": NCU_DRAM_BYTES_PER_NORMAL * n}
    else:
        dom = {"kernel": "sdf_kernel (kd-nearest signed distance)", "bytes": sb, "ms": sdf_ms,
               "traffic": NCU_DRAM_BYTES_PER_SDF_VERTEX * nq}
    achieved = dom["bytes"] / (dom["ms"] / 1000.0) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "normals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config(n, {"parallelism": "replicas" if world > 1 else "single", "bucket": args.bucket,
                             "seed_radius": args.seed_radius}),
        "stages_ms": {"lbvh_build": float(stage[0]), "normals": normals_ms, "interpolation": float(stage[2]),
                      "grid_build": float(stage[3]), "signed_distance": sdf_ms, "culling": float(stage[5]),
                      "marching_cubes": float(stage[6]), "planar_post_pass": float(stage[7])},
        "rates": {"normals_per_s_stage": n / ((stage[0] + stage[1] + stage[2]) / 1000.0),
                  "sdf_evals_per_s_stage": nq / (sdf_ms / 1000.0),
                  "mc_cells_per_s_stage": ncv / (stage[6] / 1000.0) if stage[6] > 0 else None,
                  "pmc_cells_per_s_stage": ncv / ((stage[6] + stage[7]) / 1000.0) if stage[6] > 0 else None},
        "counts": {"grid_vertices": int(nq), "cells_valid": int(ncv), "faces": int(nf), "vertices": int(nv),
                   "fitted_per_round": [int(x) for x in stats[:5]], "fp64_eigensolves": int(stats[5]),
                   "normals_buckets_per_warp": float(stats[8]) / max(1.0, n / 32.0),
                   "normals_nodes_per_warp": float(stats[9]) / max(1.0, n / 32.0),
                   "normals_heap_pushes_per_query": float(stats[10]) / max(1.0, n),
                   "normals_chunks_per_warp": float(stats[11]) / max(1.0, n / 32.0),
                   "normals_push_rounds_per_warp": float(stats[12]) / max(1.0, n / 32.0),
                   "sdf_buckets_per_warp": float(sdf_stats[0]) / max(1.0, nq / 32.0),
                   "sdf_nodes_per_warp": float(sdf_stats[1]) / max(1.0, nq / 32.0),
                   "sdf_heap_pushes_per_query": float(sdf_stats[2]) / max(1.0, nq),
                   "sdf_chunks_per_warp": float(sdf_stats[3]) / max(1.0, nq / 32.0),
                   "sdf_push_rounds_per_warp": float(sdf_stats[4]) / max(1.0, nq / 32.0)},
        "roofline": {"bound": "hbm", "kernel": dom["kernel"], "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "algorithmic_bytes": int(dom["bytes"]),
                     "traffic": int(dom["traffic"]) if dom["traffic"] else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a 2M-point capture, "
                                       "scaled per point (normals) or per grid vertex (signed distance)"},
        # both kNN stages against the same HBM roofline; ncu shows them issue-bound
        # (57% and 71% issue active), not bandwidth-bound
        "stage_rooflines": [
            {"stage": "normals", "kernel": "normals_kernel", "algorithmic_bytes": int(nb),
             "achieved_gbs": nb / (normals_ms / 1000.0) / 1e9, "frac": nb / (normals_ms / 1000.0) / 1e9 / peak,
             "traffic": int(NCU_DRAM_BYTES_PER_NORMAL * n)},
            {"stage": "signed_distance", "kernel": "sdf_kernel", "algorithmic_bytes": int(sb),
             "achieved_gbs": sb / (sdf_ms / 1000.0) / 1e9, "frac": sb / (sdf_ms / 1000.0) / 1e9 / peak,
             "traffic": int(NCU_DRAM_BYTES_PER_SDF_VERTEX * nq)},
        ],
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "e2e": e2e,
    }
    if not args.no_full_form:
        _, _, centroid = s.bounding_box()
        line["full_form"] = full_form_measurement(d_pts, centroid, ms, args.steps)
    if not args.no_scan_scene:
        line["scan_scene"] = scan_scene_measurement(args, args.steps)
    if not args.no_batched:
        line["batched"] = batched_measurement(args, args.steps)
    if not args.no_adjoint:
        line["adjoint"] = adjoint_measurement(args, args.steps)
    if not args.no_precision:
        line["precision"] = precision_measurement(args, args.steps)
    if not args.no_reference_gpu:
        line["reference_gpu"] = reference_gpu_measurement()
    if not args.no_cpu_baseline:
        sample = cpu_sample(pts)
        dt, _ = cpu_reference_step(sample)
        line["cpu_baseline"] = {"value": len(sample) / dt, "unit": "normals/s", "cores": os.cpu_count(),
                                "kind": "port",
                                "sample": "spatial crop of the cloud (%d points, same density), one pass of "
                                          "the full CPU pipeline (oracle/ restatement of the reference)"
                                          % len(sample)}
    print(json.dumps(line))
    s.close()
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
