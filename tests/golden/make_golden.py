"""Writes the frozen oracle outputs and the reference tables used by the tests.

  tests/golden/ref_tables.json   the lvr2 marching-cubes / grid tables, printed
                                 by oracle/_ref/ref_tables, which is compiled
                                 from the lvr2 headers by `make -C oracle ref`
                                 (run here, where the lvr2 tree is present).
  tests/golden/oracle_small.npz  oracle results on small seeded clouds: kNN
                                 rows, normals (nem 0/1/2/3, adaptive k), the
                                 interpolation, signed distances, the grid and
                                 the marching-cubes mesh.

The lvr2 reference ships no tests or golden vectors for this path and its CPU
code cannot be compiled here (Eigen, Boost and FLANN are absent), so these
files freeze the CPU restatement; the tables are the only values taken from
the reference itself.

Usage: python tests/golden/make_golden.py
"""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from lvr2_gb300 import synthetic  # noqa: E402
from oracle import oracle as O  # noqa: E402


def clouds():
    rng = np.random.Generator(np.random.PCG64(11))
    v = rng.normal(size=(3000, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    sphere = (0.5 + 0.3 * v + rng.normal(scale=2e-3, size=v.shape)).astype(np.float32)
    scan, _ = synthetic.scan_scene(20_000, seed=7)
    g = np.stack(np.meshgrid(np.arange(12), np.arange(12), np.arange(3), indexing="ij"), -1).reshape(-1, 3)
    lattice = (g * 0.5).astype(np.float32)  # exact ties
    return {"sphere": sphere, "scan": scan, "lattice": lattice}


def main():
    subprocess.run(["make", "-C", str(ROOT / "oracle"), "ref"], check=True, capture_output=True)
    tables = O.reference_tables()
    (HERE / "ref_tables.json").write_text(json.dumps(tables, separators=(",", ":")) + "\n")
    O.build()
    out = {}
    for name, pts in clouds().items():
        s = O.OracleSurface(pts, threads=1)
        q = pts[::7]
        idx, dist, cnt = s.knn(q, 8)
        out[name + "/points"] = pts
        out[name + "/knn_idx"] = idx
        out[name + "/knn_dist"] = dist
        flip = np.array([0.5, 0.5, 0.5], np.float32) if name == "sphere" else np.zeros(3, np.float32)
        for nem in (0, 1, 2, 3):
            n, k = s.normals(5, nem=nem, adaptive=True, flip=flip, with_k=True)
            out["%s/normals_nem%d" % (name, nem)] = n
            out["%s/kused_nem%d" % (name, nem)] = k
        raw = out[name + "/normals_nem3"]
        inter = s.interpolate(raw, 6)
        out[name + "/interp"] = inter
        lo, hi, _ = s.bbox()
        vs = float(np.max(hi - lo) / 12.0)
        out[name + "/voxelsize"] = np.float32(vs)
        qd = q + np.float32(0.1 * vs)
        proj, eucl = s.distance(inter, 4, qd)
        out[name + "/dist_q"] = qd
        out[name + "/dist_proj"] = proj
        out[name + "/dist_eucl"] = eucl
        for dec in ("MC", "PMC"):
            r = s.reconstruct(inter, voxelsize=vs, kd=4, decomposition=dec)
            for key in ("cells_all", "cells_valid", "qp_lattice", "qp_pos", "qp_dist", "qp_invalid", "vkeys",
                        "vpos", "faces"):
                out["%s/%s/%s" % (name, dec, key)] = r[key]
    np.savez_compressed(HERE / "oracle_small.npz", **out)
    print("wrote", HERE / "oracle_small.npz", len(out), "arrays")


if __name__ == "__main__":
    main()
