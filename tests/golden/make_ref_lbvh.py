"""Golden vectors and timings from lvr2's own CUDA LBVH, run on a GB300.

lvr2's LBVHIndex (src/liblvr2/reconstruction/cuda/LBVHIndex.cu) is the one
part of the reference's hot path that compiles here: `oracle/Makefile`
copies its sources (`make -C oracle ref-lbvh-src REF=<lvr2 tree>`, where the
lvr2 tree is present) and builds `oracle/_ref/ref_lbvh` from that copy
(`make -C oracle ref-lbvh`, on the GPU machine).  This script runs it.

  python tests/golden/make_ref_lbvh.py golden <out_dir>
      three seeded clouds; for each: LBVHIndex::kSearch (K = 20, leaf size 1,
      as SearchTreeLBVH builds it) on a sample of the points plus random
      queries, and LBVHIndex::knn_normals (K = 20) on every point, also on a
      leaf-size-1 tree (oracle/ref_lbvh.cu says why not CudaKSearchSurface's
      32).  Writes
      <out_dir>/ref_lbvh.npz, which is committed as tests/golden/ref_lbvh.npz
      (points included: the clouds are made with transcendental functions
      whose last bits may differ between machines).
  python tests/golden/make_ref_lbvh.py timing <out_dir> <n> [<n> ...]
      spheres-and-tori clouds of n points: wall-clock times of
      LBVHIndex::build, kSearch (every point as a query) and knn_normals,
      K = 20; one JSON line per size.

The reference's kernels run unmodified; `ref_lbvh` checks each tree it
builds on the host before any query runs on it.
"""
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from lvr2_gb300 import synthetic  # noqa: E402

EXE = ROOT / "oracle" / "_ref" / "ref_lbvh"
K = 20


def write_points(path, p):
    p = np.ascontiguousarray(p, np.float32).reshape(-1, 3)
    with open(path, "wb") as f:
        f.write(np.int64(len(p)).tobytes())
        f.write(p.tobytes())


def run(args, timeout=1800):
    r = subprocess.run([str(EXE)] + [str(a) for a in args], capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("ref_lbvh %s failed (%d):\n%s\n%s" % (args, r.returncode, r.stdout[-2000:], r.stderr[-2000:]))
    # the reference prints the NVRTC log on stdout; the report is the last line
    return json.loads(r.stdout.strip().splitlines()[-1])


def clouds():
    rng = np.random.Generator(np.random.PCG64(21))
    v = rng.normal(size=(12_000, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    sphere = (0.5 + 0.3 * v + rng.normal(scale=1e-3, size=v.shape)).astype(np.float32)
    scan, _ = synthetic.scan_scene(20_000, seed=8)
    st = synthetic.spheres_tori(24_000, seed=9)
    return {"sphere": sphere, "scan": np.ascontiguousarray(scan, np.float32), "spheres_tori": st}


def golden(out_dir):
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    arrays = {}
    report = {}
    for name, P in clouds().items():
        rng = np.random.Generator(np.random.PCG64(len(P)))
        sel = np.sort(rng.choice(len(P), 1200, replace=False)).astype(np.int64)
        lo, hi = P.min(0), P.max(0)
        rq = rng.uniform(lo, hi, size=(200, 3)).astype(np.float32)
        Q = np.concatenate([P[sel], rq])
        tmp = Path(tempfile.mkdtemp())
        pf, qf, pre = tmp / (name + "_pts.bin"), tmp / (name + "_q.bin"), tmp / name
        write_points(pf, P)
        write_points(qf, Q)
        rep = run(["run", pf, pre, K, qf])
        idx = np.fromfile(str(pre) + "_knn_idx.bin", np.uint32).reshape(len(Q), K)
        dist = np.fromfile(str(pre) + "_knn_dist.bin", np.float32).reshape(len(Q), K)
        cnt = np.fromfile(str(pre) + "_knn_cnt.bin", np.uint32)
        nrm = np.fromfile(str(pre) + "_normals.bin", np.float32).reshape(len(P), 3)
        arrays.update({name + "_points": P, name + "_queries": Q, name + "_idx": idx, name + "_dist": dist,
                       name + "_cnt": cnt, name + "_normals": nrm})
        report[name] = rep
        for f in [pf, qf] + [Path(str(pre) + s) for s in ("_knn_idx.bin", "_knn_dist.bin", "_knn_cnt.bin",
                                                          "_normals.bin")]:
            f.unlink()
    np.savez_compressed(out_dir / "ref_lbvh.npz", K=np.int64(K), **arrays)
    print(json.dumps(report))


def timing(out_dir, sizes):
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    jit = run(["jit", K])
    for n in sizes:
        P = synthetic.spheres_tori(int(n), seed=2)
        pf = Path(tempfile.mkdtemp()) / "timing_pts.bin"
        write_points(pf, P)
        rep = run(["run", pf, "-", K])
        rep["jit_ms_both_kernels"] = jit["ms"]
        pf.unlink()
        print(json.dumps(rep), flush=True)


if __name__ == "__main__":
    if len(sys.argv) >= 3 and sys.argv[1] == "golden":
        golden(sys.argv[2])
    elif len(sys.argv) >= 4 and sys.argv[1] == "timing":
        timing(sys.argv[2], sys.argv[3:])
    else:
        sys.exit(__doc__)
