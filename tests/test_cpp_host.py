"""The C++ host side: lvr2_gb300/cpp/lvr2gb.hpp (lvr2-style classes over the
C ABI) and the lvr2gb_reconstruct command-line tool."""
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def built(lib, tmp_path_factory):
    from lvr2_gb300 import build as B
    cli = B.build_cli()
    test_bin = tmp_path_factory.mktemp("cpp") / "test_adapters"
    B.cpp_compile(ROOT / "tests/cpp/test_adapters.cpp", test_bin)
    return cli, test_bin


def test_cpp_programs_compile_and_parse_flags(built):
    cli, _ = built
    r = subprocess.run([str(cli), "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "--voxelsize" in r.stdout and "--flipPoint" in r.stdout
    r = subprocess.run([str(cli), "/nonexistent/scan.pts"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr
    r = subprocess.run([str(cli), "x.pts", "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2


def read_ply_counts(path):
    data = Path(path).read_bytes()
    head = data[:data.index(b"end_header\n")].decode()
    nv = int(head.split("element vertex ")[1].split()[0])
    nf = int(head.split("element face ")[1].split()[0])
    return nv, nf


def read_ply_mesh(path):
    """Vertex records (a numpy structured array with the header's float and
    uchar properties) and faces (uchar 3 + int32 x 3) of a binary
    little-endian PLY written by lvr2gb_reconstruct."""
    data = Path(path).read_bytes()
    end = data.index(b"end_header\n") + len(b"end_header\n")
    head = data[:end].decode().split("element face")[0]
    types = {"float": "<f4", "uchar": "u1"}
    fields = [(ln.split()[2], types[ln.split()[1]]) for ln in head.splitlines() if ln.startswith("property ")]
    nv, nf = read_ply_counts(path)
    v = np.frombuffer(data, np.dtype(fields), nv, end)
    rec = np.dtype([("n", "u1"), ("i", "<i4", 3)])
    f = np.frombuffer(data, rec, nf, end + v.nbytes)
    assert np.all(f["n"] == 3)
    return v, f["i"]


@pytest.mark.gpu
def test_cpp_adapters_on_gpu(built):
    _, test_bin = built
    r = subprocess.run([str(test_bin)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr + r.stdout


@pytest.mark.gpu
def test_cli_matches_python_path(built, tmp_path):
    """lvr2gb_reconstruct with lvr2_reconstruct's default flags gives the same
    mesh as the same calls made through the Python mirror."""
    import lvr2_gb300
    from lvr2_gb300 import synthetic
    cli, _ = built
    pts, _ = synthetic.scan_scene(40_000, seed=9)
    src = tmp_path / "scan.xyz"
    with open(src, "w") as f:
        f.write("%d\n" % len(pts))
        np.savetxt(f, pts, fmt="%.9g")
    out = tmp_path / "mesh.ply"
    r = subprocess.run([str(cli), str(src), "-v", "10", "--outputFile", str(out), "-e"], capture_output=True,
                       text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "Grid Cells:" in r.stdout
    nv, nf = read_ply_counts(out)
    pts_read = np.loadtxt(src, skiprows=1, dtype=np.float32)
    with lvr2_gb300.Surface(pts_read, kn=10, ki=10, kd=5, nem=0, flip_point=(0, 0, 0)) as s:
        s.calculate_normals()
        info = s.reconstruct(voxelsize=10.0, decomposition="PMC")
        s.optimize_planar_faces(5)
        v, f, _ = s.mesh(with_edges=False)
        vn = s.vertex_normals()
    assert (nv, nf) == (info.vertices, info.faces)
    pv, pf = read_ply_mesh(out)
    assert pv.dtype.names == ("x", "y", "z", "nx", "ny", "nz")
    assert np.array_equal(np.c_[pv["x"], pv["y"], pv["z"]], v) and np.array_equal(pf, f.astype(np.int32))
    assert np.array_equal(np.c_[pv["nx"], pv["ny"], pv["nz"]], vn)
    assert (tmp_path / "pointnormals.ply").exists()


@pytest.mark.gpu
def test_cli_colours(built, tmp_path):
    """A .pts with r g b columns (AsciiIO autodetection; the first line is
    skipped): the PLY carries red green blue per vertex, the colour of the
    vertex's nearest point."""
    import lvr2_gb300
    from lvr2_gb300 import synthetic
    cli, _ = built
    P = synthetic.spheres_tori(30_000, seed=14)
    rng = np.random.Generator(np.random.PCG64(3))
    C = rng.integers(0, 256, size=(len(P), 3))
    src = tmp_path / "scan.pts"
    with open(src, "w") as fh:
        fh.write("x y z r g b\n")
        for p, c in zip(P.tolist(), C.tolist()):
            fh.write("%.9g %.9g %.9g %d %d %d\n" % (*p, *c))
    out = tmp_path / "mesh.ply"
    r = subprocess.run([str(cli), str(src), "-v", "0.02", "--nem", "3", "--outputFile", str(out)], capture_output=True,
                       text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    pv, _ = read_ply_mesh(out)
    assert pv.dtype.names == ("x", "y", "z", "red", "green", "blue", "nx", "ny", "nz")
    pts = np.loadtxt(src, skiprows=1, dtype=np.float64)
    with lvr2_gb300.Surface(pts[:, :3].astype(np.float32), kn=10, ki=10, kd=5, nem=3, flip_point=(0, 0, 0)) as s:
        s.calculate_normals()
        s.reconstruct(voxelsize=0.02, decomposition="PMC")
        s.optimize_planar_faces(5)
        v, _, _ = s.mesh(with_edges=False)
        vc = s.vertex_colors(pts[:, 3:].astype(np.uint8))
    assert np.array_equal(np.c_[pv["x"], pv["y"], pv["z"]], v)
    assert np.array_equal(np.c_[pv["red"], pv["green"], pv["blue"]], vc)


@pytest.mark.gpu
def test_cli_scan_pose_file(built, tmp_path):
    """--scanPoseFile: poses read as lvr2's parseScanPoses reads them (the read
    that meets the end of the file appends the last pose again), normals
    flipped as with Surface.set_scan_poses."""
    import lvr2_gb300
    from lvr2_gb300 import synthetic
    cli, _ = built
    P = synthetic.spheres_tori(20_000, seed=52)
    src = tmp_path / "cloud.xyz"
    with open(src, "w") as fh:
        fh.write("%d\n" % len(P))
        np.savetxt(fh, P, fmt="%.9g")
    poses = np.array([[0.1, 0.2, 0.3], [0.9, 0.8, 0.7]], np.float32)
    pf = tmp_path / "poses.txt"
    pf.write_text("".join("%g %g %g\n" % tuple(p) for p in poses))
    r = subprocess.run([str(cli), str(src), "-v", "0.05", "--nem", "3", "-e", "--scanPoseFile", str(pf),
                        "--outputFile", str(tmp_path / "m.ply")], capture_output=True, text=True, timeout=300,
                       cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "3 scan poses" in r.stdout
    data = (tmp_path / "pointnormals.ply").read_bytes()
    end = data.index(b"end_header\n") + len(b"end_header\n")
    rec = np.frombuffer(data, np.float32, offset=end).reshape(-1, 6)
    pts_read = np.loadtxt(src, skiprows=1, dtype=np.float32)
    lvr_poses = np.concatenate([poses, poses[-1:]]).astype(np.float32)
    with lvr2_gb300.Surface(pts_read, kn=10, ki=10, kd=5, nem=3, flip_point=(0, 0, 0)) as s:
        s.set_scan_poses(lvr_poses)
        s.calculate_normals()
        n = s.normals()
    assert np.array_equal(rec[:, 3:], n)


def test_save_grid_stream_format(built, tmp_path):
    """--saveGrid writes HashGrid::saveGrid's stream: the cell count, then each
    cell's centre and 8 corner distances, every number as operator<< prints
    a float (%g, 6 significant digits) with no separator."""
    from lvr2_gb300 import build as B
    exe = tmp_path / "test_write_grid"
    B.cpp_compile(ROOT / "tests/cpp/test_write_grid.cpp", exe)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    centers = np.float32([0.5, -1.25, 1e-7, 1234567.0, 0.1, -0.0])
    tsdf = (np.arange(16) - 7).astype(np.float32) * np.float32(0.3)
    want = "2"
    for i in range(2):
        want += "".join("%g" % float(x) for x in centers[3 * i:3 * i + 3])
        want += "".join("%g" % float(x) for x in tsdf[8 * i:8 * i + 8])
    assert r.stdout == want
    cli, _ = built
    r = subprocess.run([str(cli), "/nonexistent/scan.pts", "-g"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr  # -g parsed, the file is missing
