"""Builds liblvrgb.so (the C ABI of include/lvrgb.h) in-tree with nvcc for sm_103a.

Every .cu file under lvr2_gb300/csrc is compiled in parallel to an object
file, then linked into lvr2_gb300/liblvrgb.so (CUDA runtime linked
statically).  Run as `python -m lvr2_gb300.build` or call build().
"""
import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "liblvrgb.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
              "-I" + str(PKG.parent / "include")]


def nvcc():
    for cand in [os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"]:
        if cand and (Path(cand).exists() or cand == "nvcc"):
            return cand
    return "nvcc"


def _compile(src, extra):
    obj = BUILD / (src.stem + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", str(src), "-o", str(obj)]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src.name, " ".join(cmd), out.stderr))
    return obj, out.stderr


def build(verbose=False, ptxas_info=False, jobs=None):
    BUILD.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    deps = sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(CSRC.glob("*.inc")) +
                  [PKG.parent / "include" / "lvrgb.h"])
    newest_dep = max((p.stat().st_mtime for p in deps), default=0)
    todo = []
    objs = []
    for s in srcs:
        obj = BUILD / (s.stem + ".o")
        objs.append(obj)
        if ptxas_info or not obj.exists() or obj.stat().st_mtime < max(s.stat().st_mtime, newest_dep):
            todo.append(s)
    logs = []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(todo) or 1)) as ex:
        for obj, err in ex.map(lambda s: _compile(s, extra), todo):
            logs.append((obj.name, err))
    if todo or not LIB.exists():
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("link failed:\n" + out.stderr)
    if verbose or ptxas_info:
        for name, err in logs:
            if err.strip():
                print("==", name)
                print(err)
    return LIB


CPP = PKG / "cpp"
CLI = PKG / "lvr2gb_reconstruct"


def cpp_compile(src, out, extra=()):
    """Compiles a C++ host program against include/lvrgb.h and liblvrgb.so."""
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", str(PKG.parent / "include"), "-I", str(CPP), str(src),
           "-L", str(PKG), "-llvrgb", "-Wl,-rpath," + str(PKG), "-o", str(out)] + list(extra)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed for %s:\n%s" % (src, r.stderr))
    return out


def build_cli():
    """The lvr2gb_reconstruct command-line tool (lvr2_gb300/cpp)."""
    src = CPP / "lvr2gb_reconstruct.cpp"
    deps = [src, CPP / "lvr2gb.hpp", PKG.parent / "include" / "lvrgb.h", LIB]
    if CLI.exists() and CLI.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return CLI
    return cpp_compile(src, CLI)


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    build_cli()
    print(LIB)
