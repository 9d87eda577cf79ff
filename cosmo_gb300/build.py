"""Build libcosmo_gb300.so in-tree for sm_103a (GB300).

Each translation unit is compiled in parallel with nvcc (host .cpp files with
the host compiler through nvcc), then linked into one shared library with the
CUDA runtime linked statically.  Outputs go to cosmo_gb300/_build/ and
cosmo_gb300/libcosmo_gb300.so (both git-ignored).

    python -m cosmo_gb300.build [--force] [--jobs N]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
SRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcosmo_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["model.cpp", "dense.cpp", "capi.cpp", "basis.cu", "hbuild.cu", "spmm.cu", "davidson.cu", "virtual.cu", "jt.cu", "xshljt.cpp", "batched.cu", "hhread.cpp", "tiled.cu", "sf.cu", "xshlsf.cpp", "em.cpp", "xshlemb.cpp", "wide.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(src: str) -> list[str]:
    host = "-fPIC,-Wall,-Wno-unused-function"
    if src == "xshljt.cpp":
        # the level listing's RMS over one experimental level is the difference
        # of two equal squares: without fused multiply-adds it is 0 on x86-64
        # and aarch64 hosts alike, as the reference prints it
        host += ",-ffp-contract=off"
    common = ["-std=c++17", "-O3", "-I", os.path.join(ROOT, "include"), "-I", SRC, "-Xcompiler", host]
    if src.endswith(".cu"):
        return common + ARCH + ["-lineinfo", "--expt-relaxed-constexpr", "-Xptxas", "-O3"]
    return common


def _compile(src: str) -> str:
    obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), "-c", os.path.join(SRC, src), "-o", obj] + _flags(src)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(ROOT, "include", "cosmo_gb300.h"),
                                                                os.path.abspath(__file__)]
    deps += [os.path.join(PKG, "cli", f) for f in os.listdir(os.path.join(PKG, "cli"))]
    if not all(os.path.exists(os.path.join(PKG, "bin", c)) for c in CLIS):
        return True
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    if verbose:
        print("built", LIB)
    return LIB


CLI_DIR = os.path.join(PKG, "cli")
BIN_DIR = os.path.join(PKG, "bin")
CLIS = ["cg_dexhvjt", "cg_xsysmbs", "cg_xhhjj", "cg_davidson_vfile", "cg_xshljt", "cg_xshlsf", "cg_xshlemb", "cg_xshlao", "cg_xlevels"]


def build_cli() -> list[str]:
    """The command-line drop-ins (C++ over the C ABI) into cosmo_gb300/bin/."""
    os.makedirs(BIN_DIR, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")

    def one(name: str) -> str:
        out = os.path.join(BIN_DIR, name)
        cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
               os.path.join(CLI_DIR, name + ".cpp"), "-o", out, "-L", PKG, "-lcosmo_gb300",
               "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"cli build failed: {name}\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return out

    with cf.ThreadPoolExecutor(max_workers=len(CLIS)) as ex:
        return list(ex.map(one, CLIS))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    a = ap.parse_args()
    build(force=a.force, jobs=a.jobs, verbose=True)


if __name__ == "__main__":
    main()
