"""Builds libcochlea_gb300.so (the CUDA kernels + C ABI) for sm_103a, in tree.

Each translation unit under csrc/ is compiled by nvcc in parallel, then the
objects are linked into cochlearmodel_gb300/_lib/libcochlea_gb300.so.
Device code is compiled with --fmad=false: every fused multiply-add in the
kernels is an explicit __fmaf_rn, so the floating-point order is the one the
CPU oracle reproduces.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
BUILD = PKG / "_build"
LIBNAME = "libcochlea_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = [
    "-O3", "-std=c++17", "-lineinfo", "--fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-I", str(ROOT / "include"), "-I", str(CSRC),
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build")
    return cand


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _compile(src: Path) -> Path:
    obj = BUILD / (src.name + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, "-c", str(src), "-o", str(obj)]
    if os.environ.get("CGB_PTXAS_VERBOSE") and src.suffix == ".cu":
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    if res.stderr.strip():
        sys.stderr.write(res.stderr)
    return obj


def lib_path() -> Path:
    return LIBDIR / LIBNAME


HARNESS = PKG / "harness" / "run_cuda_harness.cpp"


def harness_path() -> Path:
    return LIBDIR / "run_cuda_harness"


def build_harness() -> Path:
    """The Run_Cuda-order host harness over the reference-named API."""
    out = harness_path()
    cmd = [nvcc(), "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(HARNESS), "-o",
           str(out), "-L", str(LIBDIR), "-lcochlea_gb300", "-lcudart",
           "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"harness build failed:\n{res.stdout}\n{res.stderr}")
    return out


def up_to_date() -> bool:
    lib = lib_path()
    if not lib.exists():
        return False
    t = lib.stat().st_mtime
    deps = sources() + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + \
        list((ROOT / "include").glob("*.h")) + [Path(__file__), HARNESS]
    return harness_path().exists() and all(d.stat().st_mtime <= t for d in deps)


def build(force: bool = False, jobs: int | None = None) -> Path:
    if not force and up_to_date():
        return lib_path()
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIBDIR / (LIBNAME + ".tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib_path())
    build_harness()
    return lib_path()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
