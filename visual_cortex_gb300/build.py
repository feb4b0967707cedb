"""Builds the native library of the package (CUDA kernels + C ABI) in-tree for sm_103a.

The library is compiled with nvcc straight from visual_cortex_gb300/csrc/*.cu into
visual_cortex_gb300/_lib/libpatchv1_gb300.so (one -gencode, translation units compiled in
parallel).  No CMake and no torch extension machinery are involved, so the same recipe runs
on the x86 build host and on the aarch64 GB300 host.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
BUILD = PKG.parent / "_build" / "native"
LIBNAME = "libpatchv1_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
# --fmad=false: every float expression is evaluated as the rounded operations written in the
# source (no contraction into FMA), as the reference's expressions are read; the host side
# likewise keeps -ffp-contract=off so x86 and aarch64 hosts compute the same table values.
NVCC_FLAGS = [ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
              "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
              "-Xptxas", "-O3", "--expt-relaxed-constexpr"]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and (Path(root) / "bin" / "nvcc").exists():
            return str(Path(root) / "bin" / "nvcc")
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the native library")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def library_path() -> Path:
    return LIBDIR / LIBNAME


def _stale(lib: Path) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + \
        list((PKG.parent / "include").glob("*.h")) + [Path(__file__)]
    return any(d.stat().st_mtime > t for d in deps)


def build_native(force: bool = False, verbose: bool = False) -> Path:
    """Compiles the native library if it is missing or older than its sources."""
    lib = library_path()
    if not force and not _stale(lib):
        return lib
    nvcc = nvcc_path()
    BUILD.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    objs = []

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        cmd = [nvcc, *NVCC_FLAGS, "-I", str(PKG.parent / "include"), "-c", str(src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            print(res.stdout, res.stderr)
        return obj

    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc, ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build_native(force=True, verbose=True))
