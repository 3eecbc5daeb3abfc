"""Builds libpyre_cuda.so (sm_103a kernels + C ABI) in-tree with nvcc.

Translation units compile in parallel, then link into
``pyre_gb300/lib/libpyre_cuda.so``. All of them build without FMA contraction
(``--fmad=false`` for device code, ``-ffp-contract=off`` for host code) so the
kernels and the host BVH builder round exactly like binary32 code that does not
fuse multiply-adds, which is what bit-exact hit parity needs.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
LIB_DIR = HERE / "lib"
LIB = LIB_DIR / "libpyre_cuda.so"
OBJ_DIR = HERE / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "integrator.cu", "bvh_host.cpp", "bvh_device.cu"]
HEADERS = ["pyre_math.cuh", "device_scene.cuh", "shading.cuh", "adjoint.cuh", "internal.h", "bvh_host.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpyre_cuda.so")


def common_flags() -> list[str]:
    return [
        "-O3", "-std=c++17", "-lineinfo", "--fmad=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
        "-I", str(CSRC), "-I", str(HERE.parent / "include"),
    ] + ARCH


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> Path:
    """Compiles the library if a source changed; returns its path."""
    OBJ_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    exe = nvcc()
    headers = [CSRC / h for h in HEADERS] + [HERE.parent / "include" / "pyre_cuda.h"]
    jobs = []
    for src in SOURCES:
        obj = OBJ_DIR / (src + ".o")
        if force or ptxas_info or _stale(obj, [CSRC / src] + headers):
            cmd = [exe, *common_flags(), "-c", str(CSRC / src), "-o", str(obj)]
            if ptxas_info and src.endswith(".cu"):
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_info:
                sys.stdout.write(r.stdout)
                sys.stderr.write(r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed ({r.returncode}):\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    objs = [OBJ_DIR / (s + ".o") for s in SOURCES]
    if force or jobs or _stale(LIB, objs):
        cmd = [exe, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv, force="--force" in sys.argv))
