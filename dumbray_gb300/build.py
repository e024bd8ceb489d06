"""In-tree build of the native library ``dumbray_gb300/_build/libdumbray_gb300.so``.

nvcc compiles the CUDA translation units for sm_103a only; the host octree builder is plain C++.
Translation units compile in parallel; no cmake, no torch extension machinery.

FP contraction: host code is compiled with ``-ffp-contract=off`` (the host octree build rounds like
DumbRay's host code on x86-64 and aarch64, where gcc would otherwise fuse multiply-adds).  On the
device only the GPU octree builder (``octree_gpu.cu``, sharing its plain-operator geometry with the
host builder through ``octree_geom.h``) is compiled with ``-fmad=false``, so its tree stays
bit-identical to the host build.  The cast predicate and the traversal are written with explicitly
rounded intrinsics (``__fadd_rn`` / ``__fmul_rn`` / ``__fdiv_rn`` / ``__fsqrt_rn``), which the compiler
never contracts, so the render and adjoint kernels may fuse multiply-adds elsewhere.
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
OUT = HERE / "_build"
LIB = OUT / "libdumbray_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NO_FMAD = {"octree_gpu.cu"}   # translation units whose bit-exactness rests on plain operators


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build dumbray_gb300")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")) + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh"))
                  + [HERE.parent / "include" / "dr_api.h"])


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in sources())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", str(HERE.parent / "include")]
    cu_flags = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                "-Xptxas", "-v"] + ARCH + inc
    jobs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = OUT / (src.stem + ".o")
        fmad = ["-fmad=false"] if src.name in NO_FMAD else ["-fmad=true"]
        jobs.append([nvcc, "-c", str(src), "-o", str(obj)] + cu_flags + fmad)
    for src in sorted(CSRC.glob("*.cpp")):
        obj = OUT / (src.stem + ".o")
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-pthread", "-c", str(src), "-o", str(obj)] + inc)
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    (OUT / "ptxas.log").write_text("\n".join(logs))
    objs = [str(OUT / (s.stem + ".o")) for s in sorted(CSRC.glob("*.cu"))] + \
           [str(OUT / (s.stem + ".o")) for s in sorted(CSRC.glob("*.cpp"))]
    tmp = OUT / (LIB.name + ".tmp")
    _run([nvcc, "-shared", "-o", str(tmp)] + objs + ARCH + ["-Xcompiler", "-pthread", "-lcudart"])
    os.replace(tmp, LIB)
    if verbose:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    p = build(force=force, verbose="-v" in sys.argv)
    print(p)
