"""In-tree build of the native library ``dumbray_gb300/_build/libdumbray_gb300.so``.

nvcc compiles the CUDA translation units for sm_103a only; the host octree builder is plain C++.
Translation units compile in parallel; no cmake, no torch extension machinery.

FP contraction is off everywhere: host code is compiled with ``-ffp-contract=off`` (the host octree
build rounds like DumbRay's host code on x86-64 and aarch64, where gcc would otherwise fuse
multiply-adds) and device code with ``-fmad=false``.  The GPU octree builder needs it for trees
bit-identical to the host build; the cast predicate is written with explicitly rounded intrinsics,
which are never contracted.  The render kernels would not need it: letting them fuse was measured on
a GB300 and bought
nothing on the 1080p path trace (327.4 / 327.5 Mpaths/s fused, 328.3 unfused) and about 2.5% on the
reference-mode twin (158.3 vs 154.5), while it moved same-seed per-pixel agreement with the FP64
oracle past 1% on one physical-mode lens case, so they stay unfused too.  ``NO_FMAD`` lists the
translation units that are compiled unfused; every one is, today.
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
NO_FMAD = {"octree_gpu.cu", "dr_kernels.cu", "dr_api.cu", "dr_noalloc.cu", "dr_progressive.cu"}


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
