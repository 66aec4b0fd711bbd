"""Builds libluz_gb300.so in-tree: sm_103a CUDA kernels + C ABI + C++17 host layer.

Device translation units are compiled with FMA contraction off (-fmad=false) and
IEEE division / square root, host code with -ffp-contract=off: rays generated on
the device must be bit-identical to rays generated by a CPU following the same
steps. Translation units compile in parallel; the result is linked against the
static CUDA runtime so that loading the library needs no GPU. LUZ_EXTRA_NVCC adds
flags to every device translation unit (e.g. -DLUZ_VIS_MIN_BLOCKS=2).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "libluz_gb300.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CUDA_TUS = ["lbvh.cu", "trace.cu", "visibility.cu", "lightpass.cu", "capi.cu", "blas_noalloc.cu",
            "denoise.cu", "batch.cu", "post.cu", "shadowmap.cu"]
FMA_TUS = {"denoise.cu"}
HOST_TUS = ["scene.cpp", "ingest.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libluz_gb300")


def _sources() -> list[Path]:
    return [CSRC / s for s in CUDA_TUS + HOST_TUS] + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for tu in CUDA_TUS:
        obj = BUILD / (tu + ".o")
        # The denoiser is not on the bit-exact ray path: FMA contraction is allowed there.
        fmad = "-fmad=true" if tu in FMA_TUS else "-fmad=false"
        cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", fmad, "-prec-div=true",
               "-prec-sqrt=true", "-ftz=false", "-Xptxas", "-warn-spills",
               "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", str(INCLUDE),
               "-c", str(CSRC / tu), "-o", str(obj)] + os.environ.get("LUZ_EXTRA_NVCC", "").split()
        jobs.append((tu, cmd))
        objs.append(obj)
    for tu in HOST_TUS:
        obj = BUILD / (tu + ".o")
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", str(INCLUDE),
               "-c", str(CSRC / tu), "-o", str(obj)]
        jobs.append((tu, cmd))
        objs.append(obj)
    procs = [(tu, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for tu, cmd in jobs]
    failed = []
    for tu, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stderr.write(out)
        if p.returncode != 0:
            failed.append(tu)
    if failed:
        raise RuntimeError(f"compilation failed: {failed}")
    tmp = LIB.with_suffix(".so.tmp")
    link = [nvcc, ARCH, "-shared", "-cudart", "static", "-o", str(tmp)] + [str(o) for o in objs] + \
        ["-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
