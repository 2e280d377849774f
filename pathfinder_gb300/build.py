"""Builds libpathfinder_cuda.so in-tree for sm_103a (nvcc, no cmake).

Translation units compile in parallel into ``pathfinder_gb300/_build`` and
link into ``pathfinder_gb300/libpathfinder_cuda.so``.  The tiler unit is built
with ``-fmad=false`` so that its single-precision arithmetic matches the
reference CPU tiler bit for bit.  The seeded scene generators (host code) are
a separate library, ``pathfinder_gb300/libpfscenes.so``, built with g++.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpathfinder_cuda.so")
SCENES_LIB = os.path.join(HERE, "libpfscenes.so")
SCENES_SRC = os.path.join(CSRC, "pf_scenes.cpp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code: no multiply-add contraction (gcc contracts by default on aarch64),
# so the host-side single-precision arithmetic is the same on every machine.
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                      "-I" + os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]

# (source, extra flags)
UNITS = [
    ("pf_tiler.cu", ["-fmad=false"]),
    ("pf_raster.cu", []),
    ("pf_adjoint.cu", []),
    ("pf_renderer.cu", []),
    ("pf_noalloc.cu", []),
    ("pf_paint.cu", []),
    ("pf_stroke.cu", ["-fmad=false"]),
    ("pf_pack.cu", []),
    ("pf_pipeline.cu", []),
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA renderer cannot be built")
    return cand


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _compile(src: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if _newer(obj, [path] + _headers()):
        return obj
    cmd = [nvcc(), "-c", path, "-o", obj] + NVCC_COMMON + extra
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return obj


def build_scenes(verbose: bool = False, force: bool = False) -> str:
    """The scene generator library (host code only; no multiply-add contraction,
    so that both host architectures generate the same bytes)."""
    hdr = os.path.join(ROOT, "include", "pathfinder_cuda_scenes.h")
    if not force and _newer(SCENES_LIB, [SCENES_SRC, hdr, os.path.join(ROOT, "include", "pathfinder_cuda.h")]):
        return SCENES_LIB
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-I" + os.path.join(ROOT, "include"), "-o", SCENES_LIB, SCENES_SRC]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"scene generator build failed:\n{r.stderr}")
    return SCENES_LIB


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    with ThreadPoolExecutor(max_workers=len(UNITS) + 1) as ex:
        scenes = ex.submit(build_scenes, verbose, force)
        objs = list(ex.map(lambda u: _compile(u[0], u[1], verbose), UNITS))
        scenes.result()
    if force or not _newer(LIB, objs):
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fPIC"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
