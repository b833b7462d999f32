"""In-tree build of libsst.so (CUDA, sm_103a).

    python -m seesharp_gb300.build [--force]

Compiles the translation units in seesharp_gb300/csrc in parallel with nvcc and links them into
seesharp_gb300/libsst.so next to this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "libsst.so")
BUILD = os.path.join(HERE, "_build")
UNITS = ["sst_api.cu", "sst_commit.cu", "sst_render.cu", "sst_adjoint_api.cu", "sst_query.cu", "sst_kernels.cu", "sst_shade_occ.cu", "sst_shade_split.cu", "sst_pyramid.cu",
         "sst_trace.cu", "sst_light.cu", "sst_bvh.cu"]
HEADERS = ["sst_host.h", "sst_types.h", "sst_device.cuh", "sst_adjoint.cuh", "sst_shade.cuh", "sst_kernels.h", "sst_bvh.h", os.path.join("..", "..", "include", "sst.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "--expt-relaxed-constexpr",
         "-diag-suppress", "177"]
# The units holding the shading kernels (camera, shade, light paths, film fold) divide and take
# square roots with the approximate single-precision forms (errors of a few ulp) instead of the
# correctly rounded ones, whose slow-path subroutine calls cost the shade kernel a third of its
# time.  Traversal and the BVH build keep the correctly rounded forms (the intersection criterion
# is exact primitive ids); the RNG's float conversion and the environment-map tables use the
# correctly rounded intrinsics explicitly (bit-exact streams, tables equal to a CPU build).
SHADING_UNITS = {"sst_kernels.cu", "sst_shade_occ.cu", "sst_shade_split.cu", "sst_pyramid.cu", "sst_light.cu"}
SHADING_FLAGS = ["-prec-div=false", "-prec-sqrt=false"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale():
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    deps = [os.path.join(CSRC, u) for u in UNITS] + [os.path.normpath(os.path.join(CSRC, h)) for h in HEADERS] + [__file__]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    if not force and not _stale():
        return OUT
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_unit(u):
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        extra = SHADING_FLAGS if u in SHADING_UNITS else []
        cmd = [cc] + ARCH + FLAGS + extra + ["-I", os.path.join(ROOT, "include"), "-c", os.path.join(CSRC, u), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        return obj

    with cf.ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = OUT + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
