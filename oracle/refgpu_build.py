"""Builds PARALLEM's own CUDA code for sm_103a: oracle/_ref/gpu/libref_gpu.so.

TEST AND MEASUREMENT INFRASTRUCTURE.  The reference's hot-path sources (its
FD_kernels, FA_kernels and MOD_kernels files, MEM_kernels/memory_dev.cu,
memory.cu, MapInfo.cu, Data.cpp and io.cpp, and its headers) are copied
unchanged from the reference tree ($PARALLEM_REF, else a `reference` folder
beside the repository) into oracle/_ref/gpu/src -- a build folder kept out of
git, so that a machine with only the repository's files builds from that copy
-- and compiled with nvcc for sm_103a, with three small stand-ins for what a
Linux build lacks (oracle/refgpu: the CUDA Samples' checkCudaErrors, the
lower-case data.h include of updates.cu, MSVC's fopen_s/strncpy_s), together
with oracle/refgpu/harness.cu in place of lem.cpp.  Its Visual Studio project
is not used.  Returns None where neither the reference tree nor the copy is
present.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref", "gpu")
SRC = os.path.join(OUT, "src")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libref_gpu.so")
COMPAT = os.path.join(HERE, "refgpu")
REF = os.environ.get("PARALLEM_REF") or os.path.normpath(os.path.join(ROOT, os.pardir, "reference"))
UNITS = ["FD_kernels/newflow.cu", "FD_kernels/routeflow.cu", "FA_kernels/mfd_simple.cu",
         "MOD_kernels/runoffweight.cu", "MOD_kernels/eroincidep.cu", "MOD_kernels/mfd_accum.cu",
         "MOD_kernels/updates.cu", "MOD_kernels/erosion.cu", "MEM_kernels/memory_dev.cu", "MEM_kernels/memory.cu",
         "MEM_kernels/MapInfo.cu", "MEM_kernels/Data.cpp", "MEM_kernels/io.cpp"]
# the driver itself: not part of the library, but copied so that the shim's
# link test can build lem.cpp unchanged against liblem_refshim.so
DRIVER = "lem.cpp"
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-w",
         "-x", "cu", "-include", os.path.join(COMPAT, "compat.h")]


def _copy_sources() -> bool:
    """Refreshes the copy from the reference tree; False when neither exists."""
    if os.path.isdir(os.path.join(REF, "FD_kernels")):
        for rel in UNITS + [DRIVER] + [os.path.join("headers", h) for h in os.listdir(os.path.join(REF, "headers"))]:
            src, dst = os.path.join(REF, rel), os.path.join(SRC, rel)
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(src):
                shutil.copy2(src, dst)
    return all(os.path.isfile(os.path.join(SRC, u)) for u in UNITS)


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build(force: bool = False) -> str | None:
    if not _copy_sources():
        return None
    os.makedirs(OBJ, exist_ok=True)
    inc = ["-I", COMPAT, "-I", os.path.join(SRC, "headers"), "-I", os.path.join(ROOT, "include")]
    jobs = []
    objs = []
    units = [(os.path.join(SRC, u), os.path.basename(u)) for u in UNITS]
    units.append((os.path.join(COMPAT, "harness.cu"), "harness.cu"))
    for src, name in units:
        o = os.path.join(OBJ, name.rsplit(".", 1)[0] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < os.path.getmtime(src):
            jobs.append([_nvcc()] + FLAGS + inc + ["-c", src, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if res.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + res.stdout + res.stderr)
                raise RuntimeError(f"nvcc failed on {cmd[-3]}")
    if force or jobs or not os.path.exists(LIB):
        cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-cudart", "static", "-o", LIB] + objs
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + res.stdout + res.stderr)
            raise RuntimeError("link of the reference build failed")
    return LIB


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    print(build(force="--force" in sys.argv) or "reference sources not present")
