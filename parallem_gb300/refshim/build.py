"""Builds parallem_gb300/_lib/liblem_refshim.so: PARALLEM's stage entry points
(cuFlowDirection, computeRunOffWeights, correctmfdflow, erosionGPU, the
memory_dev.cu set) on top of liblem_gb300.so.

The shim is compiled against the reference's own Data type.  Its headers
(headers/Data.h and the four it includes) are read from the reference tree --
$PARALLEM_REF, else a `reference` folder beside the repository -- and copied
into parallem_gb300/refshim/_ref/, a build folder kept out of git, so that a
machine without the reference tree (where only the repository's files are
present) builds from that copy.  Without either, there is nothing to build and
build() returns None.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
GEN = os.path.join(HERE, "_ref")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "liblem_refshim.so")
SRC = os.path.join(HERE, "lem_refshim.cpp")
HEADERS = ("Data.h", "lem.h", "config.h", "MapInfo.h", "production.h")


def reference_root() -> str:
    return os.environ.get("PARALLEM_REF") or os.path.normpath(os.path.join(ROOT, os.pardir, "reference"))


def headers_dir() -> str | None:
    """The folder holding the reference's Data.h and its includes (refreshed
    from the reference tree when present), or None."""
    src = os.path.join(reference_root(), "headers")
    if all(os.path.isfile(os.path.join(src, h)) for h in HEADERS):
        os.makedirs(GEN, exist_ok=True)
        for h in HEADERS:
            dst = os.path.join(GEN, h)
            if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(os.path.join(src, h)):
                shutil.copy2(os.path.join(src, h), dst)
    if all(os.path.isfile(os.path.join(GEN, h)) for h in HEADERS):
        return GEN
    return None


def build(force: bool = False) -> str | None:
    hdr = headers_dir()
    if hdr is None:
        return None
    from parallem_gb300 import build as core
    core_lib = core.build()
    deps = [SRC, os.path.join(ROOT, "include", "lem_refshim.h"), os.path.join(ROOT, "include", "lem_gb300.h"),
            core_lib] + [os.path.join(hdr, h) for h in HEADERS]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", "-I", hdr, "-I", os.path.join(ROOT, "include"),
           SRC, "-L", LIBDIR, "-llem_gb300", "-Wl,-rpath,$ORIGIN", "-o", LIB]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + res.stdout + res.stderr)
        raise RuntimeError("liblem_refshim.so failed to build")
    return LIB


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    print(build(force="--force" in sys.argv) or "reference headers not present")
