"""Builds oracle/_ref/libref.so from the reference's own kernel sources.

TEST INFRASTRUCTURE.  The reference's hot path is CUDA C: its kernel bodies are
plain C++ apart from the launch syntax of the host files that call them.  This
recipe copies the named kernel and helper definitions out of the reference
files where they lie ($PARALLEM_REF, else a `reference` folder beside the
repository) into
oracle/_ref/ref_kernels.inc -- a build product that stays out of git -- and
compiles them with oracle/ref_shim.h (sequential emulation of a CUDA grid) and
oracle/ref_harness.cpp (the host loops of cuFlowDirection, correctmfdflow and
erosionGPU) into a shared library.  It then serves as a second, independent
checker of the oracle on small grids.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libref.so")
# the reference tree: $PARALLEM_REF, else a `reference` folder beside the repository
REF = os.environ.get("PARALLEM_REF") or os.path.normpath(os.path.join(HERE, os.pardir, os.pardir, "reference"))

# (file, list of definition-start regexes) in the order they are emitted
PIECES = [
    ("headers/newflow.h", [r"^class watershed_edge\b", r"^class union_set\b"]),
    ("FD_kernels/newflow.cu", [
        r"^__global__ void FlowDirs\s*\(", r"^__global__ void shortest_paths_plateaus_initMFD\s*\(",
        r"^__global__ void route_plateausMFD\s*\(", r"^__global__ void init_watershedMFD\s*\(",
        r"^__global__ void init_watershed_sinkMFD\s*\(", r"^__global__ void identify_watershedMFD\s*\(",
        r"^using namespace std;",
        r"^watershed_edge::watershed_edge\(\)", r"^watershed_edge::~watershed_edge\(\)",
        r"^watershed_edge::watershed_edge\(int n1", r"^int watershed_edge::get_node1\(",
        r"^int watershed_edge::get_node2\(", r"^HASH_TYPE watershed_edge::get_weight\(",
        r"^void watershed_edge::set_node1\(", r"^void watershed_edge::set_node2\(",
        r"^void watershed_edge::set_weight\(", r"^bool watershed_edge::operator<\(",
        r"^union_set::union_set\(", r"^union_set::~union_set\(", r"^bool union_set::in_set\(",
        r"^int union_set::find_root\(", r"^void union_set::make_set\(", r"^void union_set::merge\(",
        r"^__device__ double atomicMin\(", r"^__global__ void init_hash_tableMFD\s*\(",
        r"^__global__ void identify_watershed_boundary_write_backMFD\s*\(",
        r"^__global__ void raise_watershedMFD\s*\(", r"^bool operator<\(const watershed_edge",
        r"^int init_and_sort_watershed_bound_labelsMFD\s*\(",
    ]),
    ("MOD_kernels/runoffweight.cu", [r"^__global__ void calcrunoffweight\s*\(", r"^void calcprops\(Data\* data\)"]),
    ("FA_kernels/mfd_simple.cu", [r"^__device__ int nghbrindex\s*\(", r"^__global__ void CalcMFD\s*\("]),
    ("MOD_kernels/eroincidep.cu", [
        r"^__global__ void diff_erosion\s*\(", r"^__global__ void conc_erosion\s*\(",
        r"^__global__ void gelifluction\s*\(", r"^__global__ void surface_change\s*\(",
        r"^__global__ void weathering\s*\(",
    ]),
    ("MOD_kernels/mfd_accum.cu", [r"^__device__ int inghbr\s*\(", r"^__global__ void MFDsedbud\s*\("]),
    ("MOD_kernels/updates.cu", [
        r"^__global__ void Update_Surface\s*\(", r"^__global__ void update_nutrient_content\s*\(",
        r"^__global__  ?void grow_vegetation\s*\(",
    ]),
]


def _extract(text: str, start_re: str) -> str:
    m = re.search(start_re, text, flags=re.M)
    if not m:
        raise RuntimeError(f"definition not found: {start_re}")
    i = m.start()
    if start_re.startswith("^using"):
        return text[i:text.index("\n", i) + 1]
    depth = 0
    j = text.index("{", i)
    while True:
        c = text[j]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                end = j + 1
                if text[end:end + 1] == ";":
                    end += 1
                return text[i:end] + "\n"
        j += 1


def generate() -> str:
    os.makedirs(OUT, exist_ok=True)
    parts = ["// generated by oracle/ref_build.py from the reference sources; do not edit\n"]
    for rel, starts in PIECES:
        path = os.path.join(REF, rel)
        text = open(path, encoding="latin-1").read()
        for s in starts:
            parts.append(f"// {rel}\n")
            piece = _extract(text, s)
            # calcprops reads only mapInfo, mask, Slopes, prop and fd of Data
            piece = piece.replace("void calcprops(Data* data)", "void calcprops(DataProps* data)")
            parts.append(piece)
    inc = os.path.join(OUT, "ref_kernels.inc")
    with open(inc, "w") as f:
        f.write("".join(parts))
    return inc


def build(force: bool = False) -> str | None:
    """Returns the library path, or None when the reference tree is absent."""
    if not os.path.isdir(os.path.join(REF, "FD_kernels")):
        return None
    deps = [os.path.join(HERE, "ref_harness.cpp"), os.path.join(HERE, "ref_shim.h"), os.path.join(HERE, "lem_oracle.h"),
            os.path.abspath(__file__)]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    generate()
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w",
           "-include", os.path.join(HERE, "ref_shim.h"),
           "-I", os.path.join(REF, "headers"), "-I", OUT, "-I", HERE,
           os.path.join(HERE, "ref_harness.cpp"), "-o", LIB]
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv) or "reference sources not present")
