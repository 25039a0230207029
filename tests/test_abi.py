"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/lem_gb300.h declares (no GPU needed)."""
import os
import re
import subprocess

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "lem_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lem_[a-z_]+)\s*\(", text)))


def test_header_declares_the_stage_calls():
    names = declared_functions()
    for n in ("lem_create", "lem_destroy", "lem_set_field", "lem_get_field", "lem_flow_direction",
              "lem_flow_accumulation", "lem_erosion", "lem_step", "lem_get_totals", "lem_synchronize"):
        assert n in names


def test_library_exports_every_declared_symbol(gpu_lib):
    from parallem_gb300 import lem
    out = subprocess.run(["nm", "-D", "--defined-only", lem.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\b[TW] (lem_[a-z_]+)\b", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"not exported: {missing}"
    # the Python mirror binds exactly the declared set
    assert sorted(lem.SIGNATURES) == declared_functions()


def test_struct_layouts_match_header():
    """ctypes mirrors have the sizes a C compiler gives the header structs."""
    import ctypes as C
    import tempfile
    from parallem_gb300 import lem
    src = r'''
#include <stdio.h>
#include "lem_gb300.h"
int main(void){printf("%zu %zu %zu %zu\n", sizeof(lem_grid_desc), sizeof(lem_params), sizeof(lem_climate), sizeof(lem_totals));return 0;}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "s")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        sizes = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert sizes == [C.sizeof(lem.GridDesc), C.sizeof(lem.Params), C.sizeof(lem.Climate), C.sizeof(lem.Totals)]


def test_no_gpu_means_error_not_crash(gpu_lib):
    """Without a usable device every call reports LEM_ERR_CUDA instead of aborting."""
    import pytest
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    import numpy as np
    from parallem_gb300 import lem
    with pytest.raises(lem.LemError) as e:
        lem.Model(np.zeros((4, 4)), 30.0, 600.0, 10.0)
    assert e.value.code == 4
