"""The reference's own stage entry points on the C ABI (liblem_refshim.so).

cpu: the shim builds against the reference's Data type and exports every name
include/lem_refshim.h declares, with the reference's C++ signatures.
gpu: tests/refshim/driver.cpp runs the timestep loop of lem.cpp (45-97, 114) --
the same calls in the same order on a Data struct -- and the host arrays it
ends with equal, bit for bit, the grids of the same steps on a lem_gb300
handle, over three climate-series steps (the first moves the outlet, as
correctmfdflow's first iteration does) and over two run-in steps; one step
from the same state also matches the FP64 oracle at the parity tolerances.
Skipped where the reference headers are not present (neither the reference
tree nor the copy the build made of them).
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT

SOIL = ("stone", "fines", "soilT", "soilM", "soilB", "nut", "totB")
OUT = ("dem", "fa", "runoff", "slopeptr", "stone", "fines", "soilT", "soilM", "soilB", "nut", "totB", "ero", "inci",
       "geli", "depo", "dz")
ROWS = ("tot_e", "tot_i", "tot_g", "tot_d", "tot_weather_c", "tot_weather_p", "tot_bio", "fa_max", "sinkcount",
        "outlet")


def _shim():
    from parallem_gb300.refshim import build as rb
    lib = rb.build()
    if lib is None:
        pytest.skip("the reference headers are not present")
    return rb, lib


def declared():
    text = open(os.path.join(ROOT, "include", "lem_refshim.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:void|int|lem_status|lem_handle\*)\s+(\w+)\s*\(", text, flags=re.M)))


def test_shim_exports_the_reference_names():
    rb, lib = _shim()
    out = subprocess.run(["nm", "-DC", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = {}
    for line in out.splitlines():
        parts = line.split(" ", 2)
        if len(parts) == 3 and parts[1] in ("T", "W"):
            exported[parts[2].split("(")[0]] = parts[2]
    names = declared()
    for n in ("cuFlowDirection", "computeRunOffWeights", "calcpropsSFD", "calcwater", "correctmfdflow", "erosionGPU",
              "createDeviceSpace", "clearDeviceSpace", "copyMask", "copylastclimate", "setdevicespace_FD",
              "cleardevicespace_Process", "zerogrids"):
        assert n in names
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    # C++ linkage with the reference's Data type, as lem.cpp's objects expect
    assert exported["cuFlowDirection"] == "cuFlowDirection(DataS*, DataS*, int)"
    assert exported["erosionGPU"] == "erosionGPU(DataS*, DataS*, int)"
    assert exported["computeRunOffWeights"] == "computeRunOffWeights(DataS*, DataS*)"
    assert exported["lem_refshim_status"] == "lem_refshim_status"  # extern "C"


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    rb, lib = _shim()
    d = tmp_path_factory.mktemp("refshim")
    so = str(d / "driver.so")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", "-I", rb.headers_dir(), "-I",
           os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "refshim", "driver.cpp"), "-L", rb.LIBDIR,
           "-llem_refshim", "-llem_gb300", "-Wl,-rpath," + rb.LIBDIR, "-o", so]
    subprocess.run(cmd, check=True)
    L = C.CDLL(so)
    P = C.c_void_p
    L.refshim_run.argtypes = [C.c_int, C.c_int, C.c_double, P, P, C.c_int, P, C.c_double, C.c_double, C.c_int,
                              C.c_int, P, P, P, P, P, P]
    L.refshim_run.restype = C.c_int
    return L


def run_driver(L, dem, st, params, init_rain, init_temp, first_iter, rain, temp, stage_ms=None):
    H, W = dem.shape
    N = H * W
    steps = len(rain)
    dem = np.ascontiguousarray(dem, np.float64)
    soil = np.ascontiguousarray(np.stack([st[f] for f in SOIL]), np.float64)
    out = np.zeros((16, H, W))
    codes = np.zeros((2, H, W), np.int32)
    rows = np.zeros((steps, 10))
    r = np.ascontiguousarray(rain, np.float64)
    t = np.ascontiguousarray(temp, np.float64)
    rc = L.refshim_run(W, H, 30.0, dem.ctypes.data, soil.ctypes.data, int(st["outlet"]), C.addressof(params),
                       init_rain, init_temp, first_iter, steps, r.ctypes.data, t.ctypes.data, out.ctypes.data,
                       codes.ctypes.data, rows.ctypes.data, None if stage_ms is None else stage_ms.ctypes.data)
    assert rc == 0, f"lem_refshim_status {rc}"
    res = {f: out[k] for k, f in enumerate(OUT)}
    res["fd"], res["sfd"] = codes[0], codes[1]
    return res, [dict(zip(ROWS, row)) for row in rows]


def handle_path(dem, st, init_rain, init_temp, first_iter, rain, temp):
    from parallem_gb300 import lem
    g = lem.Model(dem, 30.0, init_rain, init_temp)
    g.set_state(st)
    rows = []
    for k in range(len(rain)):
        i = first_iter + k
        flags = lem.STEP_KEEP_DIAGNOSTICS | (lem.STEP_SET_OUTLET_FROM_FA if k == 0 else 0)
        g.step(float(rain[k]), float(temp[k]), i >= 0, flags)
        t = g.totals()
        rows.append({k2: t[k2] for k2 in ROWS})
    res = {f: g.get(f) for f in OUT + ("fd", "sfd")}
    g.close()
    return res, rows


@pytest.mark.gpu
@pytest.mark.parametrize("first_iter,steps", [(0, 3), (-2, 2)])
def test_driver_loop_on_the_shim_equals_the_handle_path(driver, first_iter, steps):
    from parallem_gb300 import build, lem
    from parallem_gb300 import scenario as S
    build.build()
    dem = S.make_dem(128, 0.8, 500.0, 0.05, 20, 3, 71)
    st = S.initial_state(dem, 30.0, 900.0, 9.0)
    rng = np.random.default_rng(3)
    rain, temp = rng.uniform(600, 1200, steps), rng.uniform(5, 12, steps)
    got, got_rows = run_driver(driver, dem, st, lem.make_params(), 900.0, 9.0, first_iter, rain, temp)
    want, want_rows = handle_path(dem, st, 900.0, 9.0, first_iter, rain, temp)
    for f in want:
        np.testing.assert_array_equal(got[f], want[f], err_msg=f)
    for a, b in zip(got_rows, want_rows):
        for k in ROWS:
            assert a[k] == b[k] or (np.isnan(a[k]) and np.isnan(b[k])), (k, a[k], b[k])


@pytest.mark.gpu
def test_driver_loop_on_the_shim_matches_the_oracle(driver):
    from oracle import oracle
    from parallem_gb300 import build, lem
    from parallem_gb300 import scenario as S
    from tests.test_gpu_parity import CANCELLING, close
    build.build()
    oracle.build()
    dem = S.make_dem(160, 0.7, 800.0, 0.03, 30, 4, 73)
    st = S.initial_state(dem, 30.0, 900.0, 9.0)
    got, rows = run_driver(driver, dem, st, lem.make_params(), 900.0, 9.0, 0, np.array([950.0]), np.array([8.5]))
    o = oracle.OracleModel(dem, 30.0, st, 900.0, 9.0)
    o.step(950.0, 8.5, True, lem.STEP_SET_OUTLET_FROM_FA | lem.STEP_KEEP_DIAGNOSTICS)
    mask = st["mask"] == 1
    np.testing.assert_array_equal(got["fd"], o["fd"])
    np.testing.assert_array_equal(got["sfd"], o["sfd"])
    close("fa", got["fa"], o["fa"], mask, rtol=1e-5, afrac=0.0)
    close("runoff", got["runoff"], o["runoff"], mask, rtol=1e-6, afrac=0.0)
    for f, of in (("slopeptr", "slopeptr"), ("stone", "stone"), ("fines", "fines"), ("soilT", "soilT"),
                  ("soilM", "soilM"), ("soilB", "soilB"), ("nut", "nut"), ("totB", "totB"), ("ero", "ero"),
                  ("inci", "inci"), ("geli", "geli"), ("depo", "depo")):
        close(f, got[f], o[of], mask, afrac=1e-6 if f in CANCELLING else 0.0)
    close("dz", got["dz"], o["dz"], mask, afrac=1e-6)
    close("dem", got["dem"], o["dem"], mask, rtol=1e-9, afrac=0.0, atol=1e-6)
    r = rows[0]
    assert r["sinkcount"] == o.s.sinkcount and r["outlet"] == o.outlet
    for k, ok in (("tot_e", "totE"), ("tot_i", "totI"), ("tot_g", "totG"), ("tot_d", "totD"),
                  ("tot_weather_c", "totWC"), ("tot_weather_p", "totWP"), ("tot_bio", "totbio"),
                  ("fa_max", "FA_max")):
        assert abs(r[k] - getattr(o.s, ok)) <= 1e-5 * abs(getattr(o.s, ok)) + 1e-12, (k, r[k], getattr(o.s, ok))


def test_reference_driver_links_unchanged_against_the_shim(tmp_path):
    """The reference's own lem.cpp, with its host files Data.cpp, io.cpp,
    memory.cu and MapInfo.cu, compiles and links against liblem_refshim.so in
    place of its FD_kernels, FA_kernels, MOD_kernels and memory_dev.cu objects:
    every stage name it calls is resolved by the shim (no GPU needed).
    Skipped where the reference sources are not present."""
    import shutil
    from oracle import refgpu_build as rg
    rb, lib = _shim()
    if not rg._copy_sources() or not os.path.isfile(os.path.join(rg.SRC, rg.DRIVER)):
        pytest.skip("the reference sources are not present")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = rg.SRC
    exe = str(tmp_path / "lem_on_shim")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O1", "-std=c++17", "-w", "-x", "cu",
           "-include", os.path.join(rg.COMPAT, "compat.h"), "-I", rg.COMPAT, "-I", os.path.join(src, "headers"),
           os.path.join(src, "lem.cpp")] + [os.path.join(src, "MEM_kernels", f) for f in
                                            ("Data.cpp", "io.cpp", "memory.cu", "MapInfo.cu")] + \
          ["-L", rb.LIBDIR, "-llem_refshim", "-llem_gb300", "-Xlinker", "-rpath," + rb.LIBDIR, "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout[-3000:] + res.stderr[-3000:]
    undefined = subprocess.run(["nm", "-uC", exe], capture_output=True, text=True, check=True).stdout
    for name in ("cuFlowDirection", "correctmfdflow", "erosionGPU", "computeRunOffWeights", "createDeviceSpace"):
        assert name in undefined  # taken from the shim library, not from objects of its own
