"""PARALLEM's own CUDA build on the GPU, beside this path, through the same loop.

oracle/refgpu_build.py compiles the reference's hot-path sources unchanged for
sm_103a, with oracle/refgpu/harness.cu in place of lem.cpp.  The harness runs
lem.cpp's set-up and timestep loop on them; tests/refshim/driver.cpp runs the
same loop on liblem_refshim.so (this path behind the reference's names).  Both
start from the same DEM and state.

gpu checks, one step: wherever the reference's direction code differs from the
oracle's, it points to another neighbour that attains the cell's plateau
distance on the routed DEM (a plateau tie, whose winner depends on the
reference's thread order), and its budget totals agree with the oracle's to
2 % (concentrated erosion 10 %) and with this path's after three steps to 5 %
(15 %): the tie choices move water and sediment between paths.  Lines starting
REFGPU give the wall-clock milliseconds per stage of both implementations
(each stage call with its setdevicespace_*/cleardevicespace_* calls, host
mirrors included).  LEM_REFGPU_LARGE=1 adds the 4080x4096 grid.

Sizes the reference's kernels need.  init_watershedMFD and
init_watershed_sinkMFD (FD_kernels/newflow.cu:352-460) test only the row
bound, and every launch has one spare block column (FD_kernels/routeflow.cu:718:
ncell_x / 16 + 1 blocks).  Threads past the last column wrap onto the first 16
cells of the next row, and on the last row they reach up to 16 elements past
the end of the mask, SFD, watershed and DEM arrays.  So the inputs here keep
their first 16 columns nodata (wrapped threads then meet nodata cells and write
what those cells' own threads write), and have sizes whose int and double
arrays are at least 2 MiB and end inside a 2 MiB page, so the elements read or
written past the end are mapped memory of the same allocation.
init_hash_tableMFD (newflow.cu:734-746) writes one row and column past its
30000 x 800 x 3 table (routeflow.cu:398-407); that table ends 700 KB short of a
page boundary.  Skipped where the reference sources are not present.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

from tests.test_refshim import OUT, ROWS, SOIL, run_driver

pytestmark = pytest.mark.gpu

PAGE = 2 << 20


def safe_shape(w, h):
    """(w, h) is a size the reference's kernels stay in mapped memory at."""
    n = w * h
    for elem, over in ((4, 16 * 4), (8, 16 * 8)):
        rem = (n * elem) % PAGE
        if n * elem < PAGE or rem == 0 or PAGE - rem < over:
            return False
    return True


def prepared_dem(w, h, seed):
    from parallem_gb300 import scenario as S
    assert safe_shape(w, h)
    dem = S.make_dem(max(w, h), 0.7, 1500.0, 0.02, int(5000 * w * h / 4096 ** 2), int(300 * w * h / 4096 ** 2),
                     seed)[:h, :w].copy()
    dem[:, :16] = S.NODATA  # the first 16 columns nodata (see the module docstring)
    dem[:2, :] = dem[-2:, :] = S.NODATA
    dem[:, -2:] = S.NODATA
    return dem


@pytest.fixture(scope="module")
def ref_gpu():
    from oracle import refgpu_build
    lib = refgpu_build.build()
    if lib is None:
        pytest.skip("the reference sources are not present")
    L = C.CDLL(lib)
    P = C.c_void_p
    L.refgpu_run.argtypes = [C.c_int, C.c_int, C.c_double, P, P, P, C.c_double, C.c_double, C.c_int, C.c_int, P, P,
                             P, P, P, P, C.c_char_p]
    L.refgpu_run.restype = C.c_int
    return L


def run_reference(L, dem, st, params, rain, temp, first_iter=0):
    H, W = dem.shape
    steps = len(rain)
    soil = np.ascontiguousarray(np.stack([st[f] for f in SOIL]), np.float64)
    out = np.zeros((16, H, W))
    codes = np.zeros((2, H, W), np.int32)
    rows = np.zeros((steps, 10))
    ms = np.zeros((steps, 4))
    d = np.ascontiguousarray(dem, np.float64)
    r = np.ascontiguousarray(rain, np.float64)
    t = np.ascontiguousarray(temp, np.float64)
    rc = L.refgpu_run(W, H, 30.0, d.ctypes.data, soil.ctypes.data, C.addressof(params), 900.0, 9.0, first_iter, steps,
                      r.ctypes.data, t.ctypes.data, out.ctypes.data, codes.ctypes.data, rows.ctypes.data,
                      ms.ctypes.data, None)
    assert rc == 0
    res = {f: out[k] for k, f in enumerate(OUT)}
    res["fd"], res["sfd"] = codes[0], codes[1]
    return res, [dict(zip(ROWS, row)) for row in rows], ms


def compare_and_time(ref_gpu, w, h, steps, seed):
    """One step of the reference build against the oracle; returns the inputs
    for the timed runs."""
    from oracle import oracle
    from parallem_gb300 import build, lem
    from parallem_gb300 import scenario as S
    build.build()
    oracle.build()
    dem = prepared_dem(w, h, seed)
    st = S.initial_state(dem, 30.0, 900.0, 9.0)
    mask = st["mask"] == 1
    rng = np.random.default_rng(seed)
    rain, temp = rng.uniform(700, 1100, steps), rng.uniform(7, 11, steps)
    params = lem.make_params()
    ref, ref_rows, ref_ms = run_reference(ref_gpu, dem, st, params, rain[:1], temp[:1])
    # one step from the same state: the reference against the oracle
    o = oracle.OracleModel(dem, 30.0, st, 900.0, 9.0)
    o.step(float(rain[0]), float(temp[0]), True, lem.STEP_SET_OUTLET_FROM_FA)
    differ = (ref["sfd"] != o["sfd"]) & mask
    share = float(differ.sum()) / float(mask.sum())
    bad = plateau_tie_violations(ref["sfd"], o, differ)
    # totals: 2 %, concentrated erosion 10 %: incision starts at an accumulation
    # threshold and grows as its 1.3th power, so it concentrates on the flow
    # paths that the tie choices move across filled basins
    tot = {"tot_e": ("totE", 0.02), "tot_i": ("totI", 0.10), "tot_g": ("totG", 0.02), "tot_d": ("totD", 0.02),
           "tot_bio": ("totbio", 0.02)}
    far = {k: (ref_rows[0][k], getattr(o.s, ok)) for k, (ok, rel) in tot.items()
           if abs(ref_rows[0][k] - getattr(o.s, ok)) > rel * abs(getattr(o.s, ok)) + 1e-9}
    return dem, st, params, rain, temp, ref_ms, share, bad, far


def plateau_tie_violations(ref_sfd, o, differ) -> int:
    """Cells where the reference's direction differs from the oracle's and is
    not another neighbour attaining the cell's plateau distance on the routed
    DEM (the oracle's distances are the relaxation's unique fixpoint, so the
    reference's are the same; only the winner among tied neighbours depends on
    its thread order)."""
    H, W = ref_sfd.shape
    z, sp = o["dem_routed"], o["shortest_paths"].astype(np.float32)
    dxl, dyl, dcl, okl = (np.zeros(256, np.int64), np.zeros(256, np.int64), np.zeros(256, np.float32),
                          np.zeros(256, bool))
    for code, (dx, dy, dc) in {64: (0, -1, 1.0), 128: (1, -1, 1.41), 1: (1, 0, 1.0), 2: (1, 1, 1.41),
                               4: (0, 1, 1.0), 8: (-1, 1, 1.41), 16: (-1, 0, 1.0), 32: (-1, -1, 1.41)}.items():
        dxl[code], dyl[code], dcl[code], okl[code] = dx, dy, dc, True
    ys, xs = np.nonzero(differ)
    codes = ref_sfd[ys, xs]
    single = (codes >= 0) & (codes < 256)
    c = np.where(single, codes, 0)
    valid = single & okl[c]
    ny, nx = ys + dyl[c], xs + dxl[c]
    inside = valid & (nx >= 0) & (nx < W) & (ny >= 0) & (ny < H)
    nyc, nxc = np.clip(ny, 0, H - 1), np.clip(nx, 0, W - 1)
    tie = inside & (z[nyc, nxc] == z[ys, xs]) & ((sp[nyc, nxc] + dcl[c]).astype(np.float32) == sp[ys, xs])
    return int((~tie).sum())


def test_reference_build_runs_and_agrees_with_the_oracle_and_this_path(ref_gpu, tmp_path_factory):
    w, h, steps = 1000, 1024, 3
    dem, st, params, rain, temp, _, share, bad, far = compare_and_time(ref_gpu, w, h, steps, 81)
    # timing: the same loop, several steps, both implementations
    _, ref_rows, ref_ms = run_reference(ref_gpu, dem, st, params, rain, temp)
    L = _driver(tmp_path_factory)
    ms = np.zeros((steps, 4))
    ours, rows = run_driver(L, dem, st, params, 900.0, 9.0, 0, rain, temp, stage_ms=ms)
    report(w, h, dem, ref_ms, ms, share, bad)
    assert bad == 0, f"{bad} cells take a direction that is not a plateau tie"
    assert not far, far
    for k, rel in (("tot_e", 0.05), ("tot_i", 0.15), ("tot_g", 0.05), ("tot_d", 0.05), ("tot_bio", 0.05)):
        for a, b in zip(rows, ref_rows):
            assert abs(a[k] - b[k]) <= rel * abs(b[k]) + 1e-9, (k, a[k], b[k])


def _driver(tmp_path_factory):
    import subprocess
    from parallem_gb300.refshim import build as rb
    from tests.conftest import ROOT
    lib = rb.build()
    if lib is None:
        pytest.skip("the reference headers are not present")
    d = tmp_path_factory.mktemp("refshim_t")
    so = str(d / "driver.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", "-I", rb.headers_dir(), "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "refshim", "driver.cpp"), "-L",
                    rb.LIBDIR, "-llem_refshim", "-llem_gb300", "-Wl,-rpath," + rb.LIBDIR, "-o", so], check=True)
    L = C.CDLL(so)
    P = C.c_void_p
    L.refshim_run.argtypes = [C.c_int, C.c_int, C.c_double, P, P, C.c_int, P, C.c_double, C.c_double, C.c_int,
                              C.c_int, P, P, P, P, P, P]
    L.refshim_run.restype = C.c_int
    return L


def report(w, h, dem, ref_ms, ms, share, bad):
    cells = int((dem != -9999).sum())
    line = {"grid": f"{w}x{h}", "active_cells": cells, "steps": len(ms), "direction_differs_share": share,
            "differs_not_a_plateau_tie": bad,
            "reference_ms_per_stage": ref_ms.mean(axis=0).round(3).tolist(),
            "this_path_via_shim_ms_per_stage": ms.mean(axis=0).round(3).tolist(),
            "stages": ["flow direction", "accumulation", "erosion", "step"],
            "reference_cell_timesteps_per_s": cells / (ref_ms[:, 3].mean() / 1e3),
            "this_path_via_shim_cell_timesteps_per_s": cells / (ms[:, 3].mean() / 1e3)}
    print("REFGPU " + json.dumps(line))


@pytest.mark.skipif(os.environ.get("LEM_REFGPU_LARGE") != "1", reason="LEM_REFGPU_LARGE=1 runs the 4080x4096 grid")
def test_reference_build_on_the_large_grid(ref_gpu, tmp_path_factory):
    w, h, steps = 4080, 4096, 2
    dem, st, params, rain, temp, _, share, bad, far = compare_and_time(ref_gpu, w, h, 1, 82)
    _, ref_rows, ref_ms = run_reference(ref_gpu, dem, st, params, rain[:1].repeat(steps), temp[:1].repeat(steps))
    L = _driver(tmp_path_factory)
    ms = np.zeros((steps, 4))
    run_driver(L, dem, st, params, 900.0, 9.0, 0, rain[:1].repeat(steps), temp[:1].repeat(steps), stage_ms=ms)
    report(w, h, dem, ref_ms, ms, share, bad)
    assert bad == 0, f"{bad} cells take a direction that is not a plateau tie"
    assert not far, far
