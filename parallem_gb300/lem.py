"""Python host mirror of the C ABI in include/lem_gb300.h (ctypes).

The reference drives its path from C++ (lem.cpp) through cuFlowDirection,
computeRunOffWeights/calcpropsSFD/correctmfdflow and erosionGPU on a host Data
struct.  ``Model`` offers the same three stage calls and a whole ``step`` on a
handle whose state stays resident on the GPU; fields are copied to or from
numpy arrays only on request.  There is no CPU path: without the CUDA library
every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liblem_gb300.so")

# lem_field
FIELDS = {
    "dem": 0, "mask": 1, "fd": 2, "sfd": 3, "slopes": 4, "slopeptr": 5, "fa": 6, "runoff": 7,
    "stone": 8, "fines": 9, "soilT": 10, "soilM": 11, "soilB": 12, "nut": 13, "totB": 14,
    "ero": 15, "inci": 16, "geli": 17, "depo": 18, "dz": 19, "wC": 20, "wP": 21,
    "contrib": 22, "watershed": 23, "dem_routed": 24, "sfd_pass1": 25,
}
INT_FIELDS = {"mask", "fd", "sfd", "contrib", "watershed", "sfd_pass1"}
STATE_FIELDS = ("stone", "fines", "soilT", "soilM", "soilB", "nut", "totB")

STEP_SET_OUTLET_FROM_FA = 0x1
STEP_KEEP_DIAGNOSTICS = 0x2
STEP_CONTRIB = 0x4

STATUS = {0: "ok", 1: "invalid argument", 2: "capacity exceeded", 3: "iteration cap reached",
          4: "CUDA error", 5: "out of memory", 6: "call out of order"}


class LemError(RuntimeError):
    def __init__(self, code: int, what: str, detail: str = ""):
        super().__init__(f"{what}: {STATUS.get(code, code)} {detail}".strip())
        self.code = code


class GridDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("cellsize", C.c_double)]


class Params(C.Structure):
    _fields_ = [
        ("flow_direction_type", C.c_int32), ("mfd_proportions", C.c_int32),
        ("soil_struct", C.c_int32), ("profile_permeability", C.c_int32),
        ("q_threshold", C.c_double), ("g_slope", C.c_double), ("kappa", C.c_double),
        ("g_flowlim", C.c_double), ("flow_a", C.c_double), ("flow_b", C.c_double),
        ("max_incision", C.c_double), ("ddk", C.c_double), ("dck", C.c_double), ("dgk", C.c_double),
        ("temp_inflex", C.c_double), ("temp_sens", C.c_double),
    ]


class Climate(C.Structure):
    _fields_ = [("rain", C.c_double), ("temp", C.c_double), ("recompute", C.c_int32)]


class Totals(C.Structure):
    _fields_ = [
        ("tot_e", C.c_double), ("tot_i", C.c_double), ("tot_g", C.c_double), ("tot_d", C.c_double),
        ("tot_weather_c", C.c_double), ("tot_weather_p", C.c_double), ("tot_bio", C.c_double),
        ("fa_max", C.c_double), ("rain", C.c_double), ("temp", C.c_double),
        ("sinkcount", C.c_int32), ("outlet", C.c_int32), ("initial_sinks", C.c_int32),
        ("initial_flats", C.c_int32), ("plateau_sweeps", C.c_int32), ("flood_edges", C.c_int32),
        ("fa_uncomputed", C.c_int32), ("sed_uncomputed", C.c_int32),
        ("merge_rounds", C.c_int32), ("label_rounds", C.c_int32), ("spill_rounds", C.c_int32), ("pad", C.c_int32),
    ]


class Tuning(C.Structure):
    _fields_ = [("state", C.c_int32), ("steps_left", C.c_int32), ("coop_blocks", C.c_int32 * 8),
                ("default_ms", C.c_double), ("tuned_ms", C.c_double), ("flowdirs_tile_rows", C.c_int32),
                ("pad", C.c_int32)]


COOP_KERNELS = ("k_plateau_relax", "k_flood_merge", "k_flood_jump", "k_flood_spill", "k_fat_coarse", "k_fa_walk",
                "k_sedt_coarse", "k_sed_walk")


def _tuning(h) -> dict:
    t = Tuning()
    _check(load().lem_get_tuning(h, C.byref(t)), "lem_get_tuning")
    return {"state": ("default", "tuning", "tuned")[t.state], "steps_left": t.steps_left,
            "coop_blocks": dict(zip(COOP_KERNELS, list(t.coop_blocks))),
            "default_ms": t.default_ms, "tuned_ms": t.tuned_ms, "flowdirs_tile_rows": t.flowdirs_tile_rows}


class Limits(C.Structure):
    _fields_ = [("max_rounds", C.c_int32), ("edge_table_log2", C.c_int32)]


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_uint32), ("total_ms", C.c_double)]


# every exported symbol of include/lem_gb300.h with its ctypes signature
_H = C.c_void_p
SIGNATURES = {
    "lem_create": (C.c_int, [C.POINTER(GridDesc), C.POINTER(Params), C.c_double, C.c_double, C.POINTER(_H)]),
    "lem_destroy": (C.c_int, [_H]),
    "lem_set_field": (C.c_int, [_H, C.c_int, C.c_void_p]),
    "lem_get_field": (C.c_int, [_H, C.c_int, C.c_void_p]),
    "lem_set_outlet": (C.c_int, [_H, C.c_int32]),
    "lem_flow_direction": (C.c_int, [_H]),
    "lem_flow_accumulation": (C.c_int, [_H, C.c_uint32]),
    "lem_erosion": (C.c_int, [_H, C.c_uint32]),
    "lem_set_climate": (C.c_int, [_H, C.POINTER(Climate)]),
    "lem_step": (C.c_int, [_H, C.POINTER(Climate), C.c_uint32]),
    "lem_synchronize": (C.c_int, [_H]),
    "lem_get_totals": (C.c_int, [_H, C.POINTER(Totals)]),
    "lem_stream": (C.c_void_p, [_H]),
    "lem_launch_count": (C.c_uint64, [_H]),
    "lem_status_string": (C.c_char_p, [C.c_int]),
    "lem_select_device": (C.c_int, [C.c_int32]),
    "lem_event_record": (C.c_int, [_H, C.c_int32]),
    "lem_event_elapsed": (C.c_int, [_H, C.c_int32, C.c_int32, C.POINTER(C.c_float)]),
    "lem_set_profiling": (C.c_int, [_H, C.c_int32]),
    "lem_profile_read": (C.c_int, [_H, C.POINTER(KernelStat), C.c_int32, C.POINTER(C.c_int32)]),
    "lem_accumulate_flow_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                              C.c_int32, C.c_void_p]),
    "lem_create_batch": (C.c_int, [C.POINTER(GridDesc), C.POINTER(Params), C.c_int32, C.POINTER(_H)]),
    "lem_dem_add": (C.c_int, [_H, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_double, C.c_double,
                              C.POINTER(C.c_int32)]),
    "lem_dem_remove": (C.c_int, [_H, C.c_int32]),
    "lem_dem_set_field": (C.c_int, [_H, C.c_int32, C.c_int, C.c_void_p]),
    "lem_dem_get_field": (C.c_int, [_H, C.c_int32, C.c_int, C.c_void_p]),
    "lem_dem_set_outlet": (C.c_int, [_H, C.c_int32, C.c_int32]),
    "lem_dem_set_climate": (C.c_int, [_H, C.c_int32, C.POINTER(Climate)]),
    "lem_dem_set_step_flags": (C.c_int, [_H, C.c_int32, C.c_uint32]),
    "lem_dem_get_totals": (C.c_int, [_H, C.c_int32, C.POINTER(Totals)]),
    "lem_dem_get_totals_n": (C.c_int, [_H, C.POINTER(C.c_int32), C.c_int32, C.POINTER(Totals)]),
    "lem_step_batch": (C.c_int, [_H, C.c_uint32]),
    "lem_set_graphs": (C.c_int, [_H, C.c_int32]),
    "lem_set_limits": (C.c_int, [_H, C.POINTER(Limits)]),
    "lem_autotune": (C.c_int, [_H, C.c_int32]),
    "lem_get_tuning": (C.c_int, [_H, C.c_void_p]),
    "lem_dem_export": (C.c_int, [_H, C.c_int32, C.POINTER(C.c_int), C.c_int32, C.POINTER(C.c_void_p)]),
    "lem_export_ready": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "lem_export_wait": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "lem_device_bytes": (C.c_size_t, [_H]),
    "lem_snapshot_bytes": (C.c_size_t, [_H, C.c_int32]),
    "lem_snapshot_save": (C.c_int, [_H, C.c_int32, C.c_void_p, C.c_size_t]),
    "lem_snapshot_load": (C.c_int, [_H, C.c_int32, C.c_void_p, C.c_size_t]),
}


def snapshot_save(h, i: int = 0) -> bytes:
    """The restart snapshot of DEM `i` of handle `h` (0 for a single grid)."""
    L = load()
    n = int(L.lem_snapshot_bytes(h, i))
    if n == 0:
        raise LemError(1, "lem_snapshot_bytes")
    buf = (C.c_char * n)()
    _check(L.lem_snapshot_save(h, i, buf, n), "lem_snapshot_save")
    return bytes(buf)


def snapshot_load(h, data: bytes, i: int = 0):
    buf = (C.c_char * len(data)).from_buffer_copy(data)
    _check(load().lem_snapshot_load(h, i, buf, len(data)), "lem_snapshot_load")

class Export:
    """A DEM's fields on their way to the host (lem_dem_export): the copy runs on
    the library's second stream while the handle steps on; wait() returns them."""

    def __init__(self, h, i: int, names, shape):
        self.names = tuple(names)
        self.shape = shape
        fields = (C.c_int * len(self.names))(*[FIELDS[f] for f in self.names])
        e = C.c_void_p()
        _check(load().lem_dem_export(h, i, fields, len(self.names), C.byref(e)), "lem_dem_export")
        self.e = e

    def ready(self) -> bool:
        r = C.c_int32()
        _check(load().lem_export_ready(self.e, C.byref(r)), "lem_export_ready")
        return bool(r.value)

    def wait(self) -> dict:
        hgt, wid = self.shape
        out = {}
        for f in self.names:
            if f in INT_FIELDS:
                out[f] = np.empty((hgt, wid), np.int32)
            elif f == "slopes":
                out[f] = np.empty((hgt, wid, 8), np.float64)
            else:
                out[f] = np.empty((hgt, wid), np.float64)
        ptrs = (C.c_void_p * len(self.names))(*[out[f].ctypes.data for f in self.names])
        e, self.e = self.e, None
        _check(load().lem_export_wait(e, ptrs), "lem_export_wait")
        return out


_lib = None


def load(path: str = LIB_PATH):
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with parallem_gb300.build.build()")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(code: int, what: str):
    if code != 0:
        detail = load().lem_status_string(code).decode() if code == 4 else ""
        raise LemError(code, what, detail)


def make_params(**kw) -> Params:
    from .scenario import DEFAULT_PAR
    d = dict(DEFAULT_PAR, **kw)
    return Params(**{k: d[k] for k, _ in Params._fields_})


class Model:
    """One DEM and its model state resident on the current CUDA device."""

    def __init__(self, dem: np.ndarray, cellsize: float, init_rain: float, init_temp: float,
                 params: Params | None = None, upload: bool = True):
        L = load()
        self.H, self.W = dem.shape
        self.N = self.H * self.W
        self.params = params if params is not None else make_params()
        h = _H()
        _check(L.lem_create(C.byref(GridDesc(self.W, self.H, float(cellsize))), C.byref(self.params),
                            float(init_rain), float(init_temp), C.byref(h)), "lem_create")
        self.h = h
        if upload:
            self.set("dem", dem)

    def snapshot(self) -> bytes:
        return snapshot_save(self.h, 0)

    def restore(self, data: bytes):
        snapshot_load(self.h, data, 0)

    def close(self):
        if getattr(self, "h", None):
            load().lem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- fields ---------------------------------------------------------------
    def set(self, name: str, arr: np.ndarray):
        n = 8 * self.N if name == "slopes" else self.N
        a = np.ascontiguousarray(arr, dtype=np.int32 if name in INT_FIELDS else np.float64).reshape(-1)
        if a.size != n:
            raise ValueError(f"{name}: expected {n} values, got {a.size}")
        _check(load().lem_set_field(self.h, FIELDS[name], a.ctypes.data), f"lem_set_field({name})")

    def get(self, name: str) -> np.ndarray:
        if name in INT_FIELDS:
            out = np.empty((self.H, self.W), np.int32)
        elif name == "slopes":
            out = np.empty((self.H, self.W, 8), np.float64)
        else:
            out = np.empty((self.H, self.W), np.float64)
        _check(load().lem_get_field(self.h, FIELDS[name], out.ctypes.data), f"lem_get_field({name})")
        return out

    def set_state(self, state: dict):
        for f in STATE_FIELDS:
            if f in state:
                self.set(f, state[f])
        if "slopes" in state:
            self.set("slopes", state["slopes"])
        if "outlet" in state:
            _check(load().lem_set_outlet(self.h, int(state["outlet"])), "lem_set_outlet")

    # -- the path ---------------------------------------------------------------
    def flow_direction(self):
        _check(load().lem_flow_direction(self.h), "lem_flow_direction")

    def flow_accumulation(self, flags: int = 0):
        _check(load().lem_flow_accumulation(self.h, flags), "lem_flow_accumulation")

    def erosion(self, flags: int = 0):
        _check(load().lem_erosion(self.h, flags), "lem_erosion")

    def set_climate(self, rain: float, temp: float, recompute: bool):
        _check(load().lem_set_climate(self.h, C.byref(Climate(rain, temp, int(bool(recompute))))), "lem_set_climate")

    def step(self, rain: float, temp: float, recompute: bool, flags: int = 0):
        _check(load().lem_step(self.h, C.byref(Climate(rain, temp, int(bool(recompute)))), flags), "lem_step")

    def synchronize(self):
        _check(load().lem_synchronize(self.h), "lem_synchronize")

    def totals(self) -> dict:
        t = Totals()
        _check(load().lem_get_totals(self.h, C.byref(t)), "lem_get_totals")
        return {k: getattr(t, k) for k, _ in Totals._fields_}

    @property
    def stream(self) -> int:
        return int(load().lem_stream(self.h) or 0)

    @property
    def launches(self) -> int:
        return int(load().lem_launch_count(self.h))

    def record(self, slot: int):
        _check(load().lem_event_record(self.h, slot), "lem_event_record")

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        _check(load().lem_event_elapsed(self.h, a, b, C.byref(ms)), "lem_event_elapsed")
        return float(ms.value)

    def profiling(self, on: bool):
        _check(load().lem_set_profiling(self.h, int(bool(on))), "lem_set_profiling")

    def graphs(self, on: bool):
        """Steps launch as one captured CUDA graph (lem_set_graphs)."""
        _check(load().lem_set_graphs(self.h, int(bool(on))), "lem_set_graphs")

    def autotune(self, cycles: int = 1):
        """The next 1 + 4 * cycles steps tune the launch schedule (lem_autotune)."""
        _check(load().lem_autotune(self.h, int(cycles)), "lem_autotune")

    def tuning(self) -> dict:
        return _tuning(self.h)

    def limits(self, max_rounds: int = 0, edge_table_log2: int = 0):
        """Caps of the device loops and of the basin-pair table (lem_set_limits; 0 = default)."""
        _check(load().lem_set_limits(self.h, C.byref(Limits(int(max_rounds), int(edge_table_log2)))),
               "lem_set_limits")

    def profile(self) -> dict:
        """{kernel name: (launches, total device ms)} since the previous read."""
        arr = (KernelStat * 64)()
        n = C.c_int32()
        _check(load().lem_profile_read(self.h, arr, 64, C.byref(n)), "lem_profile_read")
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms)) for i in range(min(n.value, 64))}


def select_device(device: int):
    _check(load().lem_select_device(int(device)), "lem_select_device")


class Batch:
    """Many DEMs stepped together (lem_create_batch): one canvas grid, each DEM
    in its own 32-aligned region with its own outlet, climate and totals.  One
    step runs every active DEM with one launch per kernel."""

    def __init__(self, width: int, height: int, cellsize: float, max_dems: int = 256,
                 params: Params | None = None):
        from .packing import TilePacker
        L = load()
        self.W, self.H = int(width), int(height)
        self.params = params if params is not None else make_params()
        h = _H()
        _check(L.lem_create_batch(C.byref(GridDesc(self.W, self.H, float(cellsize))), C.byref(self.params),
                                  int(max_dems), C.byref(h)), "lem_create_batch")
        self.h = h
        self.packer = TilePacker(self.W, self.H)
        self.shape = {}   # id -> (height, width)
        self.place = {}   # id -> region handle of the packer

    def close(self):
        if getattr(self, "h", None):
            load().lem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, dem: np.ndarray, init_rain: float, init_temp: float, at: tuple | None = None) -> int:
        """Places the DEM (first fit unless `at` = (x0, y0)) and uploads it; None when it does not fit."""
        hgt, wid = dem.shape
        if at is None:
            r = self.packer.alloc(wid, hgt)
            if r is None:
                return None
            x0, y0 = r[0], r[1]
        else:
            x0, y0 = at
            r = self.packer.take(x0, y0, wid, hgt)
        a = np.ascontiguousarray(dem, dtype=np.float64)
        i = C.c_int32()
        code = load().lem_dem_add(self.h, x0, y0, wid, hgt, a.ctypes.data, float(init_rain), float(init_temp),
                                  C.byref(i))
        if code != 0:
            self.packer.free(r)
            _check(code, "lem_dem_add")
        self.shape[i.value] = (hgt, wid)
        self.place[i.value] = r
        return i.value

    def export(self, i: int, names) -> Export:
        """Starts the asynchronous copy of DEM i's fields `names` to the host."""
        return Export(self.h, i, names, self.shape[i])

    def device_bytes(self) -> int:
        return int(load().lem_device_bytes(self.h))

    def remove(self, i: int):
        _check(load().lem_dem_remove(self.h, i), "lem_dem_remove")
        self.packer.free(self.place.pop(i))
        self.shape.pop(i)

    def set(self, i: int, name: str, arr: np.ndarray):
        hgt, wid = self.shape[i]
        n = 8 * hgt * wid if name == "slopes" else hgt * wid
        a = np.ascontiguousarray(arr, dtype=np.int32 if name in INT_FIELDS else np.float64).reshape(-1)
        if a.size != n:
            raise ValueError(f"{name}: expected {n} values, got {a.size}")
        _check(load().lem_dem_set_field(self.h, i, FIELDS[name], a.ctypes.data), f"lem_dem_set_field({name})")

    def get(self, i: int, name: str) -> np.ndarray:
        hgt, wid = self.shape[i]
        if name in INT_FIELDS:
            out = np.empty((hgt, wid), np.int32)
        elif name == "slopes":
            out = np.empty((hgt, wid, 8), np.float64)
        else:
            out = np.empty((hgt, wid), np.float64)
        _check(load().lem_dem_get_field(self.h, i, FIELDS[name], out.ctypes.data), f"lem_dem_get_field({name})")
        return out

    def set_state(self, i: int, state: dict):
        for f in STATE_FIELDS:
            if f in state:
                self.set(i, f, state[f])
        if "slopes" in state:
            self.set(i, "slopes", state["slopes"])
        _check(load().lem_dem_set_outlet(self.h, i, int(state["outlet"])), "lem_dem_set_outlet")

    def set_climate(self, i: int, rain: float, temp: float, recompute: bool):
        _check(load().lem_dem_set_climate(self.h, i, C.byref(Climate(rain, temp, int(bool(recompute))))),
               "lem_dem_set_climate")

    def set_step_flags(self, i: int, flags: int):
        _check(load().lem_dem_set_step_flags(self.h, i, int(flags)), "lem_dem_set_step_flags")

    def step(self, flags: int = 0):
        _check(load().lem_step_batch(self.h, int(flags)), "lem_step_batch")

    def synchronize(self):
        _check(load().lem_synchronize(self.h), "lem_synchronize")

    def snapshot(self, i: int) -> bytes:
        return snapshot_save(self.h, i)

    def restore(self, i: int, data: bytes):
        snapshot_load(self.h, data, i)

    def totals(self, i: int) -> dict:
        t = Totals()
        _check(load().lem_dem_get_totals(self.h, i, C.byref(t)), "lem_dem_get_totals")
        return {k: getattr(t, k) for k, _ in Totals._fields_}

    def totals_n(self, ids) -> list:
        """The budget rows of several DEMs after one synchronisation."""
        n = len(ids)
        idv = (C.c_int32 * n)(*ids)
        out = (Totals * n)()
        _check(load().lem_dem_get_totals_n(self.h, idv, n, out), "lem_dem_get_totals_n")
        return [{k: getattr(t, k) for k, _ in Totals._fields_} for t in out]

    @property
    def stream(self) -> int:
        return int(load().lem_stream(self.h) or 0)

    @property
    def launches(self) -> int:
        return int(load().lem_launch_count(self.h))

    def record(self, slot: int):
        _check(load().lem_event_record(self.h, slot), "lem_event_record")

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        _check(load().lem_event_elapsed(self.h, a, b, C.byref(ms)), "lem_event_elapsed")
        return float(ms.value)

    def profiling(self, on: bool):
        _check(load().lem_set_profiling(self.h, int(bool(on))), "lem_set_profiling")

    def graphs(self, on: bool):
        """Steps launch as one captured CUDA graph (lem_set_graphs)."""
        _check(load().lem_set_graphs(self.h, int(bool(on))), "lem_set_graphs")

    def autotune(self, cycles: int = 1):
        """The next 1 + 4 * cycles steps tune the launch schedule (lem_autotune)."""
        _check(load().lem_autotune(self.h, int(cycles)), "lem_autotune")

    def tuning(self) -> dict:
        return _tuning(self.h)

    def profile(self) -> dict:
        arr = (KernelStat * 64)()
        n = C.c_int32()
        _check(load().lem_profile_read(self.h, arr, 64, C.byref(n)), "lem_profile_read")
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms)) for i in range(min(n.value, 64))}
