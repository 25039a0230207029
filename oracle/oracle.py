"""ctypes binding of the FP64 CPU oracle (oracle/lem_oracle.cpp).

TEST INFRASTRUCTURE: used by tests/, __graft_entry__.smoke() and bench.py's CPU
legs as the checker.  The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liblem_oracle.so")

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)
_F = C.POINTER(C.c_float)


class LemParams(C.Structure):
    _fields_ = [
        ("flow_direction_type", C.c_int32), ("mfd_proportions", C.c_int32),
        ("soil_struct", C.c_int32), ("profile_permeability", C.c_int32),
        ("q_threshold", C.c_double), ("g_slope", C.c_double), ("kappa", C.c_double),
        ("g_flowlim", C.c_double), ("flow_a", C.c_double), ("flow_b", C.c_double),
        ("max_incision", C.c_double), ("ddk", C.c_double), ("dck", C.c_double), ("dgk", C.c_double),
        ("temp_inflex", C.c_double), ("temp_sens", C.c_double),
    ]


class LemClimate(C.Structure):
    _fields_ = [("rain", C.c_double), ("temp", C.c_double), ("recompute", C.c_int32)]


_FP_FIELDS = ["dem", "mask", "slopes", "prop", "fd", "sfd", "fa", "runoff", "slopeptr", "stone", "fines",
              "soilT", "soilM", "soilB", "nut", "totB", "ero", "inci", "geli", "depo", "dz", "wC", "wP",
              "rainmat", "tempmat", "last_rainmat", "last_tempmat", "shortest_paths", "watershed", "contrib",
              "dem_routed", "sfd_pass1"]
_TYPES = {"mask": _I, "fd": _I, "sfd": _I, "shortest_paths": _F, "watershed": _I, "contrib": _I, "sfd_pass1": _I}


class OracleStateC(C.Structure):
    _fields_ = ([("W", C.c_int32), ("H", C.c_int32), ("cellsize", C.c_double)]
                + [(f, _TYPES.get(f, _D)) for f in _FP_FIELDS]
                + [("outlet", C.c_int32), ("rain", C.c_double), ("temp", C.c_double),
                   ("last_rain", C.c_double), ("last_temp", C.c_double),
                   ("totE", C.c_double), ("totI", C.c_double), ("totG", C.c_double), ("totD", C.c_double),
                   ("totWC", C.c_double), ("totWP", C.c_double), ("totbio", C.c_double), ("FA_max", C.c_double),
                   ("sinkcount", C.c_int32), ("init_sinks", C.c_int32), ("init_flats", C.c_int32),
                   ("plateau_sweeps", C.c_int32), ("flood_basins", C.c_int32),
                   ("fa_uncomputed", C.c_int32), ("sed_uncomputed", C.c_int32)])


def build(quiet: bool = True) -> str:
    """Compile the oracle library with its Makefile (idempotent)."""
    cmd = ["make", "-C", _HERE]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL if quiet else None)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        P = C.POINTER(OracleStateC)
        L.oracle_set_climate.argtypes = [P, C.c_int]
        L.oracle_flow_direction.argtypes = [P, C.POINTER(LemParams)]
        L.oracle_flow_accumulation.argtypes = [P, C.POINTER(LemParams), C.c_uint32]
        L.oracle_erosion.argtypes = [P, C.POINTER(LemParams)]
        L.oracle_step.argtypes = [P, C.POINTER(LemParams), C.POINTER(LemClimate), C.c_uint32]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_num_threads.restype = C.c_int
        _lib = L
    return _lib


def make_params(**kw) -> LemParams:
    from parallem_gb300.scenario import DEFAULT_PAR
    d = dict(DEFAULT_PAR, **kw)
    return LemParams(**{k: d[k] for k, _ in LemParams._fields_})


class OracleModel:
    """The reference's host Data state as fp64 numpy arrays plus the oracle calls."""

    def __init__(self, dem: np.ndarray, cellsize: float, state: dict, init_rain: float, init_temp: float,
                 params: LemParams | None = None, diagnostics: bool = True):
        h, w = dem.shape
        n = h * w
        self.H, self.W, self.cellsize = h, w, float(cellsize)
        self.params = params if params is not None else make_params()
        a = {}
        a["dem"] = np.ascontiguousarray(dem, dtype=np.float64).copy()
        a["mask"] = np.ascontiguousarray(state["mask"], dtype=np.int32).reshape(h, w).copy()
        for f in ("fa", "runoff", "slopeptr", "ero", "inci", "geli", "depo", "dz", "wC", "wP",
                  "rainmat", "tempmat", "last_rainmat", "last_tempmat"):
            a[f] = np.zeros((h, w), np.float64)
        for f in ("stone", "fines", "soilT", "soilM", "soilB", "nut", "totB"):
            a[f] = np.ascontiguousarray(state[f], dtype=np.float64).reshape(h, w).copy()
        a["slopes"] = np.zeros((h, w, 8), np.float64)
        a["prop"] = np.zeros((h, w, 8), np.float64)
        a["fd"] = np.zeros((h, w), np.int32)
        a["sfd"] = np.zeros((h, w), np.int32)
        a["shortest_paths"] = np.zeros((h, w), np.float32) if diagnostics else None
        a["watershed"] = np.zeros((h, w), np.int32) if diagnostics else None
        a["contrib"] = np.zeros((h, w), np.int32) if diagnostics else None
        a["dem_routed"] = np.zeros((h, w), np.float64) if diagnostics else None
        a["sfd_pass1"] = np.zeros((h, w), np.int32) if diagnostics else None
        self.a = a
        self.s = OracleStateC()
        self.s.W, self.s.H, self.s.cellsize = w, h, self.cellsize
        for f in _FP_FIELDS:
            arr = a[f]
            setattr(self.s, f, arr.ctypes.data_as(_TYPES.get(f, _D)) if arr is not None else None)
        self.s.outlet = int(state["outlet"])
        self.s.rain, self.s.temp = float(init_rain), float(init_temp)
        self.s.last_rain, self.s.last_temp = float(init_rain), float(init_temp)
        lib().oracle_set_climate(C.byref(self.s), 1)

    def __getitem__(self, name):
        return self.a[name]

    @property
    def outlet(self):
        return int(self.s.outlet)

    def set_arrays(self, **fields):
        for k, v in fields.items():
            self.a[k][...] = np.asarray(v).reshape(self.a[k].shape)

    def flow_direction(self):
        lib().oracle_flow_direction(C.byref(self.s), C.byref(self.params))

    def flow_accumulation(self, flags: int = 0):
        lib().oracle_flow_accumulation(C.byref(self.s), C.byref(self.params), flags)

    def erosion(self):
        lib().oracle_erosion(C.byref(self.s), C.byref(self.params))

    def step(self, rain: float, temp: float, recompute: bool, flags: int = 0):
        c = LemClimate(rain, temp, 1 if recompute else 0)
        lib().oracle_step(C.byref(self.s), C.byref(self.params), C.byref(c), flags)

    def totals(self) -> dict:
        s = self.s
        return dict(tot_e=s.totE, tot_i=s.totI, tot_g=s.totG, tot_d=s.totD, tot_weather_c=s.totWC,
                    tot_weather_p=s.totWP, tot_bio=s.totbio, fa_max=s.FA_max, sinkcount=s.sinkcount,
                    outlet=s.outlet, initial_sinks=s.init_sinks, initial_flats=s.init_flats,
                    flood_basins=s.flood_basins, fa_uncomputed=s.fa_uncomputed,
                    sed_uncomputed=s.sed_uncomputed)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def num_threads() -> int:
    return int(lib().oracle_num_threads())


# --- the reference's own kernels run on the CPU (oracle/_ref, built from the
# reference sources by oracle/ref_build.py; absent where the sources are) ---
_ref = None


def ref_lib():
    """ctypes handle of oracle/_ref/libref.so, or None when it cannot be built."""
    global _ref
    if _ref is None:
        from oracle import ref_build
        path = ref_build.build()
        if path is None:
            return None
        L = C.CDLL(path)
        P = C.POINTER(OracleStateC)
        L.ref_flow_direction.argtypes = [P, C.POINTER(LemParams)]
        L.ref_flow_accumulation.argtypes = [P, C.POINTER(LemParams), C.c_uint32]
        L.ref_erosion.argtypes = [P, C.POINTER(LemParams)]
        _ref = L
    return _ref


class RefModel(OracleModel):
    """Same state as OracleModel; the stages run the reference's kernels."""

    def flow_direction(self):
        ref_lib().ref_flow_direction(C.byref(self.s), C.byref(self.params))

    def flow_accumulation(self, flags: int = 0):
        ref_lib().ref_flow_accumulation(C.byref(self.s), C.byref(self.params), flags)

    def erosion(self):
        ref_lib().ref_erosion(C.byref(self.s), C.byref(self.params))

    def step(self, rain: float, temp: float, recompute: bool, flags: int = 0):
        if recompute:
            self.s.last_rain, self.s.last_temp = self.s.rain, self.s.temp
            self.s.rain, self.s.temp = float(rain), float(temp)
            lib().oracle_set_climate(C.byref(self.s), 0)
        self.flow_direction()
        self.flow_accumulation(flags)
        self.erosion()
