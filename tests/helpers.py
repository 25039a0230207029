"""Shared set-up of the tests: identical initial states for the oracle and the GPU."""
from __future__ import annotations

import numpy as np

from parallem_gb300 import scenario as S

NODATA = -9999.0
CODE = {0: 64, 1: 128, 2: 1, 3: 2, 4: 4, 5: 8, 6: 16, 7: 32}  # direction index -> MFD bit


def state_for(dem: np.ndarray, cellsize: float = 30.0, rain: float = 800.0, temp: float = 10.0, **soil):
    st = S.initial_state(dem, cellsize, rain, temp, soil=soil or None)
    return st


def oracle_model(dem, cellsize=30.0, rain=800.0, temp=10.0, params=None, **soil):
    from oracle.oracle import OracleModel, make_params
    st = state_for(dem, cellsize, rain, temp, **soil)
    return OracleModel(dem, cellsize, st, rain, temp, params if params is not None else make_params())


def ringed(interior: np.ndarray, width: int = 1) -> np.ndarray:
    """Surrounds a block of elevations with a nodata border."""
    h, w = interior.shape
    out = np.full((h + 2 * width, w + 2 * width), NODATA)
    out[width:width + h, width:width + w] = interior
    return out
