"""Placement of DEMs in a batch canvas, at the 32-cell granularity of the tiles.

A DEM of w x h cells occupies ceil(w/32) x ceil(h/32) tiles of the canvas, so
two DEMs never share a tile.  First fit in row-major tile order, with an
integral image of the occupied tiles to test a block in O(1).
"""
from __future__ import annotations

import numpy as np

TILE = 32


class TilePacker:
    def __init__(self, width: int, height: int):
        self.tw, self.th = width // TILE, height // TILE
        self.occ = np.zeros((self.th, self.tw), np.int32)

    def _free_blocks(self, bw: int, bh: int) -> np.ndarray:
        s = np.zeros((self.th + 1, self.tw + 1), np.int64)
        s[1:, 1:] = self.occ.cumsum(0).cumsum(1)
        if bh > self.th or bw > self.tw:
            return np.zeros((0, 0), bool)
        area = s[bh:, bw:] - s[:-bh, bw:] - s[bh:, :-bw] + s[:-bh, :-bw]
        return area == 0

    def alloc(self, w: int, h: int):
        """(x0, y0, bw, bh) of a free block for a w x h DEM, or None."""
        bw, bh = -(-w // TILE), -(-h // TILE)
        free = self._free_blocks(bw, bh)
        if free.size == 0 or not free.any():
            return None
        ty, tx = np.unravel_index(int(np.argmax(free)), free.shape)
        self.occ[ty:ty + bh, tx:tx + bw] = 1
        return (int(tx) * TILE, int(ty) * TILE, bw, bh)

    def take(self, x0: int, y0: int, w: int, h: int):
        bw, bh = -(-w // TILE), -(-h // TILE)
        tx, ty = x0 // TILE, y0 // TILE
        self.occ[ty:ty + bh, tx:tx + bw] = 1
        return (x0, y0, bw, bh)

    def free(self, r):
        x0, y0, bw, bh = r
        tx, ty = x0 // TILE, y0 // TILE
        self.occ[ty:ty + bh, tx:tx + bw] = 0

    def used_fraction(self) -> float:
        return float(self.occ.mean())
