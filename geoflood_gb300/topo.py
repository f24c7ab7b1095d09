"""Topography (DEM) sets: GeoClaw topo files read on the host and the
cell-averaged bathymetry computed on the device (``gf_topo_*`` in
include/geoflood_gb300.h).

    topo = Topo()
    topo.read_data("topo.data")            # or read_file(path, topo_type)
    b = topo.raster(ctx, nx, ny, 2, x0, y0, dx, dy, xupper, yupper)
    forest = Forest(ctx, mx, nbx, nby, lmin, lmax, dx0, dy0, None, None)
    forest.set_topo(topo)                  # setaux + sea-level qinit per level
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import GeoFloodError, _lib
from ._lib import dptr


def _ok(rc: int, what: str):
    if rc != 0:
        raise GeoFloodError(rc, what)


class Topo:
    def __init__(self, topo_missing: float | None = None):
        self._lib = _lib.load()
        h = C.c_void_p()
        _ok(self._lib.gf_topo_create(C.byref(h)), "gf_topo_create")
        self.h = h
        if topo_missing is not None:
            self.set_missing(topo_missing)

    def close(self):
        if getattr(self, "h", None):
            self._lib.gf_topo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_missing(self, topo_missing: float):
        _ok(self._lib.gf_topo_set_missing(self.h, topo_missing), "gf_topo_set_missing")

    def read_file(self, path: str, topo_type: int):
        _ok(self._lib.gf_topo_read_file(self.h, os.fsencode(path), topo_type),
            "gf_topo_read_file(%s)" % path)

    def read_data(self, path: str):
        _ok(self._lib.gf_topo_read_data(self.h, os.fsencode(path)), "gf_topo_read_data(%s)" % path)

    def add_grid(self, z: np.ndarray, xll: float, yll: float, dx: float, dy: float):
        """z: (my, mx) node values, row 0 the northernmost (file order)."""
        z = np.ascontiguousarray(z, np.float64)
        my, mx = z.shape
        _ok(self._lib.gf_topo_add_grid(self.h, mx, my, xll, yll, dx, dy, dptr(z)), "gf_topo_add_grid")

    def __len__(self) -> int:
        return int(self._lib.gf_topo_count(self.h))

    def grid(self, k: int) -> dict:
        mx, my = C.c_int(), C.c_int()
        v = [C.c_double() for _ in range(6)]
        _ok(self._lib.gf_topo_grid_info(self.h, k, C.byref(mx), C.byref(my), *(C.byref(x) for x in v),
                                        None), "gf_topo_grid_info")
        z = np.zeros(mx.value * my.value)
        _ok(self._lib.gf_topo_grid_info(self.h, k, None, None, None, None, None, None, None, None,
                                        dptr(z)), "gf_topo_grid_info")
        keys = ("xlow", "ylow", "xhi", "yhi", "dx", "dy")
        out = dict(mx=mx.value, my=my.value, z=z)
        out.update({k_: x.value for k_, x in zip(keys, v)})
        return out

    def covered_area(self, x1, x2, y1, y2) -> float:
        a = C.c_double()
        _ok(self._lib.gf_topo_covered_area(self.h, x1, x2, y1, y2, C.byref(a)), "gf_topo_covered_area")
        return a.value

    def raster(self, ctx, nx: int, ny: int, halo: int, xlower: float, ylower: float, dx: float,
               dy: float, xupper: float, yupper: float) -> np.ndarray:
        """(ny + 2 halo, nx + 2 halo) cell averages, as setaux sets aux(1)."""
        out = np.empty((ny + 2 * halo, nx + 2 * halo))
        from . import _check
        _check(ctx.h, self._lib.gf_topo_raster(ctx.h, self.h, nx, ny, halo, xlower, ylower, dx, dy,
                                               xupper, yupper, dptr(out)))
        return out
