"""Topography input -- TEST INFRASTRUCTURE ONLY (the oracle).

Plain-Python restatement of GeoClaw's topo readers and the ctypes wrappers
of the oracle's C cell integrals (geoclaw_oracle_topo.c):

- read_topo_header / read_topo_file
  (src/fc2d_geoclaw/geolib_source/topo_module.f90:491-769, 785-1059) for
  topo types 1 (x y z records), 2 (one value per record) and 3 (one row per
  record), negative types flipping the sign, no-data values replaced by
  topo_missing, ESRI 'xllcorner' / 'yllcorner' headers shifted by half a
  cell to the nodes;
- parse_values (geolib_source/utility_module.f90:53-108);
- read_topo_settings' file list (topo_module.f90:160-245) from topo.data.
"""
from __future__ import annotations

import ctypes as C
import re

import numpy as np

from . import _ptr, load

_REAL = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eEdD][+-]?\d+)?$")


class orc_topo_grid(C.Structure):
    _fields_ = [("z", C.POINTER(C.c_double)), ("mx", C.c_int), ("my", C.c_int),
                ("xlow", C.c_double), ("ylow", C.c_double), ("xhi", C.c_double),
                ("yhi", C.c_double), ("dx", C.c_double), ("dy", C.c_double)]


def _num(word: str):
    """A Fortran real constant as list-directed input reads it, else None."""
    w = word.rstrip(",")
    if not _REAL.match(w):
        return None
    return float(w.replace("d", "e").replace("D", "e"))


def parse_values(line: str) -> list[float]:
    return [v for v in (_num(w) for w in line.split()) if v is not None]


def _records(path):
    with open(path) as f:
        return f.read().split("\n")


def _fortran_nint(v: float) -> int:
    return int(np.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1)


def read_topo_header(path: str, topo_type: int) -> dict:
    t = abs(topo_type)
    lines = _records(path)
    if t == 1:
        recs = [parse_values(l) for l in lines]
        recs = [r for r in recs if r]
        xll, yhi = recs[0][0], recs[0][1]
        mx = 1
        k = 1
        while True:                      # count records of the first row
            x, y = recs[k][0], recs[k][1]
            k += 1
            mx += 1
            if y != yhi:
                break
        mx -= 1
        size = len(recs)
        my = size // mx
        xhi, yll = recs[-1][0], recs[-1][1]
        dx, dy = (xhi - xll) / (mx - 1), (yhi - yll) / (my - 1)
    elif t in (2, 3):
        v = [parse_values(lines[k]) for k in range(6)]
        mx, my = _fortran_nint(v[0][0]), _fortran_nint(v[1][0])
        xll, yll = v[2][0], v[3][0]
        dx = v[4][0]
        dy = v[4][1] if len(v[4]) == 2 else dx
        if "xllcorner" in lines[2].lower():
            xll = xll + 0.5 * dx
        if "yllcorner" in lines[3].lower():
            yll = yll + 0.5 * dy
        xhi = xll + (mx - 1) * dx
        yhi = yll + (my - 1) * dy
    else:
        raise ValueError("topo type %d is not supported" % topo_type)
    return dict(mx=mx, my=my, xlow=xll, ylow=yll, xhi=xhi, yhi=yhi, dx=dx, dy=dy)


def read_netcdf_topo(path: str, topo_type: int) -> dict:
    """Topo type 4 (geolib_source/topo_module.f90:624-732 and :926-1035,
    get_dim_info :1599-1623), parsed with scipy's classic-NetCDF reader: x / y
    dimensions named lon / longitude / x and lat / latitude / y in any case,
    coordinate variables of the same names, the last 2-D variable as z in
    either dimension order, rows north first, z negated when its attribute
    positive is "down" and the type is negative. The whole grid (the
    reference crops to the domain plus one spacing)."""
    from scipy.io import netcdf_file

    with netcdf_file(path, "r", mmap=False) as f:
        xd = yd = None
        for name in f.dimensions:
            u = name.upper()
            if u in ("LON", "LONGITUDE", "X"):
                xd = name
            elif u in ("LAT", "LATITUDE", "Y"):
                yd = name
        zname = None
        for name, v in f.variables.items():
            if name in (xd, yd):
                continue
            if len(v.dimensions) == 2:
                zname = name
        xs = np.array(f.variables[xd].data, dtype=np.float64)
        ys = np.array(f.variables[yd].data, dtype=np.float64)
        zv = f.variables[zname]
        data = np.array(zv.data, dtype=np.float64)
        if tuple(zv.dimensions) == (yd, xd):
            grid = data
        elif tuple(zv.dimensions) == (xd, yd):
            grid = data.T
        else:
            raise ValueError("NetCDF z variable has dimensions that don't align with x and y")
        pos = getattr(zv, "positive", b"")
        pos = pos.decode() if isinstance(pos, bytes) else str(pos)
    z = np.ascontiguousarray(grid[::-1, :]).reshape(-1)
    if topo_type < 0 and pos.lower() == "down":
        z = -z
    return dict(mx=len(xs), my=len(ys), xlow=xs[0], ylow=ys[0], xhi=xs[-1], yhi=ys[-1],
                dx=xs[1] - xs[0], dy=ys[1] - ys[0], z=z)


def read_topo_file(path: str, topo_type: int, topo_missing: float = 99999.0) -> dict:
    """Header plus z (mx*my,) in file order: rows north to south, x fastest."""
    if abs(topo_type) == 4:
        h = read_netcdf_topo(path, topo_type)
        if topo_type < 0:
            h["z"] = -h["z"]
        return h
    h = read_topo_header(path, topo_type)
    mx, my = h["mx"], h["my"]
    t = abs(topo_type)
    lines = _records(path)
    z = np.zeros(mx * my)
    if t == 1:
        recs = [r for r in (parse_values(l) for l in lines) if r]
        for i in range(mx * my):
            z[i] = recs[i][2]
    else:
        nodata = parse_values(lines[5])[0]
        k = 6
        missing = 0
        if t == 2:
            for i in range(mx * my):
                while not parse_values(lines[k]):
                    k += 1
                z[i] = parse_values(lines[k])[0]
                k += 1
        else:
            for j in range(my):
                row = []
                while len(row) < mx:
                    row += parse_values(lines[k])
                    k += 1
                z[j * mx:(j + 1) * mx] = row[:mx]
        bad = z == nodata
        missing = int(bad.sum())
        z[bad] = topo_missing
        if missing and topo_missing == 99999.0:
            raise ValueError("missing data with the default topo_missing")
    if topo_type < 0:
        z = -z
    h["z"] = z
    return h


def read_topo_data(path: str) -> tuple[float, list[tuple[str, int]]]:
    """(topo_missing, [(file name, topo type)]) from topo.data (test_topography 0)."""
    recs = [l for l in _records(path) if l.strip() and not l.lstrip().startswith("#")]
    missing = parse_values(recs[0].split("=:")[0])[0]
    test = int(recs[1].split()[0])
    if test != 0:
        raise ValueError("analytic test topography is not supported")
    n = int(parse_values(recs[2].split("=:")[0])[0])
    files = []
    for k in range(n):
        name = recs[3 + 2 * k].strip().split("'")[1]
        ttype = int(recs[4 + 2 * k].split()[0])
        files.append((name, ttype))
    return missing, files


class TopoSet:
    """Grids in the order given; rank[] finest first as read_topo_settings ranks them."""

    def __init__(self, grids: list[dict]):
        self.grids = grids
        self._z = [np.ascontiguousarray(g["z"], np.float64) for g in grids]
        n = len(grids)
        self._c = (orc_topo_grid * max(n, 1))()
        for k, g in enumerate(grids):
            self._c[k] = orc_topo_grid(_ptr(self._z[k]), g["mx"], g["my"], g["xlow"], g["ylow"],
                                       g["xhi"], g["yhi"], g["dx"], g["dy"])
        self._order = (C.c_int * max(n, 1))()
        lib = _lib()
        lib.orc_topo_rank(self._c, n, self._order)
        self.order = list(self._order)[:n]

    def cell_integral(self, xim, xip, yjm, yjp) -> float:
        v = C.c_double()
        rc = _lib().orc_cellgridintegrate(C.byref(v), xim, xip, yjm, yjp, self._c, self._order,
                                          len(self.grids))
        if rc:
            raise ValueError("cell overlaps no topo grid")
        return v.value

    def area(self, x1, x2, y1, y2) -> float:
        return _lib().orc_topo_area(x1, x2, y1, y2, self._c, self._order, len(self.grids))

    def raster(self, nx, ny, halo, xlower, ylower, dx, dy, xupper, yupper) -> np.ndarray:
        """(ny + 2 halo, nx + 2 halo) cell averages as setaux sets aux(1)."""
        out = np.zeros((ny + 2 * halo, nx + 2 * halo))
        rc = _lib().orc_setaux_raster(self._c, self._order, len(self.grids), nx, ny, halo,
                                      xlower, ylower, dx, dy, xupper, yupper, _ptr(out))
        if rc:
            raise ValueError("a cell overlaps no topo grid")
        return out


_typed = None


def _lib():
    global _typed
    lib = load()
    if _typed is None:
        G = C.POINTER(orc_topo_grid)
        ip = C.POINTER(C.c_int)
        dp = C.POINTER(C.c_double)
        lib.orc_topo_rank.argtypes = [G, C.c_int, ip]
        lib.orc_topointegral.argtypes = [C.c_double] * 4 + [G]
        lib.orc_topointegral.restype = C.c_double
        lib.orc_cellgridintegrate.argtypes = [dp] + [C.c_double] * 4 + [G, ip, C.c_int]
        lib.orc_topo_area.argtypes = [C.c_double] * 4 + [G, ip, C.c_int]
        lib.orc_topo_area.restype = C.c_double
        lib.orc_setaux_raster.argtypes = [G, ip, C.c_int, C.c_int, C.c_int, C.c_int] + \
            [C.c_double] * 6 + [dp]
        _typed = lib
    return lib
