"""Reference file formats: ASCII frames (fort.tXXXX / fort.qXXXX), gauge files
(gaugeXXXXX.txt) and the gauges.data input, through the library's host-side
writers (``gf_write_ascii_frame``, ``gf_sample_gauge``,
``gf_write_gauge_header`` / ``_rows``, ``gf_read_gauges_data`` in
include/geoflood_gb300.h). Forests write these themselves during
``Forest.run`` (``Forest.set_output`` / ``Forest.set_gauges``); the functions
here serve single levels and user loops.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import GeoFloodError, _lib
from ._lib import dptr

_ip = C.POINTER(C.c_int)


def _enc(d) -> bytes:
    return os.fsencode(d if d is not None else "")


def _ok(rc: int, what: str):
    if rc != 0:
        raise GeoFloodError(rc, what)


def write_ascii_frame(out_dir: str, iframe: int, time: float, q: np.ndarray, aux: np.ndarray,
                      level, xlower, ylower, dx, dy, block=None, grid_number=None) -> None:
    """q: (npatch, mx+4, mx+4, 3), aux: (npatch, mx+4, mx+4, maux), Fortran
    layout per patch (ghosts included); per-patch level, corner and spacing."""
    q = np.ascontiguousarray(q, np.float64)
    aux = np.ascontiguousarray(aux, np.float64)
    n, n4 = q.shape[0], q.shape[1]
    if q.shape != (n, n4, n4, 3) or aux.shape[:3] != (n, n4, n4):
        raise ValueError("q must be (npatch, n4, n4, 3) and aux (npatch, n4, n4, maux)")
    lv = np.ascontiguousarray(np.broadcast_to(np.asarray(level, np.int32), (n,)))
    bk = None if block is None else np.ascontiguousarray(np.broadcast_to(np.asarray(block, np.int32), (n,)))
    gn = None if grid_number is None else np.ascontiguousarray(np.asarray(grid_number, np.int32))
    arr = [np.ascontiguousarray(np.broadcast_to(np.asarray(v, np.float64), (n,)))
           for v in (xlower, ylower, dx, dy)]
    ip = lambda a: a.ctypes.data_as(_ip) if a is not None else None  # noqa: E731
    _ok(_lib.load().gf_write_ascii_frame(_enc(out_dir), iframe, time, n, n4 - 4, aux.shape[3],
                                         dptr(q), dptr(aux), ip(gn), ip(lv), ip(bk),
                                         *(dptr(a) for a in arr)), "gf_write_ascii_frame")


def sample_gauge(q: np.ndarray, aux: np.ndarray, xlower: float, ylower: float, dx: float,
                 dy: float, dry_tolerance: float, xc: float, yc: float) -> tuple:
    """(h, hu, hv, bathymetry) at (xc, yc) of one patch (n4, n4, 3) / (n4, n4, maux)."""
    q = np.ascontiguousarray(q, np.float64)
    aux = np.ascontiguousarray(aux, np.float64)
    out = np.zeros(4)
    _ok(_lib.load().gf_sample_gauge(q.shape[0] - 4, aux.shape[2], dptr(q), dptr(aux), xlower,
                                    ylower, dx, dy, dry_tolerance, xc, yc, dptr(out)),
        "gf_sample_gauge")
    return tuple(float(v) for v in out)


def write_gauge_header(out_dir: str, gauge_id: int, xc: float, yc: float) -> None:
    _ok(_lib.load().gf_write_gauge_header(_enc(out_dir), gauge_id, xc, yc), "gf_write_gauge_header")


def write_gauge_rows(out_dir: str, gauge_id: int, rows) -> None:
    """rows: (level, t, h, hu, hv, bathymetry) tuples, appended in order."""
    rows = list(rows)
    if not rows:
        return
    lv = np.array([int(r[0]) for r in rows], np.int32)
    t = np.array([r[1] for r in rows], np.float64)
    qv = np.ascontiguousarray(np.array([r[2:6] for r in rows], np.float64))
    _ok(_lib.load().gf_write_gauge_rows(_enc(out_dir), gauge_id, len(rows), lv.ctypes.data_as(_ip),
                                        dptr(t), dptr(qv)), "gf_write_gauge_rows")


def read_gauges_data(path: str) -> list[tuple]:
    """[(id, x, y, t1, t2, min_time_increment)] from a GeoClaw gauges.data file."""
    lib = _lib.load()
    n = C.c_int(0)
    _ok(lib.gf_read_gauges_data(_enc(path), 0, C.byref(n), None, None, None, None, None, None),
        "gf_read_gauges_data")
    k = n.value
    if k == 0:
        return []
    ids = np.zeros(k, np.int32)
    v = [np.zeros(k) for _ in range(5)]
    _ok(lib.gf_read_gauges_data(_enc(path), k, C.byref(n), ids.ctypes.data_as(_ip),
                                *(dptr(a) for a in v)), "gf_read_gauges_data")
    return [(int(ids[i]),) + tuple(float(a[i]) for a in v) for i in range(k)]
