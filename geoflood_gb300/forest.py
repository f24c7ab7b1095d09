"""Multi-level forests on the device (``gf_forest_*`` in include/geoflood_gb300.h).

A forest is nbx x nby root blocks refined as quadtrees between minlevel and
maxlevel with patches of mx x mx cells: the ForestClaw level machinery
around the patch update (balance, ghost exchange between levels, regrid,
outstyle-1 time stepping), resident on one GPU. Static fields and the
initial state are rasters at the finest level; a coarser patch takes their
cell averages.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import GeoFloodError, Refine, _check, _lib
from ._lib import dptr


def _stats_dict(s: _lib.gf_forest_stats) -> dict:
    return {k: getattr(s, k) for k, _ in _lib.gf_forest_stats._fields_}


def forest_planes(aux, q, nx: int, ny: int, maux: int = 1):
    """(planes, maux): the (maux + 3, ny, nx) raster block gf_forest_create
    takes (aux fields, then h, hu, hv), or None for zero rasters."""
    if aux is None and q is None:
        return None, maux
    aux = np.asarray(aux, np.float64)
    if aux.ndim == 2:
        aux = aux[None]
    maux = aux.shape[0]
    if aux.shape[1:] != (ny, nx) or q.shape != (ny, nx, 3):
        raise ValueError(f"rasters must be ({ny}, {nx}) at the finest level")
    planes = np.empty((maux + 3, ny, nx))
    planes[:maux] = aux
    planes[maux:] = np.moveaxis(np.asarray(q, np.float64), 2, 0)
    return planes, maux


def forest_opts(mx: int, nbx: int, nby: int, minlevel: int, maxlevel: int, dx0: float,
                dy0: float, maux: int = 1, x0: float = 0.0, y0: float = 0.0, phys_slot: int = 0,
                mthbc=(1, 1, 1, 1), regrid_interval: int = 0, max_patches: int = 0,
                refine: Refine | None = None, subcycle: bool = False) -> _lib.gf_forest_opts:
    o = _lib.gf_forest_opts()
    _lib.load().gf_forest_opts_default(C.byref(o))
    o.mx, o.maux, o.nbx, o.nby = mx, maux, nbx, nby
    o.minlevel, o.maxlevel = minlevel, maxlevel
    o.x0, o.y0, o.dx0, o.dy0 = x0, y0, dx0, dy0
    o.phys_slot = phys_slot
    for k in range(4):
        o.mthbc[k] = int(mthbc[k])
    o.regrid_interval = regrid_interval
    o.max_patches = max_patches
    o.refine = (refine or Refine()).to_c()
    o.subcycle = int(bool(subcycle))
    return o


def footprint(o: _lib.gf_forest_opts) -> int:
    """Device bytes a forest with these options may hold at most (0: invalid)."""
    return int(_lib.load().gf_forest_footprint(C.byref(o)))


class Forest:
    """aux: (ny, nx) bathymetry or (maux, ny, nx); q: (ny, nx, 3) with h, hu,
    hv; both at the finest level: nx = nbx*mx*2^maxlevel, ny = nby*mx*2^maxlevel.
    With aux = q = None the rasters start at zero and set_topo() fills them
    from DEM files (maux then gives the number of aux fields)."""

    def __init__(self, ctx, mx: int, nbx: int, nby: int, minlevel: int, maxlevel: int,
                 dx0: float, dy0: float, aux: np.ndarray | None, q: np.ndarray | None,
                 x0: float = 0.0, y0: float = 0.0, phys_slot: int = 0, mthbc=(1, 1, 1, 1),
                 regrid_interval: int = 0, max_patches: int = 0, refine: Refine | None = None,
                 maux: int = 1, subcycle: bool = False):
        self.ctx = ctx
        self._lib = _lib.load()
        nx, ny = nbx * mx << maxlevel, nby * mx << maxlevel
        planes, maux = forest_planes(aux, q, nx, ny, maux)
        o = forest_opts(mx, nbx, nby, minlevel, maxlevel, dx0, dy0, maux, x0, y0, phys_slot, mthbc,
                        regrid_interval, max_patches, refine, subcycle)
        self.mx, self.maux = mx, maux
        self.minlevel, self.maxlevel = minlevel, maxlevel
        h = C.c_void_p()
        _check(ctx.h, self._lib.gf_forest_create(ctx.h, C.byref(o), dptr(planes), C.byref(h)))
        self.h = h
        ctx._adopt(self)

    def close(self):
        if getattr(self, "h", None):
            self._lib.gf_forest_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_hydrograph(self, time, hu, side, width: float, x0: float, y0: float):
        tm = np.ascontiguousarray(time, np.float64)
        hv = np.ascontiguousarray(hu, np.float64)
        sd = np.ascontiguousarray(side, np.int32)
        _check(self.ctx.h, self._lib.gf_forest_set_hydrograph(
            self.h, len(tm), dptr(tm), dptr(hv), sd.ctypes.data_as(C.POINTER(C.c_int)),
            width, x0, y0))

    def set_topo(self, topo, qinit: bool = True):
        """Bathymetry of every level from a Topo set (setaux per level); with
        qinit, h = max(0, sea_level - b) and zero momentum. Before init()."""
        _check(self.ctx.h, self._lib.gf_forest_set_topo(self.h, topo.h, int(qinit)))

    def init(self):
        _check(self.ctx.h, self._lib.gf_forest_init(self.h))

    def ghost_fill(self, t: float):
        _check(self.ctx.h, self._lib.gf_forest_ghost_fill(self.h, t))

    def step(self, t: float, dt: float) -> float:
        c = C.c_double()
        _check(self.ctx.h, self._lib.gf_forest_step(self.h, t, dt, C.byref(c)))
        return c.value

    def accept(self, ok: bool = True):
        _check(self.ctx.h, self._lib.gf_forest_accept(self.h, int(bool(ok))))

    def regrid(self, t: float) -> bool:
        ch = C.c_int()
        _check(self.ctx.h, self._lib.gf_forest_regrid(self.h, t, C.byref(ch)))
        return bool(ch.value)

    def run(self, t_final: float, nout: int = 1, initial_dt: float = 1.0,
            desired_cfl: float = 0.9, max_cfl: float = 1.0, max_steps: int = 0) -> dict:
        st = _lib.gf_forest_stats()
        _check(self.ctx.h, self._lib.gf_forest_run(self.h, t_final, nout, initial_dt, desired_cfl,
                                                   max_cfl, max_steps, C.byref(st)))
        return _stats_dict(st)

    def stats(self) -> dict:
        st = _lib.gf_forest_stats()
        _check(self.ctx.h, self._lib.gf_forest_get_stats(self.h, C.byref(st)))
        return _stats_dict(st)

    @property
    def npatch(self) -> int:
        return int(self._lib.gf_forest_npatch(self.h))

    def patches(self) -> np.ndarray:
        """(npatch, 3) int array of (level, I, J) in canonical order."""
        n = self.npatch
        lv, ii, jj = (np.zeros(n, np.int32) for _ in range(3))
        ip = C.POINTER(C.c_int)
        _check(self.ctx.h, self._lib.gf_forest_patches(
            self.h, lv.ctypes.data_as(ip), ii.ctypes.data_as(ip), jj.ctypes.data_as(ip)))
        return np.stack([lv, ii, jj], axis=1)

    def download(self) -> np.ndarray:
        n4 = self.mx + 4
        out = np.empty((self.npatch, n4, n4, 3))
        _check(self.ctx.h, self._lib.gf_forest_download(self.h, dptr(out)))
        return out

    def download_aux(self) -> np.ndarray:
        n4 = self.mx + 4
        out = np.empty((self.npatch, n4, n4, self.maux))
        _check(self.ctx.h, self._lib.gf_forest_download_aux(self.h, dptr(out)))
        return out

    def upload(self, q: np.ndarray):
        q = np.ascontiguousarray(q, np.float64)
        if q.shape != (self.npatch, self.mx + 4, self.mx + 4, 3):
            raise GeoFloodError(-1, "q must match the current leaves")
        _check(self.ctx.h, self._lib.gf_forest_upload(self.h, dptr(q)))

    # ---- output in the reference's file formats --------------------------
    def set_output(self, out_dir: str = "", frames: bool = True):
        """Frames fort.tXXXX / fort.qXXXX (frame 0 before the first step, one
        per output time) and gauge files go to out_dir during run()."""
        _check(self.ctx.h, self._lib.gf_forest_set_output(self.h, os.fsencode(out_dir), int(frames)))

    def set_gauges(self, gauges):
        """gauges: [(id, x, y, t1, t2, min_time_increment)], e.g. from
        output.read_gauges_data; creates the gauge files in the output dir."""
        g = list(gauges)
        ids = np.array([int(r[0]) for r in g], np.int32)
        cols = [np.ascontiguousarray(np.array([r[k] for r in g], np.float64)) for k in range(1, 6)]
        _check(self.ctx.h, self._lib.gf_forest_set_gauges(
            self.h, len(g), ids.ctypes.data_as(C.POINTER(C.c_int)), *(dptr(c) for c in cols)))

    def write_frame(self, iframe: int, out_dir: str = ""):
        _check(self.ctx.h, self._lib.gf_forest_write_ascii(self.h, os.fsencode(out_dir), iframe))

    def sample_gauges(self, t: float):
        _check(self.ctx.h, self._lib.gf_forest_sample_gauges(self.h, t))

    def flush_gauges(self):
        _check(self.ctx.h, self._lib.gf_forest_flush_gauges(self.h))


def batch_run(forests, t_final: float, nout: int = 1, initial_dt: float = 1.0,
              desired_cfl: float = 0.9, max_cfl: float = 1.0) -> dict:
    """Run several forests of one context together (gf_forest_batch_run):
    shared launches, device-side time-step control, one captured round per
    epoch. Each forest ends exactly as its own Forest.run would."""
    forests = list(forests)
    if not forests:
        raise ValueError("no forests")
    ctx = forests[0].ctx
    arr = (C.c_void_p * len(forests))(*[f.h for f in forests])
    st = _lib.gf_forest_batch_stats()
    _check(ctx.h, _lib.load().gf_forest_batch_run(arr, len(forests), t_final, nout, initial_dt,
                                                  desired_cfl, max_cfl, C.byref(st)))
    return {k: getattr(st, k) for k, _ in _lib.gf_forest_batch_stats._fields_}

