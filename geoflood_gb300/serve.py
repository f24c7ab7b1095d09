"""Served form: flood scenarios through the native continuous-batching
request loop (``gf_server_*`` in include/geoflood_gb300.h).

A scenario is a single-level forest: a brick of npx x npy patches of
mx x mx cells with its own bathymetry, Manning coefficient, inflow
hydrograph and horizon. The server keeps every admitted scenario resident
on the device and steps all active scenarios of a size lane together; see
gf_server.cpp for the round structure. Arrays handed to ``submit`` are kept
alive by the ``Server`` until the scenario ends.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import Phys, GeoFloodError, _lib
from ._lib import STATUS_NAMES


@dataclass
class Hydrograph:
    """Discharge-per-unit-width inflow on the sides with a non-zero flag
    (hydrograph/hydrograh_module.f90, discharge type)."""
    time: np.ndarray
    hu: np.ndarray
    side: tuple = (1, 0, 0, 0)
    width: float = 0.0
    x0: float = 0.0
    y0: float = 0.0


@dataclass
class Scenario:
    """q: (npatch, mx+4, mx+4, 3) and aux: (npatch, mx+4, mx+4, maux), the
    reference's per-patch Fortran layout q(meqn, i, j); patch = py*npx + px."""
    mx: int
    npx: int
    npy: int
    dx: float
    dy: float
    q: np.ndarray
    aux: np.ndarray
    t_final: float
    phys: Phys = field(default_factory=Phys)
    mthbc: tuple = (1, 1, 3, 3)
    hydro: Hydrograph | None = None
    xlower: float = 0.0
    ylower: float = 0.0
    nout: int = 1
    initial_dt: float = 0.1
    desired_cfl: float = 0.9
    max_cfl: float = 1.0
    seed: int = 0

    @property
    def cells(self) -> int:
        return self.npx * self.npy * self.mx * self.mx

    def to_c(self, q_out: np.ndarray | None) -> tuple[_lib.gf_scenario, tuple]:
        for name, a, nf in (("q", self.q, 3), ("aux", self.aux, None)):
            n4 = self.mx + 4
            want = (self.npx * self.npy, n4, n4)
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.shape[:3] != want or (
                    nf and a.shape[3] != nf):
                raise ValueError(f"{name} must be contiguous float64 of shape {want} + (fields,)")
        if q_out is not None and (q_out.shape != self.q.shape or q_out.dtype != np.float64
                                  or not q_out.flags["C_CONTIGUOUS"]):
            raise ValueError("q_out must match q")
        s = _lib.gf_scenario()
        s.mx, s.npx, s.npy, s.maux = self.mx, self.npx, self.npy, self.aux.shape[3]
        s.dx, s.dy, s.xlower, s.ylower = self.dx, self.dy, self.xlower, self.ylower
        s.q = self.q.ctypes.data
        s.aux = self.aux.ctypes.data
        s.q_out = q_out.ctypes.data if q_out is not None else None
        s.phys = self.phys.to_c()
        for k in range(4):
            s.mthbc[k] = int(self.mthbc[k])
        keep = (self.q, self.aux, q_out)
        if self.hydro is not None:
            tm = np.ascontiguousarray(self.hydro.time, np.float64)
            hu = np.ascontiguousarray(self.hydro.hu, np.float64)
            s.nhydro = len(tm)
            s.hydro_time = tm.ctypes.data
            s.hydro_hu = hu.ctypes.data
            for k in range(4):
                s.hydro_side[k] = int(self.hydro.side[k])
            s.hydro_width, s.hydro_x0, s.hydro_y0 = self.hydro.width, self.hydro.x0, self.hydro.y0
            keep = keep + (tm, hu)
        s.t_final, s.nout = self.t_final, self.nout
        s.initial_dt, s.desired_cfl, s.max_cfl = self.initial_dt, self.desired_cfl, self.max_cfl
        return s, keep


def _info_dict(i: _lib.gf_scenario_info) -> dict:
    return {"state": _lib.SCEN_STATE_NAMES.get(i.state, str(i.state)), "lane": i.lane,
            "steps": i.steps, "rejects": i.rejects, "cell_updates": i.cell_updates, "t": i.t,
            "dt": i.dt, "t_submit": i.t_submit, "t_admit": i.t_admit, "t_done": i.t_done,
            "max_cfl_seen": i.max_cfl_seen, "device_bytes": i.device_bytes}


class Server:
    """Continuous-batching scenario server on one GPU (gf_server)."""

    def __init__(self, device: int = 0, hbm_budget: int | None = None, max_active: int = 256,
                 lanes: tuple = (100_000, 1_000_000), priority: bool = True,
                 backfill: bool = True, reserve_sms: int | None = None, mixed_update: bool = False,
                 cull_dry: bool = True, split_sizes: bool = True):
        self._lib = _lib.load()
        o = _lib.gf_server_opts()
        self._lib.gf_server_opts_default(C.byref(o))
        if hbm_budget is not None:
            o.hbm_budget = int(hbm_budget)
        o.max_active = int(max_active)
        o.nlanes = len(lanes) + 1
        for k, v in enumerate(lanes):
            o.lane_cells[k] = int(v)
        o.priority = int(bool(priority))
        o.backfill = int(bool(backfill))
        if reserve_sms is not None:
            o.reserve_sms = int(reserve_sms)
        o.mixed_update = int(bool(mixed_update))
        o.cull_dry = int(bool(cull_dry))
        o.split_sizes = int(bool(split_sizes))
        h = C.c_void_p()
        rc = self._lib.gf_server_create(int(device), C.byref(o), C.byref(h))
        if rc != 0:
            raise GeoFloodError(rc, f"gf_server_create failed ({STATUS_NAMES.get(rc, rc)})")
        self.h = h
        self._keep: dict[int, tuple] = {}
        self._out: dict[int, np.ndarray | None] = {}

    def _check(self, rc: int):
        if rc != 0:
            msg = self._lib.gf_server_last_error(self.h)
            raise GeoFloodError(rc, f"{STATUS_NAMES.get(rc, rc)}: "
                                    f"{msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "h", None):
            self._lib.gf_server_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @staticmethod
    def footprint(sc: Scenario) -> int:
        s, _ = sc.to_c(None)
        return int(_lib.load().gf_scenario_footprint(C.byref(s)))

    def submit(self, sc: Scenario, q_out: np.ndarray | None = None) -> int:
        """Queue a scenario; q_out (same shape as sc.q) receives the final state."""
        s, keep = sc.to_c(q_out)
        sid = C.c_longlong()
        self._check(self._lib.gf_server_submit(self.h, C.byref(s), C.byref(sid)))
        self._keep[sid.value] = keep
        self._out[sid.value] = q_out
        return sid.value

    def pump(self) -> bool:
        busy = C.c_int()
        self._check(self._lib.gf_server_pump(self.h, C.byref(busy)))
        return bool(busy.value)

    def run_until_idle(self, timeout: float = 600.0):
        t_end = self.clock() + timeout
        while self.pump():
            if self.clock() > t_end:
                raise GeoFloodError(-5, "server did not go idle")

    def start(self):
        self._check(self._lib.gf_server_start(self.h))

    def stop(self):
        self._check(self._lib.gf_server_stop(self.h))

    def wait(self, sid: int, timeout: float = 600.0) -> dict:
        self._check(self._lib.gf_server_wait(self.h, int(sid), float(timeout)))
        info = self.poll(sid)
        if info["state"] in ("done", "failed", "cancelled"):
            self._keep.pop(sid, None)
        return info

    def poll(self, sid: int) -> dict:
        i = _lib.gf_scenario_info()
        self._check(self._lib.gf_server_poll(self.h, int(sid), C.byref(i)))
        return _info_dict(i)

    def result(self, sid: int) -> np.ndarray | None:
        return self._out.get(sid)

    def release(self, sid: int):
        """Drop the references kept for a finished scenario."""
        self._keep.pop(sid, None)
        self._out.pop(sid, None)

    def cancel(self, sid: int):
        self._check(self._lib.gf_server_cancel(self.h, int(sid)))

    def stats(self) -> dict:
        st = _lib.gf_server_stats()
        self._check(self._lib.gf_server_stats_get(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in _lib.gf_server_stats._fields_}

    def clock(self) -> float:
        return float(self._lib.gf_server_clock(self.h))


# ------------------------------------------------------------ AMR forests

@dataclass
class ForestRequest:
    """An adaptive scenario for the forest server: the options of a Forest
    (rasters at the finest level, or zero rasters plus a Topo set) and its
    outstyle-1 run. aux: (ny, nx) or (maux, ny, nx); q: (ny, nx, 3)."""
    mx: int
    nbx: int
    nby: int
    minlevel: int
    maxlevel: int
    dx0: float
    dy0: float
    t_final: float
    aux: np.ndarray | None = None
    q: np.ndarray | None = None
    topo: object | None = None
    qinit: bool = True
    maux: int = 1
    x0: float = 0.0
    y0: float = 0.0
    mthbc: tuple = (1, 1, 1, 1)
    regrid_interval: int = 0
    max_patches: int = 0
    refine: object | None = None
    phys: Phys = field(default_factory=Phys)
    hydro: Hydrograph | None = None
    nout: int = 1
    initial_dt: float = 1.0
    desired_cfl: float = 0.9
    max_cfl: float = 1.0
    subcycle: bool = False

    def opts(self, maux: int | None = None):
        from .forest import forest_opts
        return forest_opts(self.mx, self.nbx, self.nby, self.minlevel, self.maxlevel, self.dx0,
                           self.dy0, self.maux if maux is None else maux, self.x0, self.y0, 0,
                           self.mthbc, self.regrid_interval, self.max_patches, self.refine,
                           self.subcycle)

    def prepare(self) -> "ForestRequest":
        """Build the C request (and its raster block) now, so that a later
        submit only queues it; change no field after this."""
        self._prepared = None
        self._prepared = self.to_c()
        return self

    def to_c(self) -> tuple[_lib.gf_forest_request, tuple]:
        if getattr(self, "_prepared", None) is not None:
            return self._prepared
        from .forest import forest_planes
        nx, ny = self.nbx * self.mx << self.maxlevel, self.nby * self.mx << self.maxlevel
        planes, maux = forest_planes(self.aux, self.q, nx, ny, self.maux)
        r = _lib.gf_forest_request()
        r.opts = self.opts(maux)
        r.phys = self.phys.to_c()
        r.fields = planes.ctypes.data if planes is not None else None
        r.topo = self.topo.h if self.topo is not None else None
        r.qinit = int(bool(self.qinit))
        keep = (planes, self.topo)
        if self.hydro is not None:
            tm = np.ascontiguousarray(self.hydro.time, np.float64)
            hu = np.ascontiguousarray(self.hydro.hu, np.float64)
            r.nhydro = len(tm)
            r.hydro_time = tm.ctypes.data
            r.hydro_hu = hu.ctypes.data
            for k in range(4):
                r.hydro_side[k] = int(self.hydro.side[k])
            r.hydro_width, r.hydro_x0, r.hydro_y0 = self.hydro.width, self.hydro.x0, self.hydro.y0
            keep = keep + (tm, hu)
        r.t_final, r.nout = self.t_final, self.nout
        r.initial_dt, r.desired_cfl, r.max_cfl = self.initial_dt, self.desired_cfl, self.max_cfl
        return r, keep


class ForestServer:
    """Request loop over adaptive scenarios on one GPU (gf_fserver): every
    admitted forest steps in the batched forest engine's shared rounds; a
    finished forest stays on the device until release()."""

    def __init__(self, device: int = 0, hbm_budget: int | None = None, max_active: int = 256,
                 backfill: bool = True, exact: bool | None = None, lane_cells: int | None = None,
                 reserve_sms: int | None = None):
        """lane_cells: ascending cell counts after initial refinement that
        split the forests into up to three lanes (0 or (): one lane);
        reserve_sms: SMs a lane's update leaves per smaller running lane."""
        self._lib = _lib.load()
        o = _lib.gf_fserver_opts()
        self._lib.gf_fserver_opts_default(C.byref(o))
        if hbm_budget is not None:
            o.hbm_budget = int(hbm_budget)
        o.max_active = int(max_active)
        o.backfill = int(bool(backfill))
        if lane_cells is not None:
            cells = (lane_cells,) if np.ndim(lane_cells) == 0 else tuple(lane_cells)
            for k in range(2):
                o.lane_cells[k] = int(cells[k]) if k < len(cells) else 0
        if reserve_sms is not None:
            o.reserve_sms = int(reserve_sms)
        h = C.c_void_p()
        rc = self._lib.gf_fserver_create(int(device), C.byref(o), C.byref(h))
        if rc != 0:
            raise GeoFloodError(rc, f"gf_fserver_create failed ({STATUS_NAMES.get(rc, rc)})")
        self.h = h
        self.ctx_h = C.c_void_p(self._lib.gf_fserver_ctx(h))
        if exact is not None:
            self._check(self._lib.gf_ctx_set_fp_contract(self.ctx_h, int(not exact)))
        self._keep: dict[int, tuple] = {}
        self._req: dict[int, ForestRequest] = {}

    def _check(self, rc: int):
        if rc != 0:
            msg = self._lib.gf_fserver_last_error(self.h)
            raise GeoFloodError(rc, f"{STATUS_NAMES.get(rc, rc)}: "
                                    f"{msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "h", None):
            self._lib.gf_fserver_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @staticmethod
    def footprint(req: ForestRequest) -> int:
        from .forest import footprint
        r, _ = req.to_c()
        return footprint(r.opts)

    def submit(self, req: ForestRequest) -> int:
        r, keep = req.to_c()
        sid = C.c_longlong()
        self._check(self._lib.gf_fserver_submit(self.h, C.byref(r), C.byref(sid)))
        self._keep[sid.value] = keep
        self._req[sid.value] = req
        return sid.value

    def pump(self) -> bool:
        busy = C.c_int()
        self._check(self._lib.gf_fserver_pump(self.h, C.byref(busy)))
        return bool(busy.value)

    def run_until_idle(self, timeout: float = 600.0):
        t_end = self.clock() + timeout
        while self.pump():
            if self.clock() > t_end:
                raise GeoFloodError(-5, "forest server did not go idle")

    def start(self):
        self._check(self._lib.gf_fserver_start(self.h))

    def stop(self):
        self._check(self._lib.gf_fserver_stop(self.h))

    def wait(self, sid: int, timeout: float = 600.0) -> dict:
        self._check(self._lib.gf_fserver_wait(self.h, int(sid), float(timeout)))
        return self.poll(sid)

    def poll(self, sid: int) -> dict:
        i = _lib.gf_forest_request_info()
        self._check(self._lib.gf_fserver_poll(self.h, int(sid), C.byref(i)))
        d = {k: getattr(i, k) for k, _ in _lib.gf_forest_request_info._fields_}
        d["state"] = _lib.SCEN_STATE_NAMES.get(i.state, str(i.state))
        if d["state"] != "queued":
            self._keep.pop(sid, None)   # the server no longer reads the rasters
        return d

    def download(self, sid: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(patches (n, 3) of level, I, J; q; aux) of a done request, in the
        canonical leaf order."""
        n = C.c_int()
        self._check(self._lib.gf_fserver_download(self.h, int(sid), C.byref(n), None, None, None,
                                                  None, None))
        req = self._req[sid]
        maux = req.aux.shape[0] if req.aux is not None and np.ndim(req.aux) == 3 else (
            1 if req.aux is not None else req.maux)
        n4 = req.mx + 4
        lv, ii, jj = (np.zeros(n.value, np.int32) for _ in range(3))
        q = np.empty((n.value, n4, n4, 3))
        aux = np.empty((n.value, n4, n4, maux))
        ip = C.POINTER(C.c_int)
        self._check(self._lib.gf_fserver_download(
            self.h, int(sid), None, lv.ctypes.data_as(ip), ii.ctypes.data_as(ip),
            jj.ctypes.data_as(ip), _lib.dptr(q), _lib.dptr(aux)))
        return np.stack([lv, ii, jj], axis=1), q, aux

    def release(self, sid: int):
        self._check(self._lib.gf_fserver_release(self.h, int(sid)))
        self._keep.pop(sid, None)
        self._req.pop(sid, None)

    def cancel(self, sid: int):
        self._check(self._lib.gf_fserver_cancel(self.h, int(sid)))

    def stats(self) -> dict:
        st = _lib.gf_fserver_stats()
        self._check(self._lib.gf_fserver_stats_get(self.h, C.byref(st)))
        d = {k: getattr(st, k) for k, _ in _lib.gf_fserver_stats._fields_}
        d["lane_admitted"] = list(st.lane_admitted)
        return d

    def clock(self) -> float:
        return float(self._lib.gf_fserver_clock(self.h))
