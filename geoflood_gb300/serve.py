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
                 backfill: bool = True, reserve_sms: int | None = None):
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
