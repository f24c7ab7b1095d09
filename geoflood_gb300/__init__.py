"""geoflood_gb300: GB300-native GeoClaw patch update behind the GeoFlood solver hooks.

Host-side mirror of the reference plugin interface for the patch-update path:

* :class:`Phys`    - the geoclaw_module / [geoclaw] options a step needs.
* :class:`Context` - one CUDA device; ``patch_update`` is the plain per-patch
  drop-in for ``geoclaw_update`` (src/fc2d_geoclaw/fc2d_geoclaw.cpp:352-387),
  ``patch_update_batch`` the buffered GPU hook ``cudaclaw_update``
  (src/fc2d_cpu_cuda/fc2d_cpucuda.cpp:410-495).
* :class:`Level`   - a device-resident batch of patches stepped in one launch.

Arrays follow the reference's Fortran layout q(meqn, 1-mbc:mx+mbc, 1-mbc:my+mbc),
which as a C-ordered numpy array is shaped ``(my+4, mx+4, 3)`` per patch
(``(npatch, my+4, mx+4, 3)`` for a batch). All compute runs in the CUDA
library; there is no host fallback.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import STATUS_NAMES, dptr, iptr

MBC = 2
MEQN = 3


class GeoFloodError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


@dataclass
class Phys:
    """Physics of one scenario (geoclaw_module.f90 set_geo, friction_module.f90)."""
    grav: float = 9.81
    dry_tolerance: float = 1.0e-3
    sea_level: float = 0.0
    friction_depth: float = 1.0e6
    manning_coefficient: tuple = (0.035,)
    manning_break: tuple = (1.0e10,)
    friction_forcing: bool = True
    variable_friction: bool = False
    friction_index: int = 0
    order: int = 2
    transverse: int = 2
    mthlim: tuple = (4, 4, 4)
    src_term: int = 1
    maxcfl_cap: float = 100.0

    def to_c(self) -> _lib.gf_phys:
        p = _lib.gf_phys()
        p.grav = self.grav
        p.dry_tolerance = self.dry_tolerance
        p.sea_level = self.sea_level
        p.friction_depth = self.friction_depth
        n = len(self.manning_coefficient)
        if n != len(self.manning_break) or n > _lib.GF_MAX_MANNING:
            raise ValueError("manning_coefficient / manning_break mismatch")
        for k in range(n):
            p.manning_coefficient[k] = self.manning_coefficient[k]
            p.manning_break[k] = self.manning_break[k]
        p.num_manning = n
        p.friction_forcing = int(bool(self.friction_forcing))
        p.variable_friction = int(bool(self.variable_friction))
        p.friction_index = int(self.friction_index)
        p.order = int(self.order)
        p.transverse = int(self.transverse)
        for k in range(3):
            p.mthlim[k] = int(self.mthlim[k])
        p.src_term = int(self.src_term)
        p.maxcfl_cap = self.maxcfl_cap
        return p


@dataclass
class Refine:
    """Refinement criteria (refinement_data_module) and regions (regions_module).
    regions: iterable of (x_low, x_hi, y_low, y_hi, t_low, t_hi, min_level, max_level)."""
    wave_tolerance: float = 0.1
    speed_tolerance: tuple = (1e12,)
    deep_depth: float = 1e2
    max_level_deep: int = 3
    max_velocity_depth_product: float = 1e20
    flowgrades: tuple = ()   # (value, variable, type, minlevel)
    regions: tuple = ()

    def to_c(self) -> _lib.gf_refine:
        r = _lib.gf_refine()
        r.wave_tolerance = self.wave_tolerance
        if len(self.speed_tolerance) > 8 or len(self.flowgrades) > 4 or len(self.regions) > 16:
            raise ValueError("too many speed tolerances / flowgrades / regions")
        for k, v in enumerate(self.speed_tolerance):
            r.speed_tolerance[k] = v
        r.num_speed_tolerance = len(self.speed_tolerance)
        r.deep_depth = self.deep_depth
        r.max_level_deep = self.max_level_deep
        r.max_velocity_depth_product = self.max_velocity_depth_product
        r.num_flowgrades = len(self.flowgrades)
        for k, (val, var, typ, ml) in enumerate(self.flowgrades):
            r.flowgradevalue[k], r.flowgradevariable[k] = val, var
            r.flowgradetype[k], r.flowgrademinlevel[k] = typ, ml
        r.num_regions = len(self.regions)
        for k, g in enumerate(self.regions):
            rr = r.regions[k]
            (rr.x_low, rr.x_hi, rr.y_low, rr.y_hi, rr.t_low, rr.t_hi,
             rr.min_level, rr.max_level) = g
        return r


def _check(ctx_handle, rc: int):
    if rc != 0:
        lib = _lib.load()
        msg = lib.gf_ctx_last_error(ctx_handle) if ctx_handle else b""
        raise GeoFloodError(rc, (msg or b"").decode())


class Context:
    """A CUDA device context (gf_ctx)."""

    def __init__(self, device: int = 0, phys: Phys | None = None):
        self._lib = _lib.load()
        h = C.c_void_p()
        rc = self._lib.gf_ctx_create(int(device), C.byref(h))
        if rc != 0:
            raise GeoFloodError(rc, f"gf_ctx_create(device={device}) failed")
        self.h = h
        # levels and forests live on this context: they are closed before it
        self._children = weakref.WeakSet()
        self.set_phys(0, phys or Phys())

    def _adopt(self, child):
        self._children.add(child)

    def close(self):
        if getattr(self, "h", None):
            for ch in list(self._children):
                ch.close()
            self._lib.gf_ctx_destroy(self.h)
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

    def set_phys(self, slot: int, phys: Phys):
        p = phys.to_c()
        _check(self.h, self._lib.gf_ctx_set_phys(self.h, int(slot), C.byref(p)))

    def autotune(self, reps: int = 5) -> list:
        """Time every tile shape of the patch kernel per patch size on this
        device and install the fastest (gf_autotune); returns per-mx results."""
        res = (_lib.gf_tile_result * 3)()
        _check(self.h, self._lib.gf_autotune(self.h, int(reps), res))
        out = []
        for r in res:
            n = r.nvariant
            out.append({"mx": r.mx,
                        "tiles": [(r.threads[v], r.band[v], r.cluster[v]) for v in range(n)],
                        "throughput": [r.throughput[v] for v in range(n)],
                        "latency_us": [r.latency_us[v] for v in range(n)],
                        "best_throughput": r.best_throughput, "best_latency": r.best_latency})
        return out

    @staticmethod
    def tile_count(mx: int) -> int:
        """Number of tile variants of the patch kernel for patch size mx."""
        return int(_lib.load().gf_tile_count(int(mx)))

    @staticmethod
    def tile(mx: int, goal: int = 0) -> int:
        """Selected tile variant for patch size mx (goal 0 throughput, 1 latency)."""
        return int(_lib.load().gf_tile_get(int(mx), int(goal)))

    @staticmethod
    def set_tile(mx: int, goal: int, variant: int):
        rc = _lib.load().gf_tile_set(int(mx), int(goal), int(variant))
        if rc != 0:
            raise GeoFloodError(rc, "no such tile variant")

    def set_fp_contract(self, allow: bool):
        """False: run the contraction-free build (bit-level parity mode)."""
        _check(self.h, self._lib.gf_ctx_set_fp_contract(self.h, int(bool(allow))))

    def set_mixed_update(self, on: bool):
        """Batched forest rounds: one persistent update launch for all patch
        sizes (True, the default) or one launch per size."""
        _check(self.h, self._lib.gf_ctx_set_mixed_update(self.h, int(bool(on))))

    @property
    def stream(self) -> int:
        """cudaStream_t of this context as an integer handle."""
        v = C.c_void_p()
        _check(self.h, self._lib.gf_ctx_stream(self.h, C.byref(v)))
        return int(v.value or 0)

    # -- plain per-patch drop-in (single_step_update) --------------------
    def patch_update(self, q: np.ndarray, aux: np.ndarray, dx: float, dy: float,
                     t: float, dt: float) -> float:
        """geoclaw_update on one patch; q is updated in place, returns the CFL."""
        my4, mx4, meqn = q.shape
        maux = aux.shape[-1]
        cfl = C.c_double()
        _check(self.h, self._lib.gf_patch_update(
            self.h, mx4 - 2 * MBC, my4 - 2 * MBC, MBC, meqn, maux, dx, dy, t, dt,
            dptr(q), dptr(aux), C.byref(cfl)))
        return cfl.value

    def patch_update_batch(self, qs: list, auxs: list, dx, dy, t: float, dt: float):
        """Buffered GPU hook: update all patches in one launch. Returns
        (per-patch CFL array, max CFL)."""
        n = len(qs)
        my4, mx4, meqn = qs[0].shape
        maux = auxs[0].shape[-1]
        dxa = np.ascontiguousarray(np.broadcast_to(np.asarray(dx, np.float64), (n,)))
        dya = np.ascontiguousarray(np.broadcast_to(np.asarray(dy, np.float64), (n,)))
        qp = (_lib._dp * n)(*[dptr(a) for a in qs])
        ap = (_lib._dp * n)(*[dptr(a) for a in auxs])
        cfl = np.zeros(n)
        mc = C.c_double()
        _check(self.h, self._lib.gf_patch_update_batch(
            self.h, n, mx4 - 2 * MBC, my4 - 2 * MBC, MBC, meqn, maux, dptr(dxa), dptr(dya),
            t, dt, qp, ap, dptr(cfl), C.byref(mc)))
        return cfl, mc.value


class StepBuffer:
    """The buffered per-patch hook of the reference's GPU build
    (cudaclaw_update, src/fc2d_cpu_cuda/fc2d_cpucuda.cpp:410-495) over
    gf_step_buffer: ``update(iter, total, q, aux, ...)`` records a patch and
    every ``buffer_len``-th call (and the last of a level step) updates the
    recorded patches in one batch, returning its largest CFL (0 otherwise).
    The arrays must stay alive and unmoved until the flush."""

    def __init__(self, ctx: Context, buffer_len: int = 1024):
        self.ctx = ctx
        self._lib = ctx._lib
        h = C.c_void_p()
        _check(ctx.h, self._lib.gf_step_buffer_create(ctx.h, int(buffer_len), C.byref(h)))
        self.h = h
        self.buffer_len = int(buffer_len)
        self._held = []

    def update(self, it: int, total: int, q: np.ndarray, aux: np.ndarray, dx: float, dy: float,
               t: float, dt: float) -> float:
        my4, mx4, meqn = q.shape
        if it == 0:
            self._held = []
        self._held.append((q, aux))
        mc = C.c_double()
        _check(self.ctx.h, self._lib.gf_step_buffer_update(
            self.h, int(it), int(total), mx4 - 2 * MBC, my4 - 2 * MBC, MBC, meqn,
            aux.shape[-1], float(dx), float(dy), float(t), float(dt), dptr(q), dptr(aux),
            C.byref(mc)))
        if (it + 1) % self.buffer_len == 0 or it + 1 == total:
            self._held = []   # flushed: the library holds no pointer to them now
        return mc.value

    def close(self):
        if getattr(self, "h", None):
            self._lib.gf_step_buffer_destroy(self.h)
            self.h = None


class Level:
    """Device-resident batch of patches (gf_level)."""

    def __init__(self, ctx: Context, npatch: int, m: int, maux: int = 1):
        self.ctx = ctx
        self._lib = ctx._lib
        self.npatch, self.m, self.maux = int(npatch), int(m), int(maux)
        h = C.c_void_p()
        _check(ctx.h, self._lib.gf_level_create(ctx.h, self.npatch, self.m, self.m, self.maux,
                                                C.byref(h)))
        self.h = h
        ctx._adopt(self)

    @property
    def shape_q(self):
        return (self.npatch, self.m + 2 * MBC, self.m + 2 * MBC, MEQN)

    @property
    def shape_aux(self):
        return (self.npatch, self.m + 2 * MBC, self.m + 2 * MBC, self.maux)

    def close(self):
        if getattr(self, "h", None):
            self._lib.gf_level_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_geometry(self, dx, dy, phys=None):
        dxa = np.ascontiguousarray(np.broadcast_to(np.asarray(dx, np.float64), (self.npatch,)))
        dya = np.ascontiguousarray(np.broadcast_to(np.asarray(dy, np.float64), (self.npatch,)))
        ph = None if phys is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(phys, np.int32), (self.npatch,)))
        _check(self.ctx.h, self._lib.gf_level_set_geometry(self.h, dptr(dxa), dptr(dya), iptr(ph)))

    def upload(self, q: np.ndarray, aux: np.ndarray | None = None):
        q = np.ascontiguousarray(q, dtype=np.float64)
        assert q.shape == self.shape_q, (q.shape, self.shape_q)
        a = None
        if aux is not None:
            a = np.ascontiguousarray(aux, dtype=np.float64)
            assert a.shape == self.shape_aux
        _check(self.ctx.h, self._lib.gf_level_upload(self.h, dptr(q), dptr(a)))

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.shape_q)
        _check(self.ctx.h, self._lib.gf_level_download(self.h, dptr(out)))
        return out

    def download_aux(self) -> np.ndarray:
        out = np.empty(self.shape_aux)
        _check(self.ctx.h, self._lib.gf_level_download_aux(self.h, dptr(out)))
        return out

    def step(self, t: float, dt: float) -> float:
        mc = C.c_double()
        _check(self.ctx.h, self._lib.gf_level_step(self.h, t, dt, C.byref(mc)))
        return mc.value

    def step_async(self, t: float, dt: float):
        _check(self.ctx.h, self._lib.gf_level_step_async(self.h, t, dt))

    def sync(self) -> float:
        mc = C.c_double()
        _check(self.ctx.h, self._lib.gf_level_sync(self.h, C.byref(mc)))
        return mc.value

    def step_host(self, q: np.ndarray, t: float, dt: float) -> float:
        mc = C.c_double()
        _check(self.ctx.h, self._lib.gf_level_step_host(self.h, dptr(q), t, dt, C.byref(mc)))
        return mc.value

    def set_pipeline(self, nchunks: int = 0):
        """Chunks of step_host (0 auto, 1 no overlap); results do not depend on it."""
        _check(self.ctx.h, self._lib.gf_level_set_pipeline(self.h, int(nchunks)))

    def set_layout(self, nbr: np.ndarray, xlower=None, ylower=None):
        nb = np.ascontiguousarray(nbr, dtype=np.int32).reshape(self.npatch, 8)
        xl = None if xlower is None else np.ascontiguousarray(xlower, dtype=np.float64)
        yl = None if ylower is None else np.ascontiguousarray(ylower, dtype=np.float64)
        _check(self.ctx.h, self._lib.gf_level_set_layout(self.h, iptr(nb), dptr(xl), dptr(yl)))

    def set_hydrograph(self, time, hu, side, width: float, x0: float, y0: float):
        tm = np.ascontiguousarray(time, dtype=np.float64)
        hv = np.ascontiguousarray(hu, dtype=np.float64)
        sd = np.ascontiguousarray(side, dtype=np.int32)
        _check(self.ctx.h, self._lib.gf_level_set_hydrograph(
            self.h, len(tm), dptr(tm), dptr(hv), iptr(sd), width, x0, y0))

    def set_bc(self, mthbc):
        mb = np.ascontiguousarray(mthbc, dtype=np.int32)
        _check(self.ctx.h, self._lib.gf_level_set_bc(self.h, iptr(mb)))

    def ghost_fill(self, t: float):
        _check(self.ctx.h, self._lib.gf_level_ghost_fill(self.h, t))

    def ghost_fill_async(self, t: float):
        _check(self.ctx.h, self._lib.gf_level_ghost_fill_async(self.h, t))

    # -- coarse/fine transfers, time interpolation, tags ------------------
    def transfer(self, fine: "Level", tasks):
        """tasks: iterable of (kind, coarse_patch, fine_patch, code, ox, oy);
        self is the coarse level."""
        tasks = list(tasks)
        arr = (_lib.gf_transfer * max(1, len(tasks)))()
        for k, t in enumerate(tasks):
            arr[k] = _lib.gf_transfer(*[int(v) for v in t])
        _check(self.ctx.h, self._lib.gf_level_transfer(self.h, fine.h, len(tasks), arr))

    def qad(self, fine: "Level", tasks, dt: float, svdflx: np.ndarray):
        """qad (qad.f:4-371) on sides of fine patches over this coarse level:
        tasks iterable of (fine_patch, coarse_patch, side, ox, oy); svdflx
        (ntask, mx/2, 3) float64, accumulated in place."""
        tasks = list(tasks)
        arr = (_lib.gf_qad_task * max(1, len(tasks)))()
        for k, t in enumerate(tasks):
            arr[k] = _lib.gf_qad_task(*[int(v) for v in t])
        if svdflx.shape != (len(tasks), self.m // 2, 3) or not svdflx.flags["C_CONTIGUOUS"]:
            raise ValueError("svdflx must be contiguous (ntask, mx/2, 3)")
        _check(self.ctx.h, self._lib.gf_level_qad(self.h, fine.h, len(tasks), arr, float(dt),
                                                  dptr(svdflx)))

    def timeinterp(self, curr: "Level", last: "Level", alpha: float):
        _check(self.ctx.h, self._lib.gf_level_timeinterp(self.h, curr.h, last.h, alpha))

    def tag4refinement(self, refine: "Refine", level: int, maxlevel: int, init_flag: int,
                       t: float) -> np.ndarray:
        r = refine.to_c()
        out = np.zeros(self.npatch, np.int32)
        _check(self.ctx.h, self._lib.gf_level_tag4refinement(self.h, C.byref(r), level, maxlevel,
                                                             init_flag, t, iptr(out)))
        return out

    def tag4coarsening(self, refine: "Refine", families, level: int, maxlevel: int,
                       init_flag: int, t: float) -> np.ndarray:
        r = refine.to_c()
        fam = np.ascontiguousarray(families, dtype=np.int32).reshape(-1, 4)
        out = np.zeros(len(fam), np.int32)
        _check(self.ctx.h, self._lib.gf_level_tag4coarsening(
            self.h, C.byref(r), len(fam), iptr(fam), level, maxlevel, init_flag, t, iptr(out)))
        return out

    def patch_cfl(self) -> np.ndarray:
        out = np.empty(self.npatch)
        _check(self.ctx.h, self._lib.gf_level_patch_cfl(self.h, dptr(out)))
        return out


from .serve import Hydrograph, Scenario, Server  # noqa: E402
from .forest import Forest  # noqa: E402

__all__ = ["Phys", "Refine", "Context", "Level", "GeoFloodError", "MBC", "MEQN", "Hydrograph",
           "Scenario", "Server", "Forest"]
