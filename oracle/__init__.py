"""CPU oracle for the GeoClaw patch update -- TEST INFRASTRUCTURE ONLY.

Loads ``liboracle.so`` built from ``geoclaw_oracle.c`` (a plain-C restatement
of the reference's Fortran patch update). Only the tests, the smoke check and
the CPU-baseline leg of bench.py use it, as the checker / the timed CPU
reference; the shipped library never does.

Parity status: the reference's own Fortran cannot be compiled here and its
tests hold no golden vectors for this path. The Riemann-solver core is pinned
against the reference's CUDA device functions compiled for the host
(``oracle/_ref``, built by ``build_ref.sh`` where the reference tree is
present; the generated vectors live in ``tests/golden/``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
MBC = 2


class orc_params(C.Structure):
    _fields_ = [
        ("grav", C.c_double), ("dry_tolerance", C.c_double), ("sea_level", C.c_double),
        ("friction_depth", C.c_double), ("friction_forcing", C.c_int),
        ("num_manning", C.c_int), ("manning_coefficient", C.c_double * 4),
        ("manning_break", C.c_double * 4), ("variable_friction", C.c_int),
        ("friction_index", C.c_int), ("order", C.c_int), ("transverse", C.c_int),
        ("mthlim", C.c_int * 3), ("src_term", C.c_int), ("maxcfl_cap", C.c_double),
    ]


def build(force: bool = False) -> Path:
    srcs = [HERE / "geoclaw_oracle.c", HERE / "geoclaw_oracle_ghost.c", HERE / "geoclaw_oracle_amr.c",
            HERE / "geoclaw_oracle_topo.c", HERE / "geoclaw_oracle_qad.c"]
    deps = srcs + [HERE / "geoclaw_oracle.h"]
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    tmp = LIB.with_suffix(f".so.{os.getpid()}")
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-std=c99", "-Wall", "-o", str(tmp), *map(str, srcs), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


_dp = C.POINTER(C.c_double)
_lib = None


class orc_region(C.Structure):
    _fields_ = [("x_low", C.c_double), ("x_hi", C.c_double), ("y_low", C.c_double),
                ("y_hi", C.c_double), ("t_low", C.c_double), ("t_hi", C.c_double),
                ("min_level", C.c_int), ("max_level", C.c_int)]


class orc_refine(C.Structure):
    _fields_ = [("wave_tolerance", C.c_double), ("speed_tolerance", C.c_double * 8),
                ("num_speed_tolerance", C.c_int), ("deep_depth", C.c_double),
                ("max_level_deep", C.c_int), ("max_velocity_depth_product", C.c_double),
                ("num_flowgrades", C.c_int), ("flowgradevalue", C.c_double * 4),
                ("flowgradevariable", C.c_int * 4), ("flowgradetype", C.c_int * 4),
                ("flowgrademinlevel", C.c_int * 4), ("num_regions", C.c_int),
                ("regions", orc_region * 16)]


def refine(r) -> orc_refine:
    """orc_refine from a geoflood_gb300.Refine."""
    o = orc_refine()
    C.memmove(C.byref(o), C.byref(r.to_c()), C.sizeof(o))
    return o


class orc_hydro(C.Structure):
    _fields_ = [("use", C.c_int), ("side", C.c_int * 4), ("width", C.c_double),
                ("x0", C.c_double), ("y0", C.c_double), ("n", C.c_int),
                ("time", _dp), ("hu", _dp)]


def hydro(time=None, hu=None, side=(0, 0, 0, 0), width=0.0, x0=0.0, y0=0.0):
    """orc_hydro for a discharge hydrograph (keeps the arrays alive on the struct)."""
    h = orc_hydro()
    if time is None:
        h.use = 0
        h.n = 0
        return h
    tm = np.ascontiguousarray(time, dtype=np.float64)
    hv = np.ascontiguousarray(hu, dtype=np.float64)
    h.use = 1
    for k in range(4):
        h.side[k] = int(side[k])
    h.width, h.x0, h.y0 = width, x0, y0
    h.n = len(tm)
    h.time = tm.ctypes.data_as(_dp)
    h.hu = hv.ctypes.data_as(_dp)
    h._keep = (tm, hv)
    return h


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        P = C.POINTER(orc_params)
        lib.orc_default_params.argtypes = [P]
        lib.orc_patch_update.restype = C.c_double
        lib.orc_patch_update.argtypes = [P, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int,
                                         C.c_double, C.c_double, C.c_double, C.c_double]
        lib.orc_level_update.restype = C.c_double
        lib.orc_level_update.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.c_long,
                                         _dp, C.c_int, C.c_long, _dp, _dp, C.c_double,
                                         C.c_double, C.c_int]
        lib.orc_b4step2.argtypes = [P, C.c_int, C.c_int, C.c_int, _dp]
        lib.orc_step2.restype = C.c_double
        lib.orc_step2.argtypes = [P, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_double,
                                  C.c_double, C.c_double]
        lib.orc_src2.argtypes = [P, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_double]
        lib.orc_riemann_aug_JCP.argtypes = [C.c_int] + [C.c_double] * 18 + [_dp, _dp]
        lib.orc_riemanntype.argtypes = ([C.c_double] * 4 + [_dp, _dp, _dp, C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), C.c_int, C.c_double, C.c_double])
        lib.orc_rpn2.argtypes = [P, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int, _dp, _dp, _dp,
                                 _dp]
        lib.orc_rpt2.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp,
                                 C.c_int, _dp, _dp, _dp]
        lib.orc_qad_side.restype = None
        lib.orc_qad_side.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp,
                                     _dp, _dp, C.c_double, C.c_double, C.c_double, _dp]
        lib.orc_rpn2_face.argtypes = [P, C.c_int, _dp, _dp, C.c_double, C.c_double, _dp, _dp,
                                      _dp, _dp]
        lib.orc_rpt2_face.argtypes = [P, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                      _dp]
        RF = C.POINTER(orc_refine)
        lib.orc_average_ghost.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp,
                                          _dp, C.c_int, C.c_int, C.c_int, C.c_int]
        lib.orc_interpolate_ghost.argtypes = lib.orc_average_ghost.argtypes
        lib.orc_interpolate2fine.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp,
                                             _dp, _dp, C.c_int]
        lib.orc_average2coarse.argtypes = lib.orc_interpolate2fine.argtypes
        lib.orc_timeinterp.restype = C.c_int
        lib.orc_timeinterp.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp,
                                       C.c_double]
        lib.orc_tag4refinement.restype = C.c_int
        lib.orc_tag4refinement.argtypes = [P, RF, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp,
                                           C.c_double, C.c_double, C.c_double, C.c_double,
                                           C.c_double, C.c_int, C.c_int, C.c_int]
        lib.orc_tag4coarsening.restype = C.c_int
        lib.orc_tag4coarsening.argtypes = [P, RF, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.POINTER(_dp), C.POINTER(_dp), _dp, _dp, C.c_double,
                                           C.c_double, C.c_double, C.c_int, C.c_int, C.c_int]
        H = C.POINTER(orc_hydro)
        ip = C.POINTER(C.c_int)
        lib.orc_bc2.argtypes = [P, H, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                C.c_double, C.c_double, _dp, _dp, C.c_int, C.c_double, ip]
        lib.orc_level_ghost_fill.argtypes = [P, H, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp,
                                             C.c_int, ip, _dp, _dp, C.c_double, C.c_double,
                                             C.c_double, ip]
        _lib = lib
    return _lib


def params(phys=None) -> orc_params:
    """orc_params from a geoflood_gb300.Phys-like object (or defaults)."""
    p = orc_params()
    load().orc_default_params(C.byref(p))
    if phys is not None:
        p.grav = phys.grav
        p.dry_tolerance = phys.dry_tolerance
        p.sea_level = phys.sea_level
        p.friction_depth = phys.friction_depth
        p.friction_forcing = int(bool(phys.friction_forcing))
        p.num_manning = len(phys.manning_coefficient)
        for k in range(p.num_manning):
            p.manning_coefficient[k] = phys.manning_coefficient[k]
            p.manning_break[k] = phys.manning_break[k]
        p.variable_friction = int(bool(phys.variable_friction))
        p.friction_index = int(phys.friction_index)
        p.order = int(phys.order)
        p.transverse = int(phys.transverse)
        for k in range(3):
            p.mthlim[k] = int(phys.mthlim[k])
        p.src_term = int(phys.src_term)
        p.maxcfl_cap = phys.maxcfl_cap
    return p


def _ptr(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def patch_update(q: np.ndarray, aux: np.ndarray, dx: float, dy: float, t: float, dt: float,
                 phys=None) -> float:
    """geoclaw_update on one patch (Fortran layout, shape (my+4, mx+4, 3)); in place."""
    p = params(phys)
    my4, mx4, _ = q.shape
    return load().orc_patch_update(C.byref(p), MBC, mx4 - 2 * MBC, my4 - 2 * MBC, _ptr(q),
                                   _ptr(aux), aux.shape[-1], dx, dy, t, dt)


def level_update(q: np.ndarray, aux: np.ndarray, dx, dy, t: float, dt: float, phys=None,
                 nthreads: int = 0) -> float:
    """One level step over patches (npatch, my+4, mx+4, 3), in place; returns max CFL."""
    p = params(phys)
    n, my4, mx4, _ = q.shape
    dxa = np.ascontiguousarray(np.broadcast_to(np.asarray(dx, np.float64), (n,)))
    dya = np.ascontiguousarray(np.broadcast_to(np.asarray(dy, np.float64), (n,)))
    maux = aux.shape[-1]
    return load().orc_level_update(C.byref(p), n, MBC, mx4 - 2 * MBC, my4 - 2 * MBC, _ptr(q),
                                   my4 * mx4 * 3, _ptr(aux), maux, my4 * mx4 * maux, _ptr(dxa),
                                   _ptr(dya), t, dt, nthreads)


def riemann_aug_JCP(hL, hR, huL, huR, hvL, hvR, bL, bR, uL, uR, vL, vR, phiL, phiR, sE1, sE2,
                    drytol=1e-3, g=9.81):
    sw = np.zeros(3)
    fw = np.zeros(9)
    load().orc_riemann_aug_JCP(1, hL, hR, huL, huR, hvL, hvR, bL, bR, uL, uR, vL, vR, phiL,
                               phiR, sE1, sE2, drytol, g, _ptr(sw), _ptr(fw))
    return sw, fw.reshape(3, 3)  # fw[mw, m]


def rpn2(ixy: int, q1d: np.ndarray, aux1d: np.ndarray, phys=None):
    """rpn2 over a slice q1d (n, 3) with n = mx + 2*mbc; returns fwave (n,3,3)
    [i, mw, m], s (n,3), amdq (n,3), apdq (n,3). q1d is modified like the Fortran."""
    p = params(phys)
    n = q1d.shape[0]
    mx = n - 2 * MBC
    fwave = np.zeros((n, 3, 3))
    s = np.zeros((n, 3))
    amdq = np.zeros((n, 3))
    apdq = np.zeros((n, 3))
    load().orc_rpn2(C.byref(p), ixy, MBC, mx, _ptr(q1d), _ptr(aux1d), aux1d.shape[-1],
                    _ptr(fwave), _ptr(s), _ptr(amdq), _ptr(apdq))
    return fwave, s, amdq, apdq


def level_ghost_fill(q: np.ndarray, aux: np.ndarray, nbr: np.ndarray, xlower, ylower, dx: float,
                     dy: float, t: float, mthbc=(1, 1, 1, 1), phys=None, hy=None):
    """Ghost fill of a same-level batch (in place): copies, then bc2."""
    p = params(phys)
    n, my4, mx4, _ = q.shape
    nb = np.ascontiguousarray(nbr, dtype=np.int32).reshape(n, 8)
    xl = np.ascontiguousarray(xlower, dtype=np.float64)
    yl = np.ascontiguousarray(ylower, dtype=np.float64)
    mb = np.ascontiguousarray(mthbc, dtype=np.int32)
    h = hy if hy is not None else hydro()
    ip = C.POINTER(C.c_int)
    load().orc_level_ghost_fill(C.byref(p), C.byref(h), n, MBC, mx4 - 2 * MBC, my4 - 2 * MBC,
                                _ptr(q), _ptr(aux), aux.shape[-1], nb.ctypes.data_as(ip),
                                _ptr(xl), _ptr(yl), dx, dy, t, mb.ctypes.data_as(ip))


def qad_side(side: int, qf: np.ndarray, af: np.ndarray, qc1d: np.ndarray, auxc1d: np.ndarray,
             hx: float, hy: float, delt: float, svdflx: np.ndarray, phys=None):
    """qad (qad.f:4-371) on one side of a fine patch qf (my+4, mx+4, 3) with
    aux af (my+4, mx+4, maux): qc1d (n, 3) / auxc1d (n, maux) are the coarse
    cells along the side; svdflx (n, 3) accumulates in place."""
    p = params(phys)
    my4, mx4, _ = qf.shape
    load().orc_qad_side(C.byref(p), int(side), MBC, mx4 - 2 * MBC, my4 - 2 * MBC, af.shape[-1],
                        _ptr(qf), _ptr(af), _ptr(qc1d), _ptr(auxc1d), hx, hy, delt, _ptr(svdflx))


def rpn2_face(ixy: int, ql, qr, bl: float, br: float, phys=None):
    """Normal solve at one face; returns fwave (3 waves x 3 comps), s, amdq, apdq."""
    p = params(phys)
    ql = np.ascontiguousarray(ql, dtype=np.float64)
    qr = np.ascontiguousarray(qr, dtype=np.float64)
    fw, s, am, ap = np.zeros(9), np.zeros(3), np.zeros(3), np.zeros(3)
    load().orc_rpn2_face(C.byref(p), ixy, _ptr(ql), _ptr(qr), bl, br, _ptr(fw), _ptr(s),
                         _ptr(am), _ptr(ap))
    return fw.reshape(3, 3), s, am, ap


def rpt2_face(ixy: int, imp: int, ql, qr, aux1, aux2, aux3, asdq, phys=None):
    """Transverse split at one face (imp 1: left cell, 2: right cell)."""
    p = params(phys)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (ql, qr, aux1, aux2, aux3, asdq)]
    bm, bp = np.zeros(3), np.zeros(3)
    load().orc_rpt2_face(C.byref(p), ixy, imp, *[_ptr(a) for a in arrs], _ptr(bm), _ptr(bp))
    return bm, bp


def average_ghost(qc, ac, qf, af, kind, code, ox, oy, phys=None):
    """kind 0 face / 1 corner; coarse ghost cells from fine (in place on qc)."""
    p = params(phys)
    m = qc.shape[0] - 2 * MBC
    load().orc_average_ghost(C.byref(p), MBC, m, m, ac.shape[-1], _ptr(qc), _ptr(ac), _ptr(qf),
                             _ptr(af), kind, code, ox, oy)


def interpolate_ghost(qc, ac, qf, af, kind, code, ox, oy, phys=None):
    """kind 0 face / 1 corner; fine ghost cells from coarse (in place on qf)."""
    p = params(phys)
    m = qc.shape[0] - 2 * MBC
    load().orc_interpolate_ghost(C.byref(p), MBC, m, m, ac.shape[-1], _ptr(qc), _ptr(ac),
                                 _ptr(qf), _ptr(af), kind, code, ox, oy)


def interpolate2fine(qc, ac, qf, af, igrid, phys=None):
    p = params(phys)
    m = qc.shape[0] - 2 * MBC
    load().orc_interpolate2fine(C.byref(p), MBC, m, m, ac.shape[-1], _ptr(qc), _ptr(ac),
                                _ptr(qf), _ptr(af), igrid)


def average2coarse(qc, ac, qf, af, igrid, phys=None):
    p = params(phys)
    m = qc.shape[0] - 2 * MBC
    load().orc_average2coarse(C.byref(p), MBC, m, m, ac.shape[-1], _ptr(qc), _ptr(ac),
                              _ptr(qf), _ptr(af), igrid)


def timeinterp(qcurr, qlast, qinterp, alpha):
    m = qcurr.shape[0] - 2 * MBC
    psize = 3 * 8 * (m - 2)  # meqn x the strip cell count the Fortran expects
    return load().orc_timeinterp(MBC, m, m, psize, _ptr(qcurr), _ptr(qlast), _ptr(qinterp), alpha)


def tag4refinement(q, aux, xlower, ylower, dx, dy, t, level, maxlevel, init_flag, rf, phys=None):
    p = params(phys)
    m = q.shape[0] - 2 * MBC
    return load().orc_tag4refinement(C.byref(p), C.byref(rf), MBC, m, m, aux.shape[-1], _ptr(q),
                                     _ptr(aux), xlower, ylower, dx, dy, t, level, maxlevel,
                                     init_flag)


def tag4coarsening(qs, auxs, xlowers, ylowers, dx, dy, t, level, maxlevel, init_flag, rf,
                   phys=None):
    p = params(phys)
    m = qs[0].shape[0] - 2 * MBC
    qp = (_dp * 4)(*[_ptr(a) for a in qs])
    ap = (_dp * 4)(*[_ptr(a) for a in auxs])
    xl = np.ascontiguousarray(xlowers, dtype=np.float64)
    yl = np.ascontiguousarray(ylowers, dtype=np.float64)
    return load().orc_tag4coarsening(C.byref(p), C.byref(rf), MBC, m, m, auxs[0].shape[-1], qp, ap,
                                     _ptr(xl), _ptr(yl), dx, dy, t, level, maxlevel, init_flag)


def brick_neighbours(npx: int, npy: int, mx: int, dx: float, dy: float, x0: float = 0.0,
                     y0: float = 0.0):
    """Neighbour table (left, right, bottom, top, ll, lr, ul, ur; -1 physical)
    and patch origins of an npx x npy brick, patch = py*npx + px."""
    n = npx * npy
    nbr = -np.ones((n, 8), np.int32)
    xl, yl = np.zeros(n), np.zeros(n)

    def at(px, py):
        return py * npx + px if 0 <= px < npx and 0 <= py < npy else -1

    for py in range(npy):
        for px in range(npx):
            k = py * npx + px
            nbr[k] = [at(px - 1, py), at(px + 1, py), at(px, py - 1), at(px, py + 1),
                      at(px - 1, py - 1), at(px + 1, py - 1), at(px - 1, py + 1),
                      at(px + 1, py + 1)]
            xl[k], yl[k] = x0 + px * mx * dx, y0 + py * mx * dy
    return nbr, xl, yl


def run_scenario(q, aux, mx, npx, npy, dx, dy, t_final, nout, initial_dt, desired_cfl,
                 max_cfl, mthbc, phys=None, hy=None, xlower=0.0, ylower=0.0, nthreads=0):
    """Single-level run with ForestClaw's outstyle-1 time stepping
    (src/fc2d_geoclaw/fc2d_geoclaw_run.c:190-395, variable dt, reduce_cfl on):
    per step, ghost fill at the step's start time, level update, CFL test.

    q (npatch, mx+4, mx+4, 3) is advanced in place; returns
    (accepted steps, rejected steps, list of accepted dt)."""
    nbr, xl, yl = brick_neighbours(npx, npy, mx, dx, dy, xlower, ylower)
    dt_outer = t_final / nout
    t_curr = 0.0
    dt_minlevel = initial_dt
    steps, rejects, dts = 0, 0, []
    for _ in range(nout):
        tend = t_curr + dt_outer
        while t_curr < tend:
            dt_step = dt_minlevel
            tol = 1e-2 * dt_step
            took_small = False
            small_step = tend - (t_curr + dt_step)
            if small_step < tol:
                dt_step = tend - t_curr
                if small_step < 0:
                    took_small = True
            save = q.copy()
            level_ghost_fill(q, aux, nbr, xl, yl, dx, dy, t_curr, mthbc, phys, hy)
            cfl = level_update(q, aux, dx, dy, t_curr, dt_step, phys, nthreads)
            if cfl > max_cfl:
                q[...] = save
                dt_minlevel = dt_minlevel * desired_cfl / cfl
                rejects += 1
                continue
            steps += 1
            t_curr += dt_step
            dts.append(dt_step)
            dt_new = dt_minlevel * desired_cfl / cfl if cfl > 0.0 else float("inf")
            if not took_small:
                dt_minlevel = dt_new
    return steps, rejects, dts
