"""Generate tests/golden/patch_pin.npz from the reference's own patch update.

Runs the reference's CUDA patch kernel body cudaclaw_flux2_and_update
(src/fc2d_cpu_cuda/cuda_source/cudaclaw_flux2.cu:63-1160) with its limiter
(cudaclaw_limiters.cu), Riemann solvers (riemann_source/geoflood_rp2.cu) and
friction source (riemann_source/geoflood_src2.cu), compiled for the host by
oracle/build_ref.sh (oracle/_ref/libref_patch.so), on seeded one-step patch
problems: dam breaks on a fractal DEM at t = 0 and after the flood has
developed, random wet/dry states with momentum, a partly dry lake at rest,
with friction on (everywhere or only in shallow cells) and off, every MC /
minmod / superbee / van Leer limiter, first order and no transverse waves,
at mx = 8, 16 and 32. Stores inputs, the reference's updated interior and
its patch CFL; tests/test_patch_pin.py replays them on the oracle.

The reference's CUDA port departs from the Fortran in ways that show here
only at rounding level (the sum orders of the second-order and transverse
parts) and in ways these cases avoid: its y-direction second-order term
uses dt/dx (so only dx = dy is pinned) and its friction reads one Manning
coefficient (so the Manning table and variable friction are not pinned).

Usage: GF_REFERENCE_ROOT=<GeoFlood tree> python tests/golden/make_patch_pin.py
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
OUT = Path(__file__).resolve().parent / "patch_pin.npz"
G, DRYTOL = 9.81, 1e-3

import oracle  # noqa: E402
from geoflood_gb300 import Phys, synth  # noqa: E402


def load_ref():
    lib_path = ROOT / "oracle" / "_ref" / "libref_patch.so"
    if not lib_path.exists():
        ref = os.environ.get("GF_REFERENCE_ROOT", "")
        subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh"), ref], check=True)
    if not lib_path.exists():
        raise SystemExit("reference tree not available (set GF_REFERENCE_ROOT): cannot build oracle/_ref")
    lib = C.CDLL(str(lib_path))
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    lib.ref_patch_update.restype = C.c_double
    lib.ref_patch_update.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                     C.c_double, ip, ip, C.c_int, C.c_double, C.c_double,
                                     C.c_double, C.c_double, dp, dp]
    return lib


def ref_step(lib, q, b, dx, dt, order, transverse, mthlim, src_term, manning, friction_depth):
    """One reference patch update of q (my+4, mx+4, 3) over b (my+4, mx+4);
    returns the updated q in the same layout and the kernel's patch CFL."""
    m = q.shape[0] - 4
    qs = np.ascontiguousarray(np.transpose(q, (2, 0, 1)))
    bs = np.ascontiguousarray(b)
    dp = C.POINTER(C.c_double)
    cfl = lib.ref_patch_update(m, m, dx, dx, 0.0, dt, (C.c_int * 2)(order, transverse),
                               (C.c_int * 3)(*mthlim), src_term, DRYTOL, G, manning,
                               friction_depth, qs.ctypes.data_as(dp), bs.ctypes.data_as(dp))
    return np.ascontiguousarray(np.transpose(qs, (1, 2, 0))), cfl


def states(m: int, rng: np.random.Generator):
    """(name, q, b, dx) one-patch problems of m x m cells with their halo."""
    dx = 64.0 / m
    out = []
    # dam break on the fractal DEM with its channel: the patch across the front
    q, b, _, _ = synth.uniform_dam_break_level(2, 1, m, dx, seed=int(rng.integers(1 << 30)),
                                               x_dam=0.9 * m * dx)
    out.append(("dambreak", q[0], b[0, ..., 0], dx))
    out.append(("dambreak_dry_side", q[1], b[1, ..., 0], dx))
    # the same flood after 12 oracle steps: shocks, rarefactions, moving fronts
    qd = q.copy()
    aux = b.copy()
    nbr, xl, yl = synth.brick_layout(1, 2, m, dx)
    for _ in range(12):
        oracle.level_ghost_fill(qd, aux, nbr, xl, yl, dx, dx, 0.0, mthbc=(3, 3, 3, 3))
        oracle.level_update(qd, aux, dx, dx, 0.0, 0.25 * dx / 12.0, nthreads=1)
    oracle.level_ghost_fill(qd, aux, nbr, xl, yl, dx, dx, 0.0, mthbc=(3, 3, 3, 3))
    out.append(("developed", qd[0].copy(), b[0, ..., 0], dx))
    out.append(("developed_front", qd[1].copy(), b[1, ..., 0], dx))
    # random wet/dry cells with momentum over rough bathymetry
    n = m + 4
    bb = rng.normal(0.0, 0.5, (n, n))
    h = np.where(rng.random((n, n)) < 0.25, rng.uniform(0.0, 2 * DRYTOL, (n, n)),
                 rng.uniform(0.05, 3.0, (n, n)))
    qr = np.stack([h, h * rng.normal(0, 1.5, (n, n)), h * rng.normal(0, 1.5, (n, n))], -1)
    out.append(("random_wetdry", qr, bb, dx))
    # lake at rest over the same rough bed, partly dry
    eta = 0.3
    hl = np.maximum(eta - bb, 0.0)
    ql = np.stack([hl, np.zeros_like(hl), np.zeros_like(hl)], -1)
    out.append(("lake_at_rest", ql, bb, dx))
    return out


METHODS = [  # (order, transverse, mthlim, src_term, friction_depth)
    (2, 2, (4, 4, 4), 1, 1.0e6),
    (2, 2, (4, 4, 4), 0, 1.0e6),
    (2, 2, (4, 4, 4), 1, 0.5),
    (2, 2, (1, 2, 3), 1, 1.0e6),
    (2, 0, (4, 4, 4), 1, 1.0e6),
    (1, 2, (4, 4, 4), 1, 1.0e6),
]


def main():
    lib = load_ref()
    rng = np.random.Generator(np.random.PCG64(20261204))
    rows = {k: [] for k in ("m", "dx", "dt", "method", "q", "b", "out", "cfl", "name")}
    for m in (8, 16, 32):
        for name, q, b, dx in states(m, rng):
            for mi, (order, tr, lim, src, fdepth) in enumerate(METHODS):
                if name.startswith("dambreak") and mi not in (0, 1):
                    continue
                dt = float(rng.uniform(0.15, 0.3)) * dx / 12.0
                manning = float(rng.uniform(0.02, 0.08))
                qout, cfl = ref_step(lib, q.copy(), b, dx, dt, order, tr, lim, src, manning, fdepth)
                rows["m"].append(m)
                rows["dx"].append(dx)
                rows["dt"].append(dt)
                rows["method"].append([order, tr, *lim, src, fdepth, manning])
                pad = np.zeros((36, 36, 3))
                pad[:m + 4, :m + 4] = q
                rows["q"].append(pad)
                padb = np.zeros((36, 36))
                padb[:m + 4, :m + 4] = b
                rows["b"].append(padb)
                po = np.zeros((32, 32, 3))
                po[:m, :m] = qout[2:2 + m, 2:2 + m]
                rows["out"].append(po)
                rows["cfl"].append(cfl)
                rows["name"].append(name)
    np.savez_compressed(OUT, **{k: np.array(v) for k, v in rows.items()}, grav=G, drytol=DRYTOL)
    print(f"wrote {OUT} ({len(rows['m'])} patch steps)")


if __name__ == "__main__":
    main()
