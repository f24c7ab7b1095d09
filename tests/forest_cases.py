"""Small multi-level forest cases shared by the CPU and GPU forest tests."""
import numpy as np

import geoflood_gb300 as gf
from geoflood_gb300 import synth

M, NBX, NBY, LMIN, LMAX = 8, 2, 1, 1, 3
DX0 = 1000.0 / M            # 1000 m root blocks


def rasters(kind="dambreak", seed=3, m=M, lmax=LMAX):
    nx, ny = NBX * m << lmax, NBY * m << lmax
    dxf = 1000.0 / m / (1 << lmax)
    b = synth.bump_ramp_dem(nx, ny, dxf, dxf, seed=seed)
    q = np.zeros((ny, nx, 3))
    if kind == "lake":
        q[..., 0] = np.maximum(8.0 - b, 0.0)
    else:
        x = (np.arange(nx) + 0.5) * dxf
        q[..., 0] = np.where(x[None, :] < 600.0, 10.0, 0.0)
    return b, q


def balanced(leaves, nbx, nby, lmax):
    """Leaves tile the domain and touching leaves differ by at most a level."""
    rects = [(l, I << (lmax - l), J << (lmax - l), 1 << (lmax - l)) for (l, I, J) in leaves]
    if sum(r[3] ** 2 for r in rects) != (nbx << lmax) * (nby << lmax):
        return False
    for a in rects:
        for b in rects:
            if a is b:
                continue
            if (a[1] <= b[1] + b[3] and b[1] <= a[1] + a[3] and a[2] <= b[2] + b[3]
                    and b[2] <= a[2] + a[3] and abs(a[0] - b[0]) > 1):
                return False
    return True


FRONT = gf.Refine(wave_tolerance=1e9, flowgrades=((1.0, 2, 1, LMAX),))
LAKE_REGION = gf.Refine(wave_tolerance=1e9, regions=((0.0, 600.0, 0.0, 400.0, 0.0, 1e9, 3, 3),))
