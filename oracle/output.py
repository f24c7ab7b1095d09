"""Output formats -- TEST INFRASTRUCTURE ONLY (the oracle).

A plain-Python restatement of the reference's frame and gauge files:

- fort.tXXXX / fort.qXXXX, written by fc2d_geoclaw_fort_write_header and
  fc2d_geoclaw_fort_write_file
  (src/fc2d_geoclaw/fclaw2d_source/fc2d_geoclaw_output_ascii_fort.f:1-117)
  for every patch of the domain
  (src/fc2d_geoclaw/fc2d_geoclaw_output_ascii.c:38-109);
- gaugeXXXXX.txt headers and rows
  (src/fc2d_geoclaw/fc2d_geoclaw_gauges_default.c:172-200, 275-305) with
  values from fc2d_geoclaw_update_gauge
  (src/fc2d_geoclaw/fortran_source/geoclaw_gauges_fort.f90:1-77);
- gauges.data as geoclaw_read_gauges_data_default reads it
  (src/fc2d_geoclaw/fc2d_geoclaw_gauges_default.c:56-167).

Fortran Ew.d edit descriptors are formed here from the exact decimal value
of the double (decimal module), rounded half-even to d significant digits --
an independent route from the library's printf-based one. Patch order in a
forest frame follows p4est (tree along the brick's Morton curve, leaves by
the Morton index of their lower-left corner); p4est and ForestClaw's gauge
scheduling are not in the reference tree, so those two rules are unpinned.
"""
from __future__ import annotations

import decimal
import math
import os

import numpy as np

MBC = 2


def fort_e(x: float, w: int, d: int) -> str:
    """Fortran Ew.d of x: [-]0.<d digits>E+xx, right-justified in w
    characters; a three-digit exponent drops the E."""
    x = float(x)
    neg = math.copysign(1.0, x) < 0
    if x == 0.0:
        digits, e10 = "0" * d, 0
    else:
        ctx = decimal.Context(prec=d, rounding=decimal.ROUND_HALF_EVEN)
        v = ctx.plus(decimal.Decimal(abs(x)))        # exact value, rounded to d digits
        _, dig, exp = v.as_tuple()
        s = "".join(map(str, dig))
        digits = s.ljust(d, "0")
        e10 = exp + len(s)                           # value = 0.<s> x 10^e10
    ae = abs(e10)
    expo = ("E%s%02d" if ae <= 99 else "%s%03d") % ("-" if e10 < 0 else "+", ae)
    s = ("-" if neg else "") + "0." + digits + expo
    return s.rjust(w)


def fort_i(v: int, w: int) -> str:
    return ("%d" % v).rjust(w)


def _tiny0(v: float) -> float:
    return 0.0 if abs(v) < 1e-99 else v


def frame_text(time: float, q: np.ndarray, aux: np.ndarray, level, block, xlower, ylower, dx, dy,
               grid_number=None) -> tuple[str, str]:
    """(fort.t text, fort.q text) for patches in the given order.
    q: (npatch, n4, n4, 3), aux: (npatch, n4, n4, maux), ghosts included."""
    npatch, n4 = q.shape[0], q.shape[1]
    mx = n4 - 2 * MBC
    maux = aux.shape[3]
    t = (fort_e(time, 30, 20) + "    time\n"
         + fort_i(4, 5) + "                 meqn\n"
         + fort_i(npatch, 5) + "                 ngrids\n"
         + fort_i(maux, 5) + "                 num_aux\n"
         + fort_i(2, 5) + "                 num_dim\n"
         + fort_i(MBC, 5) + "                 num_ghost\n")
    out = []
    for k in range(npatch):
        gn = k if grid_number is None else int(grid_number[k])
        out.append(fort_i(gn, 5) + "                 grid_number\n")
        out.append(fort_i(int(level[k]), 5) + "                 AMR_level\n")
        out.append(fort_i(int(block[k]), 5) + "                 block_number\n")
        out.append(fort_i(0, 5) + "                 mpi_rank\n")
        out.append(fort_i(mx, 5) + "                 mx\n")
        out.append(fort_i(mx, 5) + "                 my\n")
        out.append(fort_e(xlower[k], 24, 16) + "    xlow\n")
        out.append(fort_e(ylower[k], 24, 16) + "    ylow\n")
        out.append(fort_e(dx[k], 24, 16) + "    dx\n")
        out.append(fort_e(dy[k], 24, 16) + "    dy\n\n")
        for j in range(MBC, MBC + mx):
            for i in range(MBC, MBC + mx):
                h, hu, hv = (_tiny0(float(v)) for v in q[k, j, i])
                eta = _tiny0(h + float(aux[k, j, i, 0]))
                out.append("".join(fort_e(v, 26, 16) for v in (h, hu, hv, eta)) + "\n")
            out.append("  \n")          # list-directed write of ' '
    return t, "".join(out)


def write_frame(dirname: str, iframe: int, time: float, *args, **kw) -> None:
    t, q = frame_text(time, *args, **kw)
    with open(os.path.join(dirname, "fort.t%04d" % (iframe % 10000)), "w") as f:
        f.write(t)
    with open(os.path.join(dirname, "fort.q%04d" % (iframe % 10000)), "w") as f:
        f.write(q)


def gauge_header(gid: int, xc: float, yc: float) -> str:
    return ("# gauge_id= %5d location=( %17.10e %17.10e ) num_eqn= %2d\n" % (gid, xc, yc, 4)
            + "# Columns: level time h    hu    hv    eta\n")


def gauge_rows(rows) -> str:
    """rows: iterable of (level, t, h, hu, hv, bathymetry)."""
    out = []
    for lev, t, h, hu, hv, b in rows:
        eta = _tiny0(h + b)
        out.append("%5d %15.7e %15.7e %15.7e %15.7e %15.7e\n" % (lev, t, h, hu, hv, eta))
    return "".join(out)


def gauge_cell(mx, xlower, ylower, dx, dy, xc, yc):
    """(ii, jj, xoff, yoff) of fc2d_geoclaw_update_gauge (geoclaw_gauges_fort.f90:19-25),
    clamped to the cells the stencil can reach."""
    ii = min(max(int((xc - xlower) / dx) + 1, 1), mx + 1)
    jj = min(max(int((yc - ylower) / dy) + 1, 1), mx + 1)
    xoff = (xc - (xlower + (ii - .5) * dx)) / dx
    yoff = (yc - (ylower + (jj - .5) * dy)) / dy
    return ii, jj, xoff, yoff


def sample_gauge(q, aux, ii, jj, xoff, yoff, dry_tolerance):
    """(h, hu, hv, bathymetry) at one gauge (geoclaw_gauges_fort.f90:27-75).
    q: (n4, n4, 3), aux: (n4, n4, maux) of the patch; (ii, jj) 1-based."""
    drytol2 = 0.1 * dry_tolerance
    a, b = ii + MBC - 1, jj + MBC - 1          # array index of cell (ii, jj)
    cells = ((b, a), (b, a + 1), (b + 1, a), (b + 1, a + 1))
    if any(float(q[c][0]) < drytol2 for c in cells):
        v = [float(x) for x in q[b, a]]
        topo = float(aux[b, a, 0])
    else:
        w = ((1.0 - xoff) * (1.0 - yoff), xoff * (1.0 - yoff), (1.0 - xoff) * yoff, xoff * yoff)
        v = []
        for m in range(3):
            s = w[0] * float(q[cells[0]][m])
            s = s + w[1] * float(q[cells[1]][m])
            s = s + w[2] * float(q[cells[2]][m])
            s = s + w[3] * float(q[cells[3]][m])
            v.append(s)
        topo = w[0] * float(aux[cells[0]][0])
        topo = topo + w[1] * float(aux[cells[1]][0])
        topo = topo + w[2] * float(aux[cells[2]][0])
        topo = topo + w[3] * float(aux[cells[3]][0])
    return tuple(_tiny0(x) for x in v) + (topo,)


def read_gauges_data(path: str) -> list[tuple]:
    """[(id, x, y, t1, t2, min_time_increment)] from a gauges.data file."""
    with open(path) as f:
        lines = f.read().split("\n")
    for k in range(5):
        if not lines[k].startswith("#"):
            raise ValueError("gauges.data: bad header")
    n = int(float(lines[6].split()[0]))
    gauges = []
    for k in range(n):
        p = lines[7 + k].split()
        gauges.append([int(float(p[0])), float(p[1]), float(p[2]), float(p[3]), float(p[4])])
    incr = lines[7 + n + 8].split()
    return [tuple(g) + (float(incr[k]),) for k, g in enumerate(gauges)]


def brick_tree_ids(mi: int, mj: int) -> dict:
    """{(bx, by): tree} along the Morton curve over the brick's power-of-two box."""
    lx = max(0, (mi - 1).bit_length())
    ly = max(0, (mj - 1).bit_length())
    ids, nxt = {}, 0
    for ti in range(1 << (lx + ly)):
        x = y = c = 0
        for i in range(max(lx, ly)):
            if i < lx:
                x |= ((ti >> c) & 1) << i
                c += 1
            if i < ly:
                y |= ((ti >> c) & 1) << i
                c += 1
        if x < mi and y < mj:
            ids[(x, y)] = nxt
            nxt += 1
    return ids


def _morton(x: int, y: int) -> int:
    k = 0
    for b in range(32):
        k |= ((x >> b) & 1) << (2 * b) | ((y >> b) & 1) << (2 * b + 1)
    return k


def p4est_order(keys, nbx: int, nby: int, maxlevel: int):
    """keys: [(level, I, J)] -> (order of the keys, tree of each key)."""
    tid = brick_tree_ids(nbx, nby)
    trees, sort_keys = [], []
    for n, (l, I, J) in enumerate(keys):
        bx, by = I >> l, J >> l
        sx = (I - (bx << l)) << (maxlevel - l)
        sy = (J - (by << l)) << (maxlevel - l)
        t = tid[(bx, by)]
        trees.append(t)
        sort_keys.append((t, _morton(sx, sy), n))
    return [k[2] for k in sorted(sort_keys)], trees
