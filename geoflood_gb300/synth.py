"""Seeded synthetic flood inputs: DEMs, initial states and patch tilings.

No public dataset is used; these generators produce inputs with the shapes,
sizes and value ranges of the workloads the patch update is measured on:

* ``bump_ramp_dem``   - b = 0.001 x + 8 seeded Gaussian bumps (amplitude
  U[0.5, 3] m, sigma U[20, 80] m): the dam-break workload on a ramp.
* ``fractal_dem``     - diamond-square fractal DEM (Hurst exponent, relief)
  with an optional straight carved channel.
* ``dam_break_state`` - water surface 10 m above b for x < x_dam, dry beyond.
* ``tile_level``      - cut a global cell array (with a 2-cell halo) into
  patches with ghost cells, in the Fortran layout the hooks use.
"""
from __future__ import annotations

import numpy as np

MBC = 2


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def diamond_square(levels: int, hurst: float, seed: int) -> np.ndarray:
    """(2^levels + 1)^2 lattice of a diamond-square fractal with displacement
    scale 2^(-hurst) per level, normalised to zero mean and unit deviation."""
    n = 2 ** levels
    g = rng(seed)
    a = np.zeros((n + 1, n + 1))
    a[::n, ::n] = g.standard_normal((2, 2))
    step, scale = n, 1.0
    while step > 1:
        half = step // 2
        scale *= 0.5 ** hurst
        # diamond step: centres of the squares
        c = 0.25 * (a[0:n:step, 0:n:step] + a[step::step, 0:n:step]
                    + a[0:n:step, step::step] + a[step::step, step::step])
        a[half::step, half::step] = c + scale * g.standard_normal(c.shape)
        # square step: edge midpoints (their neighbours are corners and centres)
        for rr, cc in ((np.arange(0, n + 1, step), np.arange(half, n, step)),
                       (np.arange(half, n, step), np.arange(0, n + 1, step))):
            R, Cc = np.meshgrid(rr, cc, indexing="ij")
            acc = np.zeros(R.shape)
            cnt = np.zeros(R.shape)
            for dr, dc in ((-half, 0), (half, 0), (0, -half), (0, half)):
                r2, c2 = R + dr, Cc + dc
                ok = (r2 >= 0) & (r2 <= n) & (c2 >= 0) & (c2 <= n)
                acc += np.where(ok, a[np.clip(r2, 0, n), np.clip(c2, 0, n)], 0.0)
                cnt += ok
            a[R, Cc] = acc / cnt + scale * g.standard_normal(acc.shape)
        step = half
    a -= a.mean()
    sd = a.std()
    return a / sd if sd > 0 else a


def fractal_dem(nx: int, ny: int, dx: float, hurst: float, relief: float, seed: int,
                channel_depth: float = 0.0, channel_width: float = 0.0,
                x0: float = 0.0, y0: float = 0.0) -> np.ndarray:
    """Cell-centred bathymetry (ny, nx): a diamond-square surface scaled to
    `relief` metres peak to peak, plus a straight channel along x at the
    domain centre `channel_depth` deep and `channel_width` wide."""
    n = max(nx, ny)
    lv = int(np.ceil(np.log2(max(n, 2))))
    lat = diamond_square(lv, hurst, seed)
    cell = 0.25 * (lat[:-1, :-1] + lat[1:, :-1] + lat[:-1, 1:] + lat[1:, 1:])
    b = cell[:ny, :nx]
    b = (b - b.min()) / max(b.max() - b.min(), 1e-300) * relief
    if channel_depth > 0.0 and channel_width > 0.0:
        y = y0 + (np.arange(ny) + 0.5) * dx
        yc = y0 + 0.5 * ny * dx
        inside = np.abs(y - yc) <= 0.5 * channel_width
        b = b - channel_depth * inside[:, None]
    return np.ascontiguousarray(b)


def bump_ramp_dem(nx: int, ny: int, dx: float, dy: float, seed: int, nbump: int = 8,
                  x0: float = 0.0, y0: float = 0.0) -> np.ndarray:
    """b = 0.001 x + sum of nbump Gaussian bumps (amplitude U[0.5,3] m,
    sigma U[20,80] m, centres uniform over the domain)."""
    g = rng(seed)
    x = x0 + (np.arange(nx) + 0.5) * dx
    y = y0 + (np.arange(ny) + 0.5) * dy
    X, Y = np.meshgrid(x, y)
    lx, ly = nx * dx, ny * dy
    b = 0.001 * X
    for _ in range(nbump):
        amp = g.uniform(0.5, 3.0)
        sig = g.uniform(20.0, 80.0)
        cx, cy = x0 + g.uniform(0, lx), y0 + g.uniform(0, ly)
        b = b + amp * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * sig * sig))
    return np.ascontiguousarray(b)


def dam_break_state(b: np.ndarray, dx: float, x_dam: float = 600.0, depth: float = 10.0,
                    x0: float = 0.0) -> np.ndarray:
    """q (ny, nx, 3): surface `depth` metres above b for x < x_dam, dry beyond."""
    ny, nx = b.shape
    x = x0 + (np.arange(nx) + 0.5) * dx
    h = np.where(x[None, :] < x_dam, depth, 0.0) * np.ones_like(b)
    q = np.zeros((ny, nx, 3))
    q[..., 0] = h
    return q


def pad_extrap(a: np.ndarray, mbc: int = MBC) -> np.ndarray:
    """Add a halo by zero-order extrapolation (the mthbc = 1 rule)."""
    pad = [(mbc, mbc), (mbc, mbc)] + [(0, 0)] * (a.ndim - 2)
    return np.pad(a, pad, mode="edge")


def pad_wall(q: np.ndarray, mbc: int = MBC) -> np.ndarray:
    """Halo for q by the solid-wall rule (mthbc = 3): mirror, negate the
    normal momentum (geoflood_bc2_fort.f90:118-131 and the y analogue)."""
    out = np.pad(q, [(mbc, mbc), (mbc, mbc), (0, 0)], mode="symmetric")
    ny, nx = q.shape[:2]
    out[:, :mbc, 1] *= -1
    out[:, nx + mbc:, 1] *= -1
    out[:mbc, :, 2] *= -1
    out[ny + mbc:, :, 2] *= -1
    return out


def tile_level(field: np.ndarray, m: int, mbc: int = MBC, out: np.ndarray | None = None) -> np.ndarray:
    """Cut a haloed global array (NY+2mbc, NX+2mbc, nf) into patches of m x m
    interior cells, each with its mbc-wide ghost ring taken from the global
    array. Returns (npatch, m+2mbc, m+2mbc, nf), patches row-major in (py, px),
    written into `out` when given."""
    NY, NX = field.shape[0] - 2 * mbc, field.shape[1] - 2 * mbc
    assert NX % m == 0 and NY % m == 0
    py, px = NY // m, NX // m
    n4 = m + 2 * mbc
    f = np.ascontiguousarray(field)
    s0, s1, s2 = f.strides
    view = np.lib.stride_tricks.as_strided(f, shape=(py, px, n4, n4, f.shape[2]),
                                           strides=(m * s0, m * s1, s0, s1, s2), writeable=False)
    if out is None:
        return np.ascontiguousarray(view).reshape(py * px, n4, n4, f.shape[2])
    np.copyto(out.reshape(py, px, n4, n4, f.shape[2]), view)
    return out


def untile_level(patches: np.ndarray, py: int, px: int, mbc: int = MBC) -> np.ndarray:
    """Inverse of tile_level for the interiors: (py*m, px*m, nf)."""
    n4 = patches.shape[1]
    m = n4 - 2 * mbc
    out = np.empty((py * m, px * m, patches.shape[3]))
    k = 0
    for j in range(py):
        for i in range(px):
            out[j * m:(j + 1) * m, i * m:(i + 1) * m] = patches[k, mbc:mbc + m, mbc:mbc + m]
            k += 1
    return out


def uniform_dam_break_level(npx: int, npy: int, m: int, dx: float, seed: int,
                            dem: str = "fractal", x_dam: float = 600.0,
                            depth: float = 10.0):
    """A single uniform level of npx x npy patches of m x m cells for the
    dam-break workload. Returns (q_patches, aux_patches, py, px)."""
    nx, ny = npx * m, npy * m
    if dem == "fractal":
        b = fractal_dem(nx, ny, dx, hurst=0.8, relief=30.0, seed=seed,
                        channel_depth=5.0, channel_width=40.0)
    else:
        b = bump_ramp_dem(nx, ny, dx, dx, seed)
    q = dam_break_state(b, dx, x_dam=x_dam, depth=depth)
    qh = pad_extrap(q)
    bh = pad_extrap(b[..., None])
    return tile_level(qh, m), tile_level(bh, m), npy, npx


def brick_layout(py: int, px: int, m: int, dx: float, dy: float | None = None,
                 x0: float = 0.0, y0: float = 0.0, periodic_x: bool = False,
                 periodic_y: bool = False):
    """Neighbour table (npatch, 8) and patch origins of a uniform py x px grid
    of m x m patches (row-major, as tile_level orders them). Entries: faces
    left, right, bottom, top, corners ll, lr, ul, ur; -1 = physical side."""
    dy = dx if dy is None else dy
    n = py * px
    nbr = -np.ones((n, 8), np.int32)
    xl = np.zeros(n)
    yl = np.zeros(n)

    def idx(j, i):
        if periodic_x:
            i %= px
        if periodic_y:
            j %= py
        if 0 <= i < px and 0 <= j < py:
            return j * px + i
        return -1

    for j in range(py):
        for i in range(px):
            k = j * px + i
            nbr[k] = [idx(j, i - 1), idx(j, i + 1), idx(j - 1, i), idx(j + 1, i),
                      idx(j - 1, i - 1), idx(j - 1, i + 1), idx(j + 1, i - 1), idx(j + 1, i + 1)]
            xl[k] = x0 + i * m * dx
            yl[k] = y0 + j * m * dy
    nbr[nbr == np.arange(n)[:, None]] = -1  # a 1-wide periodic grid has no true neighbour
    return nbr, xl, yl


_LATTICE_CACHE: dict = {}


def _lattice_window(nx: int, ny: int, hurst: float, seed: int, pool: int = 2) -> np.ndarray:
    """(ny, nx) window of one of `pool` cached diamond-square lattices, picked
    and offset by `seed`; large scenarios share lattices instead of growing
    a new 4097^2 surface each."""
    n = max(nx, ny)
    lv = max(int(np.ceil(np.log2(max(n, 2)))), 8)
    if lv >= 11:
        key = (12, hurst, seed % pool)
        lv = 12
    else:
        key = (lv, hurst, seed)
    lat = _LATTICE_CACHE.get(key)
    if lat is None:
        lat = diamond_square(key[0], hurst, 7919 * key[2] + 17)
        cell = 0.25 * (lat[:-1, :-1] + lat[1:, :-1] + lat[:-1, 1:] + lat[1:, 1:])
        lat = cell
        if len(_LATTICE_CACHE) > 8:
            _LATTICE_CACHE.clear()
        _LATTICE_CACHE[key] = lat
    g = rng(seed + 1)
    oy = int(g.integers(0, lat.shape[0] - ny + 1))
    ox = int(g.integers(0, lat.shape[1] - nx + 1))
    return lat[oy:oy + ny, ox:ox + nx]


def flood_scenario_params(seed: int, cells: float, mx: int | None = None, dx: float = 5.0,
                          time_scale: float = 1.0 / 150.0) -> dict:
    """The scalar draws of flood_scenario (sizes, channel, hydrograph,
    friction, horizon) without building any arrays."""
    g = rng(seed)
    if mx is None:
        mx = int(g.choice([8, 16, 32]))
    npt = max(1, int(round(cells / (mx * mx))))
    npy = max(1, int(round(np.sqrt(npt / 2.0))))
    npx = max(1, int(round(npt / npy)))
    ly = npy * mx * dx
    width = float(max(g.uniform(30.0, 80.0), 3 * dx))
    width = min(width, 0.5 * ly)
    amp = 0.15 * ly * float(g.uniform(0.3, 1.0))
    peak = float(g.uniform(10.0, 500.0))
    t_rise = float(g.uniform(0.5, 2.0)) * 3600.0 * time_scale
    horizon = float(g.uniform(1.0, 6.0)) * 3600.0 * time_scale
    n = float(g.uniform(0.02, 0.08))
    return dict(mx=mx, npx=npx, npy=npy, dx=dx, width=width, amp=amp, peak=peak, t_rise=t_rise,
                horizon=horizon, manning=n)


def flood_scenario(seed: int, cells: float, mx: int | None = None, dx: float = 5.0,
                   time_scale: float = 1.0 / 150.0, relief: float = 10.0, alloc=None):
    """One served flood scenario: a river valley on a fractal DEM fed by an
    inflow hydrograph on the left side (mthbc 0 there, extrapolation on the
    right, walls top and bottom).

    - mx drawn from {8, 16, 32} unless given; npx x npy patches (about 2:1)
      with about `cells` interior cells at `dx` metres.
    - DEM: fractal surface (Hurst 0.8, `relief` m) on a 0.002 down-valley
      slope, with a meandering channel 3 m deep and U[30, 80] m wide.
    - Water: 2 m in the channel at t = 0, dry elsewhere.
    - Hydrograph: discharge rising from 10 % of a peak Q ~ U[10, 500] m^3/s
      to the peak at t_rise ~ U[0.5, 2] h and back by 3 t_rise, per unit
      channel width; Manning n ~ U[0.02, 0.08]; horizon U[1, 6] h.
    - All times (rise, horizon) are multiplied by `time_scale`.

    `alloc(shape)` (optional) provides the q and aux arrays (e.g. pinned).
    """
    from . import Phys
    from .serve import Hydrograph, Scenario
    p = flood_scenario_params(seed, cells, mx, dx, time_scale)
    mx, npx, npy, width = p["mx"], p["npx"], p["npy"], p["width"]
    nx, ny = npx * mx, npy * mx
    lx, ly = nx * dx, ny * dx
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dx
    surf = _lattice_window(nx, ny, 0.8, seed)
    surf = (surf - surf.min()) / max(surf.max() - surf.min(), 1e-300) * relief
    yc = 0.5 * ly + p["amp"] * np.sin(2.0 * np.pi * x / max(lx, 1.0))
    inside = np.abs(y[:, None] - yc[None, :]) <= 0.5 * width
    b = surf + 0.002 * (lx - x)[None, :] - 3.0 * inside
    q = np.zeros((ny, nx, 3))
    q[..., 0] = np.where(inside, 2.0, 0.0)
    peak, t_rise = p["peak"], p["t_rise"]
    hy = Hydrograph(time=np.array([0.0, t_rise, 3.0 * t_rise]),
                    hu=np.array([0.1 * peak, peak, 0.1 * peak]) / width,
                    side=(1, 0, 0, 0), width=width, x0=0.0, y0=0.5 * ly)
    n4 = mx + 2 * MBC
    qt = alloc((npx * npy, n4, n4, 3)) if alloc else None
    at = alloc((npx * npy, n4, n4, 1)) if alloc else None
    qt = tile_level(pad_extrap(q), mx, out=qt)
    at = tile_level(pad_extrap(b[..., None]), mx, out=at)
    return Scenario(mx=mx, npx=npx, npy=npy, dx=dx, dy=dx, q=qt, aux=at, t_final=p["horizon"],
                    phys=Phys(manning_coefficient=(p["manning"],), manning_break=(1.0e10,)),
                    mthbc=(0, 1, 3, 3), hydro=hy, nout=4, initial_dt=0.2, seed=seed)


def flood_forest(seed: int, target_patches: float, mx: int | None = None, minlevel: int = 2,
                 maxlevel: int = 5, wet_fraction: float = 0.5):
    """One batched-AMR forest: nbx x nby root blocks (at most 4 x 2) sized so
    that refining the wet part of the domain to maxlevel gives about
    `target_patches` patches; fractal valley DEM (Hurst 0.8, 10 m relief,
    0.002 slope), a reservoir at the left end sized for the target (surface
    0.5 m above the 70th percentile of its bed), inflow hydrograph on the left
    (peak Q ~ U[10, 500] m^3/s over a 40 m window, per unit width), n ~
    U[0.02, 0.08]; finest cells are 2 m. Refinement: depth > 0.01 m up to
    maxlevel. Returns the Forest keyword arguments plus 'hydro' and 'phys'."""
    from . import Phys, Refine
    g = rng(seed)
    if mx is None:
        mx = int(g.choice([8, 16, 32]))
    full_per_block = 4 ** maxlevel
    need = target_patches / max(wet_fraction, 1e-3)
    layouts = [(1, 1), (2, 1), (2, 2), (4, 2)]
    nbx, nby = next(((a, b) for a, b in layouts if a * b * full_per_block >= need), layouts[-1])
    dxf = 2.0
    nx, ny = nbx * mx << maxlevel, nby * mx << maxlevel
    dx0 = dxf * (1 << maxlevel)
    x = (np.arange(nx) + 0.5) * dxf
    surf = _lattice_window(nx, ny, 0.8, seed)
    surf = (surf - surf.min()) / max(surf.max() - surf.min(), 1e-300) * 10.0
    b = surf + 0.002 * (nx * dxf - x)[None, :]
    frac = min(1.0, target_patches / (0.7 * nbx * nby * full_per_block))
    x_res = max(frac, 1.0 / nx) * nx * dxf
    inres = np.broadcast_to(x[None, :] < x_res, b.shape)
    level = float(np.percentile(b[inres], 70.0)) + 0.5
    q = np.zeros((ny, nx, 3))
    q[..., 0] = np.where(inres, np.maximum(level - b, 0.0), 0.0)
    peak = float(g.uniform(10.0, 500.0))
    width = 40.0
    n = float(g.uniform(0.02, 0.08))
    hydro = ([0.0, 60.0, 600.0], [0.1 * peak / width, peak / width, 0.1 * peak / width],
             [1, 0, 0, 0], width, 0.0, 0.5 * ny * dxf)
    return dict(mx=mx, nbx=nbx, nby=nby, minlevel=minlevel, maxlevel=maxlevel, dx0=dx0, dy0=dx0,
                aux=b, q=q, mthbc=(0, 1, 3, 3), regrid_interval=4,
                refine=Refine(wave_tolerance=1e9, flowgrades=((0.01, 1, 1, maxlevel),)),
                hydro=hydro, phys=Phys(manning_coefficient=(n,), manning_break=(1e10,)))


def _carve(b: np.ndarray, pts: np.ndarray, dx: float, width: float, depth: float):
    """Lower b by `depth` within width/2 of a polyline given by cell-centre
    points (k, 2) in metres (a channel of the dendritic network)."""
    ny, nx = b.shape
    r = max(1, int(round(0.5 * width / dx)))
    done = np.zeros_like(b, dtype=bool)
    for x, y in pts:
        i, j = int(x / dx), int(y / dx)
        i0, i1, j0, j1 = max(i - r, 0), min(i + r + 1, nx), max(j - r, 0), min(j + r + 1, ny)
        if i0 >= i1 or j0 >= j1:
            continue
        done[j0:j1, i0:i1] = True
    b[done] -= depth


def _walk(g, start, heading, length, step, wiggle, lx, ly):
    """A seeded meandering polyline of `length` metres from `start`."""
    pts = [np.array(start, float)]
    ang = heading
    for _ in range(int(length / step)):
        ang += g.normal(0.0, wiggle)
        ang = heading + np.clip(ang - heading, -0.6, 0.6)
        p = pts[-1] + step * np.array([np.cos(ang), np.sin(ang)])
        if not (0.0 <= p[0] < lx and 0.0 <= p[1] < ly):
            break
        pts.append(p)
    return np.array(pts)


def large_scenario(seed: int = 7, mx: int = 32, minlevel: int = 3, maxlevel: int = 7,
                   wet_fraction: float = 0.25):
    """The large single scenario: a 2 x 2 brick at 2 m finest cells (8192^2
    at maxlevel 7, mx = 32), fractal DEM (Hurst 0.85, 50 m relief) draining
    to the upper right, a dendritic channel network (two trunks from the
    left and bottom inflow points, seeded tributaries), a Manning field of
    two land-cover classes (0.03 / 0.07) used through variable friction
    (aux field 2), and the inundated state of peak flooding: water up to the
    bed's `wet_fraction` quantile plus full channels. One discharge
    hydrograph (peak 800 m^3/s over 60 m windows) enters on the left and
    bottom sides, the reference's single hydrograph applied on two flagged
    sides. Refinement: depth > 0.01 m to maxlevel. Returns the Forest
    keyword arguments plus 'hydro' and 'phys'."""
    from . import Phys, Refine
    g = rng(seed)
    nb = 2
    n = nb * mx << maxlevel
    dxf = 2.0
    L = n * dxf
    lv = int(np.ceil(np.log2(n)))
    lat = diamond_square(lv, 0.85, seed)
    b = 0.25 * (lat[:-1, :-1] + lat[1:, :-1] + lat[:-1, 1:] + lat[1:, 1:])[:n, :n]
    del lat
    b -= b.min()
    b *= 50.0 / max(b.max(), 1e-300)
    x = (np.arange(n) + 0.5) * dxf
    b += 0.001 * (L - x)[None, :] + 0.001 * (L - x)[:, None]
    # dendritic network: two trunks and tributaries joining them
    trunks = [_walk(g, (0.0, 0.5 * L), 0.25, 2 * L, 4.0, 0.05, L, L),
              _walk(g, (0.5 * L, 0.0), 1.3, 2 * L, 4.0, 0.05, L, L)]
    for tr in trunks:
        _carve(b, tr, dxf, 60.0, 5.0)
        for _ in range(6):
            k = int(g.integers(len(tr) // 8, max(len(tr) - 1, len(tr) // 8 + 1)))
            head = float(g.uniform(-2.5, 2.5))
            trib = _walk(g, tr[k], head, float(g.uniform(0.1, 0.3)) * L, 4.0, 0.08, L, L)
            _carve(b, trib, dxf, 20.0, 2.0)
    # land cover: two classes from a coarse seeded fractal, nearest-cell upsampled
    cover = diamond_square(8, 0.8, seed + 11)[:256, :256]
    rep = n // 256
    nman = np.where(np.kron(cover > 0.0, np.ones((rep, rep), bool)), 0.03, 0.07)
    level = float(np.quantile(b[::8, ::8], wet_fraction))
    q = np.zeros((n, n, 3))
    q[..., 0] = np.maximum(level - b, 0.0)
    aux = np.stack([b, nman])
    peak = 800.0
    width = 60.0
    hydro = ([0.0, 1800.0, 7200.0], [0.1 * peak / width, peak / width, 0.1 * peak / width],
             [1, 0, 1, 0], width, 0.5 * L, 0.5 * L)
    phys = Phys(manning_coefficient=(0.035,), manning_break=(1e10,), variable_friction=True,
                friction_index=2)
    return dict(mx=mx, nbx=nb, nby=nb, minlevel=minlevel, maxlevel=maxlevel,
                dx0=dxf * (1 << maxlevel), dy0=dxf * (1 << maxlevel), aux=aux, q=q,
                mthbc=(0, 1, 0, 1), regrid_interval=4,
                refine=Refine(wave_tolerance=1e9, flowgrades=((0.01, 1, 1, maxlevel),)),
                hydro=hydro, phys=phys)
