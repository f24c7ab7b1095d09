"""Topography on the CPU: the library's topo readers against what the
reference's own topotools reads from files it wrote (fixtures made by
tests/golden/make_topo_golden.py), the oracle's readers against the
library's, and the oracle's cell integrals (restating setaux /
cellgridintegrate / rectintegral / topointegral) against exact integrals
of bilinear surfaces. No GPU is used."""
from pathlib import Path

import numpy as np
import pytest

from oracle import topo as ot

GOLD = Path(__file__).resolve().parent / "golden" / "topo"
FILES = {"A": ("A.tt3", 3), "B": ("B.tt2", 2), "C": ("C.tt1", 1), "D": ("D.asc", -3)}
MISSING = 25.0


@pytest.fixture(scope="module")
def parsed():
    d = np.load(GOLD / "parsed.npz")
    return {k: d[k] for k in d.files}


def native_set(gpu_lib):
    from geoflood_gb300.topo import Topo

    t = Topo()
    t.read_data(str(GOLD / "topo.data"))
    return t


def test_native_readers_match_reference_topotools(gpu_lib, parsed):
    t = native_set(gpu_lib)
    assert len(t) == 4
    for k, key in enumerate("ABCD"):
        g = t.grid(k)
        x, y, Z = parsed[key + "_x"], parsed[key + "_y"], parsed[key + "_Z"]
        assert (g["mx"], g["my"]) == (len(x), len(y)), key
        # (topotools lists a type-1 file's y from north to south)
        assert g["xlow"] == pytest.approx(x.min(), rel=0, abs=1e-9)
        assert g["ylow"] == pytest.approx(y.min(), rel=0, abs=1e-9)
        assert g["xhi"] == pytest.approx(x.max(), rel=0, abs=1e-9)
        assert g["yhi"] == pytest.approx(y.max(), rel=0, abs=1e-9)
        assert g["dx"] == pytest.approx(abs(x[1] - x[0]), rel=1e-12)
        assert g["dy"] == pytest.approx(abs(y[1] - y[0]), rel=1e-12)
        want = np.flipud(Z).ravel().copy()          # file order: north to south
        neg = FILES[key][1] < 0
        if neg:
            want = -want                            # topotools negated already
        if key + "_nodata" in parsed:
            want[want == float(parsed[key + "_nodata"])] = MISSING
        if neg:
            want = -want
        assert np.array_equal(g["z"], want), key
    # the four no-data nodes of D became -topo_missing
    assert np.sum(t.grid(3)["z"] == -MISSING) == 4


def test_oracle_readers_equal_native(gpu_lib):
    t = native_set(gpu_lib)
    missing, files = ot.read_topo_data(str(GOLD / "topo.data"))
    assert missing == MISSING and [f[1] for f in files] == [3, 2, 1, -3]
    for k, (name, ttype) in enumerate(files):
        o = ot.read_topo_file(str(GOLD / name), ttype, missing)
        g = t.grid(k)
        for f in ("mx", "my", "xlow", "ylow", "xhi", "yhi", "dx", "dy"):
            assert g[f] == o[f], (name, f)
        assert np.array_equal(g["z"], o["z"]), name


def test_reader_errors(gpu_lib, tmp_path):
    from geoflood_gb300 import GeoFloodError
    from geoflood_gb300.topo import Topo

    t = Topo()
    with pytest.raises(GeoFloodError):
        t.read_file(str(GOLD / "D.asc"), 3)        # no-data with the default 99999
    with pytest.raises(GeoFloodError):
        t.read_file(str(tmp_path / "absent.tt3"), 3)
    with pytest.raises(GeoFloodError):
        t.read_file(str(GOLD / "A.tt3"), 4)        # not a NetCDF file
    hdf = tmp_path / "nc4.nc"
    hdf.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes(64))
    with pytest.raises(GeoFloodError):
        t.read_file(str(hdf), 4)                   # NetCDF-4 (HDF5) is not read
    bad = tmp_path / "short.tt3"
    bad.write_text("4 ncols\n3 nrows\n0 xll\n0 yll\n1 cellsize\n-9999 nodata\n1 2 3 4\n")
    with pytest.raises(GeoFloodError):
        t.read_file(str(bad), 3)
    assert len(t) == 0
    with pytest.raises(ValueError):
        ot.read_topo_file(str(GOLD / "D.asc"), 3)


def test_header_value_forms(gpu_lib, tmp_path):
    """parse_values takes the numbers of a line whatever the label order,
    Fortran D exponents included; two values on the cellsize line give dx, dy."""
    from geoflood_gb300.topo import Topo

    p = tmp_path / "h.tt2"
    p.write_text("ncols 3\n2 nrows\nxllcenter 1.5D+01\nyll -2.0e1 yllcenter\n"
                 "2.0 4.0 cellsize\nnodata -1\n1\n2\n\n3\n4 9 9\n5\n6\n")
    t = Topo(topo_missing=-7.0)
    t.read_file(str(p), 2)
    g = t.grid(0)
    assert (g["mx"], g["my"], g["xlow"], g["ylow"], g["dx"], g["dy"]) == (3, 2, 15.0, -20.0, 2.0, 4.0)
    assert list(g["z"]) == [1, 2, 3, 4, 5, 6]
    o = ot.read_topo_file(str(p), 2, -7.0)
    assert list(o["z"]) == [1, 2, 3, 4, 5, 6] and o["xlow"] == 15.0


def bil(a, b, c, d):
    return lambda X, Y: a + b * X + c * Y + d * X * Y


def bil_integral(f_coef, x1, x2, y1, y2):
    a, b, c, d = f_coef
    xm, ym = 0.5 * (x1 + x2), 0.5 * (y1 + y2)
    return (x2 - x1) * (y2 - y1) * (a + b * xm + c * ym + d * xm * ym)


def grid_of(coef, x0, y0, dx, dy, mx, my):
    x = x0 + dx * np.arange(mx)
    y = y0 + dy * np.arange(my)
    X, Y = np.meshgrid(x, y)
    Z = bil(*coef)(X, Y)
    return dict(mx=mx, my=my, xlow=x0, ylow=y0, xhi=x0 + (mx - 1) * dx, yhi=y0 + (my - 1) * dy,
                dx=dx, dy=dy, z=np.flipud(Z).ravel().copy())


def test_cell_average_of_bilinear_surface_is_exact():
    """The bilinear interpolant of a bilinear surface is the surface: every
    cell average equals the surface at the cell centre, for cells finer and
    coarser than the grid and cells straddling grid lines."""
    coef = (3.0, 0.01, -0.02, 1e-4)
    ts = ot.TopoSet([grid_of(coef, -10.0, -10.0, 7.0, 5.0, 40, 50)])
    for (nx, dx) in ((13, 17.0), (50, 3.3), (7, 31.0)):
        ny, dy = nx, dx * 0.75
        r = ts.raster(nx, ny, 2, 0.0, 0.0, dx, dy, nx * dx, ny * dy)
        xc = (np.arange(nx) + 0.5) * dx
        yc = (np.arange(ny) + 0.5) * dy
        X, Y = np.meshgrid(xc, yc)
        assert np.allclose(r[2:-2, 2:-2], bil(*coef)(X, Y), rtol=1e-13, atol=1e-12)
        # cells outside the domain copy the nearest cell inside
        assert np.array_equal(r[:2, 2:-2], np.repeat(r[2:3, 2:-2], 2, 0))
        assert np.array_equal(r[:, :2], np.repeat(r[:, 2:3], 2, 1))
        assert np.array_equal(r[-2:, :], np.repeat(r[-3:-2, :], 2, 0))


def test_finer_grid_takes_priority():
    """Two grids, a coarse one over everything and a fine one over a window:
    a cell's integral is the coarse surface outside the fine grid's extent
    plus the fine surface inside (inclusion-exclusion of rectintegral)."""
    c1, c2 = (1.0, 0.02, 0.01, 0.0), (-5.0, 0.0, 0.03, 2e-4)
    coarse = grid_of(c1, -20.0, -20.0, 20.0, 20.0, 20, 20)
    fine = grid_of(c2, 95.0, 102.0, 2.5, 2.0, 41, 31)    # [95, 195] x [102, 162]
    ts = ot.TopoSet([coarse, fine])
    assert ts.order == [1, 0]
    fx1, fx2, fy1, fy2 = fine["xlow"], fine["xhi"], fine["ylow"], fine["yhi"]
    for (x1, x2, y1, y2) in ((100, 110, 110, 120), (80, 120, 90, 130), (180, 230, 150, 170),
                             (0, 40, 0, 40), (90, 200, 100, 165)):
        want = bil_integral(c1, x1, x2, y1, y2)
        ix1, ix2, iy1, iy2 = max(x1, fx1), min(x2, fx2), max(y1, fy1), min(y2, fy2)
        if ix2 > ix1 and iy2 > iy1:
            want += bil_integral(c2, ix1, ix2, iy1, iy2) - bil_integral(c1, ix1, ix2, iy1, iy2)
        got = ts.cell_integral(x1, x2, y1, y2)
        assert got == pytest.approx(want, rel=1e-12, abs=1e-9), (x1, x2, y1, y2)


def test_equal_resolution_later_file_first():
    g1 = grid_of((1, 0, 0, 0), 0, 0, 1.0, 1.0, 5, 5)
    g2 = grid_of((2, 0, 0, 0), 0, 0, 1.0, 1.0, 5, 5)
    ts = ot.TopoSet([g1, g2])
    assert ts.order == [1, 0]
    assert ts.cell_integral(0.5, 1.5, 0.5, 1.5) == pytest.approx(2.0)


def test_coverage_and_uncovered_cell():
    ts = ot.TopoSet([grid_of((1, 0, 0, 0), 0, 0, 1.0, 1.0, 11, 11)])
    assert ts.area(0, 20, 0, 10) == pytest.approx(100.0)
    with pytest.raises(ValueError):
        ts.cell_integral(12, 13, 2, 3)


def test_native_covered_area_matches_oracle(gpu_lib, parsed):
    t = native_set(gpu_lib)
    missing, files = ot.read_topo_data(str(GOLD / "topo.data"))
    ts = ot.TopoSet([ot.read_topo_file(str(GOLD / n), ty, missing) for n, ty in files])
    for rect in ((0, 800, 0, 600), (-200, 1000, -100, 800), (320, 420, 250, 480)):
        assert t.covered_area(*rect) == ts.area(*rect)


def write_nc(path, version, dims, z, zdims, ztype, positive=None, extra_2d=False):
    """A classic NetCDF topo file written by scipy (an independent writer)."""
    from scipy.io import netcdf_file

    with netcdf_file(str(path), "w", version=version) as f:
        for name, vals in dims:
            f.createDimension(name, len(vals))
        for name, vals in dims:
            v = f.createVariable(name, "d", (name,))
            v[:] = vals
        if extra_2d:                               # an earlier 2-D variable: the last one is z
            e = f.createVariable("mask", "i", zdims)
            e[:] = np.zeros(z.shape, dtype=np.int32)
        v = f.createVariable("elevation", ztype, zdims)
        v[:] = z.astype(ztype)
        if positive is not None:
            v.positive = positive


@pytest.mark.parametrize("case", range(5))
def test_netcdf_topo_native_equals_oracle(gpu_lib, tmp_path, case):
    """Topo type +-4: the native classic-NetCDF reader and the oracle (scipy's
    parser, the reference's rules) give the same grid; the grid holds the
    written nodes, rows north first."""
    from geoflood_gb300.topo import Topo

    rng = np.random.default_rng(case)
    mx, my = 7 + case, 5 + 2 * case
    xs = -120.0 + 0.25 * np.arange(mx)
    ys = 40.0 + 0.5 * np.arange(my)
    zyx = rng.uniform(-50.0, 30.0, (my, mx)).round(2)       # z[y][x]
    spec = [
        dict(version=1, names=("lon", "lat"), order="yx", ztype="d", positive=None, ttype=4),
        dict(version=2, names=("x", "y"), order="xy", ztype="f", positive="down", ttype=-4),
        dict(version=1, names=("LONGITUDE", "Latitude"), order="yx", ztype="h", positive="down", ttype=4),
        dict(version=2, names=("lon", "lat"), order="yx", ztype="d", positive=None, ttype=-4),
        dict(version=1, names=("x", "y"), order="xy", ztype="i", positive="Down", ttype=-4),
    ][case]
    xn, yn = spec["names"]
    z_store = zyx if spec["order"] == "yx" else zyx.T
    zdims = (yn, xn) if spec["order"] == "yx" else (xn, yn)
    dims = [(yn, ys), (xn, xs)] if case % 2 else [(xn, xs), (yn, ys)]
    path = tmp_path / f"t{case}.nc"
    write_nc(path, spec["version"], dims, z_store, zdims, spec["ztype"], spec["positive"], extra_2d=case == 3)
    t = Topo()
    t.read_file(str(path), spec["ttype"])
    g = t.grid(0)
    o = ot.read_topo_file(str(path), spec["ttype"])
    for f in ("mx", "my", "xlow", "ylow", "xhi", "yhi", "dx", "dy"):
        assert g[f] == o[f], f
    assert np.array_equal(g["z"], o["z"])
    want = zyx.astype(spec["ztype"]).astype(np.float64)[::-1, :].reshape(-1)
    neg = spec["ttype"] < 0
    if neg and spec["positive"] is not None and spec["positive"].lower() == "down":
        neg = False                                  # negated twice, as the reference does
    assert np.array_equal(g["z"], -want if neg else want)
    assert (g["mx"], g["my"], g["xlow"], g["ylow"]) == (mx, my, xs[0], ys[0])
