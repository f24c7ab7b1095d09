"""Cell-averaged topography on the GPU against the oracle (GPU required):
rasters of the fixture DEM set (four files of three types and three
resolutions, no-data nodes, a negative type) at cell sizes coarser and finer
than every file, bit for bit; forests whose levels take their bathymetry and
sea-level initial state from the DEMs; a lake at rest over the real-format
DEM staying at rest; and a contraction-free forest run from the DEMs equal
to the oracle forest's."""
from pathlib import Path

import numpy as np
import pytest

import geoflood_gb300 as gf
from geoflood_gb300.topo import Topo
from oracle import forest as of
from oracle import topo as ot

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden" / "topo"
SLOT = 9
M, NBX, NBY, LMIN, LMAX, DX0 = 8, 4, 3, 0, 3, 25.0     # 800 m x 600 m


def sets():
    t = Topo()
    t.read_data(str(GOLD / "topo.data"))
    missing, files = ot.read_topo_data(str(GOLD / "topo.data"))
    ts = ot.TopoSet([ot.read_topo_file(str(GOLD / n), ty, missing) for n, ty in files])
    return t, ts


@pytest.mark.parametrize("nx,ny,dx", [(8, 6, 100.0), (32, 24, 25.0), (160, 120, 5.0),
                                      (256, 192, 3.125), (7, 5, 114.0)])
def test_raster_matches_oracle(ctx, nx, ny, dx):
    t, ts = sets()
    xu, yu = nx * dx, ny * dx
    got = t.raster(ctx, nx, ny, 2, 0.0, 0.0, dx, dx, xu, yu)
    want = ts.raster(nx, ny, 2, 0.0, 0.0, dx, dx, xu, yu)
    assert np.array_equal(got, want)


def test_uncovered_cell_is_an_error(ctx):
    t, _ = sets()
    with pytest.raises(gf.GeoFloodError):
        t.raster(ctx, 4, 4, 0, 5000.0, 5000.0, 10.0, 10.0, 5040.0, 5040.0)


LAKE = gf.Refine(wave_tolerance=1e9, regions=((250.0, 450.0, 150.0, 350.0, 0.0, 1e9, 3, 3),))


def forests(ctx, phys, regrid=0, refine=LAKE, lmin=LMIN, lmax=LMAX):
    t, ts = sets()
    ctx.set_phys(SLOT, phys)
    G = gf.Forest(ctx, M, NBX, NBY, lmin, lmax, DX0, DX0, None, None, mthbc=(3, 3, 3, 3),
                  regrid_interval=regrid, refine=refine, phys_slot=SLOT)
    G.set_topo(t)
    nx, ny = NBX * M << lmax, NBY * M << lmax
    O = of.Forest(M, NBX, NBY, lmin, lmax, DX0, DX0, np.zeros((ny, nx)), np.zeros((ny, nx, 3)),
                  phys=phys, mthbc=(3, 3, 3, 3), regrid_interval=regrid, rf=refine)
    O.set_topo(ts)
    G.init()
    O.init()
    return G, O, ts


def test_forest_levels_take_setaux_and_sea_level_qinit(ctx):
    phys = gf.Phys(sea_level=30.0)
    G, O, ts = forests(ctx, phys)
    P = G.patches()
    assert np.array_equal(P, O.patches()) and set(P[:, 0]) == {1, 2, 3}
    aux, q = G.download_aux(), G.download()
    xu, yu = NBX * M * DX0, NBY * M * DX0
    for k, (l, I, J) in enumerate(P):
        r = ts.raster(NBX * M << l, NBY * M << l, 2, 0.0, 0.0, DX0 / (1 << l), DX0 / (1 << l), xu, yu)
        win = r[J * M:J * M + M + 4, I * M:I * M + M + 4]
        assert np.array_equal(aux[k, ..., 0], win), (l, I, J)
        assert np.array_equal(q[k, ..., 0], np.maximum(0.0, 30.0 - win))
        assert not q[k, ..., 1:].any()
    assert np.array_equal(aux, O.download_aux())
    G.close()


def test_lake_at_rest_over_dem(ctx):
    """Still water at sea level 60 over the whole DEM set (pits, file
    seams, four levels, regrids): momentum stays at round-off and the
    surface stays at 60. (With shorelines the reference's solver moves water
    wherever a cell holds less than the dry tolerance below sea level, so a
    partly dry lake is held to the oracle instead, below.)"""
    phys = gf.Phys(sea_level=60.0)
    G, O, _ = forests(ctx, phys, regrid=2)
    st = G.run(60.0, 2, 1.0, 0.9, 1.0, max_steps=40)
    assert st["steps"] == 40 and st["regrids"] == 20
    q, aux = G.download(), G.download_aux()
    S = (slice(None), slice(2, -2), slice(2, -2))
    assert np.abs(q[S][..., 1:]).max() < 1e-10
    assert np.abs((q[S][..., 0] + aux[S][..., 0]) - 60.0).max() < 1e-11
    G.close()


def test_exact_build_dem_dam_break_matches_oracle(ctx):
    """A wave released over the DEM terrain (water raised in one corner),
    refinement following it, contraction-free build: the device forest and
    the oracle forest agree bit for bit."""
    phys = gf.Phys(sea_level=30.0, friction_forcing=False)
    rf = gf.Refine(wave_tolerance=0.5)
    ctx.set_fp_contract(False)
    try:
        G, O, _ = forests(ctx, phys, regrid=2, refine=rf)
        q = G.download()
        ql = O.download()
        assert np.array_equal(q, ql)
        # raise the water in the lower-left block of every leaf there
        P = G.patches()
        for k, (l, I, J) in enumerate(P):
            if (I >> l) == 0 and (J >> l) == 0:
                q[k, ..., 0] = np.where(q[k, ..., 0] > 0, q[k, ..., 0] + 2.0, 0.0)
        G.upload(q)
        O.upload(q)
        for _ in range(2):
            st = G.run(10.0, 1, 1.0, 0.9, 1.0)
            O.run(10.0, 1, 1.0, 0.9, 1.0)
            assert np.array_equal(G.patches(), O.patches())
            assert (st["steps"], st["rejects"], st["regrids"]) == (O.steps, O.rejects, O.regrids)
            assert np.array_equal(G.download()[:, 2:-2, 2:-2], O.download()[:, 2:-2, 2:-2])
        G.close()
    finally:
        ctx.set_fp_contract(True)
