"""Forest-server host logic without a GPU: the device-footprint bound that
admission uses, and request validation through the Python wrapper."""
import numpy as np

from geoflood_gb300.forest import footprint, forest_opts


def pools_and_pyramid(mx, nbx, nby, lmin, lmax, maux, cap=None):
    full = nbx * nby << (2 * lmax)
    cap = cap or full + (full + 3) // 4
    S = (mx + 4) ** 2
    pyr = sum((maux + 3) * ((nbx * mx << l) + 4) * ((nby * mx << l) + 4) for l in range(lmin, lmax + 1))
    return 8 * (cap * (6 + maux) * S + pyr)


def test_footprint_covers_pools_and_pyramid(gpu_lib):
    for mx, nbx, nby, lmin, lmax, maux in ((8, 2, 1, 1, 3, 1), (16, 4, 3, 0, 4, 2), (32, 1, 1, 0, 0, 3)):
        o = forest_opts(mx, nbx, nby, lmin, lmax, 10.0, 10.0, maux)
        fp = footprint(o)
        base = pools_and_pyramid(mx, nbx, nby, lmin, lmax, maux)
        assert base < fp < 1.25 * base + (2 << 20), (mx, fp, base)


def test_footprint_grows_with_depth_and_shrinks_with_max_patches(gpu_lib):
    a = footprint(forest_opts(16, 2, 2, 0, 3, 1.0, 1.0))
    b = footprint(forest_opts(16, 2, 2, 0, 4, 1.0, 1.0))
    assert b > 3 * a
    c = footprint(forest_opts(16, 2, 2, 0, 4, 1.0, 1.0, max_patches=64))
    assert c < b and c > pools_and_pyramid(16, 2, 2, 0, 4, 1, cap=64)


def test_footprint_zero_for_invalid_options(gpu_lib):
    assert footprint(forest_opts(12, 1, 1, 0, 1, 1.0, 1.0)) == 0
    assert footprint(forest_opts(8, 1, 1, 2, 1, 1.0, 1.0)) == 0
    assert footprint(forest_opts(8, 0, 1, 0, 1, 1.0, 1.0)) == 0
    assert footprint(forest_opts(8, 1, 1, 0, 1, 1.0, 1.0, maux=4)) == 0
    assert footprint(forest_opts(8, 64, 64, 0, 10, 1.0, 1.0)) == 0   # > 2^22 slots


def test_request_struct_carries_options(gpu_lib):
    from geoflood_gb300.serve import ForestRequest, Hydrograph

    b = np.zeros((16, 32))
    q = np.zeros((16, 32, 3))
    r = ForestRequest(mx=8, nbx=2, nby=1, minlevel=0, maxlevel=1, dx0=5.0, dy0=5.0, t_final=3.0,
                      aux=b, q=q, mthbc=(0, 1, 3, 3), regrid_interval=4,
                      hydro=Hydrograph(np.array([0.0, 1.0]), np.array([1.0, 2.0])))
    c, keep = r.to_c()
    assert (c.opts.mx, c.opts.nbx, c.opts.maxlevel, c.opts.regrid_interval) == (8, 2, 1, 4)
    assert list(c.opts.mthbc) == [0, 1, 3, 3] and c.nhydro == 2 and c.hydro_side[0] == 1
    assert keep[0].shape == (4, 16, 32) and c.fields == keep[0].ctypes.data
    assert c.t_final == 3.0 and c.topo is None
