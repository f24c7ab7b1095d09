"""The oracle's multi-level forest driver on its own (no GPU): tiling and
2:1 balance through regrids, the raster pyramid, and well-balancing across
coarse/fine interfaces."""
import numpy as np

import geoflood_gb300 as gf
from oracle import forest as of

from forest_cases import (DX0, FRONT, LAKE_REGION, LMAX, LMIN, M, NBX, NBY, balanced,
                          rasters)


def test_pyramid_is_blockwise_mean():
    rng = np.random.default_rng(1)
    f = rng.standard_normal((2, 16, 32))
    p = of.pyramid(f, 3)
    assert p[0].shape == (2, 20, 36) and p[2].shape == (2, 8, 12)
    assert np.array_equal(p[0][:, 2:-2, 2:-2], f)
    assert np.allclose(p[2][:, 2:-2, 2:-2], f.reshape(2, 4, 4, 8, 4).mean(axis=(2, 4)),
                       rtol=0, atol=1e-15)
    assert np.array_equal(p[1][:, 0, 2:-2], p[1][:, 2, 2:-2])      # edge-extended halo


def test_lake_at_rest_across_levels():
    b, q = rasters("lake")
    F = of.Forest(M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, phys=gf.Phys(), mthbc=(3, 3, 3, 3),
                  regrid_interval=2, rf=LAKE_REGION)
    F.init()
    assert {k[0] for k in F.leaves} == {1, 2, 3}
    assert balanced(F.leaves, NBX, NBY, LMAX)
    F.run(50.0, 2, 5.0, 0.9, 1.0, max_steps=12)
    qq, aa = F.download(), F.download_aux()
    s = (slice(None), slice(2, -2), slice(2, -2))
    assert np.abs(qq[s][..., 1:]).max() < 1e-12
    wet = qq[s][..., 0] > 1e-3
    eta = qq[s][..., 0] + aa[s][..., 0]
    assert np.abs(eta[wet] - 8.0).max() < 1e-12


def test_front_refines_and_stays_balanced():
    b, q = rasters("dambreak")
    F = of.Forest(M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, phys=gf.Phys(), mthbc=(3, 3, 3, 3),
                  regrid_interval=2, rf=FRONT)
    F.init()
    seen = set()
    for k in range(3):
        F.run(20.0, 1, 5.0, 0.9, 1.0)
        seen |= {lk[0] for lk in F.leaves}
        assert balanced(F.leaves, NBX, NBY, LMAX)
    assert LMAX in seen and F.regrids > 5
    assert balanced(F.leaves, NBX, NBY, LMAX)
    assert list(map(tuple, F.patches())) == sorted(F.leaves, key=lambda k: (k[0], k[2], k[1]))
