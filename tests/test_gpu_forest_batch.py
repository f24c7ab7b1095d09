"""Batched forests on the GPU (GPU required): shared launches, device-side
time-step control and captured rounds give each forest exactly the result
of its own run, alone or in a mix of patch sizes."""
import numpy as np
import pytest

import geoflood_gb300 as gf
from geoflood_gb300.forest import batch_run
from oracle import forest as of

from forest_cases import FRONT, LMAX, LMIN, NBX, NBY, rasters

pytestmark = pytest.mark.gpu
S = (slice(None), slice(2, -2), slice(2, -2))
SLOT = 7
PHYS = gf.Phys(manning_coefficient=(0.035,), manning_break=(1e10,))


def make(ctx, m=8, seed=3, regrid=2, mthbc=(3, 3, 3, 3), hydro=None, rf=FRONT):
    b, q = rasters("dambreak", seed, m)
    F = gf.Forest(ctx, m, NBX, NBY, LMIN, LMAX, 1000.0 / m, 1000.0 / m, b, q, mthbc=mthbc,
                  regrid_interval=regrid, refine=rf, phys_slot=SLOT)
    if hydro is not None:
        F.set_hydrograph(*hydro)
    F.init()
    return F


def same(F, G):
    assert np.array_equal(F.patches(), G.patches())
    assert np.array_equal(F.download()[S], G.download()[S])
    a, b = F.stats(), G.stats()
    for k in ("steps", "rejects", "regrids", "cell_updates", "t"):
        assert a[k] == b[k], k


def test_batch_of_one_equals_its_own_run(ctx):
    ctx.set_phys(SLOT, PHYS)
    A, B = make(ctx), make(ctx)
    A.run(40.0, 2, 5.0, 0.9, 1.0)
    st = batch_run([B], 40.0, 2, 5.0, 0.9, 1.0)
    assert st["rounds"] > 0 and st["epochs"] >= 2
    same(A, B)
    A.close()
    B.close()


def test_forest_alone_and_in_a_mixed_batch(ctx):
    ctx.set_phys(SLOT, PHYS)
    hydro = ([0.0, 30.0, 90.0], [2.0, 20.0, 2.0], [1, 0, 0, 0], 120.0, 0.0, 500.0)
    alone = make(ctx, m=16, seed=5, mthbc=(0, 3, 3, 3), hydro=hydro)
    batch_run([alone], 30.0, 1, 5.0, 0.9, 1.0)
    mix = [make(ctx, m=8, seed=4, regrid=3), make(ctx, m=16, seed=5, mthbc=(0, 3, 3, 3),
                                                   hydro=hydro),
           make(ctx, m=32, seed=6, regrid=4)]
    st = batch_run(mix, 30.0, 1, 5.0, 0.9, 1.0)
    same(alone, mix[1])
    assert st["regrids"] == sum(f.stats()["regrids"] for f in mix)
    for f in mix + [alone]:
        f.close()


def test_batch_matches_oracle_forests_bitwise(ctx):
    """Contraction-free build, friction off: two forests in one batch against
    two oracle forest runs."""
    phys = gf.Phys(friction_forcing=False)
    ctx.set_phys(SLOT, phys)
    ctx.set_fp_contract(False)
    try:
        fs = [make(ctx, m=8, seed=3, regrid=2), make(ctx, m=8, seed=9, regrid=3)]
        batch_run(fs, 30.0, 1, 5.0, 0.9, 1.0)
        for F, (seed, regrid) in zip(fs, ((3, 2), (9, 3))):
            b, q = rasters("dambreak", seed, 8)
            O = of.Forest(8, NBX, NBY, LMIN, LMAX, 125.0, 125.0, b, q, phys=phys,
                          mthbc=(3, 3, 3, 3), regrid_interval=regrid, rf=FRONT)
            O.init()
            O.run(30.0, 1, 5.0, 0.9, 1.0)
            assert np.array_equal(F.patches(), O.patches())
            assert F.stats()["steps"] == O.steps and F.stats()["regrids"] == O.regrids
            assert np.array_equal(F.download()[S], O.download()[S])
            F.close()
    finally:
        ctx.set_fp_contract(True)


@pytest.mark.parametrize("exact", [False, True])
def test_mixed_and_per_size_updates_agree(ctx, exact):
    """The one-launch update over all patch sizes (a device cursor over the
    concatenated work list) and the per-size launches give the same bits."""
    ctx.set_phys(SLOT, PHYS)
    ctx.set_fp_contract(not exact)
    outs = []
    try:
        for mixed in (True, False):
            ctx.set_mixed_update(mixed)
            fs = [make(ctx, m=8, seed=4, regrid=3), make(ctx, m=16, seed=5, regrid=2),
                  make(ctx, m=32, seed=6, regrid=4), make(ctx, m=8, seed=7, regrid=2)]
            batch_run(fs, 25.0, 1, 5.0, 0.9, 1.0)
            outs.append([(F.patches(), F.download(), F.stats()) for F in fs])
            for F in fs:
                F.close()
    finally:
        ctx.set_mixed_update(True)
        ctx.set_fp_contract(True)
    for (pa, qa, sa), (pb, qb, sb) in zip(*outs):
        assert np.array_equal(pa, pb) and np.array_equal(qa[S], qb[S])
        assert sa["steps"] == sb["steps"] and sa["regrids"] == sb["regrids"]
