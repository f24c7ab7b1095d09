"""Multi-level forests on the GPU against the oracle's forest driver (GPU
required). In the contraction-free build with the friction term off (the
only FP difference left is pow in src2), whole runs with regrids agree bit
for bit: patch lists, step counts and states. The production build is held
to the per-step bar from identical states."""
import numpy as np
import pytest

import geoflood_gb300 as gf
import oracle
from oracle import forest as of

from forest_cases import (DX0, FRONT, LAKE_REGION, LMAX, LMIN, M, NBX, NBY, balanced,
                          rasters)

pytestmark = pytest.mark.gpu
S = (slice(None), slice(2, -2), slice(2, -2))
SLOT = 7   # a physics slot of its own in the shared context


def pair(ctx, kind, rf, phys, mthbc=(3, 3, 3, 3), regrid=2, hydro=None):
    b, q = rasters(kind)
    ctx.set_phys(SLOT, phys)
    G = gf.Forest(ctx, M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, mthbc=mthbc,
                  regrid_interval=regrid, refine=rf, phys_slot=SLOT)
    hy = None
    if hydro is not None:
        G.set_hydrograph(*hydro)
        hy = oracle.hydro(*hydro)
    O = of.Forest(M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, phys=phys, mthbc=mthbc,
                  regrid_interval=regrid, rf=rf, hy=hy)
    G.init()
    O.init()
    return G, O


def test_initial_refinement_and_pyramid(ctx):
    G, O = pair(ctx, "lake", LAKE_REGION, gf.Phys())
    assert np.array_equal(G.patches(), O.patches())
    assert np.array_equal(G.download_aux()[S], O.download_aux()[S])
    assert np.array_equal(G.download()[S], O.download()[S])
    G.close()


def test_lake_at_rest_across_levels(ctx):
    G, O = pair(ctx, "lake", LAKE_REGION, gf.Phys())
    st = G.run(50.0, 2, 5.0, 0.9, 1.0, max_steps=12)
    assert st["steps"] == 12 and st["regrids"] == 6
    qq, aa = G.download(), G.download_aux()
    assert np.abs(qq[S][..., 1:]).max() < 1e-12
    wet = qq[S][..., 0] > 1e-3
    assert np.abs((qq[S][..., 0] + aa[S][..., 0])[wet] - 8.0).max() < 1e-12
    G.close()


def test_exact_build_run_with_regrids_is_bitwise(ctx):
    """Dam break whose refinement follows the front: the device forest and
    the oracle agree on every patch list, step count and value."""
    phys = gf.Phys(friction_forcing=False)
    ctx.set_fp_contract(False)
    try:
        G, O = pair(ctx, "dambreak", FRONT, phys)
        for k in range(3):
            st = G.run(20.0, 1, 5.0, 0.9, 1.0)
            O.run(20.0, 1, 5.0, 0.9, 1.0)
            assert np.array_equal(G.patches(), O.patches()), k
            assert (st["steps"], st["rejects"], st["regrids"]) == (O.steps, O.rejects, O.regrids)
            assert st["t"] == O.t
            assert np.array_equal(G.download()[S], O.download()[S]), k
        assert st["levels_used"] == LMAX and balanced(map(tuple, G.patches()), NBX, NBY, LMAX)
        G.close()
    finally:
        ctx.set_fp_contract(True)


def test_production_build_per_step_with_inflow(ctx):
    """FMA build, Manning friction, hydrograph inflow on the left: every
    step from the oracle's state agrees within the FP64 bar, and regrids
    from identical states give identical patch lists."""
    phys = gf.Phys(manning_coefficient=(0.035,), manning_break=(1e10,))
    hydro = ([0.0, 30.0, 90.0], [2.0, 20.0, 2.0], [1, 0, 0, 0], 120.0, 0.0, 500.0)
    G, O = pair(ctx, "dambreak", FRONT, phys, mthbc=(0, 3, 3, 3), hydro=hydro)
    t, dt = 0.0, 0.4
    for k in range(12):
        G.upload(O.download())
        cg = G.step(t, dt)
        co = O.step(t, dt)
        assert abs(cg - co) <= 1e-12 * max(co, 1e-300)
        G.accept(True)            # the step's result becomes the current state
        qg, qo = G.download()[S], O.download()[S]
        scale = max(float(np.abs(qo[..., 0]).max()), 1.0)
        assert np.abs(qg - qo).max() <= 1e-10 * scale, k
        assert np.array_equal(qg[..., 0] > phys.dry_tolerance, qo[..., 0] > phys.dry_tolerance)
        t += dt
        if k % 3 == 2:
            G.upload(O.download())
            G.regrid(t)
            O.regrid(t)
            assert np.array_equal(G.patches(), O.patches()), k
    G.close()


def test_regrid_to_full_refinement_fits_default_pool(ctx):
    """A forest that refines everywhere: the regrid holds the new children
    and their parents at once, which the default slot pool must allow."""
    b, q = rasters("lake")
    ctx.set_phys(SLOT, gf.Phys())
    everywhere = gf.Refine(wave_tolerance=1e9, regions=((0.0, 2000.0, 0.0, 1000.0, 0.0, 1e9, 3, 3),))
    G = gf.Forest(ctx, M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, mthbc=(3, 3, 3, 3),
                  regrid_interval=1, refine=everywhere, phys_slot=SLOT)
    G.init()
    G.run(20.0, 1, 5.0, 0.9, 1.0, max_steps=3)
    P = G.patches()
    assert len(P) == NBX * NBY * 4 ** LMAX and set(P[:, 0]) == {LMAX}
    G.close()


def test_config1_regrids_match_oracle_from_identical_states(ctx):
    """The 200-attempt config-1 dam break (2 x 1 blocks, mx 16, levels 1-3,
    regrid every 2 accepted steps) in the production build: before every
    regrid the oracle restarts from the device forest's leaves and state,
    and every regrid must give the same patch list on both sides."""
    import bench

    c = bench.forest_dambreak_config()
    ctx.set_phys(0, c["phys"])
    try:
        regrids, mismatches = bench.regrid_parity(ctx, c, 200, resync=True)
    finally:
        ctx.set_phys(0, gf.Phys())
    assert regrids >= 50
    assert mismatches == 0, f"{mismatches} of {regrids} regrids differ"
