"""Subcycled forests on the GPU against the oracle's subcycled schedule (GPU
required). In the contraction-free build with friction off and walls, whole
runs agree bit for bit: every level's sub-steps, the time-interpolated
coarse ghost cells at the midpoints, retakes and regrids. Runs with the
hydrograph inflow (evaluated at each sub-step's time, through pow) and the
production build are held to the FP64 bar."""
import numpy as np
import pytest

import geoflood_gb300 as gf
import oracle
from oracle import forest as of

from forest_cases import DX0, FRONT, LMAX, LMIN, M, NBX, NBY, balanced, rasters

pytestmark = pytest.mark.gpu
S = (slice(None), slice(2, -2), slice(2, -2))
SLOT = 10
HYDRO = ([0.0, 30.0, 90.0], [2.0, 20.0, 2.0], [1, 0, 0, 0], 120.0, 0.0, 500.0)


def pair(ctx, phys, mthbc=(3, 3, 3, 3), hydro=None, regrid=2):
    b, q = rasters("dambreak")
    ctx.set_phys(SLOT, phys)
    G = gf.Forest(ctx, M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, mthbc=mthbc, regrid_interval=regrid,
                  refine=FRONT, phys_slot=SLOT, subcycle=True)
    hy = None
    if hydro is not None:
        G.set_hydrograph(*hydro)
        hy = oracle.hydro(*hydro)
    O = of.Forest(M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, phys=phys, mthbc=mthbc, regrid_interval=regrid,
                  rf=FRONT, hy=hy, subcycle=True)
    G.init()
    O.init()
    return G, O


def test_exact_build_subcycled_run_is_bitwise(ctx):
    phys = gf.Phys(friction_forcing=False)
    ctx.set_fp_contract(False)
    try:
        G, O = pair(ctx, phys)
        for k in range(3):
            st = G.run(15.0, 1, 5.0, 0.9, 1.0)
            O.run(15.0, 1, 5.0, 0.9, 1.0)
            assert np.array_equal(G.patches(), O.patches()), k
            assert (st["steps"], st["rejects"], st["regrids"]) == (O.steps, O.rejects, O.regrids), k
            assert st["t"] == O.t and st["cell_updates"] == O.cell_updates
            assert np.array_equal(G.download()[S], O.download()[S]), k
        assert st["levels_used"] == LMAX and balanced(map(tuple, G.patches()), NBX, NBY, LMAX)
        assert st["rejects"] > 0          # retakes restore every level
        G.close()
    finally:
        ctx.set_fp_contract(True)


def test_subcycled_inflow_within_fp64_bar(ctx):
    """Hydrograph inflow evaluated at every sub-step's time. Its boundary
    state comes from pow and a Newton solve on the device (pow is not
    correctly rounded there), so the bar is the FP64 one: equal step counts,
    retakes, regrids and patch lists, states within 1e-8 of the depth scale."""
    phys = gf.Phys(friction_forcing=False)
    ctx.set_fp_contract(False)
    try:
        G, O = pair(ctx, phys, mthbc=(0, 3, 3, 3), hydro=HYDRO)
        for k in range(3):
            st = G.run(15.0, 1, 5.0, 0.9, 1.0)
            O.run(15.0, 1, 5.0, 0.9, 1.0)
            assert np.array_equal(G.patches(), O.patches()), k
            assert (st["steps"], st["rejects"], st["regrids"]) == (O.steps, O.rejects, O.regrids), k
            qg, qo = G.download()[S], O.download()[S]
            scale = max(float(np.abs(qo[..., 0]).max()), 1.0)
            assert np.abs(qg - qo).max() <= 1e-8 * scale, k
        G.close()
    finally:
        ctx.set_fp_contract(True)


def test_production_build_subcycled_within_fp64_bar(ctx):
    """FMA build with Manning friction and inflow: after 20 coarse steps the
    states differ from the oracle's only at round-off amplified by the
    flow (the step count and patch lists must agree)."""
    phys = gf.Phys(manning_coefficient=(0.035,), manning_break=(1e10,))
    G, O = pair(ctx, phys, mthbc=(0, 3, 3, 3), hydro=HYDRO)
    st = G.run(1e9, 1, 2.0, 0.9, 1.0, max_steps=20)
    O.run(1e9, 1, 2.0, 0.9, 1.0, max_steps=20)
    assert (st["steps"], st["rejects"]) == (O.steps, O.rejects)
    assert np.array_equal(G.patches(), O.patches())
    qg, qo = G.download()[S], O.download()[S]
    scale = max(float(np.abs(qo[..., 0]).max()), 1.0)
    assert np.abs(qg - qo).max() <= 1e-8 * scale
    G.close()


def test_subcycling_takes_fewer_coarse_steps(ctx):
    """The same horizon with and without subcycling: the subcycled forest
    takes coarse steps 2^(levels - 1) times longer, its finest level the
    same number of sub-steps per unit time, and both end at the horizon with
    water still in the domain (walls)."""
    phys = gf.Phys(friction_forcing=False)
    ctx.set_phys(SLOT, phys)
    b, q = rasters("dambreak")
    runs = {}
    for sub in (False, True):
        G = gf.Forest(ctx, M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, mthbc=(3, 3, 3, 3),
                      regrid_interval=2, refine=FRONT, phys_slot=SLOT, subcycle=sub)
        G.init()
        runs[sub] = G.run(30.0, 1, 5.0, 0.9, 1.0)
        G.close()
    assert runs[True]["t"] == runs[False]["t"] == 30.0
    assert runs[True]["steps"] < runs[False]["steps"]


def forest(ctx, m=M, seed=3, regrid=2, subcycle=True, mthbc=(3, 3, 3, 3), hydro=None):
    b, q = rasters("dambreak", seed, m)
    F = gf.Forest(ctx, m, NBX, NBY, LMIN, LMAX, 1000.0 / m, 1000.0 / m, b, q, mthbc=mthbc,
                  regrid_interval=regrid, refine=FRONT, phys_slot=SLOT, subcycle=subcycle)
    if hydro is not None:
        F.set_hydrograph(*hydro)
    F.init()
    return F


def test_subcycled_forests_in_a_batch_equal_their_own_runs(ctx):
    """Subcycled forests of different patch sizes in gf_forest_batch_run
    (each in a launch group of its own), beside forests that share rounds:
    every forest ends as its own gf_forest_run."""
    from geoflood_gb300.forest import batch_run

    ctx.set_phys(SLOT, gf.Phys(manning_coefficient=(0.035,), manning_break=(1e10,)))
    specs = [dict(m=8, seed=3, regrid=2), dict(m=16, seed=5, regrid=3, mthbc=(0, 3, 3, 3), hydro=HYDRO),
             dict(m=8, seed=7, regrid=2, subcycle=False), dict(m=32, seed=6, regrid=4)]
    alone = []
    for sp in specs:
        F = forest(ctx, **sp)
        st = F.run(30.0, 2, 5.0, 0.9, 1.0)
        alone.append((F.patches(), F.download(), st))
        F.close()
    fs = [forest(ctx, **sp) for sp in specs]
    bst = batch_run(fs, 30.0, 2, 5.0, 0.9, 1.0)
    for F, (P, q, st) in zip(fs, alone):
        got = F.stats()
        assert np.array_equal(F.patches(), P)
        assert np.array_equal(F.download()[S], q[S])
        for k in ("steps", "rejects", "regrids", "cell_updates", "t"):
            assert got[k] == st[k], k
    assert bst["regrids"] == sum(F.stats()["regrids"] for F in fs)
    for F in fs:
        F.close()


@pytest.mark.parametrize("exact", [False, True])
def test_subcycled_forests_share_launches_and_equal_their_own_runs(ctx, exact):
    """Six subcycled forests of one patch size (different beds, regrid
    cadences, one with hydrograph inflow) in gf_forest_batch_run: forests
    whose leaves span the same levels step in shared launches, and the groups
    change as regrids add and remove levels; every forest ends as its own
    gf_forest_run, bit for bit, in both builds."""
    from geoflood_gb300.forest import batch_run

    ctx.set_phys(SLOT, gf.Phys(manning_coefficient=(0.035,), manning_break=(1e10,)))
    ctx.set_fp_contract(not exact)
    try:
        specs = [dict(m=16, seed=3 + k, regrid=2 + k % 2) for k in range(5)]
        specs.append(dict(m=16, seed=11, regrid=2, mthbc=(0, 3, 3, 3), hydro=HYDRO))
        alone = []
        for sp in specs:
            F = forest(ctx, **sp)
            st = F.run(30.0, 2, 5.0, 0.9, 1.0)
            alone.append((F.patches(), F.download(), st))
            F.close()
        fs = [forest(ctx, **sp) for sp in specs]
        bst = batch_run(fs, 30.0, 2, 5.0, 0.9, 1.0)
        for F, (P, q, st) in zip(fs, alone):
            got = F.stats()
            assert np.array_equal(F.patches(), P)
            assert np.array_equal(F.download()[S], q[S])
            for k in ("steps", "rejects", "regrids", "cell_updates", "t"):
                assert got[k] == st[k], k
        assert bst["regrids"] == sum(F.stats()["regrids"] for F in fs)
        for F in fs:
            F.close()
    finally:
        ctx.set_fp_contract(True)
