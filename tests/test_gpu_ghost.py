"""Ghost fill on the device against the oracle (GPU required).

Copies and the extrapolation / wall / periodic rules move values without
arithmetic, so they must agree bit for bit. The hydrograph inflow solves a
Newton iteration with pow(); it is held to 1e-10 of the depth scale.
"""
import numpy as np
import pytest

import geoflood_gb300 as gf
import oracle
from geoflood_gb300 import synth

pytestmark = pytest.mark.gpu
MBC = 2


def scrambled(q, seed):
    """Same interiors, garbage ghost cells (so every ghost must be written)."""
    g = synth.rng(seed)
    out = q.copy()
    ring = np.ones(q.shape[1:3], bool)
    m = q.shape[1] - 2 * MBC
    ring[MBC:MBC + m, MBC:MBC + m] = False
    out[:, ring] = g.standard_normal(out[:, ring].shape) * 50.0
    return out


def gpu_fill(ctx, q, aux, m, nbr, xl, yl, dx, t, mthbc, hydro=None):
    lev = gf.Level(ctx, q.shape[0], m, aux.shape[-1])
    lev.set_geometry(dx, dx)
    lev.upload(q, aux)
    lev.set_layout(nbr, xl, yl)
    if hydro is not None:
        lev.set_hydrograph(**hydro)
    lev.set_bc(mthbc)
    lev.ghost_fill(t)
    out, a = lev.download(), lev.download_aux()
    lev.close()
    return out, a


@pytest.mark.parametrize("m", [8, 16, 32])
@pytest.mark.parametrize("mthbc", [(1, 1, 1, 1), (3, 3, 3, 3), (1, 3, 3, 1)])
def test_copy_and_physical_bc_bitwise(ctx, m, mthbc):
    q, aux, py, px = synth.uniform_dam_break_level(3, 4, m, 1.0, seed=5, x_dam=1.7 * m)
    q[..., 1] = 0.3 * q[..., 0]
    q[..., 2] = -0.2 * q[..., 0]
    nbr, xl, yl = synth.brick_layout(py, px, m, 1.0)
    qs = scrambled(q, 3)
    out, a = gpu_fill(ctx, qs, aux.copy(), m, nbr, xl, yl, 1.0, 0.0, mthbc)
    ref, ra = qs.copy(), aux.copy()
    oracle.level_ghost_fill(ref, ra, nbr, xl, yl, 1.0, 1.0, 0.0, mthbc)
    assert np.array_equal(out, ref)
    assert np.array_equal(a, ra)


def test_periodic_x(ctx):
    m = 16
    q, aux, py, px = synth.uniform_dam_break_level(3, 2, m, 1.0, seed=6, x_dam=20.0)
    nbr, xl, yl = synth.brick_layout(py, px, m, 1.0, periodic_x=True)
    qs = scrambled(q, 4)
    mthbc = (2, 2, 3, 3)
    out, a = gpu_fill(ctx, qs, aux.copy(), m, nbr, xl, yl, 1.0, 0.0, mthbc)
    ref, ra = qs.copy(), aux.copy()
    oracle.level_ghost_fill(ref, ra, nbr, xl, yl, 1.0, 1.0, 0.0, mthbc)
    assert np.array_equal(out, ref) and np.array_equal(a, ra)


@pytest.mark.parametrize("t", [0.0, 150.0, 900.0, 5000.0])
def test_hydrograph_inflow_left(ctx, t):
    m = 16
    q, aux, py, px = synth.uniform_dam_break_level(2, 4, m, 2.0, seed=7, x_dam=40.0)
    # a wet strip and a dry strip along the inflow side
    q[..., 0] = np.where(np.arange(m + 4)[None, :, None] < 10, 2.5, q[..., 0])
    q[..., 1] = 0.4 * q[..., 0]
    nbr, xl, yl = synth.brick_layout(py, px, m, 2.0)
    hyd = dict(time=[0.0, 600.0, 1800.0], hu=[0.0, 4.0, 1.5], side=(1, 0, 0, 0),
               width=40.0, x0=0.0, y0=64.0)
    qs = scrambled(q, 5)
    mthbc = (0, 1, 3, 3)
    out, a = gpu_fill(ctx, qs, aux.copy(), m, nbr, xl, yl, 2.0, t, mthbc, hyd)
    ref, ra = qs.copy(), aux.copy()
    hy = oracle.hydro(hyd["time"], hyd["hu"], hyd["side"], hyd["width"], hyd["x0"], hyd["y0"])
    oracle.level_ghost_fill(ref, ra, nbr, xl, yl, 2.0, 2.0, t, mthbc, hy=hy)
    sc = max(1.0, float(np.abs(q).max()))
    assert np.abs(out - ref).max() <= 1e-10 * sc
    assert np.array_equal(a, ra)


def test_bc_rule0_without_hydrograph_is_rejected(ctx):
    lev = gf.Level(ctx, 1, 8)
    with pytest.raises(gf.GeoFloodError):
        lev.set_bc((0, 1, 1, 1))
    lev.close()


def test_ghost_fill_needs_layout(ctx):
    lev = gf.Level(ctx, 1, 8)
    with pytest.raises(gf.GeoFloodError):
        lev.ghost_fill(0.0)
    lev.close()


@pytest.mark.parametrize("mthbc", [(1, 1, 1, 1), (3, 3, 3, 3)])
def test_level_steps_with_ghost_fill_resynced(ctx, mthbc):
    """Update + ghost fill for 8 steps; each step the oracle restarts from the
    GPU state and both must agree (update within 1e-10, ghosts exactly)."""
    m, dx, dt = 16, 1.0, 0.05
    q, aux, py, px = synth.uniform_dam_break_level(4, 3, m, dx, seed=9, x_dam=20.0)
    nbr, xl, yl = synth.brick_layout(py, px, m, dx)
    ctx.set_phys(0, gf.Phys())
    lev = gf.Level(ctx, q.shape[0], m)
    lev.set_geometry(dx, dx)
    lev.upload(q, aux)
    lev.set_layout(nbr, xl, yl)
    lev.set_bc(mthbc)
    lev.ghost_fill(0.0)
    state, aux_state = lev.download(), lev.download_aux()
    for step in range(8):
        ref, ra = state.copy(), aux_state.copy()
        oracle.level_update(ref, ra, dx, dx, 0.0, dt, gf.Phys(), nthreads=1)
        oracle.level_ghost_fill(ref, ra, nbr, xl, yl, dx, dx, (step + 1) * dt, mthbc)
        lev.step(0.0, dt)
        lev.ghost_fill((step + 1) * dt)
        out = lev.download()
        sc = max(1.0, float(np.abs(state).max()))
        assert np.abs(out - ref).max() <= 1e-10 * sc
        state = out
        lev.upload(state)
