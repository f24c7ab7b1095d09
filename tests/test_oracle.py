"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no golden vectors for the patch update, so the oracle is
checked against properties that follow from the mathematics of the scheme:
well-balancing (lake at rest), dry-bed invariance, conservation with wall
ghost cells, x/y symmetry and the analytic Stoker dam-break solution.
"""
import numpy as np
import pytest
from scipy.optimize import brentq

import oracle
from geoflood_gb300 import Phys, synth

MBC = 2


def _lake(m, seed, eta=15.0, dx=10.0):
    b = synth.fractal_dem(m, m, dx, 0.8, 30.0, seed)
    h = np.maximum(eta - b, 0.0)
    q = np.zeros((m, m, 3))
    q[..., 0] = h
    return synth.pad_extrap(q), synth.pad_extrap(b[..., None])


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("m", [8, 16, 32])
def test_lake_at_rest_is_preserved(m, seed):
    q, aux = _lake(m, seed)
    q0 = q.copy()
    cfl = oracle.patch_update(q, aux, 10.0, 10.0, 0.0, 0.5)
    s = slice(MBC, MBC + m)
    eta0 = q0[s, s, 0] + aux[s, s, 0]
    wet = q0[s, s, 0] > 1e-3
    eta1 = q[s, s, 0] + aux[s, s, 0]
    assert np.abs(eta1 - eta0)[wet].max() < 1e-12
    assert np.abs(q[s, s, 1:]).max() < 1e-12
    assert 0.0 < cfl < 1.0


def test_dry_bed_stays_dry():
    m = 16
    b = synth.fractal_dem(m, m, 5.0, 0.8, 10.0, 4)
    q = np.zeros((m + 4, m + 4, 3))
    q[..., 0] = 1e-4  # below the dry tolerance
    q[..., 1] = 0.3   # momenta in dry cells are zeroed by b4step2
    aux = synth.pad_extrap(b[..., None])
    cfl = oracle.patch_update(q, aux, 5.0, 5.0, 0.0, 0.1)
    assert cfl == 0.0
    s = slice(MBC, MBC + m)
    assert np.all(q[s, s, 0] == 1e-4)
    assert np.all(q[s, s, 1:] == 0.0)


def test_mass_conserved_with_wall_ghosts():
    """With mirrored walls the only mass source is b4step2's clipping of
    negative depths (geoclaw_b4step2_fort.f90:183-186)."""
    m = 32
    b = synth.fractal_dem(m, m, 10.0, 0.8, 30.0, 3)
    bw = synth.pad_wall(np.repeat(b[..., None], 3, axis=2))[..., :1].copy()
    q = synth.dam_break_state(b, 10.0, x_dam=160.0)
    mass0 = q[..., 0].sum()
    clipped = 0.0
    for _ in range(20):
        clipped += -np.minimum(q[..., 0], 0.0).sum()
        qh = synth.pad_wall(q)
        oracle.patch_update(qh, bw, 10.0, 10.0, 0.0, 0.2)
        q = qh[MBC:-MBC, MBC:-MBC].copy()
    assert abs(q[..., 0].sum() - mass0 - clipped) / mass0 < 1e-13


def test_flat_bed_walls_conserve_exactly():
    m = 32
    aux = np.zeros((m + 4, m + 4, 1))
    x = np.arange(m) + 0.5
    q = np.zeros((m, m, 3))
    q[..., 0] = np.where(x[None, :] < 16, 10.0, 2.0) + 0.5 * np.sin(np.arange(m))[:, None]
    mass0 = q[..., 0].sum()
    for _ in range(50):
        qh = synth.pad_wall(q)
        oracle.patch_update(qh, aux, 1.0, 1.0, 0.0, 0.05)
        q = qh[MBC:-MBC, MBC:-MBC].copy()
    assert abs(q[..., 0].sum() - mass0) / mass0 < 1e-14


def test_xy_transpose_symmetry():
    m = 16
    g = synth.rng(11)
    b = synth.fractal_dem(m, m, 4.0, 0.7, 6.0, 5)
    q = np.zeros((m, m, 3))
    q[..., 0] = np.maximum(4.0 - b + 0.5 * g.standard_normal((m, m)), 0.0)
    q[..., 1] = g.standard_normal((m, m))
    q[..., 2] = g.standard_normal((m, m))
    qa, ba = synth.pad_extrap(q), synth.pad_extrap(b[..., None])
    qt = np.ascontiguousarray(qa.transpose(1, 0, 2)[..., [0, 2, 1]])
    bt = np.ascontiguousarray(ba.transpose(1, 0, 2))
    c1 = oracle.patch_update(qa, ba, 4.0, 4.0, 0.0, 0.1)
    c2 = oracle.patch_update(qt, bt, 4.0, 4.0, 0.0, 0.1)
    back = qt.transpose(1, 0, 2)[..., [0, 2, 1]]
    s = slice(MBC, MBC + m)
    assert np.abs(back[s, s] - qa[s, s]).max() < 1e-12
    assert abs(c1 - c2) < 1e-14


def _stoker(x, t, hl, hr, x0, g=9.81):
    cl = np.sqrt(g * hl)

    def f(hm):
        um_r = 2 * (cl - np.sqrt(g * hm))
        um_s = (hm - hr) * np.sqrt(0.5 * g * (hm + hr) / (hm * hr))
        return um_r - um_s

    hm = brentq(f, hr, hl)
    um = 2 * (cl - np.sqrt(g * hm))
    cm = np.sqrt(g * hm)
    S = hm * um / (hm - hr)
    xi = (x - x0) / t
    h = np.where(xi < -cl, hl, 0.0)
    fan = (xi >= -cl) & (xi < um - cm)
    h = np.where(fan, (2 * cl - xi) ** 2 / (9 * g), h)
    h = np.where((xi >= um - cm) & (xi < S), hm, h)
    h = np.where(xi >= S, hr, h)
    return h


def test_stoker_dam_break_flat_bed():
    """1-D wet dam break (hL = 2 m, hR = 1 m) against the analytic solution."""
    mx, my, dx = 400, 4, 0.5
    x = (np.arange(mx) + 0.5) * dx
    q = np.zeros((my, mx, 3))
    q[..., 0] = np.where(x < 100.0, 2.0, 1.0)[None, :]
    aux = np.zeros((my + 4, mx + 4, 1))
    phys = Phys(friction_forcing=False)
    t, tend = 0.0, 10.0
    while t < tend - 1e-12:
        qh = synth.pad_extrap(q)
        dt = min(0.05, tend - t)
        cfl = oracle.patch_update(qh, aux, dx, dx, t, dt, phys)
        assert cfl < 1.0
        q = qh[MBC:-MBC, MBC:-MBC].copy()
        t += dt
    h_exact = _stoker(x, tend, 2.0, 1.0, 100.0)
    l1 = np.abs(q[1, :, 0] - h_exact).sum() / np.abs(h_exact).sum()
    assert l1 < 5e-3
    assert np.abs(q[..., 2]).max() < 1e-12  # no transverse momentum


def test_riemann_known_answers():
    """Single-face augmented solver: a still lake over a step is a steady
    state (zero f-waves); a symmetric collision gives symmetric speeds."""
    g, tol = 9.81, 1e-3
    # lake at rest across a bathymetry step: eta = 5, bL = 0, bR = 1
    hL, hR = 5.0, 4.0
    phiL, phiR = 0.5 * g * hL * hL, 0.5 * g * hR * hR
    cL, cR = np.sqrt(g * hL), np.sqrt(g * hR)
    uhat = 0.0
    chat = np.sqrt(g * 0.5 * (hL + hR))
    sE1, sE2 = min(-cL, uhat - chat), max(cR, uhat + chat)
    s, fw = oracle.riemann_aug_JCP(hL, hR, 0, 0, 0, 0, 0.0, 1.0, 0, 0, 0, 0, phiL, phiR,
                                   sE1, sE2, tol, g)
    assert np.abs(fw).max() < 1e-12
    # symmetric collision: u = +-1 on equal depths
    h, u = 3.0, 1.0
    phi = 0.5 * g * h * h + h * u * u
    c = np.sqrt(g * h)
    chat = np.sqrt(g * h)
    s, fw = oracle.riemann_aug_JCP(h, h, h * u, -h * u, 0, 0, 0, 0, u, -u, 0, 0, phi, phi,
                                   min(u - c, -chat), max(-u + c, chat), tol, g)
    assert abs(s[0] + s[2]) < 1e-14
    assert abs(s[1]) < 1e-14
