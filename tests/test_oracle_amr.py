"""Known-answer tests of the oracle's coarse/fine transfers, time
interpolation and refinement tags (no GPU)."""
import numpy as np
import pytest

import geoflood_gb300 as gf
import oracle

MBC = 2


def flat_state(m, h, hu, hv, b):
    q = np.zeros((m + 4, m + 4, 3))
    q[..., 0], q[..., 1], q[..., 2] = h, hu, hv
    aux = np.full((m + 4, m + 4, 1), float(b))
    return q, aux


def test_average2coarse_of_uniform_children():
    m = 16
    qc, ac = flat_state(m, 0.0, 0.0, 0.0, 1.0)
    qf, af = flat_state(m, 2.0, 0.6, -0.4, 1.0)
    for igrid in range(4):
        oracle.average2coarse(qc, ac, qf, af, igrid)
    s = slice(MBC, MBC + m)
    assert np.allclose(qc[s, s, 0], 2.0, atol=0, rtol=0)
    assert np.allclose(qc[s, s, 1], 0.6, rtol=1e-15)
    assert np.allclose(qc[s, s, 2], -0.4, rtol=1e-15)


def test_average_of_dry_children_is_dry():
    m = 8
    qc, ac = flat_state(m, 5.0, 1.0, 1.0, 0.0)
    qf, af = flat_state(m, 5e-4, 0.3, 0.3, 0.0)
    oracle.average2coarse(qc, ac, qf, af, 0)
    s = slice(MBC, MBC + m // 2)
    assert np.all(qc[s, s] == 0.0)


def test_interpolate2fine_preserves_flat_surface():
    m = 16
    rng = np.random.default_rng(3)
    qc, ac = flat_state(m, 0.0, 0.5, 0.25, 0.0)
    bc = rng.uniform(0, 2, (m + 4, m + 4))
    ac[..., 0] = bc
    qc[..., 0] = 5.0 - bc                      # eta = 5 everywhere
    qf, af = flat_state(m, 0.0, 0.0, 0.0, 0.0)
    af[..., 0] = rng.uniform(0, 2, (m + 4, m + 4))
    oracle.interpolate2fine(qc, ac, qf, af, 0)
    s = slice(MBC, MBC + m)
    assert np.allclose(qf[s, s, 0] + af[s, s, 0], 5.0, rtol=0, atol=1e-14)
    assert np.all(qf[s, s, 1] == 0.5) and np.all(qf[s, s, 2] == 0.25)


def test_refine_then_coarsen_round_trip_lake():
    m = 16
    qc, ac = flat_state(m, 0.0, 0.0, 0.0, 0.0)
    qc[..., 0] = 3.0
    children = []
    for igrid in range(4):
        qf, af = flat_state(m, 0.0, 0.0, 0.0, 0.0)
        oracle.interpolate2fine(qc, ac, qf, af, igrid)
        children.append((qf, af))
    back, bac = flat_state(m, 0.0, 0.0, 0.0, 0.0)
    for igrid, (qf, af) in enumerate(children):
        oracle.average2coarse(back, bac, qf, af, igrid)
    s = slice(MBC, MBC + m)
    assert np.array_equal(back[s, s], qc[s, s])


def test_timeinterp_strip_and_count():
    m = 16
    rng = np.random.default_rng(5)
    cur = rng.standard_normal((m + 4, m + 4, 3))
    last = rng.standard_normal((m + 4, m + 4, 3))
    out = np.zeros_like(cur)
    assert oracle.timeinterp(cur, last, out, 0.25) == 0
    s = slice(MBC, MBC + m)
    strip = np.zeros((m, m), bool)
    strip[:2, :] = strip[-2:, :] = strip[:, :2] = strip[:, -2:] = True
    exp = last + 0.25 * (cur - last)
    assert np.array_equal(out[s, s][strip], exp[s, s][strip])
    assert np.all(out[s, s][~strip] == 0.0)


def test_face_average_fills_half_the_coarse_ghosts():
    """A fine neighbour on the coarse patch's right face covers half of it."""
    m = 8
    qc, ac = flat_state(m, 9.0, 9.0, 9.0, 0.0)
    qf, af = flat_state(m, 1.0, 0.0, 0.0, 0.0)
    oracle.average_ghost(qc, ac, qf, af, 0, 1, -2 * m, 0)   # fine patch = lower half
    ghost = qc[MBC:MBC + m, MBC + m:, 0]                     # rows j=1..m, right ghosts
    assert np.all(ghost[: m // 2] == 1.0) and np.all(ghost[m // 2:] == 9.0)


def test_tags_known_answers():
    m = 8
    q, aux = flat_state(m, 2.0, 0.0, 0.0, -2.0)       # eta = 0 = sea level
    rf = oracle.refine(gf.Refine(wave_tolerance=0.1, speed_tolerance=(1.0, 2.0)))
    assert oracle.tag4refinement(q, aux, 0, 0, 1, 1, 0.0, 1, 3, 0, rf) == 0
    q[MBC + 3, MBC + 4, 0] = 2.5                       # a wave above tolerance
    assert oracle.tag4refinement(q, aux, 0, 0, 1, 1, 0.0, 1, 3, 0, rf) == 1
    q[..., 0] = 2.0
    q[MBC + 1, MBC + 1, 1] = 3.0                       # speed 1.5 > tol(1) at level 1
    assert oracle.tag4refinement(q, aux, 0, 0, 1, 1, 0.0, 1, 3, 0, rf) == 1
    assert oracle.tag4refinement(q, aux, 0, 0, 1, 1, 0.0, 2, 3, 0, rf) == 0
    # a region forcing refinement at level < 3 wins over the criteria
    rfr = oracle.refine(gf.Refine(regions=((0.0, 4.0, 0.0, 4.0, 0.0, 10.0, 3, 5),)))
    q, aux = flat_state(m, 0.0, 0.0, 0.0, 0.0)
    assert oracle.tag4refinement(q, aux, 0, 0, 1, 1, 0.0, 2, 5, 0, rfr) == 1
    assert oracle.tag4refinement(q, aux, 0, 0, 1, 1, 20.0, 2, 5, 0, rfr) == 0


def test_coarsening_uses_integer_threshold_factor():
    """th_factor is an INTEGER in the Fortran: 0.5 truncates to 0, so any
    moving wet cell blocks coarsening."""
    m = 8
    q, aux = flat_state(m, 2.0, 1e-9, 0.0, -2.0)
    rf = oracle.refine(gf.Refine(wave_tolerance=0.1, speed_tolerance=(1.0,)))
    fam = [q, q, q, q]
    auxs = [aux] * 4
    assert oracle.tag4coarsening(fam, auxs, [0, 8, 0, 8], [0, 0, 8, 8], 1, 1, 0.0, 1, 3, 0, rf) == 0
    q2, _ = flat_state(m, 2.0, 0.0, 0.0, -2.0)
    assert oracle.tag4coarsening([q2] * 4, auxs, [0, 8, 0, 8], [0, 0, 8, 8], 1, 1, 0.0, 1, 3, 0,
                                 rf) == 1
    # initial refinement never coarsens
    assert oracle.tag4coarsening([q2] * 4, auxs, [0, 8, 0, 8], [0, 0, 8, 8], 1, 1, 0.0, 1, 3, 1,
                                 rf) == 1
