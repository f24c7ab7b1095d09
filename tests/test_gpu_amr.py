"""Coarse/fine transfers, time interpolation and refinement tags on the GPU
against the oracle (GPU required). These kernels are built without FMA
contraction, so values and tags must agree bit for bit."""
import numpy as np
import pytest

import geoflood_gb300 as gf
import oracle
from geoflood_gb300 import _lib, synth

pytestmark = pytest.mark.gpu
MBC = 2


def wet_dry_patch(m, seed, depth=2.0):
    g = np.random.default_rng(seed)
    b = synth.fractal_dem(m + 4, m + 4, 1.0, 0.7, 4.0, seed)
    q = np.zeros((m + 4, m + 4, 3))
    q[..., 0] = np.maximum(depth - b + 0.3 * g.standard_normal(b.shape), 0.0)
    q[..., 1] = q[..., 0] * g.standard_normal(b.shape)
    q[..., 2] = q[..., 0] * g.standard_normal(b.shape)
    return q, b[..., None].copy()


def make_level(ctx, qs, auxs, m, dx=1.0):
    lev = gf.Level(ctx, len(qs), m, auxs[0].shape[-1])
    lev.set_geometry(dx, dx)
    lev.upload(np.stack(qs), np.stack(auxs))
    return lev


@pytest.mark.parametrize("m", [8, 16, 32])
def test_face_average_then_interpolate(ctx, m):
    """Coarse patch with two half-size fine neighbours across its right face."""
    qc, ac = wet_dry_patch(m, 1)
    fines = [wet_dry_patch(m, 10 + k) for k in range(2)]
    C = make_level(ctx, [qc], [ac], m, 2.0)
    F = make_level(ctx, [f[0] for f in fines], [f[1] for f in fines], m, 1.0)
    avg = [(_lib.XFER_AVG_FACE, 0, k, 1, -2 * m, -k * m) for k in range(2)]
    C.transfer(F, avg)
    itp = [(_lib.XFER_INTERP_FACE, 0, k, 1, -2 * m, -k * m) for k in range(2)]
    C.transfer(F, itp)
    gc, gfq = C.download()[0], F.download()
    rc = qc.copy()
    rfs = [f[0].copy() for f in fines]
    for k in range(2):
        oracle.average_ghost(rc, ac, rfs[k], fines[k][1], 0, 1, -2 * m, -k * m)
    for k in range(2):
        oracle.interpolate_ghost(rc, ac, rfs[k], fines[k][1], 0, 1, -2 * m, -k * m)
    assert np.array_equal(gc, rc)
    for k in range(2):
        assert np.array_equal(gfq[k], rfs[k])
    C.close()
    F.close()


@pytest.mark.parametrize("face", [0, 2, 3])
def test_other_faces(ctx, face):
    m = 16
    qc, ac = wet_dry_patch(m, 2)
    qf, af = wet_dry_patch(m, 3)
    # fine patch across the given coarse face (its lower / left half): the
    # coarse patch's lower-left corner in the fine patch's cell indices
    ox, oy = {0: (m, 0), 2: (0, m), 3: (0, -2 * m)}[face]
    C = make_level(ctx, [qc], [ac], m)
    F = make_level(ctx, [qf], [af], m)
    C.transfer(F, [(_lib.XFER_AVG_FACE, 0, 0, face, ox, oy)])
    C.transfer(F, [(_lib.XFER_INTERP_FACE, 0, 0, face, ox, oy)])
    rc, rf = qc.copy(), qf.copy()
    oracle.average_ghost(rc, ac, rf, af, 0, face, ox, oy)
    oracle.interpolate_ghost(rc, ac, rf, af, 0, face, ox, oy)
    assert np.array_equal(C.download()[0], rc)
    assert np.array_equal(F.download()[0], rf)


@pytest.mark.parametrize("corner", [0, 1, 2, 3])
def test_corner_average_and_interpolate(ctx, corner):
    m = 16
    qc, ac = wet_dry_patch(m, 4)
    qf, af = wet_dry_patch(m, 5)
    ox = -2 * m if corner in (1, 3) else m
    oy = -2 * m if corner in (2, 3) else m
    C = make_level(ctx, [qc], [ac], m)
    F = make_level(ctx, [qf], [af], m)
    C.transfer(F, [(_lib.XFER_AVG_CORNER, 0, 0, corner, ox, oy)])
    C.transfer(F, [(_lib.XFER_INTERP_CORNER, 0, 0, corner, ox, oy)])
    rc, rf = qc.copy(), qf.copy()
    oracle.average_ghost(rc, ac, rf, af, 1, corner, ox, oy)
    oracle.interpolate_ghost(rc, ac, rf, af, 1, corner, ox, oy)
    assert np.array_equal(C.download()[0], rc)
    assert np.array_equal(F.download()[0], rf)


@pytest.mark.parametrize("m", [8, 16, 32])
def test_refine_and_coarsen_transfers(ctx, m):
    qc, ac = wet_dry_patch(m, 6)
    kids = [wet_dry_patch(m, 20 + k) for k in range(4)]
    C = make_level(ctx, [qc], [ac], m, 2.0)
    F = make_level(ctx, [k[0] for k in kids], [k[1] for k in kids], m, 1.0)
    C.transfer(F, [(_lib.XFER_INTERP2FINE, 0, g, g, 0, 0) for g in range(4)])
    got_f = F.download()
    rfs = [k[0].copy() for k in kids]
    for g in range(4):
        oracle.interpolate2fine(qc, ac, rfs[g], kids[g][1], g)
        assert np.array_equal(got_f[g], rfs[g])
    C.transfer(F, [(_lib.XFER_AVG2COARSE, 0, g, g, 0, 0) for g in range(4)])
    rc = qc.copy()
    for g in range(4):
        oracle.average2coarse(rc, ac, rfs[g], kids[g][1], g)
    assert np.array_equal(C.download()[0], rc)


def test_timeinterp(ctx):
    m = 16
    g = np.random.default_rng(7)
    cur = g.standard_normal((3, m + 4, m + 4, 3))
    last = g.standard_normal((3, m + 4, m + 4, 3))
    dst = np.zeros_like(cur)
    aux = np.zeros((3, m + 4, m + 4, 1))
    Lc, Ll, Ld = (make_level(ctx, list(a), list(aux), m) for a in (cur, last, dst))
    Ld.timeinterp(Lc, Ll, 0.375)
    ref = dst.copy()
    for k in range(3):
        assert oracle.timeinterp(cur[k], last[k], ref[k], 0.375) == 0
    assert np.array_equal(Ld.download(), ref)


REFINES = [
    gf.Refine(wave_tolerance=0.2, speed_tolerance=(1.0, 2.0, 3.0)),
    gf.Refine(wave_tolerance=1e9, speed_tolerance=(0.5,), max_level_deep=1, deep_depth=1.0,
              max_velocity_depth_product=2.0),
    gf.Refine(flowgrades=((1.5, 1, 1, 3), (2.0, 2, 1, 2), (0.5, 3, 1, 3))),
    gf.Refine(regions=((0.0, 20.0, 0.0, 20.0, 0.0, 5.0, 2, 3),
                       (30.0, 60.0, 0.0, 60.0, 0.0, 50.0, 1, 1))),
]


@pytest.mark.parametrize("ri", range(len(REFINES)))
@pytest.mark.parametrize("level", [1, 2, 3])
def test_refinement_and_coarsening_tags(ctx, ri, level):
    m = 16
    n = 8
    pats = [wet_dry_patch(m, 40 + k, depth=1.0 + 0.3 * k) for k in range(n)]
    nbr, xl, yl = synth.brick_layout(2, 4, m, 1.0)
    L = make_level(ctx, [p[0] for p in pats], [p[1] for p in pats], m)
    L.set_layout(nbr, xl, yl)
    rf = REFINES[ri]
    for init_flag in (0, 1):
        for t in (0.0, 10.0):
            tags = L.tag4refinement(rf, level, 4, init_flag, t)
            ref = [oracle.tag4refinement(pats[k][0], pats[k][1], xl[k], yl[k], 1.0, 1.0, t, level,
                                         4, init_flag, oracle.refine(rf)) for k in range(n)]
            assert list(tags) == ref
            fams = [[0, 1, 4, 5], [2, 3, 6, 7]]
            ctags = L.tag4coarsening(rf, fams, level, 4, init_flag, t)
            cref = [oracle.tag4coarsening([pats[k][0] for k in f], [pats[k][1] for k in f],
                                          [xl[k] for k in f], [yl[k] for k in f], 1.0, 1.0, t,
                                          level, 4, init_flag, oracle.refine(rf)) for f in fams]
            assert list(ctags) == cref


def test_transfer_rejects_bad_tasks(ctx):
    m = 8
    qc, ac = wet_dry_patch(m, 1)
    C = make_level(ctx, [qc], [ac], m)
    F = make_level(ctx, [qc], [ac], m)
    with pytest.raises(gf.GeoFloodError):
        C.transfer(F, [(_lib.XFER_AVG_FACE, 0, 3, 1, 0, 0)])   # fine index out of range
    with pytest.raises(gf.GeoFloodError):
        C.transfer(F, [(_lib.XFER_AVG_CORNER, 0, 0, 3, 0, 0)])  # corner reaching outside
