"""qad (geolib_source/qad.f:4-371) on the device against the oracle.

A coarse level and a fine level of random wet/dry patches (ghost cells
included); tasks on every side of fine patches, each side's ghost layer over
the coarse patch at the offsets a 2:1 quadtree gives (coarse neighbour left,
above, right, below; either half of its side). The device's svdflx, built
without contraction, must equal the oracle's restatement bit for bit, and it
accumulates over repeated calls.
"""
import numpy as np
import pytest

import geoflood_gb300 as gf
import oracle

pytestmark = pytest.mark.gpu


def _levels(rng, m, npatch):
    n = m + 4
    b = rng.normal(0.0, 0.4, (npatch, n, n, 1))
    h = np.where(rng.random((npatch, n, n)) < 0.2, rng.uniform(0, 2e-3, (npatch, n, n)),
                 rng.uniform(0.05, 3.0, (npatch, n, n)))
    q = np.stack([h, h * rng.normal(0, 1.5, h.shape), h * rng.normal(0, 1.5, h.shape)], -1)
    return np.ascontiguousarray(q), np.ascontiguousarray(b)


def _coarse_cells(qc, bc, m, side, ox, oy):
    """the coarse cells along a side, in qad.f's order, from the offsets"""
    cells = []
    for c in range(m // 2):
        f = 2 * c + 1                    # first of the two fine faces (1-based)
        fi, fj = {1: (0, f), 2: (f, m + 1), 3: (m + 1, f), 4: (f, 0)}[side]
        ci, cj = (fi - ox + 1) // 2, (fj - oy + 1) // 2
        cells.append((qc[cj + 1, ci + 1], bc[cj + 1, ci + 1]))
    return (np.ascontiguousarray([c[0] for c in cells]),
            np.ascontiguousarray([c[1] for c in cells]))


@pytest.mark.parametrize("m", [8, 16, 32])
def test_gpu_qad_equals_oracle(gpu_lib, m):
    rng = np.random.default_rng(100 + m)
    nc, nf = 3, 5
    qc, bc = _levels(rng, m, nc)
    qf, bf = _levels(rng, m, nf)
    hx = hy = 2.0
    dt = 0.05
    # (side, ox, oy) a 2:1 brick gives: the coarse neighbour across the side,
    # the fine side on its lower or upper half
    offs = {1: [(-2 * m, 0), (-2 * m, -m)], 2: [(0, m), (-m, m)],
            3: [(m, 0), (m, -m)], 4: [(0, -2 * m), (-m, -2 * m)]}
    tasks = []
    for k in range(nf):
        for side in (1, 2, 3, 4):
            ox, oy = offs[side][(k + side) % 2]
            tasks.append((k, (k + side) % nc, side, ox, oy))
    ctx = gf.Context(0)
    ctx.set_fp_contract(True)
    C = gf.Level(ctx, nc, m, 1)
    C.set_geometry(2 * hx, 2 * hy)
    C.upload(qc, bc)
    F = gf.Level(ctx, nf, m, 1)
    F.set_geometry(hx, hy)
    F.upload(qf, bf)
    svd = np.ascontiguousarray(rng.normal(0, 1e-3, (len(tasks), m // 2, 3)))
    want = svd.copy()
    for rep in range(2):
        C.qad(F, tasks, dt, svd)
        for t, (kf, kc, side, ox, oy) in enumerate(tasks):
            q1d, a1d = _coarse_cells(qc[kc], bc[kc], m, side, ox, oy)
            w = np.ascontiguousarray(want[t])
            oracle.qad_side(side, qf[kf], bf[kf], q1d, a1d, hx, hy, dt, w, gf.Phys())
            want[t] = w
        assert np.array_equal(svd, want), f"call {rep}: max diff {np.abs(svd - want).max():.3e}"
    assert np.abs(svd).max() > 0.0
    # a side whose ghost cells are not over the coarse patch is refused
    with pytest.raises(gf.GeoFloodError):
        C.qad(F, [(0, 0, 1, 0, 0)], dt, np.zeros((1, m // 2, 3)))
    C.close()
    F.close()
    ctx.close()
