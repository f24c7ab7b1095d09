"""Known-answer tests of the oracle's qad (geolib_source/qad.f:4-371).

qad adds, per coarse cell along a side of a fine patch, the fluctuations
amdq + apdq of the Riemann problem between the fine ghost cell and the coarse
cell, times the fine face length and dt. With the f-wave solver the
fluctuations of the depth equation sum to the jump of the normal momentum
(hu_right - hu_left), which gives an exact answer for the mass entries;
equal states give no fluctuation at all, and a lake at rest across a
bathymetry step (well-balanced solver) none beyond round-off.
"""
import numpy as np
import pytest

import oracle
from geoflood_gb300 import Phys

M = 16
PH = Phys()


def _patch(rng, m=M, wet=True):
    n = m + 4
    b = rng.normal(0.0, 0.3, (n, n, 1))
    h = rng.uniform(0.5, 3.0, (n, n)) if wet else np.zeros((n, n))
    q = np.stack([h, h * rng.normal(0, 1, (n, n)), h * rng.normal(0, 1, (n, n))], -1)
    return np.ascontiguousarray(q), np.ascontiguousarray(b)


def _ghost(q, side, f):
    """fine ghost cell f (0-based) of a side, as qad.f reads it"""
    m = q.shape[0] - 4
    if side == 1:
        return q[2 + f, 1]
    if side == 2:
        return q[m + 2, 2 + f]
    if side == 3:
        return q[2 + f, m + 2]
    return q[1, 2 + f]


@pytest.mark.parametrize("side", [1, 2, 3, 4])
def test_mass_entries_are_the_momentum_jump(side):
    rng = np.random.default_rng(10 + side)
    q, b = _patch(rng)
    nc = M // 2
    qc = np.ascontiguousarray(np.stack([rng.uniform(0.5, 3.0, nc), rng.normal(0, 2, nc),
                                        rng.normal(0, 2, nc)], -1))
    bc = np.ascontiguousarray(rng.normal(0, 0.3, (nc, 1)))
    svd = np.zeros((nc, 3))
    hx, hy, dt = 0.5, 0.75, 0.01
    oracle.qad_side(side, q, b, qc, bc, hx, hy, dt, svd, PH)
    normal = 1 if side in (1, 3) else 2
    h = hy if side in (1, 3) else hx
    sgn = 1.0 if side in (1, 4) else -1.0
    for c in range(nc):
        want = 0.0
        for l in range(2):
            g = _ghost(q, side, 2 * c + l)
            left, right = (qc[c], g) if side in (1, 4) else (g, qc[c])
            want += sgn * (right[normal] - left[normal]) * h * dt
        assert svd[c, 0] == pytest.approx(want, rel=1e-12, abs=1e-14)


@pytest.mark.parametrize("side", [1, 2, 3, 4])
def test_equal_states_give_no_fluctuation(side):
    rng = np.random.default_rng(20 + side)
    q, b = _patch(rng)
    nc = M // 2
    qc = np.zeros((nc, 3))
    bc = np.zeros((nc, 1))
    for c in range(nc):
        g = _ghost(q, side, 2 * c)
        for l in range(2):  # both fine ghosts of the coarse cell equal to it
            f = 2 * c + l
            if side == 1:
                q[2 + f, 1], b[2 + f, 1] = g, 0.25
            elif side == 2:
                q[M + 2, 2 + f], b[M + 2, 2 + f] = g, 0.25
            elif side == 3:
                q[2 + f, M + 2], b[2 + f, M + 2] = g, 0.25
            else:
                q[1, 2 + f], b[1, 2 + f] = g, 0.25
        qc[c], bc[c] = g, 0.25
    svd = np.zeros((nc, 3))
    oracle.qad_side(side, q, b, qc, bc, 1.0, 1.0, 0.1, svd, PH)
    assert np.all(svd == 0.0)


@pytest.mark.parametrize("side", [1, 2, 3, 4])
def test_lake_at_rest_stays_balanced(side):
    rng = np.random.default_rng(30 + side)
    n = M + 4
    b = rng.normal(0.0, 0.5, (n, n, 1))
    eta = 2.0
    q = np.zeros((n, n, 3))
    q[..., 0] = eta - b[..., 0]
    nc = M // 2
    bc = rng.normal(0.0, 0.5, (nc, 1))
    qc = np.zeros((nc, 3))
    qc[:, 0] = eta - bc[:, 0]
    svd = np.zeros((nc, 3))
    oracle.qad_side(side, q, b, qc, bc, 1.0, 1.0, 0.1, svd, PH)
    assert np.abs(svd).max() < 1e-12


def test_dry_against_dry_is_zero_and_accumulates():
    rng = np.random.default_rng(5)
    q, b = _patch(rng, wet=False)
    nc = M // 2
    qc = np.zeros((nc, 3))
    bc = np.zeros((nc, 1))
    svd = np.full((nc, 3), 0.125)
    oracle.qad_side(1, q, b, qc, bc, 1.0, 1.0, 0.1, svd, PH)
    assert np.all(svd == 0.125)  # accumulated into, nothing added
