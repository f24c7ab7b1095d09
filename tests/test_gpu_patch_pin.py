"""The GPU patch update against the reference's own patch kernel.

Replays tests/golden/patch_pin.npz (one-step patch problems and the results
of the reference's cudaclaw_flux2_and_update, host-built; see
tests/golden/make_patch_pin.py) through the C-ABI buffered hook
gf_patch_update_batch, in the production build (FMA contraction, the 1e-10
bar of the state's scale) and in the contraction-free build (the 1e-13 bar
the oracle meets). Wet/dry masks must be equal and the patch CFL agree to
1e-12.
"""
from pathlib import Path

import numpy as np
import pytest

import geoflood_gb300 as gf

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "patch_pin.npz"


def _phys(method, drytol, grav):
    order, tr, l1, l2, l3, src, fdepth, manning = method
    return gf.Phys(grav=float(grav), dry_tolerance=float(drytol), friction_depth=float(fdepth),
                   manning_coefficient=(float(manning),), manning_break=(1.0e10,),
                   order=int(order), transverse=int(tr), mthlim=(int(l1), int(l2), int(l3)),
                   src_term=int(src))


@pytest.mark.parametrize("contract,tol", [(1, 1e-10), (0, 1e-13)])
def test_gpu_matches_reference_patch_kernel(gpu_lib, contract, tol):
    d = np.load(GOLDEN)
    drytol = float(d["drytol"])
    ctx = gf.Context(0)
    ctx.set_fp_contract(bool(contract))
    worst = 0.0
    for k in range(len(d["m"])):
        m = int(d["m"][k])
        q = np.ascontiguousarray(d["q"][k][:m + 4, :m + 4])
        b = np.ascontiguousarray(d["b"][k][:m + 4, :m + 4, None])
        ctx.set_phys(0, _phys(d["method"][k], drytol, d["grav"]))
        qg = q.copy()
        dx = float(d["dx"][k])
        cfl, _ = ctx.patch_update_batch([qg], [b], dx, dx, 0.0, float(d["dt"][k]))
        got, ref = qg[2:2 + m, 2:2 + m], d["out"][k][:m, :m]
        scale = max(1.0, float(np.abs(q[2:2 + m, 2:2 + m]).max()))
        err = float(np.abs(got - ref).max()) / scale
        worst = max(worst, err)
        assert err <= tol, f"{d['name'][k]} mx={m} method={d['method'][k]}: {err:.3e}"
        assert np.array_equal(got[..., 0] > drytol, ref[..., 0] > drytol)
        cref = float(d["cfl"][k])
        assert abs(cfl[0] - cref) <= 1e-12 * max(1.0, cref)
    ctx.close()
