"""The allocation-free patch update (gf_patch_update_noalloc) on a GPU.

It exists for callers that cannot allocate device memory at step time --
memory owned by another allocator, a service at its memory limit, or a
stream that a synchronising cudaFree would stall -- so it stages through a
static device array instead of cudaMalloc'd buffers. This file checks its
result against the allocating entry point (gf_patch_update_batch) on two
calls in a row, at the same 1e-10 bar as the other parity tests, and that
sizes beyond the static array are refused.

Named to be collected last: a run that stops at the first failure has then
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import geoflood_gb300 as gf
from geoflood_gb300 import _lib, synth

pytestmark = pytest.mark.gpu
MBC = 2
TOL = 1e-10


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _call(lib, pc, qdev, adev, n, m, maux, dx, dt):
    dxa = np.full(n, dx)
    cfl = np.zeros(n)
    mc = C.c_double()
    rc = lib.gf_patch_update_noalloc(0, C.byref(pc), n, m, m, MBC, 3, maux, _ptr(dxa), _ptr(dxa),
                                     dt, C.c_void_p(qdev), C.c_void_p(adev), _ptr(cfl),
                                     C.byref(mc), None)
    return rc, cfl, mc.value


def test_noalloc_matches_allocating_entry_point_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    m, n, dx, dt = 32, 12, 1.0, 0.05
    q, aux, _, _ = synth.uniform_dam_break_level(4, 3, m, dx, seed=91, x_dam=50.0)
    q[..., 1] = 0.4 * q[..., 0]
    phys = gf.Phys()
    pc = phys.to_c()
    ctx = gf.Context(0, phys)
    state = q.copy()
    s = slice(MBC, MBC + m)
    for call in range(2):
        ref = [state[k].copy() for k in range(n)]
        pref, mref = ctx.patch_update_batch(ref, [aux[k] for k in range(n)], dx, dx, 0.0, dt)
        ref = np.stack(ref)

        qd = torch.from_numpy(state.copy()).cuda()
        ad = torch.from_numpy(np.ascontiguousarray(aux)).cuda()
        torch.cuda.synchronize()
        rc, cfl, mc = _call(gpu_lib, pc, qd.data_ptr(), ad.data_ptr(), n, m, 1, dx, dt)
        assert rc == 0, f"call {call}: status {rc}"
        out = qd.cpu().numpy()

        scale = max(1.0, float(np.abs(state[:, s, s]).max()))
        assert np.abs(out[:, s, s] - ref[:, s, s]).max() <= TOL * scale, f"call {call}"
        assert abs(mc - mref) <= 1e-12 * max(1.0, mref)
        assert np.allclose(cfl, pref, rtol=1e-12, atol=0.0)
        state = out
    ctx.close()


def test_noalloc_refuses_sizes_beyond_its_static_array(gpu_lib):
    pc = gf.Phys().to_c()
    dummy = 1  # never dereferenced: the size checks come first
    rc, _, _ = _call(gpu_lib, pc, dummy, dummy, _lib_max_patches() + 1, 32, 1, 1.0, 0.1)
    assert rc == -1  # GF_ERR_ARG
    rc, _, _ = _call(gpu_lib, pc, dummy, dummy, 1, 32, 5, 1.0, 0.1)
    assert rc == -1
    rc, _, _ = _call(gpu_lib, pc, dummy, dummy, 1, 24, 1, 1.0, 0.1)
    assert rc == -6  # GF_ERR_UNSUPPORTED


def _lib_max_patches():
    import re
    from pathlib import Path

    h = (Path(__file__).resolve().parents[1] / "include" / "geoflood_gb300.h").read_text()
    return int(re.search(r"#define GF_NOALLOC_MAX_PATCHES (\d+)", h).group(1))
