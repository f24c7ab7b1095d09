"""The allocation-free patch update (gf_patch_update_noalloc) on a GPU.

It exists for callers that cannot allocate device memory at step time --
memory owned by another allocator, a service at its memory limit, or a
stream that a synchronising cudaFree would stall -- so it stages through a
static device array instead of cudaMalloc'd buffers. This file checks its
result against the allocating entry point (gf_patch_update_batch) on two
calls in a row, at the same 1e-10 bar as the other parity tests, over every
patch size, one and the largest number of patches, one aux field and the
largest number (a Manning field among them), on the legacy stream and on a
side stream; that the device's free memory is the same before and after a
call; and that sizes beyond the static array and unusable physics are
refused before any device memory is touched.

Named to be collected last: a run that stops at the first failure has then
already run every other test.
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import geoflood_gb300 as gf
from geoflood_gb300 import synth

pytestmark = pytest.mark.gpu
MBC = 2
TOL = 1e-10


def _header_define(name):
    h = (Path(__file__).resolve().parents[1] / "include" / "geoflood_gb300.h").read_text()
    return int(re.search(rf"#define {name} (\d+)", h).group(1))


MAX_PATCHES = _header_define("GF_NOALLOC_MAX_PATCHES")
MAX_MAUX = _header_define("GF_NOALLOC_MAX_MAUX")


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _call(lib, pc, qdev, adev, n, m, maux, dx, dt, stream=None):
    dxa = np.full(n, dx)
    cfl = np.zeros(n)
    mc = C.c_double()
    rc = lib.gf_patch_update_noalloc(0, C.byref(pc), n, m, m, MBC, 3, maux, _ptr(dxa), _ptr(dxa),
                                     dt, C.c_void_p(qdev), C.c_void_p(adev), _ptr(cfl),
                                     C.byref(mc), stream)
    return rc, cfl, mc.value


def _case(m, n, maux):
    """A wet/dry dam break over n patches of m x m cells; with maux > 1 a
    Manning field lies in aux field 2 and the physics reads it."""
    npx = n if n < 4 else 4
    npy = max(1, n // npx)
    assert npx * npy == n
    dx = 32.0 / m
    q, b, _, _ = synth.uniform_dam_break_level(npx, npy, m, dx, seed=91 + m + n,
                                               x_dam=0.45 * npx * m * dx)
    q = np.array(q)
    q[..., 1] = 0.4 * q[..., 0]
    q[..., 2] = -0.1 * q[..., 0]
    rng = np.random.default_rng(5 * m + n)
    aux = np.zeros(b.shape[:3] + (maux,))
    aux[..., 0] = b[..., 0]
    for f in range(1, maux):
        aux[..., f] = rng.uniform(0.02, 0.08, aux.shape[:3])
    phys = gf.Phys()
    if maux > 1:
        phys = gf.Phys(variable_friction=True, friction_index=2)
    return q, aux, phys, dx


@pytest.mark.parametrize("m", [8, 16, 32])
@pytest.mark.parametrize("n", [1, MAX_PATCHES])
@pytest.mark.parametrize("maux", [1, MAX_MAUX])
def test_noalloc_matches_allocating_entry_point_twice(gpu_lib, m, n, maux):
    torch = pytest.importorskip("torch")
    q, aux, phys, dx = _case(m, n, maux)
    dt = 0.2 * dx / 10.0
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
        free_before = torch.cuda.mem_get_info()[0]
        rc, cfl, mc = _call(gpu_lib, pc, qd.data_ptr(), ad.data_ptr(), n, m, maux, dx, dt)
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == 0, f"call {call}: status {rc}"
        if call == 1:  # the first call may load kernels lazily; later ones allocate nothing
            assert free_after == free_before, f"device memory changed by {free_before - free_after} B"
        out = qd.cpu().numpy()

        scale = max(1.0, float(np.abs(state[:, s, s]).max()))
        assert np.abs(out[:, s, s] - ref[:, s, s]).max() <= TOL * scale, f"call {call}"
        assert abs(mc - mref) <= 1e-12 * max(1.0, mref)
        assert np.allclose(cfl, pref, rtol=1e-12, atol=0.0)
        state = out
    ctx.close()


def test_noalloc_on_a_side_stream(gpu_lib):
    torch = pytest.importorskip("torch")
    m, n, maux = 16, 4, 1
    q, aux, phys, dx = _case(m, n, maux)
    dt = 0.02
    ctx = gf.Context(0, phys)
    ref = [q[k].copy() for k in range(n)]
    _, mref = ctx.patch_update_batch(ref, [aux[k] for k in range(n)], dx, dx, 0.0, dt)
    ctx.close()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        qd = torch.from_numpy(q.copy()).cuda()
        ad = torch.from_numpy(np.ascontiguousarray(aux)).cuda()
    side.synchronize()
    rc, _, mc = _call(gpu_lib, phys.to_c(), qd.data_ptr(), ad.data_ptr(), n, m, maux, dx, dt,
                      stream=C.c_void_p(side.cuda_stream))
    assert rc == 0
    out = qd.cpu().numpy()
    s = slice(MBC, MBC + m)
    scale = max(1.0, float(np.abs(q[:, s, s]).max()))
    assert np.abs(out[:, s, s] - np.stack(ref)[:, s, s]).max() <= TOL * scale
    assert abs(mc - mref) <= 1e-12 * max(1.0, mref)


def test_noalloc_refuses_before_touching_device_memory(gpu_lib):
    pc = gf.Phys().to_c()
    dummy = 1  # never dereferenced: every check below comes before any device access
    assert _call(gpu_lib, pc, dummy, dummy, MAX_PATCHES + 1, 32, 1, 1.0, 0.1)[0] == -1  # GF_ERR_ARG
    assert _call(gpu_lib, pc, dummy, dummy, 1, 32, MAX_MAUX + 1, 1.0, 0.1)[0] == -1
    assert _call(gpu_lib, pc, dummy, dummy, 1, 24, 1, 1.0, 0.1)[0] == -6  # GF_ERR_UNSUPPORTED
    # variable friction reading an aux field past the ones passed
    bad = gf.Phys(variable_friction=True, friction_index=3).to_c()
    assert _call(gpu_lib, bad, dummy, dummy, 1, 32, 2, 1.0, 0.1)[0] == -1
    bad = gf.Phys(variable_friction=True, friction_index=0).to_c()
    assert _call(gpu_lib, bad, dummy, dummy, 1, 32, 2, 1.0, 0.1)[0] == -1
    bad = gf.Phys().to_c()
    bad.num_manning = 9
    assert _call(gpu_lib, bad, dummy, dummy, 1, 32, 1, 1.0, 0.1)[0] == -1
