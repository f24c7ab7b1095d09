"""The buffered per-patch hook (gf_step_buffer_update) on a GPU.

ForestClaw's level step hands patches one at a time; the reference's GPU
build (cudaclaw_update, src/fc2d_cpu_cuda/fc2d_cpucuda.cpp:410-495) records
them and updates every buffer_len of them in one batch. The hook here must
give the same bits as one gf_patch_update_batch over the same patches, return
the largest CFL of each flush (0 from the other calls) and refuse an iter out
of sequence.
"""
import numpy as np
import pytest

import geoflood_gb300 as gf
from geoflood_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,buffer_len", [(32, 16), (16, 7), (8, 1024)])
def test_buffered_hook_equals_one_batch(gpu_lib, m, buffer_len):
    dx = 64.0 / m
    q, aux, _, _ = synth.uniform_dam_break_level(8, 5, m, dx, seed=17, x_dam=4 * m * dx)
    n = q.shape[0]
    dt = 0.15 * dx / 10.0
    ctx = gf.Context(0)
    ref = [np.array(q[k]) for k in range(n)]
    pcfl, mref = ctx.patch_update_batch(ref, [np.ascontiguousarray(aux[k]) for k in range(n)],
                                        dx, dx, 0.0, dt)
    buf = gf.StepBuffer(ctx, buffer_len)
    qs = [np.array(q[k]) for k in range(n)]
    auxs = [np.ascontiguousarray(aux[k]) for k in range(n)]
    rets = [buf.update(k, n, qs[k], auxs[k], dx, dx, 0.0, dt) for k in range(n)]
    for k in range(n):
        assert np.array_equal(qs[k], ref[k]), f"patch {k}"
    flushes = [k for k in range(n) if (k + 1) % buffer_len == 0 or k + 1 == n]
    for k in range(n):
        if k not in flushes:
            assert rets[k] == 0.0
    assert max(rets) == mref
    lo = 0
    for k in flushes:
        assert rets[k] == pcfl[lo:k + 1].max()
        lo = k + 1
    buf.close()
    ctx.close()


def test_buffered_hook_refuses_iter_out_of_sequence(gpu_lib):
    q, aux, _, _ = synth.uniform_dam_break_level(2, 1, 16, 2.0, seed=3, x_dam=20.0)
    ctx = gf.Context(0)
    buf = gf.StepBuffer(ctx, 4)
    qs = [np.array(q[k]) for k in range(2)]
    auxs = [np.ascontiguousarray(aux[k]) for k in range(2)]
    buf.update(0, 3, qs[0], auxs[0], 2.0, 2.0, 0.0, 0.01)
    with pytest.raises(gf.GeoFloodError) as e:
        buf.update(2, 3, qs[1], auxs[1], 2.0, 2.0, 0.0, 0.01)
    assert e.value.status == -5  # GF_ERR_STATE
    buf.close()
    ctx.close()
