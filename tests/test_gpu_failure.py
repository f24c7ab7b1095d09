"""Failure detection on the GPU without a fault (GPU required): the bounded
device wait that every patch kernel uses gives up on a barrier phase that
nothing completes, reports it to the host, and leaves the context usable."""
import ctypes as C

import pytest

import geoflood_gb300 as gf
from geoflood_gb300 import _lib

from test_gpu_patch import compare, level_vs_oracle, random_state

pytestmark = pytest.mark.gpu


def probe(arrive, iters):
    t, ms = C.c_int(-1), C.c_double(0.0)
    rc = _lib.load().gf_probe_bounded_wait(0, int(arrive), int(iters), C.byref(t), C.byref(ms))
    assert rc == 0
    return t.value, ms.value


@pytest.mark.parametrize("iters", [1 << 10, 1 << 14])
def test_wait_nothing_completes_times_out_and_returns(ctx, iters):
    timed_out, ms = probe(0, iters)
    assert timed_out == 1 and ms < 10_000.0
    assert probe(1, iters)[0] == 0          # the same wait with the arrival succeeds
    # the context still works: a level step afterwards meets the parity bar
    q, aux = random_state(8, 16, 3)
    out, ref, cg, cr, pg, pr = level_vs_oracle(ctx, q, aux, 16, 2.0, 0.04, gf.Phys())
    compare(q, out, ref, cg, cr, 16, pcfl_gpu=pg, pcfl_ref=pr)
