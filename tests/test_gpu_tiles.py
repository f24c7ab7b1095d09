"""Tile shapes of the patch kernel (GPU required): every variant of every
patch size meets the same parity bar against the oracle, and the autotuner
measures them and installs a choice per goal."""
import numpy as np
import pytest

import geoflood_gb300 as gf
from geoflood_gb300 import synth

from test_gpu_patch import compare, level_vs_oracle, random_state

pytestmark = pytest.mark.gpu


def variants(m):
    return range(gf.Context.tile_count(m))


@pytest.mark.parametrize("m", [8, 16, 32])
def test_every_tile_meets_the_parity_bar(ctx, m):
    keep = gf.Context.tile(m, 0)
    try:
        for v in variants(m):
            gf.Context.set_tile(m, 0, v)
            q, aux = random_state(24, m, 40 + v)
            out, ref, cg, cr, pg, pr = level_vs_oracle(ctx, q, aux, m, 2.0, 0.04, gf.Phys())
            compare(q, out, ref, cg, cr, m, pcfl_gpu=pg, pcfl_ref=pr)
            q, aux, _, _ = synth.uniform_dam_break_level(4, 4, m, 1.0, seed=v, x_dam=1.5 * m)
            out, ref, cg, cr, pg, pr = level_vs_oracle(ctx, q, aux, m, 1.0, 0.05, gf.Phys())
            compare(q, out, ref, cg, cr, m, pcfl_gpu=pg, pcfl_ref=pr)
    finally:
        gf.Context.set_tile(m, 0, keep)


@pytest.mark.parametrize("m", [8, 16, 32])
def test_tile_shapes_give_the_same_bits(ctx, m):
    """Threads per patch, slices per band and the split of one patch over a
    thread-block cluster change the work split, not the sums: every
    variant's step equals variant 0's bit for bit."""
    keep = gf.Context.tile(m, 0)
    outs = []
    try:
        for v in variants(m):
            gf.Context.set_tile(m, 0, v)
            q, aux, _, _ = synth.uniform_dam_break_level(4, 4, m, 1.0, seed=7, x_dam=1.5 * m)
            out, _, cg, _, pg, _ = level_vs_oracle(ctx, q, aux, m, 1.0, 0.05, gf.Phys())
            outs.append((out, cg, pg))
    finally:
        gf.Context.set_tile(m, 0, keep)
    for out, cg, pg in outs[1:]:
        assert np.array_equal(out, outs[0][0]) and cg == outs[0][1]
        assert np.array_equal(pg, outs[0][2])


def test_autotune_measures_and_selects(ctx):
    ctx.set_phys(0, gf.Phys())
    res = ctx.autotune(reps=2)
    assert [r["mx"] for r in res] == [8, 16, 32]
    for r in res:
        assert len(r["tiles"]) == len(variants(r["mx"]))
        assert all(v > 0 for v in r["throughput"]) and all(v > 0 for v in r["latency_us"])
        assert r["best_throughput"] == int(np.argmax(r["throughput"]))
        assert r["best_latency"] == int(np.argmin(r["latency_us"]))
        assert gf.Context.tile(r["mx"], 0) == r["best_throughput"]
        assert gf.Context.tile(r["mx"], 1) == r["best_latency"]
    with pytest.raises(gf.GeoFloodError):
        gf.Context.set_tile(8, 0, 9)


@pytest.mark.parametrize("m", [8, 16, 32])
def test_small_host_batches_take_the_latency_tile_with_the_same_bits(ctx, m):
    """gf_patch_update_batch on a handful of patches runs the latency
    choice (a patch split over a cluster for the window tiles): every
    variant installed there gives the bits of the one-CTA kernel."""
    keep = gf.Context.tile(m, 1)
    q, aux, _, _ = synth.uniform_dam_break_level(2, 2, m, 1.0, seed=5, x_dam=1.0 * m)
    outs = []
    try:
        for v in variants(m):
            gf.Context.set_tile(m, 1, v)
            qs = [np.array(q[k]) for k in range(4)]
            cfl, mc = ctx.patch_update_batch(qs, [np.ascontiguousarray(aux[k]) for k in range(4)],
                                             1.0, 1.0, 0.0, 0.05)
            outs.append((np.stack(qs), cfl, mc))
    finally:
        gf.Context.set_tile(m, 1, keep)
    for out, cfl, mc in outs[1:]:
        assert np.array_equal(out, outs[0][0])
        assert np.array_equal(cfl, outs[0][1]) and mc == outs[0][2]
