"""Host side of the served form (no GPU): scenario footprint through the C
ABI, the generator, and the oracle's outstyle-1 driver."""
import ctypes as C

import numpy as np

import geoflood_gb300 as gf
import oracle
from geoflood_gb300 import _lib, synth


def test_footprint_counts_two_state_buffers_aux_layout_and_flags():
    sc = synth.flood_scenario(5, 2048, mx=16)
    s, _ = sc.to_c(None)
    lib = _lib.load()
    S = (sc.mx + 4) ** 2
    n = sc.npx * sc.npy

    def a256(b):
        return (b + 255) // 256 * 256
    # two state buffers, aux, neighbour table, geometry, dry-patch flags
    want = 2 * a256(n * 3 * S * 8) + a256(n * 1 * S * 8) + a256(n * 32) + a256(n * 32) + a256(n * 4)
    assert lib.gf_scenario_footprint(C.byref(s)) == want
    s.mx = 12
    assert lib.gf_scenario_footprint(C.byref(s)) == 0
    s.mx = 16
    s.mthbc[0] = 0
    s.nhydro = 0
    assert lib.gf_scenario_footprint(C.byref(s)) == 0   # inflow side without a hydrograph


def test_generator_shapes_and_ranges():
    for seed in range(6):
        sc = synth.flood_scenario(seed, 20000, time_scale=1.0)
        assert sc.mx in (8, 16, 32)
        assert 0.5 * 20000 <= sc.cells <= 2.0 * 20000
        assert 3600.0 <= sc.t_final <= 6 * 3600.0
        assert 0.02 <= sc.phys.manning_coefficient[0] <= 0.08
        peak = sc.hydro.hu.max() * sc.hydro.width
        assert 10.0 <= peak <= 500.0
        assert sc.q.shape == (sc.npx * sc.npy, sc.mx + 4, sc.mx + 4, 3)
        assert sc.aux.shape[:3] == sc.q.shape[:3]


def test_oracle_outstyle1_lands_on_output_times_and_keeps_a_lake():
    m, npx, npy = 8, 3, 2
    b = synth.fractal_dem(npx * m, npy * m, 1.0, 0.8, 4.0, 3)
    q = np.zeros(b.shape + (3,))
    q[..., 0] = np.maximum(3.0 - b, 0.0)
    qt = synth.tile_level(synth.pad_extrap(q), m)
    at = synth.tile_level(synth.pad_extrap(b[..., None]), m)
    steps, rejects, dts = oracle.run_scenario(qt, at, m, npx, npy, 1.0, 1.0, 5.0, 3, 0.5, 0.9,
                                              1.0, (3, 3, 3, 3))
    assert steps > 3
    assert abs(sum(dts) - 5.0) <= 1e-12
    s = (slice(None), slice(2, -2), slice(2, -2))
    assert np.abs(qt[s][..., 1:]).max() <= 1e-12      # round-off of eta = h + b
    eta = qt[s][..., 0] + at[s][..., 0]
    wet = qt[s][..., 0] > 1e-3
    assert np.allclose(eta[wet], 3.0, rtol=0, atol=1e-12)


def test_server_option_defaults():
    """Defaults of gf_server_opts_default as the C ABI fills them: three size
    lanes, priority streams, per-size round queues, dry-patch culling, one
    CTA per patch (no reserved SMs), the per-size updates."""
    lib = _lib.load()
    o = _lib.gf_server_opts()
    lib.gf_server_opts_default(C.byref(o))
    assert o.nlanes == 3 and list(o.lane_cells)[:2] == [100000, 1000000]
    assert o.priority == 1 and o.backfill == 1
    assert o.split_sizes == 1 and o.cull_dry == 1
    assert o.reserve_sms == 0 and o.mixed_update == 0
    assert 1 <= o.max_active <= 1024 and o.hbm_budget > 0
