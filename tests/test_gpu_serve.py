"""Served form on the GPU: scenarios through the continuous-batching server
against the oracle's outstyle-1 run, and each result the same alone and in a
mix (GPU required)."""
import numpy as np
import pytest

import geoflood_gb300 as gf
import oracle
from geoflood_gb300 import synth

pytestmark = pytest.mark.gpu

# 3.6 s of simulated time per hour of horizon: tens of steps at dx = 5 m
TS = 1.0 / 1000.0


def scen(seed, cells, mx, ts=TS):
    return synth.flood_scenario(seed, cells, mx=mx, time_scale=ts)


def oracle_run(sc):
    q = sc.q.copy()
    h = sc.hydro
    hy = oracle.hydro(h.time, h.hu, h.side, h.width, h.x0, h.y0)
    steps, rejects, dts = oracle.run_scenario(
        q, sc.aux, sc.mx, sc.npx, sc.npy, sc.dx, sc.dy, sc.t_final, sc.nout, sc.initial_dt,
        sc.desired_cfl, sc.max_cfl, sc.mthbc, sc.phys, hy, sc.xlower, sc.ylower)
    return q, steps, rejects, dts


def interior(q):
    return q[:, 2:-2, 2:-2, :]


def serve_alone(sc, **kw):
    with gf.Server(**kw) as srv:
        out = np.zeros_like(sc.q)
        sid = srv.submit(sc, out)
        info = srv.wait(sid, timeout=300)
        assert info["state"] == "done"
        return out, info


@pytest.mark.parametrize("mx,cells", [(8, 1500), (16, 2048), (32, 4096)])
def test_served_scenario_matches_oracle_run(mx, cells):
    sc = scen(11 + mx, cells, mx)
    out, info = serve_alone(sc)
    ref, steps, rejects, dts = oracle_run(sc)
    assert info["steps"] == steps and info["rejects"] == rejects
    assert steps >= 10
    assert abs(info["t"] - sum(dts)) <= 1e-12 * sc.t_final
    assert info["cell_updates"] == steps * sc.cells
    scale = max(float(np.max(sc.q[..., 0])), 1.0)
    d = np.abs(interior(out) - interior(ref)).max(axis=(0, 1, 2))
    # tens of steps of the FMA build against the contraction-free oracle
    assert np.all(d <= 1e-9 * scale), d
    hg, hr = interior(out)[..., 0], interior(ref)[..., 0]
    assert np.array_equal(hg > sc.phys.dry_tolerance, hr > sc.phys.dry_tolerance)
    mass_g, mass_r = hg.sum(), hr.sum()
    assert abs(mass_g - mass_r) <= 1e-11 * mass_r


@pytest.mark.parametrize("lanes,split", [((100_000, 1_000_000), True), ((), True), ((), False)])
def test_result_is_the_same_alone_and_in_the_mix(lanes, split):
    """Bitwise: a scenario's result does not depend on what shares its launches,
    with one round queue per patch size or the sizes as branches of one
    queue's rounds."""
    a = scen(21, 1200, 8)
    b = scen(22, 4096, 16)
    c = scen(23, 9000, 32)
    alone, info_a = serve_alone(a, lanes=lanes)
    with gf.Server(lanes=lanes, split_sizes=split) as srv:
        outs = {k: np.zeros_like(s.q) for k, s in (("a", a), ("b", b), ("c", c))}
        ids = {"b": srv.submit(b, outs["b"]), "a": srv.submit(a, outs["a"]),
               "c": srv.submit(c, outs["c"])}
        srv.run_until_idle()
        infos = {k: srv.poll(v) for k, v in ids.items()}
    assert all(i["state"] == "done" for i in infos.values())
    assert np.array_equal(outs["a"], alone)
    assert infos["a"]["steps"] == info_a["steps"] and infos["a"]["rejects"] == info_a["rejects"]
    b_alone, _ = serve_alone(b, lanes=lanes)
    assert np.array_equal(outs["b"], b_alone)


@pytest.mark.parametrize("reserve_sms", [0, 24])
def test_one_launch_update_of_later_lanes_gives_the_same_bits(reserve_sms):
    """Lanes after the first update every patch size in one persistent launch,
    or per size (one CTA per patch, or a grid capped to leave reserve_sms
    SMs): every form and each scenario alone give the same bits."""
    scs = [scen(31, 1200, 8), scen(32, 4096, 16), scen(33, 9000, 32), scen(34, 3000, 8)]
    runs = []
    for mixed in (True, False):
        with gf.Server(lanes=(1000,), mixed_update=mixed, reserve_sms=reserve_sms) as srv:
            outs = [np.zeros_like(s.q) for s in scs]
            ids = [srv.submit(s, o) for s, o in zip(scs, outs)]
            srv.run_until_idle()
            infos = [srv.poll(i) for i in ids]
        assert all(i["state"] == "done" for i in infos)
        assert {i["lane"] for i in infos} == {1}
        runs.append((outs, [i["steps"] for i in infos]))
    for a, b in zip(runs[0][0], runs[1][0]):
        assert np.array_equal(a, b)
    assert runs[0][1] == runs[1][1]
    alone, _ = serve_alone(scs[2], lanes=(1000,))
    assert np.array_equal(runs[0][0][2], alone)


def test_admission_waits_for_hbm_budget():
    a = scen(31, 2048, 16)
    b = scen(32, 2048, 16)
    fa, fb = gf.Server.footprint(a), gf.Server.footprint(b)
    assert fa > 0 and fb > 0
    with gf.Server(hbm_budget=max(fa, fb) + 1024) as srv:
        ia, ib = srv.submit(a, np.zeros_like(a.q)), srv.submit(b, np.zeros_like(b.q))
        srv.run_until_idle()
        pa, pb = srv.poll(ia), srv.poll(ib)
        assert pa["state"] == pb["state"] == "done"
        assert pb["t_admit"] >= pa["t_done"]          # b waited for a's memory
        st = srv.stats()
        assert st["bytes_in_use"] == 0 and st["bytes_peak"] <= max(fa, fb) + 1024
        big = scen(33, 40000, 32)
        with pytest.raises(gf.GeoFloodError):
            srv.submit(big)                             # can never fit


def test_cancel_and_background_loop():
    long_sc = scen(41, 4096, 32, ts=1.0 / 200.0)
    short = [scen(42 + k, 1500, 8) for k in range(3)]
    with gf.Server() as srv:
        srv.start()
        lid = srv.submit(long_sc)
        sids = [srv.submit(s, np.zeros_like(s.q)) for s in short]
        infos = [srv.wait(s, timeout=300) for s in sids]
        assert all(i["state"] == "done" for i in infos)
        srv.cancel(lid)
        info = srv.wait(lid, timeout=60)
        assert info["state"] in ("cancelled", "done")
        srv.stop()
        assert srv.stats()["bytes_in_use"] == 0
    # the background loop gives the same bits as the pumped loop
    ref, _ = serve_alone(short[0])
    with gf.Server() as srv:
        srv.start()
        out = np.zeros_like(short[0].q)
        srv.wait(srv.submit(short[0], out), timeout=300)
        srv.stop()
    assert np.array_equal(out, ref)


def test_submit_rejects_bad_scenarios():
    sc = scen(51, 1500, 8)
    with gf.Server() as srv:
        for bad in (dict(mx=12), dict(t_final=0.0), dict(mthbc=(0, 1, 3, 3), hydro=None),
                    dict(mthbc=(2, 2, 3, 3))):
            kw = dict(sc.__dict__)
            kw.update(bad)
            with pytest.raises((gf.GeoFloodError, ValueError)):
                srv.submit(gf.Scenario(**kw))


@pytest.mark.parametrize("mx", [8, 16, 32])
def test_dry_patch_culling_gives_the_same_interior(mx):
    """A valley mostly dry at the start, its channel fed by the hydrograph:
    with the dry-patch culling on (the default) the run takes the same steps
    and ends in the same interior bits as with every patch updated every
    step."""
    sc = scen(77 + mx, 40000, mx, ts=1.0 / 100.0)
    on, info_on = serve_alone(sc)
    off, info_off = serve_alone(sc, cull_dry=False)
    assert (info_on["steps"], info_on["rejects"]) == (info_off["steps"], info_off["rejects"])
    assert info_on["t"] == info_off["t"]
    assert np.array_equal(interior(on), interior(off))
    wet = interior(on)[..., 0] > sc.phys.dry_tolerance
    assert 0.0 < wet.mean() < 0.5  # water arrived, and most of the valley stayed dry
