"""Served AMR forests on the GPU (GPU required): requests admitted into the
batched forest engine by device footprint, joining and leaving between
iterations, give each forest exactly the result of its own gf_forest_run
(same leaves, same state bit for bit, same step and regrid counts)."""
from pathlib import Path

import numpy as np
import pytest

import geoflood_gb300 as gf
from geoflood_gb300.forest import footprint
from geoflood_gb300.serve import ForestRequest, ForestServer, Hydrograph
from geoflood_gb300.topo import Topo

from forest_cases import FRONT, LMAX, LMIN, NBX, NBY, rasters

pytestmark = pytest.mark.gpu
S = (slice(None), slice(2, -2), slice(2, -2))
PHYS = gf.Phys(manning_coefficient=(0.035,), manning_break=(1e10,))
HYDRO = Hydrograph(time=np.array([0.0, 30.0, 90.0]), hu=np.array([2.0, 20.0, 2.0]),
                   side=(1, 0, 0, 0), width=120.0, x0=0.0, y0=500.0)
GOLD = Path(__file__).resolve().parent / "golden" / "topo"


def request(m=8, seed=3, regrid=2, mthbc=(3, 3, 3, 3), hydro=None, t_final=30.0):
    b, q = rasters("dambreak", seed, m)
    return ForestRequest(mx=m, nbx=NBX, nby=NBY, minlevel=LMIN, maxlevel=LMAX, dx0=1000.0 / m,
                         dy0=1000.0 / m, t_final=t_final, aux=b, q=q, mthbc=mthbc,
                         regrid_interval=regrid, refine=FRONT, phys=PHYS, hydro=hydro, nout=1,
                         initial_dt=5.0)


MIX = (dict(m=8, seed=4, regrid=3), dict(m=16, seed=5, mthbc=(0, 3, 3, 3), hydro=HYDRO),
       dict(m=32, seed=6, regrid=4))


def own_run(ctx, req: ForestRequest):
    """The request run alone through gf_forest_run."""
    ctx.set_phys(5, req.phys)
    F = gf.Forest(ctx, req.mx, req.nbx, req.nby, req.minlevel, req.maxlevel, req.dx0, req.dy0,
                  req.aux, req.q, mthbc=req.mthbc, regrid_interval=req.regrid_interval,
                  refine=req.refine, phys_slot=5, subcycle=req.subcycle)
    if req.hydro is not None:
        h = req.hydro
        F.set_hydrograph(h.time, h.hu, h.side, h.width, h.x0, h.y0)
    F.init()
    st = F.run(req.t_final, req.nout, req.initial_dt, req.desired_cfl, req.max_cfl)
    out = (F.patches(), F.download(), st)
    F.close()
    return out


def pump_until(srv, cond, timeout=60.0):
    """pump() never waits on the device: pass until cond() holds."""
    t_end = srv.clock() + timeout
    while not cond():
        srv.pump()
        assert srv.clock() < t_end, "condition not reached"


def check_same(srv, sid, want):
    P, q, st = want
    info = srv.poll(sid)
    assert info["state"] == "done"
    p, qq, _ = srv.download(sid)
    assert np.array_equal(p, P)
    assert np.array_equal(qq[S], q[S])
    for k in ("steps", "rejects", "regrids", "cell_updates", "t"):
        assert info[k] == st[k], k
    assert info["npatch"] == len(P)
    assert 0 < info["device_bytes"] <= info["footprint"]


def test_mixed_requests_equal_their_own_runs(ctx):
    reqs = [request(**kw) for kw in MIX]
    want = [own_run(ctx, r) for r in reqs]
    with ForestServer() as srv:
        ids = [srv.submit(r) for r in reqs]
        srv.run_until_idle()
        for sid, w in zip(ids, want):
            check_same(srv, sid, w)
        st = srv.stats()
        assert st["done"] == 3 and st["failed"] == 0 and st["active"] == 0 and st["held"] == 3
        assert st["regrids"] == sum(srv.poll(s)["regrids"] for s in ids)
        assert st["launches"] > 0 and st["epochs"] >= 2


@pytest.mark.parametrize("lane_cells", [0, 4096, (3000, 6000)])
def test_lanes_give_the_same_results(ctx, lane_cells):
    """One lane on the context's stream, or small and large forests in two
    lanes that overlap on the device (the large lane's update on fewer
    SMs): every result equals its own run."""
    reqs = [request(**kw) for kw in MIX] + [request(m=8, seed=11, regrid=2)]
    want = [own_run(ctx, r) for r in reqs]
    with ForestServer(lane_cells=lane_cells, reserve_sms=24) as srv:
        ids = [srv.submit(r) for r in reqs]
        srv.run_until_idle()
        for sid, w in zip(ids, want):
            check_same(srv, sid, w)
        lanes = [srv.poll(s)["lane"] for s in ids]
        st = srv.stats()
        if isinstance(lane_cells, tuple):
            assert len(set(lanes)) >= 2 and sum(st["lane_admitted"][:3]) == len(ids)
        elif lane_cells:
            assert set(lanes) == {0, 1} and st["lane_admitted"] == [lanes.count(0), lanes.count(1), 0, 0]
        else:
            assert set(lanes) == {0} and st["lane_admitted"] == [len(ids), 0, 0, 0]


def test_arrivals_join_a_running_batch(ctx):
    """Requests submitted while others run: joining mid-run (and the graph
    re-captures that follow) leaves every result unchanged."""
    reqs = [request(m=8, seed=3, regrid=2, t_final=40.0), request(m=16, seed=7, regrid=3),
            request(m=8, seed=9, regrid=2, t_final=20.0)]
    want = [own_run(ctx, r) for r in reqs]
    with ForestServer() as srv:
        ids = [srv.submit(reqs[0])]
        pump_until(srv, lambda: srv.poll(ids[0])["steps"] > 0)
        assert srv.poll(ids[0])["state"] == "active"
        ids.append(srv.submit(reqs[1]))
        pump_until(srv, lambda: srv.poll(ids[1])["steps"] > 0)
        ids.append(srv.submit(reqs[2]))
        srv.run_until_idle()
        for sid, w in zip(ids, want):
            check_same(srv, sid, w)
        i = [srv.poll(s) for s in ids]
        assert i[1]["t_admit"] > i[0]["t_admit"] and i[2]["t_submit"] > i[1]["t_submit"]


def test_admission_by_budget_and_release():
    """A budget that holds one forest: the second waits, also behind a
    finished but unreleased forest, and is admitted on release."""
    r1, r2 = request(m=8, seed=3), request(m=8, seed=4)
    fp = ForestServer.footprint(r1)
    assert fp > 0 and ForestServer.footprint(r2) == fp
    with ForestServer(hbm_budget=fp + fp // 2) as srv:
        a, b = srv.submit(r1), srv.submit(r2)
        srv.pump()
        assert srv.poll(a)["state"] == "active" and srv.poll(b)["state"] == "queued"
        assert srv.stats()["bytes_in_use"] == fp
        srv.wait(a)
        for _ in range(3):
            srv.pump()
        assert srv.poll(b)["state"] == "queued" and srv.stats()["held"] == 1
        srv.release(a)
        assert srv.stats()["bytes_in_use"] == 0
        srv.wait(b)
        assert srv.poll(b)["state"] == "done"
        st = srv.stats()
        assert st["bytes_peak"] == fp and st["bytes_in_use"] == fp
        with pytest.raises(gf.GeoFloodError):
            srv.download(a)                    # released
    with ForestServer(hbm_budget=fp - 1) as srv:
        with pytest.raises(gf.GeoFloodError):
            srv.submit(r1)                     # can never fit


def test_cancel_and_refusals(ctx):
    keep = request(m=8, seed=5, regrid=2)
    want = own_run(ctx, keep)
    with ForestServer(max_active=1) as srv:
        a, b, c = srv.submit(keep), srv.submit(request(m=16, seed=6)), srv.submit(request(m=8))
        srv.cancel(c)                          # still queued
        srv.pump()
        srv.pump()
        assert srv.poll(b)["state"] == "queued"   # max_active = 1
        srv.wait(a)
        check_same(srv, a, want)
        pump_until(srv, lambda: srv.poll(b)["steps"] > 0)
        assert srv.poll(b)["state"] == "active"
        srv.cancel(b)                          # running
        pump_until(srv, lambda: srv.poll(b)["state"] != "active")
        assert srv.poll(b)["state"] == "cancelled" and srv.poll(c)["state"] == "cancelled"
        assert srv.stats()["bytes_in_use"] == srv.poll(a)["footprint"]
        bad = request()
        bad.mthbc = (0, 3, 3, 3)               # inflow without a hydrograph
        with pytest.raises(gf.GeoFloodError):
            srv.submit(bad)
        assert ForestServer.footprint(bad) == footprint(bad.opts())


def test_topo_request_and_loop_thread(ctx):
    """DEM bathymetry and still-water qinit on admission; the request loop
    on its own thread."""
    phys = gf.Phys(sea_level=30.0)
    lake = gf.Refine(wave_tolerance=1e9, regions=((250.0, 450.0, 150.0, 350.0, 0.0, 1e9, 3, 3),))
    t = Topo()
    t.read_data(str(GOLD / "topo.data"))
    req = ForestRequest(mx=8, nbx=4, nby=3, minlevel=0, maxlevel=3, dx0=25.0, dy0=25.0,
                        t_final=10.0, topo=t, qinit=True, phys=phys, refine=lake,
                        mthbc=(3, 3, 3, 3), regrid_interval=2, initial_dt=1.0)
    ctx.set_phys(5, phys)
    F = gf.Forest(ctx, 8, 4, 3, 0, 3, 25.0, 25.0, None, None, mthbc=(3, 3, 3, 3),
                  regrid_interval=2, refine=lake, phys_slot=5)
    F.set_topo(t)
    F.init()
    st = F.run(10.0, 1, 1.0, 0.9, 1.0)
    want = (F.patches(), F.download(), st)
    F.close()
    with ForestServer() as srv:
        srv.start()
        sid = srv.submit(req)
        info = srv.wait(sid, timeout=120.0)
        srv.stop()
        assert info["state"] == "done"
        check_same(srv, sid, want)


def test_subcycled_requests_run_beside_the_batched_lanes(ctx):
    """Subcycled requests (a third lane: each coarse step the forest's own
    graph, side by side) and round-sharing requests in one server: every
    result equals its own gf_forest_run; cancelling a running subcycled
    request leaves the others unchanged."""
    reqs = [request(m=8, seed=3, regrid=2), request(m=16, seed=5, regrid=3, mthbc=(0, 3, 3, 3), hydro=HYDRO),
            request(m=8, seed=9, regrid=2), request(m=32, seed=6, regrid=4)]
    reqs[0].subcycle = reqs[1].subcycle = reqs[3].subcycle = True
    want = [own_run(ctx, r) for r in reqs]
    with ForestServer(lane_cells=4096) as srv:
        ids = [srv.submit(r) for r in reqs]
        sub_extra = request(m=8, seed=11, t_final=200.0)
        sub_extra.subcycle = True
        extra = srv.submit(sub_extra)
        pump_until(srv, lambda: srv.poll(extra)["steps"] > 0)
        srv.cancel(extra)
        srv.run_until_idle()
        for sid, w in zip(ids, want):
            check_same(srv, sid, w)
        lanes = [srv.poll(s)["lane"] for s in ids]
        assert lanes[0] == lanes[1] == lanes[3] == 3 and lanes[2] in (0, 1, 2)
        assert srv.poll(extra)["state"] == "cancelled"
        st = srv.stats()
        assert st["lane_admitted"][3] == 4 and st["sub_steps"] > 0
