"""Frames and gauges written by a device forest during its run against the
oracle forest's files, byte for byte (GPU required). The contraction-free
build with friction off agrees bit for bit with the oracle, so every value
printed -- frame cells, gauge samples, times -- must print the same."""
import os

import numpy as np
import pytest

import geoflood_gb300 as gf
from oracle import forest as of

from forest_cases import DX0, FRONT, LMAX, LMIN, M, NBX, NBY, rasters

pytestmark = pytest.mark.gpu
SLOT = 8

# (id, x, y, t1, t2, min_time_increment) on the 2000 m x 1000 m domain
GAUGES = [
    (1, 612.3, 404.1, 0.0, 1e10, 0.0),        # near the front
    (2, 1000.0 - 0.7, 250.0, 0.0, 1e10, 0.0),  # last cell of a leaf: stencil on ghost cells
    (3, 450.0, 999.9, 5.0, 30.0, 3.0),         # window and minimum increment
    (4, 2000.0, 1000.0, 0.0, 1e10, 0.0),       # upper-right corner of the domain
    (5, 1500.0, 500.0, 0.0, 1e10, 2.5),
    (6, 500.0 - 0.7, 625.0 - 0.1, 0.0, 1e10, 0.0),  # wet, last column of every leaf there
    (99, -10.0, 10.0, 0.0, 1e10, 0.0),         # outside: header only
]


def files(d):
    return sorted(os.listdir(d))


def test_forest_run_frames_and_gauges_match_oracle(ctx, tmp_path):
    phys = gf.Phys(friction_forcing=False)
    ctx.set_phys(SLOT, phys)
    ctx.set_fp_contract(False)
    gdir, odir = tmp_path / "gpu", tmp_path / "oracle"
    gdir.mkdir()
    odir.mkdir()
    try:
        b, q = rasters("dambreak")
        G = gf.Forest(ctx, M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, mthbc=(3, 3, 3, 3),
                      regrid_interval=2, refine=FRONT, phys_slot=SLOT)
        O = of.Forest(M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, phys=phys, mthbc=(3, 3, 3, 3),
                      regrid_interval=2, rf=FRONT)
        G.init()
        O.init()
        # a frame of the initial leaves through the explicit call
        G.write_frame(17, str(gdir))
        O.write_frame(str(odir), 17)
        G.set_output(str(gdir), True)
        O.set_output(str(odir), True)
        G.set_gauges(GAUGES)
        O.set_gauges(GAUGES)
        st = G.run(24.0, 4, 5.0, 0.9, 1.0)
        O.run(24.0, 4, 5.0, 0.9, 1.0)
        assert (st["steps"], st["regrids"]) == (O.steps, O.regrids) and st["regrids"] > 3
        names = files(gdir)
        assert names == files(odir)
        assert {"fort.t0000", "fort.q0004", "fort.q0017", "gauge00099.txt"} <= set(names)
        for n in names:
            assert (gdir / n).read_bytes() == (odir / n).read_bytes(), n
        rows = {g[0]: (gdir / ("gauge%05d.txt" % g[0])).read_text().count("\n") - 2
                for g in GAUGES}
        assert rows[1] == rows[2] == rows[6] == st["steps"] + 1
        assert 0 < rows[3] < st["steps"] and rows[99] == 0
        G.close()
    finally:
        ctx.set_fp_contract(True)


def test_host_loop_gauge_sampling(ctx, tmp_path):
    """gf_forest_step / accept / sample / flush from a user loop: the same
    rows as the oracle sampling at the same times."""
    phys = gf.Phys(friction_forcing=False)
    ctx.set_phys(SLOT, phys)
    ctx.set_fp_contract(False)
    gdir, odir = tmp_path / "gpu", tmp_path / "oracle"
    gdir.mkdir()
    odir.mkdir()
    try:
        b, q = rasters("dambreak")
        G = gf.Forest(ctx, M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, mthbc=(3, 3, 3, 3),
                      refine=FRONT, phys_slot=SLOT)
        O = of.Forest(M, NBX, NBY, LMIN, LMAX, DX0, DX0, b, q, phys=phys, mthbc=(3, 3, 3, 3),
                      rf=FRONT)
        G.init()
        O.init()
        G.set_output(str(gdir), False)
        O.set_output(str(odir), False)
        G.set_gauges(GAUGES[:3])
        O.set_gauges(GAUGES[:3])
        t = 0.0
        for k in range(6):
            G.step(t, 0.5)
            G.accept(True)
            O.step(t, 0.5)
            t += 0.5
            G.sample_gauges(t)
            O.sample_gauges(t)
        G.flush_gauges()
        O.flush_gauges()
        for g in GAUGES[:3]:
            n = "gauge%05d.txt" % g[0]
            assert (gdir / n).read_bytes() == (odir / n).read_bytes(), n
        G.close()
    finally:
        ctx.set_fp_contract(True)
