"""Output formats on the CPU: the oracle's restatement of the reference's
frame and gauge writers against fixtures that the reference's own Python
readers parsed (tests/golden/make_output_golden.py), and the library's
host-side writers, gauge interpolation and gauges.data reader against the
oracle, byte for byte / bit for bit. No GPU is used."""
import json
import os
from pathlib import Path

import numpy as np
import pytest

from oracle import output as oo

GOLD = Path(__file__).resolve().parent / "golden" / "output"


def inputs():
    d = np.load(GOLD / "inputs.npz")
    return {k: d[k] for k in d.files}


def big(d):
    q = d["q"].copy()
    q[2, 4, 4, 2] = 1.5e150
    return q


def frame_args(d, q=None):
    return (d["q"] if q is None else q, d["aux"], d["level"], d["block"], d["xlower"],
            d["ylower"], d["dx"], d["dy"])


def r16(v):
    """v as an E26.16 field carries it: 16 significant digits (0 below 1e-99)."""
    v = float(v)
    return 0.0 if abs(v) < 1e-99 else float("%.15e" % v)


@pytest.mark.parametrize("x,w,d,text", [
    (1.0, 24, 16, "  0.1000000000000000E+01"),
    (-0.5, 24, 16, " -0.5000000000000000E+00"),
    (0.0, 26, 16, "    0.0000000000000000E+00"),
    (1e100, 24, 16, "  0.1000000000000000+101"),     # three-digit exponent: no E
    (1.5e-120, 26, 16, "    0.1500000000000000-119"),
    (123.456, 26, 16, "    0.1234560000000000E+03"),
    (0.1, 30, 20, "    0.10000000000000000555E+00"),  # the double nearest 0.1
    (9.9999999999999999e4, 26, 16, "    0.1000000000000000E+06"),
])
def test_fortran_e_edit_descriptor(x, w, d, text):
    """Ew.d per the Fortran standard: 0.d1..dd, exponent E+xx, or +xxx
    without the E beyond 99."""
    assert oo.fort_e(x, w, d) == text


def test_oracle_writers_reproduce_fixtures(tmp_path):
    d = inputs()
    oo.write_frame(str(tmp_path), 3, float(d["time"]), *frame_args(d))
    oo.write_frame(str(tmp_path), 4, float(d["time"]), *frame_args(d, big(d)))
    for name in ("fort.t0003", "fort.q0003", "fort.t0004", "fort.q0004"):
        assert (tmp_path / name).read_bytes() == (GOLD / name).read_bytes(), name
    g = d["gauges"][0]
    text = oo.gauge_header(7, g[1], g[2]) + oo.gauge_rows([tuple(r) for r in d["grows"]])
    assert text == (GOLD / "gauge00007.txt").read_text()


def test_reference_readers_read_back_the_values():
    """parsed.json holds what the reference's readers made of the fixture
    files: every field equals the written value at the format's precision."""
    d = inputs()
    p = json.loads((GOLD / "parsed.json").read_text())
    assert (p["num_eqn"], p["nstates"], p["num_aux"], p["num_dim"], p["num_ghost"]) == (4, 3, 1, 2, 2)
    assert p["t"] == float("%.19e" % float(d["time"]))
    for k, P in enumerate(p["patches"]):
        assert (P["patch_index"], P["level"], P["block_number"], P["mpi_rank"]) == (
            k, int(d["level"][k]), int(d["block"][k]), 0)
        assert P["num_cells"] == [8, 8]
        assert P["lower"] == [r16(d["xlower"][k]), r16(d["ylower"][k])]
        # the reader's Dimension keeps (lower, lower + n * delta, n) and
        # recomputes delta from them
        lo = (r16(d["xlower"][k]), r16(d["ylower"][k]))
        dd = (r16(d["dx"][k]), r16(d["dy"][k]))
        assert P["delta"] == [((lo[i] + 8 * dd[i]) - lo[i]) / 8 for i in range(2)]
        q = np.array(P["q"])                                  # (4, mx, my) as q[m, i, j]
        inner = d["q"][k, 2:-2, 2:-2]                         # (j, i, m)
        for m in range(3):
            want = np.vectorize(r16)(inner[..., m]).T
            assert np.array_equal(q[m], want), (k, m)
        h = np.vectorize(lambda v: 0.0 if abs(v) < 1e-99 else v)(inner[..., 0])
        eta = np.vectorize(r16)(h + d["aux"][k, 2:-2, 2:-2, 0]).T
        assert np.array_equal(q[3], eta), k
    G = p["gauge"]
    g = d["gauges"][0]
    assert G["id"] == 7 and G["location"] == [float("%.10e" % g[1]), float("%.10e" % g[2])]
    rows = d["grows"]
    assert G["level"] == [int(v) for v in rows[:, 0]]
    assert G["t"] == [float("%.7e" % v) for v in rows[:, 1]]
    eta = [0.0 if abs(r[2] + r[5]) < 1e-99 else r[2] + r[5] for r in rows]
    for m, col in enumerate((rows[:, 2], rows[:, 3], rows[:, 4], eta)):
        assert G["q"][m] == [float("%.7e" % v) for v in col], m


def test_native_frame_writer_matches_oracle_bytes(gpu_lib, tmp_path):
    from geoflood_gb300 import output as go

    d = inputs()
    args = dict(level=d["level"], xlower=d["xlower"], ylower=d["ylower"], dx=d["dx"],
                dy=d["dy"], block=d["block"])
    go.write_ascii_frame(str(tmp_path), 3, float(d["time"]), d["q"], d["aux"], **args)
    go.write_ascii_frame(str(tmp_path), 10004, float(d["time"]), big(d), d["aux"], **args)
    for name in ("fort.t0003", "fort.q0003", "fort.t0004", "fort.q0004"):
        assert (tmp_path / name).read_bytes() == (GOLD / name).read_bytes(), name


def test_native_frame_writer_random_values(gpu_lib, tmp_path):
    """Random magnitudes 1e-300..1e300 with ties-prone decimals: native == oracle."""
    from geoflood_gb300 import output as go

    rng = np.random.default_rng(11)
    n, m = 4, 16
    q = rng.standard_normal((n, m + 4, m + 4, 3)) * 10.0 ** rng.integers(-300, 300, (n, m + 4, m + 4, 3))
    q[0, 2:6, 2:6, 0] = np.array([0.5, 0.25, 0.125, 1e-99]).reshape(1, 4)  # exact decimals
    aux = rng.standard_normal((n, m + 4, m + 4, 3)) * 1e3
    lv, bk = [0, 1, 2, 3], [0, 1, 2, 3]
    xl, yl = rng.uniform(-1e6, 1e6, n), rng.uniform(-1e6, 1e6, n)
    dx = dy = 1000.0 / m / 2.0 ** np.arange(n)
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    go.write_ascii_frame(str(tmp_path / "a"), 9, 1e-310, q, aux, lv, xl, yl, dx, dy, block=bk)
    oo.write_frame(str(tmp_path / "b"), 9, 1e-310, q, aux, lv, bk, xl, yl, dx, dy)
    for name in ("fort.t0009", "fort.q0009"):
        assert (tmp_path / "a" / name).read_bytes() == (tmp_path / "b" / name).read_bytes()


def test_native_gauge_files_match_oracle(gpu_lib, tmp_path):
    from geoflood_gb300 import output as go

    d = inputs()
    g = d["gauges"][0]
    go.write_gauge_header(str(tmp_path), 7, g[1], g[2])
    go.write_gauge_rows(str(tmp_path), 7, [tuple(r) for r in d["grows"][:2]])
    go.write_gauge_rows(str(tmp_path), 7, [tuple(r) for r in d["grows"][2:]])
    assert (tmp_path / "gauge00007.txt").read_bytes() == (GOLD / "gauge00007.txt").read_bytes()


def test_gauges_data_readers(gpu_lib):
    """gauges.data written by the reference's GaugeData writer: the native
    and oracle readers return the gauges at the writer's precision."""
    from geoflood_gb300 import output as go

    d = inputs()
    want = [(int(g[0]), float("%.10e" % g[1]), float("%.10e" % g[2]), float("%.6e" % g[3]),
             float("%.6e" % g[4]), float(g[5])) for g in d["gauges"]]
    assert go.read_gauges_data(str(GOLD / "gauges.data")) == want
    assert oo.read_gauges_data(str(GOLD / "gauges.data")) == want


def test_gauges_data_bad_header(gpu_lib, tmp_path):
    from geoflood_gb300 import GeoFloodError
    from geoflood_gb300 import output as go

    p = tmp_path / "gauges.data"
    p.write_text("# a\n# b\nnot a comment\n")
    with pytest.raises(GeoFloodError):
        go.read_gauges_data(str(p))
    with pytest.raises(GeoFloodError):
        go.read_gauges_data(str(tmp_path / "missing.data"))


def test_native_gauge_sample_matches_oracle(gpu_lib):
    """Bilinear and dry-neighbour branches, gauges on cell edges, in the last
    cell (stencil on ghost cells) and on the patch's upper edge."""
    from geoflood_gb300 import output as go

    rng = np.random.default_rng(5)
    m = 8
    xl, yl, dx, dy, tol = 100.0, -50.0, 2.5, 1.25, 1e-3
    for trial in range(200):
        q = rng.uniform(0.0, 3.0, (m + 4, m + 4, 3))
        q[..., 1:] = rng.standard_normal((m + 4, m + 4, 2))
        dry = rng.random((m + 4, m + 4)) < 0.15
        q[dry, 0] = rng.uniform(0.0, 2e-4, dry.sum())
        aux = rng.standard_normal((m + 4, m + 4, 2)) * 10
        kind = trial % 4
        if kind == 0:
            xc, yc = xl + rng.uniform(0, m * dx), yl + rng.uniform(0, m * dy)
        elif kind == 1:
            xc, yc = xl + rng.integers(0, m) * dx, yl + rng.integers(0, m) * dy
        elif kind == 2:
            xc, yc = xl + (m - 0.3) * dx, yl + (m - 0.1) * dy
        else:
            xc, yc = xl + m * dx, yl + m * dy
        got = go.sample_gauge(q, aux, xl, yl, dx, dy, tol, xc, yc)
        cell = oo.gauge_cell(m, xl, yl, dx, dy, xc, yc)
        want = oo.sample_gauge(q, aux, *cell, tol)
        assert got == want, (trial, got, want)


def test_p4est_order_rules():
    ids = oo.brick_tree_ids(1, 1)
    assert ids == {(0, 0): 0}
    ids = oo.brick_tree_ids(2, 2)
    assert [ids[(x, y)] for y in range(2) for x in range(2)] == [0, 1, 2, 3]
    ids = oo.brick_tree_ids(3, 2)           # box 4 x 2: Morton skips x = 3
    assert ids == {(0, 0): 0, (1, 0): 1, (0, 1): 2, (1, 1): 3, (2, 0): 4, (2, 1): 5}
    ids = oo.brick_tree_ids(1, 3)           # y bits only
    assert ids == {(0, 0): 0, (0, 1): 1, (0, 2): 2}
    # one block at level 1 with its lower-right quadrant refined to level 2
    keys = [(1, 0, 0), (1, 0, 1), (1, 1, 1), (2, 2, 0), (2, 3, 0), (2, 2, 1), (2, 3, 1)]
    order, trees = oo.p4est_order(keys, 1, 1, 2)
    assert [keys[n] for n in order] == [(1, 0, 0), (2, 2, 0), (2, 3, 0), (2, 2, 1), (2, 3, 1),
                                        (1, 0, 1), (1, 1, 1)]
    assert trees == [0] * 7
    # two blocks side by side: all of block 0 first
    keys = [(1, 2, 0), (1, 0, 0), (1, 1, 1), (1, 3, 1), (1, 0, 1), (1, 1, 0), (1, 2, 1), (1, 3, 0)]
    order, trees = oo.p4est_order(keys, 2, 1, 1)
    assert [keys[n] for n in order] == [(1, 0, 0), (1, 1, 0), (1, 0, 1), (1, 1, 1),
                                        (1, 2, 0), (1, 3, 0), (1, 2, 1), (1, 3, 1)]
