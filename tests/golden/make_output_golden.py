"""Generate the output-format fixtures under tests/golden/output/.

Run from the repository root in a checkout that has the GeoFlood reference
tree (its Python scripts are imported from REFERENCE/scripts):

    python tests/golden/make_output_golden.py /path/to/GeoFlood

1. Seeded patch data (three 8 x 8 patches, values spanning 1e-120 .. 1e5,
   signed zeros, tiny bathymetry) and a gauge record set are written with
   the oracle's restatement of the reference writers (oracle/output.py):
   fort.t0003, fort.q0003, gauge00007.txt; fort.t0004 / fort.q0004 hold the
   same patches with one value of 1.5e150 (three-digit exponent).
2. gauges.data is written by the reference's own GaugeData writer
   (scripts/amrclaw/data.py:375-520).
3. The reference's own readers parse the written files: read_t and
   read_array (scripts/pyclaw/fileio/ascii.py:243-400), ForestClaw's
   read_patch_header (scripts/forestclaw/fileio/ascii.py) and GaugeSolution
   (scripts/pyclaw/gauges.py:79-200). What they return is stored in
   parsed.json next to the inputs (inputs.npz), so the tests can check,
   without the reference tree, that the files carry exactly the values
   written at the precision of the format.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "output")

FRAME = 3
FRAME_BIG = 4       # the same patches with one value of 1.5e150
GAUGE_ID = 7


def make_inputs():
    rng = np.random.default_rng(20240531)
    n, m = 3, 8
    n4 = m + 4
    q = rng.standard_normal((n, n4, n4, 3)) * 10.0 ** rng.integers(-6, 6, (n, n4, n4, 3))
    q[0, 3, 3, 0] = 1e-120          # zeroed by the writer
    q[1, 2, 5, 1] = -0.0            # signed zero -> 0
    q[0, 5, 5, 0] = -2.5e-100       # three-digit negative exponent, kept
    q[1, 6, 6, 0] = 2.0
    aux = rng.standard_normal((n, n4, n4, 1))
    aux[1, 6, 6, 0] = -2.0          # eta = 0 exactly
    level = np.array([1, 2, 2], np.int32)
    block = np.array([0, 1, 1], np.int32)
    xlower = np.array([0.0, -1.5, 1e-3])
    ylower = np.array([2.0, 3.25, -7e5])
    dx = np.array([0.125, 0.0625, 1.0 / 3.0])
    dy = np.array([0.25, 0.0625, 2.0 / 3.0])
    time = 0.1 + 1e-17
    grows = np.array([[1, 0.0, 1.0, 0.5, -0.25, -1.0],
                      [2, 0.125, 1.0 / 3.0, 1e-120, -7.5e-3, 2.0],
                      [2, 1.0e5 / 3.0, 0.0, 0.0, 0.0, 1e-120],
                      [3, 1e10, 123.456, -9.87654321e7, 5e-8, -123.456]])
    gauges = [(GAUGE_ID, 12.5, -3.75, 0.0, 1e10, 0.5),
              (11, 1.0 / 3.0, 2.0e3, 5.0, 60.0, 0.0)]
    return dict(q=q, aux=aux, level=level, block=block, xlower=xlower, ylower=ylower, dx=dx,
                dy=dy, time=np.array(time), grows=grows,
                gauges=np.array(gauges, np.float64))


def main(reference: str) -> None:
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(reference, "scripts"))
    from oracle import output as oo

    os.makedirs(OUT, exist_ok=True)
    d = make_inputs()
    np.savez(os.path.join(OUT, "inputs.npz"), **d)
    oo.write_frame(OUT, FRAME, float(d["time"]), d["q"], d["aux"], d["level"], d["block"],
                   d["xlower"], d["ylower"], d["dx"], d["dy"])
    # A value of 1e100 or more prints with a three-digit exponent and no E
    # (Fortran Ew.d); the reference's Python reader cannot parse that field,
    # so this frame is checked as text only.
    qb = d["q"].copy()
    qb[2, 4, 4, 2] = 1.5e150
    oo.write_frame(OUT, FRAME_BIG, float(d["time"]), qb, d["aux"], d["level"], d["block"],
                   d["xlower"], d["ylower"], d["dx"], d["dy"])
    with open(os.path.join(OUT, "gauge%05d.txt" % GAUGE_ID), "w") as f:
        g = d["gauges"][0]
        f.write(oo.gauge_header(GAUGE_ID, g[1], g[2]))
        f.write(oo.gauge_rows([tuple(r) for r in d["grows"]]))

    # gauges.data by the reference's own writer
    import amrclaw.data as amr_data
    gd = amr_data.GaugeData()
    for g in d["gauges"]:
        gd.gauges.append([int(g[0]), g[1], g[2], g[3], g[4]])
    gd.min_time_increment = {int(g[0]): g[5] for g in d["gauges"]}
    path = os.path.join(OUT, "gauges.data")
    gd.write(num_eqn=3, num_aux=1, out_file=path)
    if getattr(gd, "_out_file", None) is not None:
        gd.close_data_file()

    # parse with the reference's readers
    import forestclaw.fileio.ascii as fc_ascii
    import pyclaw
    import pyclaw.fileio.ascii as pc_ascii
    from pyclaw.gauges import GaugeSolution

    t, num_eqn, nstates, num_aux, num_dim, num_ghost, _ = pc_ascii.read_t(FRAME, OUT + "/")
    parsed = dict(t=t, num_eqn=num_eqn, nstates=nstates, num_aux=num_aux, num_dim=num_dim,
                  num_ghost=num_ghost, patches=[])
    with open(os.path.join(OUT, "fort.q%04d" % FRAME)) as f:
        for _ in range(nstates):
            patch = fc_ascii.read_patch_header(f, num_dim)
            state = pyclaw.state.State(patch, num_eqn, num_aux)
            qa = pc_ascii.read_array(f, state, num_eqn)
            parsed["patches"].append(dict(
                patch_index=int(patch.patch_index), level=int(patch.level),
                block_number=int(patch.block_number), mpi_rank=int(patch.mpi_rank),
                num_cells=[int(v) for v in patch.num_cells_global],
                lower=[float(dm.lower) for dm in patch.dimensions],
                delta=[float(dm.delta) for dm in patch.dimensions],
                q=np.asarray(qa).tolist()))
    gs = GaugeSolution(GAUGE_ID, OUT)
    parsed["gauge"] = dict(id=int(gs.id), location=[float(v) for v in gs.location],
                           level=np.asarray(gs.level).tolist(), t=np.asarray(gs.t).tolist(),
                           q=np.asarray(gs.q).tolist())
    with open(os.path.join(OUT, "parsed.json"), "w") as f:
        json.dump(parsed, f, indent=0)
    print("wrote", OUT)


if __name__ == "__main__":
    import os

    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GF_REFERENCE_ROOT")
    if not ref:
        raise SystemExit("usage: name the GeoFlood reference tree (argument or GF_REFERENCE_ROOT)")
    main(ref)
