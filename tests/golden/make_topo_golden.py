"""Generate the topography fixtures under tests/golden/topo/.

Run from the repository root with the GeoFlood reference tree available
(its Python tools are imported from REFERENCE/scripts):

    python tests/golden/make_topo_golden.py /path/to/GeoFlood

1. Four seeded DEM grids over a 1 km x 0.75 km domain:
   A  41 x 31 nodes, 25 m spacing, covering the domain with margin (type 3);
   B  61 x 49 nodes, 5 m, a sub-region of A (type 2);
   C  9 x 7 nodes, 12.5 m, overlapping B's corner (type 1);
   D  12 x 10 nodes, 10 m, ESRI header written label first, 'xllcorner'
      registration, four no-data nodes, read as type -3 (depth positive).
   A, B and C are written by the reference's own Topography.write
   (scripts/geoclaw/topotools.py:960-1100); D by this script.
2. topo.data listing them is written by the reference's TopographyData
   writer (scripts/geoclaw/data.py:145-215), which stores absolute paths;
   the directory prefix is then cut so the fixture names files relative to
   topo.data.
3. Each file is read back with the reference's Topography.read
   (topotools.py:612-830); the node coordinates and values it returns are
   stored in parsed.npz for the tests.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "topo")
TOPO_MISSING = 25.0


def surface(x, y, rng, amp):
    X, Y = np.meshgrid(x, y)
    z = (30.0 - 0.02 * X + 0.015 * Y + 8.0 * np.sin(X / 90.0) * np.cos(Y / 70.0)
         + amp * rng.standard_normal(X.shape))
    return np.round(z, 3)


def grids():
    rng = np.random.default_rng(777)
    A = dict(x=-100.0 + 25.0 * np.arange(41), y=-50.0 + 25.0 * np.arange(31))
    B = dict(x=300.0 + 5.0 * np.arange(61), y=200.0 + 5.0 * np.arange(49))
    C = dict(x=560.0 + 12.5 * np.arange(9), y=400.0 + 12.5 * np.arange(7))
    for g, amp in ((A, 0.5), (B, 0.2), (C, 0.1)):
        g["Z"] = surface(g["x"], g["y"], rng, amp)       # rows south to north
    return A, B, C


def write_esri(path):
    """D: label-first ESRI header, llcorner registration, depth positive."""
    rng = np.random.default_rng(31)
    z = np.round(-20.0 + 3.0 * rng.standard_normal((10, 12)), 2)   # rows north to south
    z[2, 3] = z[7, 0] = z[9, 11] = z[0, 5] = -9999.0
    with open(path, "w") as f:
        f.write("ncols 12\nnrows 10\nxllcorner 95.0\nyllcorner 495.0\n"
                "cellsize 10.0\nNODATA_value -9999\n")
        for row in z:
            f.write(" ".join("%.2f" % v for v in row) + "\n")


def main(reference: str) -> None:
    sys.path.insert(0, os.path.join(reference, "scripts"))
    import geoclaw.data as gdata
    import geoclaw.topotools as tt

    os.makedirs(OUT, exist_ok=True)
    A, B, C = grids()
    names = {"A": ("A.tt3", 3), "B": ("B.tt2", 2), "C": ("C.tt1", 1)}
    for key, g in zip("ABC", (A, B, C)):
        t = tt.Topography()
        t.x, t.y, t.Z = g["x"], g["y"], g["Z"]
        t.write(os.path.join(OUT, names[key][0]), topo_type=names[key][1])
    write_esri(os.path.join(OUT, "D.asc"))
    names["D"] = ("D.asc", -3)

    td = gdata.TopographyData()
    td.topo_missing = TOPO_MISSING
    td.topofiles = [[names[k][1], os.path.join(OUT, names[k][0])] for k in "ABCD"]
    path = os.path.join(OUT, "topo.data")
    td.write(out_file=path)
    if getattr(td, "_out_file", None) is not None:
        td.close_data_file()
    with open(path) as f:
        text = f.read()
    with open(path, "w") as f:
        f.write(text.replace(OUT + os.sep, ""))

    parsed = {}
    for k in "ABCD":
        t = tt.Topography()
        t.read(os.path.join(OUT, names[k][0]), topo_type=names[k][1])
        parsed[k + "_x"] = np.asarray(t.x)
        parsed[k + "_y"] = np.asarray(t.y)
        parsed[k + "_Z"] = np.asarray(t.Z)          # rows south to north
        if abs(names[k][1]) in (2, 3):
            parsed[k + "_nodata"] = np.array(t.no_data_value)
    np.savez(os.path.join(OUT, "parsed.npz"), **parsed)
    print("wrote", OUT)


if __name__ == "__main__":
    import os

    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GF_REFERENCE_ROOT")
    if not ref:
        raise SystemExit("usage: name the GeoFlood reference tree (argument or GF_REFERENCE_ROOT)")
    main(ref)
