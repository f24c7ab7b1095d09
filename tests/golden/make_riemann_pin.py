"""Generate tests/golden/riemann_pin.npz from the reference's own Riemann solver.

Runs the reference's CUDA device functions cuda_flood_rpn2 / cuda_flood_rpt2
(src/fc2d_cpu_cuda/riemann_source/geoflood_rp2.cu) compiled for the host by
oracle/build_ref.sh (oracle/_ref/libref_riemann.so) on seeded single-face
problems covering the solver's regimes: wet/wet with 2-rarefaction,
2-shock and shock-rarefaction structure, wet/dry walls and overtopping, lake
at rest over steps, near-sonic states, x and y faces. Stores inputs and the
reference outputs; tests/test_reference_pin.py replays them on the oracle.

Usage: python tests/golden/make_riemann_pin.py   (needs the reference tree)
"""
from __future__ import annotations

import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent / "riemann_pin.npz"
G, DRYTOL = 9.81, 1e-3


def load_ref():
    lib_path = ROOT / "oracle" / "_ref" / "libref_riemann.so"
    if not lib_path.exists():
        subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh")], check=True)
    if not lib_path.exists():
        raise SystemExit("reference tree not available: cannot build oracle/_ref")
    lib = C.CDLL(str(lib_path))
    dp = C.POINTER(C.c_double)
    lib.ref_set_gravity.argtypes = [C.c_double]
    lib.ref_rpn2_face.argtypes = [C.c_int, dp, dp, C.c_double, C.c_double, C.c_double, dp, dp, dp, dp]
    lib.ref_rpt2_face.argtypes = [C.c_int, C.c_int, dp, dp, dp, dp, dp, dp, C.c_double, dp, dp]
    lib.ref_set_gravity(G)
    return lib


def cases(n: int, seed: int = 20261203):
    g = np.random.Generator(np.random.PCG64(seed))
    rows = []
    for k in range(n):
        kind = k % 8
        hl, hr = g.uniform(0.01, 10.0, 2)
        ul, ur = g.normal(0.0, 2.0, 2)
        vl, vr = g.normal(0.0, 1.0, 2)
        bl, br = g.normal(0.0, 1.0, 2)
        if kind == 1:    # strong dam break: shock + rarefaction
            hl, hr, ul, ur = g.uniform(5, 10), g.uniform(0.1, 1), 0.0, 0.0
        elif kind == 2:  # colliding streams: 2 shocks
            ul, ur = g.uniform(1, 5), -g.uniform(1, 5)
        elif kind == 3:  # diverging: 2 rarefactions
            ul, ur = -g.uniform(1, 4), g.uniform(1, 4)
        elif kind == 4:  # right cell dry, left may overtop or reflect
            hr, ur, vr = g.uniform(0, DRYTOL), 0.0, 0.0
            br = bl + g.uniform(-2, 3)
        elif kind == 5:  # left cell dry
            hl, ul, vl = g.uniform(0, DRYTOL), 0.0, 0.0
            bl = br + g.uniform(-2, 3)
        elif kind == 6:  # lake at rest across a step
            eta = g.uniform(2, 6)
            hl, hr = eta - bl, eta - br
            if hl <= 0 or hr <= 0:
                bl, br = 0.0, g.uniform(-1, 1)
                hl, hr = eta, eta - br
            ul = ur = vl = vr = 0.0
        elif kind == 7:  # near-critical flow
            hl = hr = g.uniform(0.5, 3)
            c = np.sqrt(G * hl)
            ul = c * (1 + g.normal(0, 1e-3))
            ur = ul * (1 + g.normal(0, 1e-3))
        idir = int(g.integers(0, 2))
        ql = [hl, 0.0, 0.0]
        qr = [hr, 0.0, 0.0]
        mu, mv = 1 + idir, 2 - idir
        ql[mu], ql[mv] = hl * ul, hl * vl
        qr[mu], qr[mv] = hr * ur, hr * vr
        topo = g.normal(0.0, 1.0, 4)  # rows below / above, left and right
        rows.append((idir, ql, qr, bl, br, topo))
    return rows


def main(n: int = 4000):
    lib = load_ref()
    dp = C.POINTER(C.c_double)

    def arr(x):
        a = np.ascontiguousarray(x, dtype=np.float64)
        return a, a.ctypes.data_as(dp)

    rs = cases(n)
    IN = np.zeros((n, 13))
    RPN = np.zeros((n, 18))   # fwave(9) s(3) amdq(3) apdq(3)
    RPT = np.zeros((n, 12))   # left: bm bp, right: bm bp
    for k, (idir, ql, qr, bl, br, topo) in enumerate(rs):
        IN[k] = [idir, *ql, *qr, bl, br, *topo]
        a_ql, p_ql = arr(ql)
        a_qr, p_qr = arr(qr)
        fw, p_fw = arr(np.zeros(9))
        s, p_s = arr(np.zeros(3))
        am, p_am = arr(np.zeros(3))
        ap, p_ap = arr(np.zeros(3))
        lib.ref_rpn2_face(idir, p_ql, p_qr, bl, br, DRYTOL, p_fw, p_s, p_am, p_ap)
        RPN[k] = np.concatenate([fw, s, am, ap])
        a1, p1 = arr([topo[0], topo[1]])
        a2, p2 = arr([bl, br])
        a3, p3 = arr([topo[2], topo[3]])
        out = []
        for imp, asdq in ((0, am), (1, ap)):
            a_d, p_d = arr(asdq)
            bm, p_bm = arr(np.zeros(3))
            bp, p_bp = arr(np.zeros(3))
            lib.ref_rpt2_face(idir, imp, p_ql, p_qr, p1, p2, p3, p_d, DRYTOL, p_bm, p_bp)
            out += [bm, bp]
        RPT[k] = np.concatenate(out)
    np.savez_compressed(OUT, inputs=IN, rpn2=RPN, rpt2=RPT, grav=G, drytol=DRYTOL)
    print(f"wrote {OUT} ({n} faces)")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 4000)
