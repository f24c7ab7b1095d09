/*
 * CPU oracle, coarse/fine conservation fix -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates qad (src/fc2d_geoclaw/geolib_source/qad.f:4-371), AMRClaw's
 * conservation fix-up as GeoClaw carries it: along each side of a fine
 * patch, solve the Riemann problem between the fine patch's first ghost
 * cell and the coarse cell that ghost cell lies in, and add the resulting
 * fluctuations, times the fine face length and time step, into svdflx, one
 * entry per coarse cell along the side. The reference tree never compiles
 * this file (absent from src/fc2d_geoclaw/CMakeLists.txt:2-52), so nothing
 * of GeoFlood calls it; it is restated here so the device kernel has a
 * checker.
 *
 * Array conventions follow qad.f: sides 1 (left), 2 (top), 3 (right),
 * 4 (bottom); along each side the coarse cells run bottom to top (sides 1,
 * 3) or left to right (sides 2, 4); the Riemann problem at face k is
 * between qr(k-1) and ql(k) (rpn2's convention), with
 *   side 1: left = coarse,     right = fine ghost  (x), svdflx += ... * hy
 *   side 2: left = fine ghost, right = coarse      (y), svdflx -= ... * hx
 *   side 3: left = fine ghost, right = coarse      (x), svdflx -= ... * hy
 *   side 4: left = coarse,     right = fine ghost  (y), svdflx += ... * hx
 * (qad.f:84-152, 166-229, 237-290, 304-356). The aux of a fine ghost cell is
 * its own (the "normal case" of qad.f:92-95; no aux field here is an
 * "xleft"/"yleft" face velocity). The source-term branch (qad.f:360-368)
 * is commented out in the reference and is not restated.
 */
#include <string.h>

#include "geoclaw_oracle.h"

/* fine patch arrays in the Fortran layout q(m, 1-mbc:mx+mbc, 1-mbc:my+mbc) */
#define QF(q, m, i, j) (q)[((m) - 1) + 3 * (((i) + mbc - 1) + (mx + 2 * mbc) * ((j) + mbc - 1))]
#define AF(a, m, i, j) (a)[((m) - 1) + maux * (((i) + mbc - 1) + (mx + 2 * mbc) * ((j) + mbc - 1))]

/* One side of qad for a fine patch of mx x my cells (mbc = 2): qc1d, auxc1d
 * hold the n coarse cells along the side (3 resp. maux values each, in the
 * side's order), svdflx (3 x n) accumulates. lratio = 2. */
void orc_qad_side(const orc_params* p, int side, int mbc, int mx, int my, int maux,
                  const double* qf, const double* af, const double* qc1d, const double* auxc1d,
                  double hx, double hy, double delt, double* svdflx)
{
    const int lratio = 2;
    const int nfine = (side == 1 || side == 3) ? my : mx;
    const int ixy = (side == 1 || side == 3) ? 1 : 2;
    const double h = (side == 1 || side == 3) ? hy : hx;
    const double sgn = (side == 1 || side == 4) ? 1.0 : -1.0;
    int r, m, l, c;
    for (c = 0; c < nfine / lratio; ++c) {
        for (l = 1; l <= lratio; ++l) {
            /* fine row / column r (1-based) of this face */
            double g[3], coarse[3], bg, bc, fw[9], s[3], am[3], ap[3];
            r = c * lratio + l;
            for (m = 1; m <= 3; ++m) {
                if (side == 1) g[m - 1] = QF(qf, m, 0, r);
                else if (side == 2) g[m - 1] = QF(qf, m, r, my + 1);
                else if (side == 3) g[m - 1] = QF(qf, m, mx + 1, r);
                else g[m - 1] = QF(qf, m, r, 0);
                coarse[m - 1] = qc1d[(m - 1) + 3 * c];
            }
            if (side == 1) bg = AF(af, 1, 0, r);
            else if (side == 2) bg = AF(af, 1, r, my + 1);
            else if (side == 3) bg = AF(af, 1, mx + 1, r);
            else bg = AF(af, 1, r, 0);
            bc = auxc1d[maux * c];
            if (side == 1 || side == 4)
                orc_rpn2_face(p, ixy, coarse, g, bc, bg, fw, s, am, ap);
            else
                orc_rpn2_face(p, ixy, g, coarse, bg, bc, fw, s, am, ap);
            for (m = 0; m < 3; ++m)
                svdflx[m + 3 * c] = svdflx[m + 3 * c] + sgn * am[m] * h * delt + sgn * ap[m] * h * delt;
        }
    }
}
