/*
 * CPU oracle, coarse/fine transfers and refinement tags -- TEST
 * INFRASTRUCTURE ONLY.
 *
 * Restates (paths relative to the GeoFlood source tree):
 *   fc2d_geoclaw_fort_average_face / _corner / _average2coarse
 *       src/fc2d_geoclaw/fclaw2d_source/fc2d_geoclaw_average_fort.f:33, 323, 482-602
 *   fc2d_geoclaw_fort_interpolate_face / _corner / _interpolate2fine
 *       src/fc2d_geoclaw/fclaw2d_source/fc2d_geoclaw_interpolate_fort.f:24, 261, 405-579
 *   fc2d_geoclaw_fort_timeinterp   fclaw2d_source/fc2d_geoclaw_timeinterp_fort.f:1-69
 *   fc2d_geoclaw_fort_tag4refinement, fc2d_geoclaw_flag2refine,
 *   fc2d_geoclaw_fort_tag4coarsening, fc2d_geoclaw_test_regions
 *       fclaw2d_source/fc2d_geoclaw_tag4refinement_fort.f90,
 *       fc2d_geoflood_flag2refine.f90, fc2d_geoclaw_tag4coarsening_fort.f90,
 *       fc2d_geoclaw_test_regions.f90; region tests of fc2d_geoclaw.cpp:405-506
 *
 * Three pieces come from ForestClaw (git tag feature_smoke3d), which is not
 * in the reference tree, and are restated here for aligned patches in a
 * brick with refinement ratio 2:
 *   - fclaw2d_clawpatch_transform_face_half / _corner_half: the four fine
 *     cells under a coarse cell, lower-left first, x fastest;
 *   - fclaw2d_clawpatch_is_valid_average / _is_valid_interp: fine interior
 *     [1, m] x [1, m] resp. fine array [1-mbc, m+mbc]^2;
 *   - fclaw2d_clawpatch_compute_slopes with mth = 5: minmod, as the
 *     reference's own comment at interpolate_fort.f:430 states.
 * mcapa = 0 throughout (capacity 1), as in every configuration here.
 */
#include <math.h>
#include <string.h>

#include "geoclaw_oracle.h"

#define QF(q, m, i, j) \
    (q)[((m) - 1) + 3 * (((i) + mbc - 1) + (mx + 2 * mbc) * ((j) + mbc - 1))]
#define AF(a, m, i, j) \
    (a)[((m) - 1) + maux * (((i) + mbc - 1) + (mx + 2 * mbc) * ((j) + mbc - 1))]

static double dmax(double a, double b) { return a > b ? a : b; }
static double dmin(double a, double b) { return a < b ? a : b; }

/* minmod slope (mth = 5) */
static double orc_slope(double sl, double sr)
{
    if (sl * sr <= 0.0) return 0.0;
    return fabs(sl) < fabs(sr) ? sl : sr;
}

/* Wet-cell-weighted average of four fine cells onto one coarse cell
 * (average_fort.f:154-198, the same block in all three averaging routines). */
static void orc_avg4(const orc_params* p, int mbc, int mx, int my, int maux, const double* qf,
                     const double* af, const int* i2, const int* j2, double bc, double* out)
{
    double etasum = 0.0, hsum = 0.0, husum = 0.0, hvsum = 0.0;
    int nwet = 0, m;
    (void)my;
    for (m = 0; m < 4; ++m) {
        double hf = QF(qf, 1, i2[m], j2[m]);
        double bf = AF(af, 1, i2[m], j2[m]);
        double huf = QF(qf, 2, i2[m], j2[m]);
        double hvf = QF(qf, 3, i2[m], j2[m]);
        double etaf;
        if (hf > p->dry_tolerance) {
            etaf = hf + bf;
            nwet = nwet + 1;
        } else {
            etaf = 0.0;
            huf = 0.0;
            hvf = 0.0;
        }
        hsum = hsum + hf;
        husum = husum + huf;
        hvsum = hvsum + hvf;
        etasum = etasum + etaf;
    }
    if (nwet > 0) {
        double etaav = etasum / (double)nwet;
        double hav = hsum / (double)nwet;
        double hc = dmin(hav, dmax(etaav - bc, 0.0));
        out[0] = hc;
        out[1] = (hc / hsum) * husum;
        out[2] = (hc / hsum) * hvsum;
    } else {
        out[0] = out[1] = out[2] = 0.0;
    }
}

/* Fine indices of the four fine cells under coarse cell (ic, jc) when the
 * coarse patch's cell (1,1) corner sits at fine index (ox+1, oy+1). */
static void orc_under(int ic, int jc, int ox, int oy, int* i2, int* j2)
{
    int m = 0, ii, jj;
    for (jj = 0; jj < 2; ++jj)
        for (ii = 0; ii < 2; ++ii) {
            i2[m] = 2 * ic - 1 + ox + ii;
            j2[m] = 2 * jc - 1 + oy + jj;
            ++m;
        }
}

void orc_average_ghost(const orc_params* p, int mbc, int mx, int my, int maux, double* qc,
                       const double* ac, const double* qf, const double* af, int kind, int code,
                       int ox, int oy)
{
    /* kind 0: face (code = iface_coarse), 1: corner (code = icorner_coarse) */
    int ic, jc, ibc, jbc, m;
    int i2[4], j2[4];
    double out[3];
    if (kind == 0) {
        const int idir = code / 2;
        if (idir == 0) {
            for (jc = 1; jc <= my; ++jc)
                for (ibc = 1; ibc <= mbc; ++ibc) {
                    int ok = 1;
                    ic = (code == 0) ? 1 - ibc : mx + ibc;
                    orc_under(ic, jc, ox, oy, i2, j2);
                    for (m = 0; m < 4; ++m)
                        if (i2[m] < 1 || i2[m] > mx || j2[m] < 1 || j2[m] > my) ok = 0;
                    if (!ok) continue;
                    orc_avg4(p, mbc, mx, my, maux, qf, af, i2, j2, AF(ac, 1, ic, jc), out);
                    for (m = 1; m <= 3; ++m) QF(qc, m, ic, jc) = out[m - 1];
                }
        } else {
            for (jbc = 1; jbc <= mbc; ++jbc)
                for (ic = 1; ic <= mx; ++ic) {
                    int ok = 1;
                    jc = (code == 2) ? 1 - jbc : my + jbc;
                    orc_under(ic, jc, ox, oy, i2, j2);
                    for (m = 0; m < 4; ++m)
                        if (i2[m] < 1 || i2[m] > mx || j2[m] < 1 || j2[m] > my) ok = 0;
                    if (!ok) continue;
                    orc_avg4(p, mbc, mx, my, maux, qf, af, i2, j2, AF(ac, 1, ic, jc), out);
                    for (m = 1; m <= 3; ++m) QF(qc, m, ic, jc) = out[m - 1];
                }
        }
    } else {
        for (ibc = 1; ibc <= mbc; ++ibc)
            for (jbc = 1; jbc <= mbc; ++jbc) {
                int i1 = (code == 0 || code == 2) ? 1 - ibc : mx + ibc;
                int j1 = (code == 0 || code == 1) ? 1 - jbc : my + jbc;
                orc_under(i1, j1, ox, oy, i2, j2);
                orc_avg4(p, mbc, mx, my, maux, qf, af, i2, j2, AF(ac, 1, i1, j1), out);
                for (m = 1; m <= 3; ++m) QF(qc, m, i1, j1) = out[m - 1];
            }
    }
}

/* eta with dry limiting on the 3x3 block around coarse cell (ic, jc) */
static void orc_etabar(const orc_params* p, int mbc, int mx, int my, int maux, const double* qc,
                       const double* ac, int ic, int jc, double eb[3][3])
{
    int ii, jj;
    (void)my;
    for (ii = -1; ii <= 1; ++ii)
        for (jj = -1; jj <= 1; ++jj) {
            double h = QF(qc, 1, ic + ii, jc + jj);
            double b = AF(ac, 1, ic + ii, jc + jj);
            eb[ii + 1][jj + 1] = (h < p->dry_tolerance) ? p->sea_level : h + b;
        }
}

/* Fill the four fine cells under coarse cell (ic, jc) from its limited
 * reconstruction (interpolate_fort.f:122-176): depth via the surface eta,
 * clipped at 0 when `clip`; momenta directly. */
static void orc_interp_cell(const orc_params* p, int mbc, int mx, int my, int maux,
                            const double* qc, const double* ac, double* qf, const double* af,
                            int ic, int jc, const int* iff, const int* jff, int clip)
{
    int mq, m;
    for (mq = 1; mq <= 3; ++mq) {
        double qcv, gradx, grady;
        if (mq == 1) {
            double eb[3][3];
            orc_etabar(p, mbc, mx, my, maux, qc, ac, ic, jc, eb);
            qcv = eb[1][1];
            gradx = orc_slope(qcv - eb[0][1], eb[2][1] - qcv);
            grady = orc_slope(qcv - eb[1][0], eb[1][2] - qcv);
        } else {
            qcv = QF(qc, mq, ic, jc);
            gradx = orc_slope(qcv - QF(qc, mq, ic - 1, jc), QF(qc, mq, ic + 1, jc) - qcv);
            grady = orc_slope(qcv - QF(qc, mq, ic, jc - 1), QF(qc, mq, ic, jc + 1) - qcv);
        }
        for (m = 0; m < 4; ++m) {
            const double shiftx = ((m & 1) - 0.5) / 2.0;
            const double shifty = ((m >> 1) - 0.5) / 2.0;
            double value = qcv + gradx * shiftx + grady * shifty;
            if (mq == 1) {
                value = value - AF(af, 1, iff[m], jff[m]);
                if (clip) value = dmax(value, 0.0);
            }
            QF(qf, mq, iff[m], jff[m]) = value;
        }
    }
}

void orc_interpolate_ghost(const orc_params* p, int mbc, int mx, int my, int maux,
                           const double* qc, const double* ac, double* qf, const double* af,
                           int kind, int code, int ox, int oy)
{
    /* kind 0: face (code = iface_coarse), 1: corner (code = icorner_coarse) */
    int i2[4], j2[4], m, ic, jc;
    if (kind == 0) {
        const int idir = code / 2;
        /* the reference loops jc (resp. ic) over 1..mx on both faces */
        for (int k = 1; k <= mx; ++k) {
            int ok = 1;
            if (idir == 0) {
                ic = (code == 0) ? 1 : mx;
                jc = k;
            } else {
                jc = (code == 2) ? 1 : my;
                ic = k;
            }
            orc_under(ic, jc, ox, oy, i2, j2);
            for (m = 0; m < 4; ++m)
                if (i2[m] < 1 - mbc || i2[m] > mx + mbc || j2[m] < 1 - mbc || j2[m] > my + mbc) ok = 0;
            if (!ok) continue;
            orc_interp_cell(p, mbc, mx, my, maux, qc, ac, qf, af, ic, jc, i2, j2, 1);
        }
    } else {
        ic = (code == 0 || code == 2) ? 1 : mx;
        jc = (code == 0 || code == 1) ? 1 : my;
        orc_under(ic, jc, ox, oy, i2, j2);
        orc_interp_cell(p, mbc, mx, my, maux, qc, ac, qf, af, ic, jc, i2, j2, 1);
    }
}

void orc_interpolate2fine(const orc_params* p, int mbc, int mx, int my, int maux,
                          const double* qc, const double* ac, double* qf, const double* af,
                          int igrid)
{
    const int ig = igrid % 2, jg = (igrid - ig) / 2;
    const int i1 = 1 - ig, i2 = mx / 2 + (1 - ig), ic_add = ig * mx / 2;
    const int j1 = 1 - jg, j2 = my / 2 + (1 - jg), jc_add = jg * my / 2;
    int i, j;
    for (i = i1; i <= i2; ++i)
        for (j = j1; j <= j2; ++j) {
            int iff[4], jff[4], m = 0, ii, jj;
            for (jj = 1; jj <= 2; ++jj)
                for (ii = 1; ii <= 2; ++ii) {
                    iff[m] = (i - 1) * 2 + ii;
                    jff[m] = (j - 1) * 2 + jj;
                    ++m;
                }
            orc_interp_cell(p, mbc, mx, my, maux, qc, ac, qf, af, i + ic_add, j + jc_add, iff,
                            jff, 0);
        }
}

void orc_average2coarse(const orc_params* p, int mbc, int mx, int my, int maux, double* qc,
                        const double* ac, const double* qf, const double* af, int igrid)
{
    const int ig = igrid % 2, jg = (igrid - ig) / 2;
    const int ic_add = ig * mx / 2, jc_add = jg * my / 2;
    int i, j, mq;
    for (j = 1; j <= my / 2; ++j)
        for (i = 1; i <= mx / 2; ++i) {
            int i2[4], j2[4], m = 0, ii, jj;
            double out[3];
            for (jj = 1; jj <= 2; ++jj)
                for (ii = 1; ii <= 2; ++ii) {
                    i2[m] = (i - 1) * 2 + ii;
                    j2[m] = (j - 1) * 2 + jj;
                    ++m;
                }
            orc_avg4(p, mbc, mx, my, maux, qf, af, i2, j2, AF(ac, 1, i + ic_add, j + jc_add), out);
            for (mq = 1; mq <= 3; ++mq) QF(qc, mq, i + ic_add, j + jc_add) = out[mq - 1];
        }
}

int orc_timeinterp(int mbc, int mx, int my, int psize, const double* qcurr, const double* qlast,
                   double* qinterp, double alpha)
{
    const int mint = 2, ng = 0;
    int i, j, m, k = 1;
    for (m = 1; m <= 3; ++m) {
        for (j = 1 - ng; j <= my - mint; ++j)
            for (i = 1 - ng; i <= mint; ++i, ++k)
                QF(qinterp, m, i, j) = QF(qlast, m, i, j) + alpha * (QF(qcurr, m, i, j) - QF(qlast, m, i, j));
        for (j = 1 - ng; j <= mint; ++j)
            for (i = mint + 1; i <= mx + ng; ++i, ++k)
                QF(qinterp, m, i, j) = QF(qlast, m, i, j) + alpha * (QF(qcurr, m, i, j) - QF(qlast, m, i, j));
        for (j = mint + 1; j <= my + ng; ++j)
            for (i = mx - mint + 1; i <= mx + ng; ++i, ++k)
                QF(qinterp, m, i, j) = QF(qlast, m, i, j) + alpha * (QF(qcurr, m, i, j) - QF(qlast, m, i, j));
        for (j = my - mint + 1; j <= my + ng; ++j)
            for (i = 1 - ng; i <= mx - mint; ++i, ++k)
                QF(qinterp, m, i, j) = QF(qlast, m, i, j) + alpha * (QF(qcurr, m, i, j) - QF(qlast, m, i, j));
    }
    return (k - 1 != psize) ? 2 : 0;
}

/* ---------------------------- refinement tags ---------------------------- */

static int orc_p_intersects_r(double xl, double yl, double xu, double yu, double t,
                              const orc_region* r)
{
    if (t < r->t_low || t > r->t_hi) return 0;
    if (xu < r->x_low || xl > r->x_hi) return 0;
    if (yu < r->y_low || yl > r->y_hi) return 0;
    return 1;
}

int orc_test_regions(const orc_refine* rf, int level, double xl, double yl, double xu, double yu,
                     double t, int refine)
{
    int m, found = 0, min_level = 100, max_level = 0;
    for (m = 0; m < rf->num_regions; ++m)
        if (orc_p_intersects_r(xl, yl, xu, yu, t, &rf->regions[m])) {
            found = 1;
            if (rf->regions[m].min_level < min_level) min_level = rf->regions[m].min_level;
            if (rf->regions[m].max_level > max_level) max_level = rf->regions[m].max_level;
        }
    if (!found) return -1;
    if (refine != 0) {
        if (level < min_level) return 1;
        if (level >= max_level) return 0;
    } else {
        if (level <= min_level) return 0;
        if (level > max_level) return 1;
    }
    return -1;
}

int orc_flag2refine(const orc_params* p, const orc_refine* rf, int mbc, int mx, int my, int maux,
                    const double* q, const double* aux, int i, int j, int level, int maxlevel,
                    int init_flag, int is_coarsening)
{
    int m, n;
    const int max_num_speeds = rf->num_speed_tolerance < maxlevel ? rf->num_speed_tolerance : maxlevel;
    double momentum, depth, eta, speed = 0.0;
    int th_factor;
    (void)my;
    if (init_flag != 0 && is_coarsening) return 0;
    /* allowflag (geolib_source/allowflag.f) is always true; the legacy
     * regions.i block is never filled, so its loop flags nothing. */
    momentum = sqrt(QF(q, 2, i, j) * QF(q, 2, i, j) + QF(q, 3, i, j) * QF(q, 3, i, j));
    depth = QF(q, 1, i, j);
    eta = depth + AF(aux, 1, i, j);
    th_factor = 1;
    if (is_coarsening) th_factor = 0; /* integer variable assigned 0.5 */
    for (m = 0; m < rf->num_flowgrades; ++m) {
        int needed = 0;
        switch (rf->flowgradevariable[m]) {
        case 1: needed = depth > rf->flowgradevalue[m]; break;
        case 2: needed = momentum > rf->flowgradevalue[m]; break;
        case 3:
            if (depth > p->dry_tolerance) needed = fabs(eta) > rf->flowgradevalue[m];
            break;
        default: break;
        }
        if (needed && level < rf->flowgrademinlevel[m]) return 1;
    }
    if (depth > p->dry_tolerance) {
        speed = momentum / depth;
        for (n = 1; n <= max_num_speeds; ++n)
            if (speed > th_factor * rf->speed_tolerance[n - 1] && level <= n) return 1;
    }
    if (rf->num_flowgrades == 0 && depth > p->dry_tolerance) {
        if (fabs(eta - p->sea_level) > th_factor * rf->wave_tolerance) {
            if (level < rf->max_level_deep) return 1;
            if (fabs(AF(aux, 1, i, j)) < rf->deep_depth) return 1;
        }
        if (fabs(AF(aux, 1, i, j)) > rf->deep_depth && speed < rf->speed_tolerance[0]) return 0;
        if (speed / depth > rf->max_velocity_depth_product) return 1;
    }
    return 0;
}

int orc_tag4refinement(const orc_params* p, const orc_refine* rf, int mbc, int mx, int my,
                       int maux, const double* q, const double* aux, double xlower,
                       double ylower, double dx, double dy, double t, int level, int maxlevel,
                       int init_flag)
{
    int i, j;
    int tag = orc_test_regions(rf, level, xlower, ylower, xlower + mx * dx, ylower + my * dy, t, 1);
    if (tag >= 0) return tag;
    for (j = 1; j <= my; ++j)
        for (i = 1; i <= mx; ++i)
            if (orc_flag2refine(p, rf, mbc, mx, my, maux, q, aux, i, j, level, maxlevel, init_flag,
                                0) > 0)
                return 1;
    return 0;
}

int orc_tag4coarsening(const orc_params* p, const orc_refine* rf, int mbc, int mx, int my,
                       int maux, const double* const* q, const double* const* aux,
                       const double* xlower, const double* ylower, double dx, double dy, double t,
                       int level, int maxlevel, int init_flag)
{
    int k, i, j;
    /* parent box from siblings 0 (ll), 1 (lr), 2 (ul): fc2d_geoclaw.cpp:485-490 */
    int tag = orc_test_regions(rf, level, xlower[0], ylower[0], xlower[1] + mx * dx,
                               ylower[2] + my * dy, t, 0);
    if (tag >= 0) return tag;
    for (k = 0; k < 4; ++k)
        for (j = 1; j <= my; ++j)
            for (i = 1; i <= mx; ++i)
                if (orc_flag2refine(p, rf, mbc, mx, my, maux, q[k], aux[k], i, j, level, maxlevel,
                                    init_flag, 1) > 0)
                    return 0;
    return 1;
}
