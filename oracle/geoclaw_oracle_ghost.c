/*
 * CPU oracle, ghost cells -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates the reference's physical boundary conditions with hydrograph
 * inflow (fortran_source/geoflood_bc2_fort.f90:7-409,
 * hydrograph/hydrograh_module.f90:155-331) and the same-level ghost copies
 * (fclaw2d_source/fc2d_geoclaw_copy_fort.f:11-107, with the identity
 * transform of aligned neighbours in a brick). The order in which ForestClaw
 * applies them (copies, then the physical boundary of each patch) lives in
 * ForestClaw itself, which is not part of the reference tree; the sequence
 * here is this project's statement of it.
 */
#include <math.h>
#include <string.h>

#include "geoclaw_oracle.h"

#define MEQN 3
#define QF(q, m, i, j) \
    (q)[((m) - 1) + MEQN * (((i) + mbc - 1) + (mx + 2 * mbc) * ((j) + mbc - 1))]
#define AF(a, m, i, j) \
    (a)[((m) - 1) + maux * (((i) + mbc - 1) + (mx + 2 * mbc) * ((j) + mbc - 1))]

/* interpolation (hydrograh_module.f90:176-221), discharge type: q0(2). */
static double orc_hydro_interp(const orc_hydro* hy, double t)
{
    double v = 0.0;
    int i;
    if (t < hy->time[0]) {
        v = hy->hu[0];
    } else if (t > hy->time[hy->n - 1]) {
        v = hy->hu[hy->n - 1];
    } else {
        for (i = 0; i < hy->n - 1; ++i) {
            if (t >= hy->time[i] && t <= hy->time[i + 1]) {
                v = hy->hu[i] + (hy->hu[i + 1] - hy->hu[i]) / (hy->time[i + 1] - hy->time[i]) *
                                    (t - hy->time[i]);
                break;
            }
        }
    }
    return v;
}

/* Riemann_invariants (hydrograh_module.f90:224-274), discharge type.
 * tol is the single-precision literal 1.0e-6 of the Fortran. */
static void orc_riemann_invariants(double g, double* q0, const double* q1)
{
    const double tol = (double)1.0e-6f;
    const double u1 = q1[1] / q1[0];
    const double Fr = 0.5;
    int i;
    q0[0] = pow(q0[1] / sqrt(g) * Fr, 2.0 / 3.0);
    for (i = 1; i <= 100; ++i) {
        double fxn = q0[1] / q0[0] - 2 * sqrt(g * q0[0]) - u1 + 2 * sqrt(g * q1[0]);
        double dfxn;
        if (fabs(fxn) < tol) return;
        dfxn = -q0[1] / (q0[0] * q0[0]) - sqrt(g / q0[0]);
        q0[0] = q0[0] - fxn / dfxn;
    }
}

/* two_shock (hydrograh_module.f90:278-331), discharge type. */
static void orc_two_shock(double g, double* q0, const double* q1)
{
    const double tol = (double)1.0e-6f;
    const double u1 = q1[1] / q1[0];
    const double Fr = 1.0;
    int i;
    q0[0] = pow(q0[1] / sqrt(g) * Fr, 2.0 / 3.0);
    for (i = 1; i <= 100; ++i) {
        double fxn = q0[1] / q0[0] - u1 -
                     (q0[0] - q1[0]) * sqrt((g / 2.0) * (1.0 / q0[0] + 1.0 / q1[0]));
        double num, deno, dfxn;
        if (fabs(fxn) < tol) return;
        num = sqrt(g * (1.0 / q0[0] + 1.0 / q1[0]));
        deno = 2 * sqrt(2.0) * (q0[0] * q0[0]) * num;
        dfxn = -q0[1] / (q0[0] * q0[0]) - num / sqrt(2.0) + g * (q0[0] - q1[0]) / deno;
        q0[0] = q0[0] - fxn / dfxn;
    }
}

/* The inflow ghost state for one boundary cell q1 (h, hu, hv); the branch
 * inside the channel window of each side of geoflood_bc2_fort.f90.
 * Returns 1 and the state in out[] for inflow, 0 for the mirror (wall) case. */
static int orc_inflow_state(const orc_params* p, double q0hu, const double* q1, double* out)
{
    const double g = p->grav;
    double q0[4];
    q0[0] = 0.0;
    q0[1] = q0hu;
    q0[2] = 0.0;
    q0[3] = 0.0;
    if (q1[0] < p->dry_tolerance) {
        double h = pow(q0[1] / sqrt(g), 2.0 / 3.0);
        out[0] = h > 0.001 ? h : 0.001;
        out[1] = q0[1];
        out[2] = 0.0;
        return 1;
    }
    if (q0[1] != 0.0) {
        orc_riemann_invariants(g, q0, q1);
        if (q0[0] > q1[0]) orc_two_shock(g, q0, q1);
        out[0] = q0[0];
        out[1] = q0[1];
        out[2] = 0.0;
        return 1;
    }
    return 0;
}

void orc_bc2(const orc_params* p, const orc_hydro* hy, int mbc, int mx, int my, double xlower,
             double ylower, double dx, double dy, double* q, double* aux, int maux, double t,
             const int* mthbc)
{
    int i, j, m, ibc, jbc;
    double st[3];
    const int hyd = hy && hy->use && hy->n > 0;
    const double q0hu = hyd ? orc_hydro_interp(hy, t) : 0.0;

    /* left boundary */
    switch (mthbc[0]) {
    case 0:
        if (hyd && hy->side[0]) {
            for (j = 1 - mbc; j <= my + mbc; ++j) {
                const double y = ylower + (j - 0.5) * dy;
                double q1[3] = {QF(q, 1, 1, j), QF(q, 2, 1, j), QF(q, 3, 1, j)};
                const int inside = fabs(y - hy->y0) <= hy->width / 2.0;
                for (ibc = 1; ibc <= mbc; ++ibc) {
                    if (inside && orc_inflow_state(p, q0hu, q1, st)) {
                        for (m = 1; m <= 3; ++m) QF(q, m, 1 - ibc, j) = st[m - 1];
                    } else {
                        AF(aux, 1, 1 - ibc, j) = AF(aux, 1, ibc, j);
                        for (m = 1; m <= 3; ++m) QF(q, m, 1 - ibc, j) = QF(q, m, ibc, j);
                        QF(q, 2, 1 - ibc, j) = -QF(q, 2, ibc, j);
                    }
                }
            }
        }
        break;
    case 1:
        for (j = 1 - mbc; j <= my + mbc; ++j)
            for (ibc = 1; ibc <= mbc; ++ibc) {
                AF(aux, 1, 1 - ibc, j) = AF(aux, 1, 1, j);
                for (m = 1; m <= 3; ++m) QF(q, m, 1 - ibc, j) = QF(q, m, 1, j);
            }
        break;
    case 3:
        for (j = 1 - mbc; j <= my + mbc; ++j)
            for (ibc = 1; ibc <= mbc; ++ibc) {
                AF(aux, 1, 1 - ibc, j) = AF(aux, 1, ibc, j);
                for (m = 1; m <= 3; ++m) QF(q, m, 1 - ibc, j) = QF(q, m, ibc, j);
            }
        for (j = 1 - mbc; j <= my + mbc; ++j)
            for (ibc = 1; ibc <= mbc; ++ibc) QF(q, 2, 1 - ibc, j) = -QF(q, 2, ibc, j);
        break;
    default:
        break;
    }

    /* right boundary */
    switch (mthbc[1]) {
    case 0:
        if (hyd && hy->side[1]) {
            for (j = 1 - mbc; j <= my + mbc; ++j) {
                const double y = ylower + (j - 0.5) * dy;
                double q1[3] = {QF(q, 1, mx, j), QF(q, 2, mx, j), QF(q, 3, mx, j)};
                const int inside = fabs(y - hy->y0) <= hy->width / 2.0;
                for (ibc = 1; ibc <= mbc; ++ibc) {
                    if (inside && orc_inflow_state(p, q0hu, q1, st)) {
                        for (m = 1; m <= 3; ++m) QF(q, m, mx + ibc, j) = st[m - 1];
                    } else {
                        AF(aux, 1, mx + ibc, j) = AF(aux, 1, mx + 1 - ibc, j);
                        for (m = 1; m <= 3; ++m) QF(q, m, mx + ibc, j) = QF(q, m, mx + 1 - ibc, j);
                        QF(q, 2, mx + ibc, j) = -QF(q, 2, mx + 1 - ibc, j);
                    }
                }
            }
        }
        break;
    case 1:
        for (j = 1 - mbc; j <= my + mbc; ++j)
            for (ibc = 1; ibc <= mbc; ++ibc) {
                AF(aux, 1, mx + ibc, j) = AF(aux, 1, mx, j);
                for (m = 1; m <= 3; ++m) QF(q, m, mx + ibc, j) = QF(q, m, mx, j);
            }
        break;
    case 3:
        for (j = 1 - mbc; j <= my + mbc; ++j)
            for (ibc = 1; ibc <= mbc; ++ibc) {
                AF(aux, 1, mx + ibc, j) = AF(aux, 1, mx + 1 - ibc, j);
                for (m = 1; m <= 3; ++m) QF(q, m, mx + ibc, j) = QF(q, m, mx + 1 - ibc, j);
            }
        for (j = 1 - mbc; j <= my + mbc; ++j)
            for (ibc = 1; ibc <= mbc; ++ibc) QF(q, 2, mx + ibc, j) = -QF(q, 2, mx + 1 - ibc, j);
        break;
    default:
        break;
    }

    /* bottom boundary (the reference tests boundary_location(4) here) */
    switch (mthbc[2]) {
    case 0:
        if (hyd && hy->side[2]) {
            for (i = 1 - mbc; i <= mx + mbc; ++i) {
                const double x = xlower + (i - 0.5) * dx;
                double q1[3] = {QF(q, 1, i, 1), QF(q, 2, i, 1), QF(q, 3, i, 1)};
                const int inside = fabs(x - hy->x0) <= hy->width / 2.0;
                for (jbc = 1; jbc <= mbc; ++jbc) {
                    if (inside && orc_inflow_state(p, q0hu, q1, st)) {
                        for (m = 1; m <= 3; ++m) QF(q, m, i, 1 - jbc) = st[m - 1];
                    } else {
                        AF(aux, 1, i, 1 - jbc) = AF(aux, 1, i, jbc);
                        for (m = 1; m <= 3; ++m) QF(q, m, i, 1 - jbc) = QF(q, m, i, jbc);
                        QF(q, 3, i, 1 - jbc) = -QF(q, 3, i, jbc);
                    }
                }
            }
        }
        break;
    case 1:
        for (jbc = 1; jbc <= mbc; ++jbc)
            for (i = 1 - mbc; i <= mx + mbc; ++i) {
                AF(aux, 1, i, 1 - jbc) = AF(aux, 1, i, 1);
                for (m = 1; m <= 3; ++m) QF(q, m, i, 1 - jbc) = QF(q, m, i, 1);
            }
        break;
    case 3:
        for (jbc = 1; jbc <= mbc; ++jbc)
            for (i = 1 - mbc; i <= mx + mbc; ++i) {
                AF(aux, 1, i, 1 - jbc) = AF(aux, 1, i, jbc);
                for (m = 1; m <= 3; ++m) QF(q, m, i, 1 - jbc) = QF(q, m, i, jbc);
            }
        for (jbc = 1; jbc <= mbc; ++jbc)
            for (i = 1 - mbc; i <= mx + mbc; ++i) QF(q, 3, i, 1 - jbc) = -QF(q, 3, i, jbc);
        break;
    default:
        break;
    }

    /* top boundary (the reference tests boundary_location(3) here) */
    switch (mthbc[3]) {
    case 0:
        if (hyd && hy->side[3]) {
            for (i = 1 - mbc; i <= mx + mbc; ++i) {
                const double x = xlower + (i - 0.5) * dx;
                double q1[3] = {QF(q, 1, i, my), QF(q, 2, i, my), QF(q, 3, i, my)};
                const int inside = fabs(x - hy->x0) <= hy->width / 2.0;
                for (jbc = 1; jbc <= mbc; ++jbc) {
                    if (inside && orc_inflow_state(p, q0hu, q1, st)) {
                        for (m = 1; m <= 3; ++m) QF(q, m, i, my + jbc) = st[m - 1];
                    } else {
                        AF(aux, 1, i, my + jbc) = AF(aux, 1, i, my + 1 - jbc);
                        for (m = 1; m <= 3; ++m) QF(q, m, i, my + jbc) = QF(q, m, i, my + 1 - jbc);
                        QF(q, 3, i, my + jbc) = -QF(q, 3, i, my + 1 - jbc);
                    }
                }
            }
        }
        break;
    case 1:
        for (jbc = 1; jbc <= mbc; ++jbc)
            for (i = 1 - mbc; i <= mx + mbc; ++i) {
                AF(aux, 1, i, my + jbc) = AF(aux, 1, i, my);
                for (m = 1; m <= 3; ++m) QF(q, m, i, my + jbc) = QF(q, m, i, my);
            }
        break;
    case 3:
        for (jbc = 1; jbc <= mbc; ++jbc)
            for (i = 1 - mbc; i <= mx + mbc; ++i) {
                AF(aux, 1, i, my + jbc) = AF(aux, 1, i, my + 1 - jbc);
                for (m = 1; m <= 3; ++m) QF(q, m, i, my + jbc) = QF(q, m, i, my + 1 - jbc);
            }
        for (jbc = 1; jbc <= mbc; ++jbc)
            for (i = 1 - mbc; i <= mx + mbc; ++i) QF(q, 3, i, my + jbc) = -QF(q, 3, i, my + 1 - jbc);
        break;
    default:
        break;
    }
}

void orc_copy_face(int mx, int my, int mbc, int meqn, double* qthis, const double* qneighbor,
                   int iface)
{
    int i, j, ibc, jbc, mq;
    (void)meqn;
    for (mq = 1; mq <= MEQN; ++mq) {
        if (iface / 2 == 0) {
            for (j = 1; j <= my; ++j)
                for (ibc = 1; ibc <= mbc; ++ibc) {
                    if (iface == 0) QF(qthis, mq, 1 - ibc, j) = QF(qneighbor, mq, mx + 1 - ibc, j);
                    else QF(qthis, mq, mx + ibc, j) = QF(qneighbor, mq, ibc, j);
                }
        } else {
            for (jbc = 1; jbc <= mbc; ++jbc)
                for (i = 1; i <= mx; ++i) {
                    if (iface == 2) QF(qthis, mq, i, 1 - jbc) = QF(qneighbor, mq, i, my + 1 - jbc);
                    else QF(qthis, mq, i, my + jbc) = QF(qneighbor, mq, i, jbc);
                }
        }
    }
}

void orc_copy_corner(int mx, int my, int mbc, int meqn, double* qthis, const double* qneighbor,
                     int icorner)
{
    int mq, ibc, jbc;
    (void)meqn;
    for (mq = 1; mq <= MEQN; ++mq)
        for (ibc = 1; ibc <= mbc; ++ibc)
            for (jbc = 1; jbc <= mbc; ++jbc) {
                int i1, j1, i2, j2;
                if (icorner == 0) { i1 = 1 - ibc; j1 = 1 - jbc; i2 = mx + 1 - ibc; j2 = my + 1 - jbc; }
                else if (icorner == 1) { i1 = mx + ibc; j1 = 1 - jbc; i2 = ibc; j2 = my + 1 - jbc; }
                else if (icorner == 2) { i1 = 1 - ibc; j1 = my + jbc; i2 = mx + 1 - ibc; j2 = jbc; }
                else { i1 = mx + ibc; j1 = my + jbc; i2 = ibc; j2 = jbc; }
                QF(qthis, mq, i1, j1) = QF(qneighbor, mq, i2, j2);
            }
}

void orc_level_ghost_fill(const orc_params* p, const orc_hydro* hy, int npatch, int mbc, int mx,
                          int my, double* q, double* aux, int maux, const int* nbr,
                          const double* xlower, const double* ylower, double dx, double dy,
                          double t, const int* mthbc)
{
    const long qs = (long)MEQN * (mx + 2 * mbc) * (my + 2 * mbc);
    const long as = (long)maux * (mx + 2 * mbc) * (my + 2 * mbc);
    int k, s;
    for (k = 0; k < npatch; ++k) {
        for (s = 0; s < 4; ++s)
            if (nbr[8 * k + s] >= 0)
                orc_copy_face(mx, my, mbc, MEQN, q + k * qs, q + (long)nbr[8 * k + s] * qs, s);
        for (s = 0; s < 4; ++s)
            if (nbr[8 * k + 4 + s] >= 0)
                orc_copy_corner(mx, my, mbc, MEQN, q + k * qs, q + (long)nbr[8 * k + 4 + s] * qs, s);
    }
    for (k = 0; k < npatch; ++k) {
        int mb[4];
        int any = 0;
        for (s = 0; s < 4; ++s) {
            mb[s] = nbr[8 * k + s] == -1 ? mthbc[s] : -1;
            any |= mb[s] >= 0;
        }
        if (any)
            orc_bc2(p, hy, mbc, mx, my, xlower[k], ylower[k], dx, dy, q + k * qs, aux + k * as, maux, t,
                    mb);
    }
}
