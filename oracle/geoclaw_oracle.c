/*
 * CPU oracle for the GeoClaw patch update -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference's Fortran patch update. Every routine
 * cites the reference file:line it follows (paths relative to the GeoFlood
 * source tree). Compiled with -ffp-contract=off so that each Fortran
 * expression is evaluated as written (no fused multiply-add).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this code, and only as the checker / the timed CPU reference.
 */
#include "geoclaw_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MEQN 3
#define MWAVES 3

/* Fortran-style 1-based, offset-origin accessors.
 *   q(m, i, j), i in 1-mbc..mx+mbc, j in 1-mbc..my+mbc               */
#define QF(q, m, i, j) \
    (q)[((m) - 1) + MEQN * (((i) + mbc - 1) + (mx + 2 * mbc) * ((j) + mbc - 1))]
#define AF(a, m, i, j) \
    (a)[((m) - 1) + maux * (((i) + mbc - 1) + (mx + 2 * mbc) * ((j) + mbc - 1))]
/* 1-D slice arrays a(meqn, 1-mbc:maxm+mbc) etc. (base index 1-mbc). */
#define S1(a, m, i) (a)[((m) - 1) + MEQN * ((i) + mbc - 1)]
#define SA(a, m, i) (a)[((m) - 1) + maux * ((i) + mbc - 1)]
#define SS(a, mw, i) (a)[((mw) - 1) + MWAVES * ((i) + mbc - 1)]
#define SW(a, m, mw, i) (a)[((m) - 1) + MEQN * (((mw) - 1) + MWAVES * ((i) + mbc - 1))]
#define S0(a, i) (a)[(i) + mbc - 1]

static double dmax(double a, double b) { return a > b ? a : b; }
static double dmin(double a, double b) { return a < b ? a : b; }
/* Fortran MAX/MIN as gfortran evaluates them for ordered operands. */
static double fsign(double a, double b) { return copysign(fabs(a), b); }

void orc_default_params(orc_params* p)
{
    memset(p, 0, sizeof(*p));
    p->grav = 9.81;
    p->dry_tolerance = 1.0e-3;
    p->sea_level = 0.0;
    p->friction_depth = 1.0e6;
    p->friction_forcing = 1;
    p->num_manning = 1;
    p->manning_coefficient[0] = 0.035;
    p->manning_break[0] = 1.0e10;
    p->variable_friction = 0;
    p->friction_index = 0;
    p->order = 2;
    p->transverse = 2;
    p->mthlim[0] = p->mthlim[1] = p->mthlim[2] = 4;
    p->src_term = 1;
    p->maxcfl_cap = 100.0;
}

/* ------------------------------------------------------------------------
 * riemanntype -- geoclaw_riemann_utils.f:566-677
 * ---------------------------------------------------------------------- */
void orc_riemanntype(double hL, double hR, double uL, double uR, double* hm_out,
                     double* s1m_out, double* s2m_out, int* rare1,
                     int* rare2, int maxiter, double drytol, double g)
{
    double hm, u1m, u2m, um, delu;
    double h_max, h_min, h0, F_max, F_min, dfdh, F0, slope, gL, gR;
    double s1m, s2m;
    int iter;
    (void)um;

    h_min = dmin(hR, hL);
    h_max = dmax(hR, hL);
    delu = uR - uL;

    if (h_min <= drytol) {
        hm = 0.0;
        um = 0.0;
        s1m = uR + uL - 2.0 * sqrt(g * hR) + 2.0 * sqrt(g * hL);
        s2m = uR + uL - 2.0 * sqrt(g * hR) + 2.0 * sqrt(g * hL);
        if (hL <= 0.0) {
            *rare2 = 1;
            *rare1 = 0;
        } else {
            *rare1 = 1;
            *rare2 = 0;
        }
    } else {
        F_min = delu + 2.0 * (sqrt(g * h_min) - sqrt(g * h_max));
        F_max = delu + (h_max - h_min) *
                           (sqrt(.5 * g * (h_max + h_min) / (h_max * h_min)));

        if (F_min > 0.0) { /* 2-rarefactions */
            double t = dmax(0.0, -delu + 2.0 * (sqrt(g * hL) + sqrt(g * hR)));
            hm = (1.0 / (16.0 * g)) * (t * t);
            um = fsign(1.0, hm) * (uL + 2.0 * (sqrt(g * hL) - sqrt(g * hm)));
            s1m = uL + 2.0 * sqrt(g * hL) - 3.0 * sqrt(g * hm);
            s2m = uR - 2.0 * sqrt(g * hR) + 3.0 * sqrt(g * hm);
            *rare1 = 1;
            *rare2 = 1;
        } else if (F_max <= 0.0) { /* 2 shocks */
            h0 = h_max;
            for (iter = 1; iter <= maxiter; ++iter) {
                gL = sqrt(.5 * g * (1 / h0 + 1 / hL));
                gR = sqrt(.5 * g * (1 / h0 + 1 / hR));
                F0 = delu + (h0 - hL) * gL + (h0 - hR) * gR;
                dfdh = gL - g * (h0 - hL) / (4.0 * (h0 * h0) * gL) + gR -
                       g * (h0 - hR) / (4.0 * (h0 * h0) * gR);
                slope = 2.0 * sqrt(h0) * dfdh;
                {
                    double t = sqrt(h0) - F0 / slope;
                    h0 = t * t;
                }
            }
            hm = h0;
            u1m = uL - (hm - hL) * sqrt((.5 * g) * (1 / hm + 1 / hL));
            u2m = uR + (hm - hR) * sqrt((.5 * g) * (1 / hm + 1 / hR));
            um = .5 * (u1m + u2m);
            s1m = u1m - sqrt(g * hm);
            s2m = u2m + sqrt(g * hm);
            *rare1 = 0;
            *rare2 = 0;
        } else { /* one shock one rarefaction */
            h0 = h_min;
            for (iter = 1; iter <= maxiter; ++iter) {
                F0 = delu + 2.0 * (sqrt(g * h0) - sqrt(g * h_max)) +
                     (h0 - h_min) * sqrt(.5 * g * (1 / h0 + 1 / h_min));
                slope = (F_max - F0) / (h_max - h_min);
                h0 = h0 - F0 / slope;
            }
            hm = h0;
            if (hL > hR) {
                um = uL + 2.0 * sqrt(g * hL) - 2.0 * sqrt(g * hm);
                s1m = uL + 2.0 * sqrt(g * hL) - 3.0 * sqrt(g * hm);
                s2m = uL + 2.0 * sqrt(g * hL) - sqrt(g * hm);
                *rare1 = 1;
                *rare2 = 0;
            } else {
                s2m = uR - 2.0 * sqrt(g * hR) + 3.0 * sqrt(g * hm);
                s1m = uR - 2.0 * sqrt(g * hR) + sqrt(g * hm);
                um = uR - 2.0 * sqrt(g * hR) + 2.0 * sqrt(g * hm);
                *rare2 = 1;
                *rare1 = 0;
            }
        }
    }
    *hm_out = hm;
    *s1m_out = s1m;
    *s2m_out = s2m;
}

/* ------------------------------------------------------------------------
 * riemann_aug_JCP -- geoclaw_riemann_utils.f:2-311 (called with maxiter=1
 * from rpn2_geoclaw.f:279-283). fw is fw(3,3) column-major: fw[(m-1)+3(mw-1)].
 * ---------------------------------------------------------------------- */
void orc_riemann_aug_JCP(int maxiter, double hL, double hR, double huL,
                         double huR, double hvL, double hvR, double bL,
                         double bR, double uL, double uR, double vL,
                         double vR, double phiL, double phiR, double sE1,
                         double sE2, double drytol, double g, double* sw,
                         double* fw)
{
    double A[3][3], r[3][3], lambda[3], del[3], beta[3];
    double delh, delhu, delphi, delb, delnorm;
    double criticaltol, convergencetol, criticaltol_2, hustar_interface;
    double s1s2bar, s1s2tilde, hbar, hLstar, hRstar, huRstar, huLstar;
    double uRstar, uLstar, hstarHLL, deldelh, deldelphi;
    double s1m, s2m, hm, det1, det2, det3, determinant;
    int rare1, rare2, rarecorrector, sonic;
    int k, mw, iter;
    (void)hvL;
    (void)hvR;

#define R(a, b) r[(a) - 1][(b) - 1]
#define AA(a, b) A[(a) - 1][(b) - 1]
#define FW(m, mw) fw[((m) - 1) + 3 * ((mw) - 1)]

    delh = hR - hL;
    delhu = huR - huL;
    delphi = phiR - phiL;
    delb = bR - bL;
    delnorm = delh * delh + delphi * delphi;

    orc_riemanntype(hL, hR, uL, uR, &hm, &s1m, &s2m, &rare1, &rare2, 1,
                    drytol, g);

    lambda[0] = dmin(sE1, s2m);
    lambda[2] = dmax(sE2, s1m);
    sE1 = lambda[0];
    sE2 = lambda[2];
    lambda[1] = 0.0;

    hstarHLL = dmax((huL - huR + sE2 * hR - sE1 * hL) / (sE2 - sE1), 0.0);

    /* rarecorrectortest is .false. (geoclaw_riemann_utils.f:89-114) */
    rarecorrector = 0;

    for (mw = 1; mw <= 3; ++mw) {
        R(1, mw) = 1.0;
        R(2, mw) = lambda[mw - 1];
        R(3, mw) = lambda[mw - 1] * lambda[mw - 1];
    }
    if (!rarecorrector) {
        lambda[1] = 0.5 * (lambda[0] + lambda[2]);
        R(1, 2) = 0.0;
        R(2, 2) = 0.0;
        R(3, 2) = 1.0;
    }

    criticaltol = dmax(drytol * g, 1e-6);
    criticaltol_2 = sqrt(criticaltol);
    deldelh = -delb;
    deldelphi = -0.5 * (hR + hL) * (g * delb);

    hLstar = hL;
    hRstar = hR;
    uLstar = uL;
    uRstar = uR;
    huLstar = uLstar * hLstar;
    huRstar = uRstar * hRstar;

    convergencetol = 1.e-6;
    for (iter = 1; iter <= maxiter; ++iter) {
        if (dmin(hLstar, hRstar) < drytol && rarecorrector) {
            rarecorrector = 0;
            hLstar = hL;
            hRstar = hR;
            uLstar = uL;
            uRstar = uR;
            huLstar = uLstar * hLstar;
            huRstar = uRstar * hRstar;
            lambda[1] = 0.5 * (lambda[0] + lambda[2]);
            R(1, 2) = 0.0;
            R(2, 2) = 0.0;
            R(3, 2) = 1.0;
        }

        hbar = dmax(0.5 * (hLstar + hRstar), 0.0);
        s1s2bar = 0.25 * ((uLstar + uRstar) * (uLstar + uRstar)) - g * hbar;
        s1s2tilde = dmax(0.0, uLstar * uRstar) - g * hbar;

        sonic = 0;
        if (fabs(s1s2bar) <= criticaltol) {
            sonic = 1;
        } else if (s1s2bar * s1s2tilde <= criticaltol * criticaltol) {
            sonic = 1;
        } else if (s1s2bar * sE1 * sE2 <= criticaltol * criticaltol) {
            sonic = 1;
        } else if (dmin(fabs(sE1), fabs(sE2)) < criticaltol_2) {
            sonic = 1;
        } else if (sE1 < criticaltol_2 && s1m > -criticaltol_2) {
            sonic = 1;
        } else if (sE2 > -criticaltol_2 && s2m < criticaltol_2) {
            sonic = 1;
        } else if ((uL + sqrt(g * hL)) * (uR + sqrt(g * hR)) < 0.0) {
            sonic = 1;
        } else if ((uL - sqrt(g * hL)) * (uR - sqrt(g * hR)) < 0.0) {
            sonic = 1;
        }

        if (sonic) {
            deldelh = -delb;
        } else {
            deldelh = delb * g * hbar / s1s2bar;
        }
        if (sE1 < -criticaltol && sE2 > criticaltol) {
            deldelh = dmin(deldelh, hstarHLL * (sE2 - sE1) / sE2);
            deldelh = dmax(deldelh, hstarHLL * (sE2 - sE1) / sE1);
        } else if (sE1 >= criticaltol) {
            deldelh = dmin(deldelh, hstarHLL * (sE2 - sE1) / sE1);
            deldelh = dmax(deldelh, -hL);
        } else if (sE2 <= -criticaltol) {
            deldelh = dmin(deldelh, hR);
            deldelh = dmax(deldelh, hstarHLL * (sE2 - sE1) / sE2);
        }

        if (sonic) {
            deldelphi = -g * hbar * delb;
        } else {
            deldelphi = -delb * g * hbar * s1s2tilde / s1s2bar;
        }
        deldelphi = dmin(deldelphi, g * dmax(-hLstar * delb, -hRstar * delb));
        deldelphi = dmax(deldelphi, g * dmin(-hLstar * delb, -hRstar * delb));

        del[0] = delh - deldelh;
        del[1] = delhu;
        del[2] = delphi - deldelphi;

        det1 = R(1, 1) * (R(2, 2) * R(3, 3) - R(2, 3) * R(3, 2));
        det2 = R(1, 2) * (R(2, 1) * R(3, 3) - R(2, 3) * R(3, 1));
        det3 = R(1, 3) * (R(2, 1) * R(3, 2) - R(2, 2) * R(3, 1));
        determinant = det1 - det2 + det3;

        for (k = 1; k <= 3; ++k) {
            for (mw = 1; mw <= 3; ++mw) {
                AA(1, mw) = R(1, mw);
                AA(2, mw) = R(2, mw);
                AA(3, mw) = R(3, mw);
            }
            AA(1, k) = del[0];
            AA(2, k) = del[1];
            AA(3, k) = del[2];
            det1 = AA(1, 1) * (AA(2, 2) * AA(3, 3) - AA(2, 3) * AA(3, 2));
            det2 = AA(1, 2) * (AA(2, 1) * AA(3, 3) - AA(2, 3) * AA(3, 1));
            det3 = AA(1, 3) * (AA(2, 1) * AA(3, 2) - AA(2, 2) * AA(3, 1));
            beta[k - 1] = (det1 - det2 + det3) / determinant;
        }

        if (fabs(del[0] * del[0] + del[2] * del[2] - delnorm) < convergencetol)
            break;
        delnorm = del[0] * del[0] + del[2] * del[2];
        hLstar = hL;
        hRstar = hR;
        uLstar = uL;
        uRstar = uR;
        huLstar = uLstar * hLstar;
        huRstar = uRstar * hRstar;
        for (mw = 1; mw <= 3; ++mw) {
            if (lambda[mw - 1] < 0.0) {
                hLstar = hLstar + beta[mw - 1] * R(1, mw);
                huLstar = huLstar + beta[mw - 1] * R(2, mw);
            }
        }
        for (mw = 3; mw >= 1; --mw) {
            if (lambda[mw - 1] > 0.0) {
                hRstar = hRstar - beta[mw - 1] * R(1, mw);
                huRstar = huRstar - beta[mw - 1] * R(2, mw);
            }
        }
        if (hLstar > drytol) {
            uLstar = huLstar / hLstar;
        } else {
            hLstar = dmax(hLstar, 0.0);
            uLstar = 0.0;
        }
        if (hRstar > drytol) {
            uRstar = huRstar / hRstar;
        } else {
            hRstar = dmax(hRstar, 0.0);
            uRstar = 0.0;
        }
    }

    for (mw = 1; mw <= 3; ++mw) {
        sw[mw - 1] = lambda[mw - 1];
        FW(1, mw) = beta[mw - 1] * R(2, mw);
        FW(2, mw) = beta[mw - 1] * R(3, mw);
        FW(3, mw) = beta[mw - 1] * R(2, mw);
    }
    FW(3, 1) = FW(3, 1) * vL;
    FW(3, 3) = FW(3, 3) * vR;
    FW(3, 2) = 0.0;

    hustar_interface = huL + FW(1, 1);
    if (hustar_interface <= 0.0) {
        FW(3, 1) = FW(3, 1) + (hR * uR * vR - hL * uL * vL - FW(3, 1) - FW(3, 3));
    } else {
        FW(3, 3) = FW(3, 3) + (hR * uR * vR - hL * uL * vL - FW(3, 1) - FW(3, 3));
    }
#undef R
#undef AA
#undef FW
}

/* ------------------------------------------------------------------------
 * rpn2 -- rpn2_geoclaw.f:84-376 (ql = qr = q1d, auxl = auxr = aux2;
 * mcapa = 0 so the latitude-longitude block at :334-353 is skipped).
 * ---------------------------------------------------------------------- */
void orc_rpn2(const orc_params* p, int ixy, int mbc, int mx, double* q1d,
              const double* aux1d, int maux, double* fwave, double* s,
              double* amdq, double* apdq)
{
    const double g = p->grav, drytol = p->dry_tolerance;
    double wall[3], fw[9], sw[3];
    double hR, hL, huR, huL, uR, uL, hvR, hvL, vR, vL, phiR, phiL;
    double bR, bL, sL, sR, sRoe1, sRoe2, sE1, sE2, uhat, chat;
    double s1m, s2m, hstar, hstartest;
    int rare1, rare2;
    int i, m, mw, mu, nv;

    for (i = 2 - mbc; i <= mx + mbc; ++i) {
        for (mw = 1; mw <= MWAVES; ++mw) {
            SS(s, mw, i) = 0.0;
            SW(fwave, 1, mw, i) = 0.0;
            SW(fwave, 2, mw, i) = 0.0;
            SW(fwave, 3, mw, i) = 0.0;
        }
        if (ixy == 1) {
            mu = 2;
            nv = 3;
        } else {
            mu = 3;
            nv = 2;
        }
        if (S1(q1d, 1, i - 1) < 0.0) {
            S1(q1d, 1, i - 1) = 0.0;
            S1(q1d, 2, i - 1) = 0.0;
            S1(q1d, 3, i - 1) = 0.0;
        }
        if (S1(q1d, 1, i) < 0.0) {
            S1(q1d, 1, i) = 0.0;
            S1(q1d, 2, i) = 0.0;
            S1(q1d, 3, i) = 0.0;
        }
        if (S1(q1d, 1, i - 1) <= drytol && S1(q1d, 1, i) <= drytol) continue;

        hL = S1(q1d, 1, i - 1);
        hR = S1(q1d, 1, i);
        huL = S1(q1d, mu, i - 1);
        huR = S1(q1d, mu, i);
        bL = SA(aux1d, 1, i - 1);
        bR = SA(aux1d, 1, i);
        hvL = S1(q1d, nv, i - 1);
        hvR = S1(q1d, nv, i);

        if (hR > drytol) {
            uR = huR / hR;
            vR = hvR / hR;
            phiR = 0.5 * g * (hR * hR) + (huR * huR) / hR;
        } else {
            hR = 0.0;
            huR = 0.0;
            hvR = 0.0;
            uR = 0.0;
            vR = 0.0;
            phiR = 0.0;
        }
        if (hL > drytol) {
            uL = huL / hL;
            vL = hvL / hL;
            phiL = 0.5 * g * (hL * hL) + (huL * huL) / hL;
        } else {
            hL = 0.0;
            huL = 0.0;
            hvL = 0.0;
            uL = 0.0;
            vL = 0.0;
            phiL = 0.0;
        }

        wall[0] = 1.0;
        wall[1] = 1.0;
        wall[2] = 1.0;
        if (hR <= drytol) {
            orc_riemanntype(hL, hL, uL, -uL, &hstar, &s1m, &s2m, &rare1,
                            &rare2, 1, drytol, g);
            hstartest = dmax(hL, hstar);
            if (hstartest + bL < bR) {
                wall[1] = 0.0;
                wall[2] = 0.0;
                hR = hL;
                huR = -huL;
                bR = bL;
                phiR = phiL;
                uR = -uL;
                vR = vL;
            } else if (hL + bL < bR) {
                bR = hL + bL;
            }
        } else if (hL <= drytol) {
            orc_riemanntype(hR, hR, -uR, uR, &hstar, &s1m, &s2m, &rare1,
                            &rare2, 1, drytol, g);
            hstartest = dmax(hR, hstar);
            if (hstartest + bR < bL) {
                wall[0] = 0.0;
                wall[1] = 0.0;
                hL = hR;
                huL = -huR;
                bL = bR;
                phiL = phiR;
                uL = -uR;
                vL = vR;
            } else if (hR + bR < bL) {
                bL = hR + bR;
            }
        }

        sL = uL - sqrt(g * hL);
        sR = uR + sqrt(g * hR);
        uhat = (sqrt(g * hL) * uL + sqrt(g * hR) * uR) /
               (sqrt(g * hR) + sqrt(g * hL));
        chat = sqrt(g * 0.5 * (hR + hL));
        sRoe1 = uhat - chat;
        sRoe2 = uhat + chat;
        sE1 = dmin(sL, sRoe1);
        sE2 = dmax(sR, sRoe2);

        orc_riemann_aug_JCP(1, hL, hR, huL, huR, hvL, hvR, bL, bR, uL, uR,
                            vL, vR, phiL, phiR, sE1, sE2, drytol, g, sw, fw);

        for (mw = 1; mw <= 3; ++mw) {
            sw[mw - 1] = sw[mw - 1] * wall[mw - 1];
            fw[0 + 3 * (mw - 1)] = fw[0 + 3 * (mw - 1)] * wall[mw - 1];
            fw[1 + 3 * (mw - 1)] = fw[1 + 3 * (mw - 1)] * wall[mw - 1];
            fw[2 + 3 * (mw - 1)] = fw[2 + 3 * (mw - 1)] * wall[mw - 1];
        }
        for (mw = 1; mw <= MWAVES; ++mw) {
            SS(s, mw, i) = sw[mw - 1];
            SW(fwave, 1, mw, i) = fw[0 + 3 * (mw - 1)];
            SW(fwave, mu, mw, i) = fw[1 + 3 * (mw - 1)];
            SW(fwave, nv, mw, i) = fw[2 + 3 * (mw - 1)];
        }
    }

    /* fluctuations (rpn2_geoclaw.f:359-376) */
    for (i = 1 - mbc; i <= mx + mbc; ++i)
        for (m = 1; m <= 3; ++m) {
            S1(amdq, m, i) = 0.0;
            S1(apdq, m, i) = 0.0;
        }
    for (i = 2 - mbc; i <= mx + mbc; ++i) {
        for (mw = 1; mw <= MWAVES; ++mw) {
            if (SS(s, mw, i) < 0.0) {
                for (m = 1; m <= 3; ++m)
                    S1(amdq, m, i) = S1(amdq, m, i) + SW(fwave, m, mw, i);
            } else if (SS(s, mw, i) > 0.0) {
                for (m = 1; m <= 3; ++m)
                    S1(apdq, m, i) = S1(apdq, m, i) + SW(fwave, m, mw, i);
            } else {
                for (m = 1; m <= 3; ++m) {
                    S1(amdq, m, i) = S1(amdq, m, i) + 0.5 * SW(fwave, m, mw, i);
                    S1(apdq, m, i) = S1(apdq, m, i) + 0.5 * SW(fwave, m, mw, i);
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------
 * rpt2 -- rpt2_geoclaw.f:46-187 (coordinate_system = 1, Cartesian).
 * ---------------------------------------------------------------------- */
void orc_rpt2(const orc_params* p, int ixy, int imp, int mbc, int mx,
              const double* q1d, const double* aux1, const double* aux2,
              const double* aux3, int maux, const double* asdq,
              double* bmasdq, double* bpasdq)
{
    const double g = p->grav, tol = p->dry_tolerance;
    double s[3], r[3][3], beta[3];
    double h, u, v, delf1, delf2, delf3, dxdcm, dxdcp, topo1, topo3, eta;
    int i, m, mw, mu, mv;

    if (ixy == 1) {
        mu = 2;
        mv = 3;
    } else {
        mu = 3;
        mv = 2;
    }
    for (i = 1 - mbc; i <= mx + mbc; ++i)
        for (m = 1; m <= 3; ++m) {
            S1(bmasdq, m, i) = 0.0;
            S1(bpasdq, m, i) = 0.0;
        }

    for (i = 2 - mbc; i <= mx + mbc; ++i) {
        int ic = (imp == 1) ? i - 1 : i;
        h = S1(q1d, 1, ic);
        if (h <= tol) continue;
        u = S1(q1d, mu, ic) / h;
        v = S1(q1d, mv, ic) / h;
        eta = h + SA(aux2, 1, ic);
        topo1 = SA(aux1, 1, ic);
        topo3 = SA(aux3, 1, ic);

        if (eta < dmin(topo1, topo3)) continue;

        dxdcp = 1.0;
        dxdcm = 1.0;

        s[0] = v - sqrt(g * h);
        s[1] = v;
        s[2] = v + sqrt(g * h);

        delf1 = S1(asdq, 1, i);
        delf2 = S1(asdq, mu, i);
        delf3 = S1(asdq, mv, i);

        beta[0] = (s[2] * delf1 - delf3) / (s[2] - s[0]);
        beta[1] = -u * delf1 + delf2;
        beta[2] = (delf3 - s[0] * delf1) / (s[2] - s[0]);

        r[0][0] = 1.0; /* r(1,1) */
        r[1][0] = u;   /* r(2,1) */
        r[2][0] = s[0];
        r[0][1] = 0.0;
        r[1][1] = 1.0;
        r[2][1] = 0.0;
        r[0][2] = 1.0;
        r[1][2] = u;
        r[2][2] = s[2];

        for (mw = 0; mw < 3; ++mw) {
            if (s[mw] < 0.0 && eta >= topo1) {
                S1(bmasdq, 1, i) = S1(bmasdq, 1, i) + dxdcm * s[mw] * beta[mw] * r[0][mw];
                S1(bmasdq, mu, i) = S1(bmasdq, mu, i) + dxdcm * s[mw] * beta[mw] * r[1][mw];
                S1(bmasdq, mv, i) = S1(bmasdq, mv, i) + dxdcm * s[mw] * beta[mw] * r[2][mw];
            } else if (s[mw] > 0.0 && eta >= topo3) {
                S1(bpasdq, 1, i) = S1(bpasdq, 1, i) + dxdcp * s[mw] * beta[mw] * r[0][mw];
                S1(bpasdq, mu, i) = S1(bpasdq, mu, i) + dxdcp * s[mw] * beta[mw] * r[1][mw];
                S1(bpasdq, mv, i) = S1(bpasdq, mv, i) + dxdcp * s[mw] * beta[mw] * r[2][mw];
            }
        }
    }
}

/* ------------------------------------------------------------------------
 * philim -- philim.f:4-65 (computed GOTO falls through to minmod for an
 * out-of-range meth).
 * ---------------------------------------------------------------------- */
static double orc_philim(double a, double b, int meth)
{
    double r, c;
    if (a == 0.0) return 0.0;
    r = b / a;
    switch (meth) {
    case 2:
        return dmax(dmax(0.0, dmin(1.0, 2.0 * r)), dmin(2.0, r));
    case 3:
        return (r + fabs(r)) / (1.0 + fabs(r));
    case 4:
        c = (1.0 + r) / 2.0;
        return dmax(0.0, dmin(dmin(c, 2.0), 2.0 * r));
    case 5:
        return r;
    case 1:
    default:
        return dmax(0.0, dmin(1.0, r));
    }
}

/* limiter -- geoclaw_limiter_fort.f:34-58 */
static void orc_limiter(int mbc, int mx, double* wave, const double* s,
                        const int* mthlim)
{
    int mw, i, m;
    double dotr, dotl, wnorm2, wlimitr;
    for (mw = 1; mw <= MWAVES; ++mw) {
        if (mthlim[mw - 1] == 0) continue;
        dotr = 0.0;
        for (i = 0; i <= mx + 1; ++i) {
            wnorm2 = 0.0;
            dotl = dotr;
            dotr = 0.0;
            for (m = 1; m <= MEQN; ++m) {
                wnorm2 = wnorm2 + SW(wave, m, mw, i) * SW(wave, m, mw, i);
                dotr = dotr + SW(wave, m, mw, i) * SW(wave, m, mw, i + 1);
            }
            if (i == 0) continue;
            if (wnorm2 == 0.0) continue;
            if (SS(s, mw, i) > 0.0)
                wlimitr = orc_philim(wnorm2, dotl, mthlim[mw - 1]);
            else
                wlimitr = orc_philim(wnorm2, dotr, mthlim[mw - 1]);
            for (m = 1; m <= MEQN; ++m)
                SW(wave, m, mw, i) = wlimitr * SW(wave, m, mw, i);
        }
    }
}

/* ------------------------------------------------------------------------
 * flux2 -- geoclaw_flux2fw_fort.f:113-267 (coordinate_system = 1,
 * relimit = .false.). The slice arrays are sized 1-mbc..mx+mbc.
 * ---------------------------------------------------------------------- */
typedef struct orc_work {
    double *fwave, *s, *amdq, *apdq, *bmasdq, *bpasdq, *cqxx;
    int n1; /* slice length maxm + 2*mbc (stride of the jside index) */
} orc_work;

static void orc_flux2(const orc_params* p, int ixy, int mbc, int mx,
                      double* q1d, double* dtdx1d, const double* aux1,
                      const double* aux2, const double* aux3, int maux,
                      double* faddm, double* faddp, double* gaddm,
                      double* gaddp, double* cfl1d, orc_work* w)
{
    double *fwave = w->fwave, *s = w->s, *amdq = w->amdq, *apdq = w->apdq;
    double *bmasdq = w->bmasdq, *bpasdq = w->bpasdq, *cqxx = w->cqxx;
    const int n = w->n1;
    int limit = 0, i, m, mw, jside;
    double gupdate;
    /* gaddm(meqn, 1-mbc:maxm+mbc, 2): jside stride = 3*n */
#define G2(a, m, i, js) (a)[((m) - 1) + MEQN * ((i) + mbc - 1) + MEQN * n * ((js) - 1)]

    for (mw = 1; mw <= MWAVES; ++mw)
        if (p->mthlim[mw - 1] > 0) limit = 1;

    for (jside = 1; jside <= 2; ++jside)
        for (i = 1 - mbc; i <= mx + mbc; ++i)
            for (m = 1; m <= MEQN; ++m) {
                S1(faddm, m, i) = 0.0;
                S1(faddp, m, i) = 0.0;
                G2(gaddm, m, i, jside) = 0.0;
                G2(gaddp, m, i, jside) = 0.0;
            }

    orc_rpn2(p, ixy, mbc, mx, q1d, aux2, maux, fwave, s, amdq, apdq);

    for (i = 2 - mbc; i <= mx + mbc - 1; ++i) {
        for (m = 1; m <= MEQN; ++m) {
            S1(faddp, m, i) = S1(faddp, m, i) - S1(apdq, m, i);
            S1(faddm, m, i) = S1(faddm, m, i) + S1(amdq, m, i);
        }
    }

    *cfl1d = 0.0;
    for (mw = 1; mw <= MWAVES; ++mw)
        for (i = 2 - mbc; i <= mx + mbc; ++i) {
            double a = S0(dtdx1d, i) * SS(s, mw, i);
            double b = -S0(dtdx1d, i - 1) * SS(s, mw, i);
            *cfl1d = dmax(dmax(*cfl1d, a), b);
        }

    if (p->order != 1) {
        if (limit) orc_limiter(mbc, mx, fwave, s, p->mthlim);
        for (i = 2 - mbc; i <= mx + mbc; ++i) {
            S0(dtdx1d, i - 1) = 0.5 * (S0(dtdx1d, i - 1) + S0(dtdx1d, i));
            for (m = 1; m <= MEQN; ++m) {
                S1(cqxx, m, i) = 0.0;
                for (mw = 1; mw <= MWAVES; ++mw) {
                    S1(cqxx, m, i) =
                        S1(cqxx, m, i) +
                        fsign(1.0, SS(s, mw, i)) *
                            (1.0 - fabs(SS(s, mw, i)) * S0(dtdx1d, i - 1)) *
                            SW(fwave, m, mw, i);
                }
                S1(faddm, m, i) = S1(faddm, m, i) + 0.5 * S1(cqxx, m, i);
                S1(faddp, m, i) = S1(faddp, m, i) + 0.5 * S1(cqxx, m, i);
            }
        }
    }

    if (p->transverse == 0) return;

    if (p->order > 1 && p->transverse == 2) {
        for (i = 2 - mbc; i <= mx + mbc - 1; ++i)
            for (m = 1; m <= MEQN; ++m) {
                S1(amdq, m, i) = S1(amdq, m, i) + S1(cqxx, m, i);
                S1(apdq, m, i) = S1(apdq, m, i) - S1(cqxx, m, i);
            }
    }

    orc_rpt2(p, ixy, 1, mbc, mx, q1d, aux1, aux2, aux3, maux, amdq, bmasdq,
             bpasdq);
    for (i = 2 - mbc; i <= mx + mbc; ++i)
        for (m = 1; m <= MEQN; ++m) {
            gupdate = 0.5 * S0(dtdx1d, i - 1) * S1(bmasdq, m, i);
            G2(gaddm, m, i - 1, 1) = G2(gaddm, m, i - 1, 1) - gupdate;
            G2(gaddp, m, i - 1, 1) = G2(gaddp, m, i - 1, 1) - gupdate;
            gupdate = 0.5 * S0(dtdx1d, i - 1) * S1(bpasdq, m, i);
            G2(gaddm, m, i - 1, 2) = G2(gaddm, m, i - 1, 2) - gupdate;
            G2(gaddp, m, i - 1, 2) = G2(gaddp, m, i - 1, 2) - gupdate;
        }

    orc_rpt2(p, ixy, 2, mbc, mx, q1d, aux1, aux2, aux3, maux, apdq, bmasdq,
             bpasdq);
    for (i = 2 - mbc; i <= mx + mbc; ++i)
        for (m = 1; m <= MEQN; ++m) {
            gupdate = 0.5 * S0(dtdx1d, i - 1) * S1(bmasdq, m, i);
            G2(gaddm, m, i, 1) = G2(gaddm, m, i, 1) - gupdate;
            G2(gaddp, m, i, 1) = G2(gaddp, m, i, 1) - gupdate;
            gupdate = 0.5 * S0(dtdx1d, i - 1) * S1(bpasdq, m, i);
            G2(gaddm, m, i, 2) = G2(gaddm, m, i, 2) - gupdate;
            G2(gaddp, m, i, 2) = G2(gaddp, m, i, 2) - gupdate;
        }
#undef G2
}

/* ------------------------------------------------------------------------
 * b4step2 -- geoclaw_b4step2_fort.f90:183-186 (all cells incl. ghosts).
 * ---------------------------------------------------------------------- */
void orc_b4step2(const orc_params* p, int mbc, int mx, int my, double* q)
{
    int i, j;
    for (j = 1 - mbc; j <= my + mbc; ++j)
        for (i = 1 - mbc; i <= mx + mbc; ++i)
            if (QF(q, 1, i, j) < p->dry_tolerance) {
                QF(q, 1, i, j) = dmax(QF(q, 1, i, j), 0.0);
                QF(q, 2, i, j) = 0.0;
                QF(q, 3, i, j) = 0.0;
            }
}

/* ------------------------------------------------------------------------
 * step2 -- geoclaw_step2_fort.f90:80-250 then the update of
 * geoclaw_step2_wrap_fort.f:95-115 (mcapa = 0).
 * ---------------------------------------------------------------------- */
double orc_step2(const orc_params* p, int mbc, int mx, int my, double* q,
                 const double* aux, int maux, double dx, double dy, double dt)
{
    const int maxm = mx > my ? mx : my;
    const int n1 = maxm + 2 * mbc;
    const long ncell = (long)(mx + 2 * mbc) * (my + 2 * mbc);
    double *fm, *fp, *gm, *gp, *q1d, *aux1, *aux2, *aux3, *dtdx1d;
    double *faddm, *faddp, *gaddm, *gaddp;
    double dtdx, dtdy, cfl1d, cflgrid;
    orc_work w;
    int i, j, m, k;
    double* pool;
    size_t pool_n;

    /* Flux arrays fm/fp/gm/gp (fc2d_geoclaw.cpp:309-318) and slice work. */
    pool_n = 4 * MEQN * ncell + (size_t)n1 * (MEQN * 3 + 3 * maux + 1 + 2 * MEQN * 3)
             + (size_t)n1 * (MEQN * MWAVES + MWAVES + 5 * MEQN);
    pool = (double*)calloc(pool_n, sizeof(double));
    fm = pool;
    fp = fm + MEQN * ncell;
    gm = fp + MEQN * ncell;
    gp = gm + MEQN * ncell;
    q1d = gp + MEQN * ncell;
    faddm = q1d + MEQN * n1;
    faddp = faddm + MEQN * n1;
    gaddm = faddp + MEQN * n1;
    gaddp = gaddm + 2 * MEQN * n1;
    aux1 = gaddp + 2 * MEQN * n1;
    aux2 = aux1 + maux * n1;
    aux3 = aux2 + maux * n1;
    dtdx1d = aux3 + maux * n1;
    w.fwave = dtdx1d + n1;
    w.s = w.fwave + MEQN * MWAVES * n1;
    w.amdq = w.s + MWAVES * n1;
    w.apdq = w.amdq + MEQN * n1;
    w.bmasdq = w.apdq + MEQN * n1;
    w.bpasdq = w.bmasdq + MEQN * n1;
    w.cqxx = w.bpasdq + MEQN * n1;
    w.n1 = n1;

    cflgrid = 0.0;
    dtdx = dt / dx;
    dtdy = dt / dy;

    /* x-sweeps (geoclaw_step2_fort.f90:92-169) */
    for (j = 2 - mbc; j <= my + mbc - 1; ++j) {
        for (i = 1 - mbc; i <= mx + mbc; ++i)
            for (m = 1; m <= MEQN; ++m) S1(q1d, m, i) = QF(q, m, i, j);
        for (i = 1 - mbc; i <= maxm + mbc; ++i) S0(dtdx1d, i) = dtdx;
        for (i = 1 - mbc; i <= mx + mbc; ++i)
            for (k = 1; k <= maux; ++k) {
                SA(aux1, k, i) = AF(aux, k, i, j - 1);
                SA(aux2, k, i) = AF(aux, k, i, j);
                SA(aux3, k, i) = AF(aux, k, i, j + 1);
            }
        orc_flux2(p, 1, mbc, mx, q1d, dtdx1d, aux1, aux2, aux3, maux, faddm,
                  faddp, gaddm, gaddp, &cfl1d, &w);
        cflgrid = dmax(cflgrid, cfl1d);
        for (i = 2 - mbc; i <= mx + mbc; ++i)
            for (m = 1; m <= MEQN; ++m) {
                QF(fm, m, i, j) = QF(fm, m, i, j) + S1(faddm, m, i);
                QF(fp, m, i, j) = QF(fp, m, i, j) + S1(faddp, m, i);
                QF(gm, m, i, j) = QF(gm, m, i, j) + gaddm[(m - 1) + MEQN * (i + mbc - 1)];
                QF(gp, m, i, j) = QF(gp, m, i, j) + gaddp[(m - 1) + MEQN * (i + mbc - 1)];
                QF(gm, m, i, j + 1) = QF(gm, m, i, j + 1) + gaddm[(m - 1) + MEQN * (i + mbc - 1) + MEQN * n1];
                QF(gp, m, i, j + 1) = QF(gp, m, i, j + 1) + gaddp[(m - 1) + MEQN * (i + mbc - 1) + MEQN * n1];
            }
    }

    /* y-sweeps (geoclaw_step2_fort.f90:175-250) */
    for (i = 2 - mbc; i <= mx + mbc - 1; ++i) {
        for (j = 1 - mbc; j <= my + mbc; ++j)
            for (m = 1; m <= MEQN; ++m) S1(q1d, m, j) = QF(q, m, i, j);
        for (j = 1 - mbc; j <= maxm + mbc; ++j) S0(dtdx1d, j) = dtdy;
        for (j = 1 - mbc; j <= my + mbc; ++j)
            for (k = 1; k <= maux; ++k) {
                SA(aux1, k, j) = AF(aux, k, i - 1, j);
                SA(aux2, k, j) = AF(aux, k, i, j);
                SA(aux3, k, j) = AF(aux, k, i + 1, j);
            }
        orc_flux2(p, 2, mbc, my, q1d, dtdx1d, aux1, aux2, aux3, maux, faddm,
                  faddp, gaddm, gaddp, &cfl1d, &w);
        cflgrid = dmax(cflgrid, cfl1d);
        for (j = 2 - mbc; j <= my + mbc; ++j)
            for (m = 1; m <= MEQN; ++m) {
                QF(gm, m, i, j) = QF(gm, m, i, j) + S1(faddm, m, j);
                QF(gp, m, i, j) = QF(gp, m, i, j) + S1(faddp, m, j);
                QF(fm, m, i, j) = QF(fm, m, i, j) + gaddm[(m - 1) + MEQN * (j + mbc - 1)];
                QF(fp, m, i, j) = QF(fp, m, i, j) + gaddp[(m - 1) + MEQN * (j + mbc - 1)];
                QF(fm, m, i + 1, j) = QF(fm, m, i + 1, j) + gaddm[(m - 1) + MEQN * (j + mbc - 1) + MEQN * n1];
                QF(fp, m, i + 1, j) = QF(fp, m, i + 1, j) + gaddp[(m - 1) + MEQN * (j + mbc - 1) + MEQN * n1];
            }
    }

    /* update q (geoclaw_step2_wrap_fort.f:95-115), ghost ring included */
    for (m = 1; m <= MEQN; ++m)
        for (i = 1 - mbc; i <= mx + mbc - 1; ++i)
            for (j = 1 - mbc; j <= my + mbc - 1; ++j)
                QF(q, m, i, j) = QF(q, m, i, j) -
                                 dtdx * (QF(fm, m, i + 1, j) - QF(fp, m, i, j)) -
                                 dtdy * (QF(gm, m, i, j + 1) - QF(gp, m, i, j));

    free(pool);
    return cflgrid;
}

/* ------------------------------------------------------------------------
 * src2 friction -- geoclaw_src2_fort.f90:41-71 (Coriolis off).
 * ---------------------------------------------------------------------- */
void orc_src2(const orc_params* p, int mbc, int mx, int my, double* q,
              const double* aux, int maux, double dt)
{
    const double g = p->grav;
    const double depth_tolerance = 1.0e-30;
    int i, j, nman;
    double gamma, dgamma, coeff = 0.0;
    if (!p->friction_forcing) return;
    for (j = 1; j <= my; ++j)
        for (i = 1; i <= mx; ++i) {
            if (QF(q, 1, i, j) < depth_tolerance) {
                QF(q, 2, i, j) = 0.0;
                QF(q, 3, i, j) = 0.0;
            } else if (QF(q, 1, i, j) <= p->friction_depth) {
                if (!p->variable_friction) {
                    for (nman = p->num_manning; nman >= 1; --nman)
                        if (AF(aux, 1, i, j) < p->manning_break[nman - 1])
                            coeff = p->manning_coefficient[nman - 1];
                } else {
                    coeff = AF(aux, p->friction_index, i, j);
                }
                gamma = sqrt(QF(q, 2, i, j) * QF(q, 2, i, j) +
                             QF(q, 3, i, j) * QF(q, 3, i, j)) *
                        g * (coeff * coeff) / pow(QF(q, 1, i, j), 7.0 / 3.0);
                dgamma = 1.0 + dt * gamma;
                QF(q, 2, i, j) = QF(q, 2, i, j) / dgamma;
                QF(q, 3, i, j) = QF(q, 3, i, j) / dgamma;
            }
        }
}

/* geoclaw_update -- fc2d_geoclaw.cpp:352-387 */
double orc_patch_update(const orc_params* p, int mbc, int mx, int my,
                        double* q, const double* aux, int maux, double dx,
                        double dy, double t, double dt)
{
    double maxcfl;
    (void)t;
    orc_b4step2(p, mbc, mx, my, q);
    maxcfl = orc_step2(p, mbc, mx, my, q, aux, maux, dx, dy, dt);
    if (maxcfl > p->maxcfl_cap) maxcfl = 0.0;
    if (p->src_term > 0) orc_src2(p, mbc, mx, my, q, aux, maux, dt);
    return maxcfl;
}

double orc_level_update(const orc_params* p, int npatch, int mbc, int mx,
                        int my, double* q, long qstride, const double* aux,
                        int maux, long astride, const double* dx,
                        const double* dy, double t, double dt, int nthreads)
{
    double maxcfl = 0.0;
    int k;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(max : maxcfl)
#endif
    for (k = 0; k < npatch; ++k) {
        double c = orc_patch_update(p, mbc, mx, my, q + (long)k * qstride,
                                    aux + (long)k * astride, maux, dx[k],
                                    dy[k], t, dt);
        if (c > maxcfl) maxcfl = c;
    }
    (void)nthreads;
    return maxcfl;
}

/* ------------------------------------------------------------------------
 * Single-face views of rpn2 / rpt2 (for the pin against the reference's
 * own solver): a slice with mx = 1 whose face 1 separates cell 0 (left
 * state) from cell 1 (right state); the other slice cells are dry.
 * fwave[3*mw + m] with m in global order (h, hu, hv).
 * ---------------------------------------------------------------------- */
void orc_rpn2_face(const orc_params* p, int ixy, const double* ql, const double* qr, double bl,
                   double br, double* fwave, double* s, double* amdq, double* apdq)
{
    const int mbc = 2, mx = 1, n = mx + 2 * mbc;
    double q1d[3 * 5], aux[5], fw[3 * 3 * 5], ss[3 * 5], am[3 * 5], ap[3 * 5];
    int m, mw;
    memset(q1d, 0, sizeof q1d);
    memset(aux, 0, sizeof aux);
    for (m = 0; m < 3; ++m) {
        q1d[m + 3 * 1] = ql[m]; /* Fortran cell 0 -> slot 0 + mbc - 1 = 1 */
        q1d[m + 3 * 2] = qr[m]; /* cell 1 -> slot 2 */
    }
    aux[1] = bl;
    aux[2] = br;
    orc_rpn2(p, ixy, mbc, mx, q1d, aux, 1, fw, ss, am, ap);
    (void)n;
    /* face 1 -> slot 1 + mbc - 1 = 2 */
    for (mw = 0; mw < 3; ++mw) {
        s[mw] = ss[mw + 3 * 2];
        for (m = 0; m < 3; ++m) fwave[3 * mw + m] = fw[m + 3 * (mw + 3 * 2)];
    }
    for (m = 0; m < 3; ++m) {
        amdq[m] = am[m + 3 * 2];
        apdq[m] = ap[m + 3 * 2];
    }
}

void orc_rpt2_face(const orc_params* p, int ixy, int imp, const double* ql, const double* qr,
                   const double* aux1, const double* aux2, const double* aux3, const double* asdq,
                   double* bmasdq, double* bpasdq)
{
    const int mbc = 2, mx = 1;
    double q1d[3 * 5], a1[5], a2[5], a3[5], as[3 * 5], bm[3 * 5], bp[3 * 5];
    int m;
    memset(q1d, 0, sizeof q1d);
    memset(a1, 0, sizeof a1);
    memset(a2, 0, sizeof a2);
    memset(a3, 0, sizeof a3);
    memset(as, 0, sizeof as);
    for (m = 0; m < 3; ++m) {
        q1d[m + 3 * 1] = ql[m];
        q1d[m + 3 * 2] = qr[m];
        as[m + 3 * 2] = asdq[m]; /* face 1 -> slot 2 */
    }
    a1[1] = aux1[0]; a1[2] = aux1[1];
    a2[1] = aux2[0]; a2[2] = aux2[1];
    a3[1] = aux3[0]; a3[2] = aux3[1];
    orc_rpt2(p, ixy, imp, mbc, mx, q1d, a1, a2, a3, 1, as, bm, bp);
    for (m = 0; m < 3; ++m) {
        bmasdq[m] = bm[m + 3 * 2];
        bpasdq[m] = bp[m + 3 * 2];
    }
}
