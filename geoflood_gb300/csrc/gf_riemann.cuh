/*
 * Face-level shallow-water Riemann solvers, FP64, device side.
 *
 * Restates the reference's GeoClaw solvers for one face at a time:
 *   - normal solve: rpn2_geoclaw.f:84-330 with riemann_aug_JCP
 *     (geoclaw_riemann_utils.f:2-311, maxiter = 1) and riemanntype
 *     (geoclaw_riemann_utils.f:566-677);
 *   - transverse split: rpt2_geoclaw.f:61-187.
 *
 * Inputs per cell come pre-digested from shared memory (gf_cell): the
 * quotients hu/h, hv/h and sqrt(g h) are computed once per cell instead of
 * once per face side. Each is the same IEEE operation the Fortran performs,
 * so the values are identical. Cramer's rule in riemann_aug_JCP is written
 * out for the fixed eigenvector pattern r(:,2) = (0,0,1), r(1,:) = 1, which
 * removes multiplications by exact 0 and 1 only.
 *
 * Component order inside these routines is LOCAL: 0 = depth, 1 = momentum
 * normal to the face, 2 = momentum along the face.
 */
#ifndef GF_RIEMANN_CUH
#define GF_RIEMANN_CUH

#include "gf_types.h"
#include "gf_cmp.cuh"

struct gf_cell {
    double h;    /* depth after b4step2                         */
    double hun;  /* momentum normal to the face                 */
    double hut;  /* momentum along the face                     */
    double un;   /* hun/h if wet else 0                         */
    double ut;   /* hut/h if wet else 0                         */
    double c;    /* sqrt(g h) if wet else 0                     */
    double b;    /* bathymetry                                  */
    double rh;   /* 1/h if wet (contracted build only)          */
    double rc;   /* 1/sqrt(g h) if wet (contracted build only)  */
    bool wet;    /* h > dry_tolerance                           */
};

/* sqrt(a): the IEEE root, or, in the contracted build and for positive
 * finite a, a * rsqrt(a) (within an ulp or two, fewer FP64 instructions;
 * zero, infinity and negative values keep the IEEE root, one integer test
 * on the bit pattern decides) */
template <bool FAST>
__device__ __forceinline__ double d_sqrt(double a)
{
    if (FAST) {
        const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(a));
        if (u - 1ull < 0x7fefffffffffffffull) return a * rsqrt(a);
    }
    return sqrt(a);
}

/* a * b < 0 for nonzero finite factors, from the sign bits on the integer
 * pipe (a product that underflows to zero aside) */
__device__ __forceinline__ bool opposite_signs(double a, double b)
{
    const unsigned long long ia = static_cast<unsigned long long>(__double_as_longlong(a));
    const unsigned long long ib = static_cast<unsigned long long>(__double_as_longlong(b));
    return ((ia ^ ib) >> 63) != 0 && (ia << 1) != 0 && (ib << 1) != 0;
}

/* riemanntype (geoclaw_riemann_utils.f:566-677), maxiter = 1.
 * cL = sqrt(g hL), cR = sqrt(g hR) are supplied by the caller (they equal
 * the Fortran's sqrt(g*hL), sqrt(g*hR) bit for bit). Returns hm, s1m, s2m. */
template <bool FAST>
__device__ __forceinline__ void gf_riemanntype(double hL, double hR, double uL,
                                               double uR, double cL, double cR,
                                               double rhL, double rhR,
                                               double g, double drytol,
                                               double c16g, double rsg, double& hm,
                                               double& s1m, double& s2m)
{
    const double h_min = d_min<FAST>(hR, hL);
    const double h_max = d_max<FAST>(hR, hL);
    const double delu = uR - uL;
    if (d_le<FAST>(h_min, drytol)) {
        hm = 0.0;
        s1m = uR + uL - 2.0 * cR + 2.0 * cL;
        s2m = s1m;
        return;
    }
    /* sqrt is monotone, so sqrt(g*h_min) = min(cL, cR). */
    const double c_min = d_min<FAST>(cR, cL);
    const double c_max = d_max<FAST>(cR, cL);
    const double F_min = delu + 2.0 * (c_min - c_max);
    /* (h_max + h_min)/(h_max h_min) = 1/h_min + 1/h_max: the contracted
     * build uses the per-cell reciprocals instead of a division. */
    double F_max = 0.0, q_fm = 0.0, s_fm = 0.0;
    if (!FAST) F_max = delu + (h_max - h_min) * sqrt(0.5 * g * (h_max + h_min) / (h_max * h_min));
    /* the contracted build forms F_max only where it is read (not for two
     * rarefactions), its root through rsqrt, whose value the two-shock step
     * reuses */
    auto f_max = [&]() {
        if (FAST) {
            const double a_fm = 0.5 * g * (d_max<FAST>(rhL, rhR) + d_min<FAST>(rhL, rhR));
            q_fm = rsqrt(a_fm);
            s_fm = a_fm * q_fm;
            F_max = delu + (h_max - h_min) * s_fm;
        }
    };
    if (d_gtz<FAST>(F_min)) { /* 2-rarefactions */
        const double t = d_max<FAST>(0.0, -delu + 2.0 * (cL + cR));
        hm = c16g * (t * t);
        /* sqrt(g hm) = t / 4 up to rounding: the contracted build takes it */
        const double cm = FAST ? 0.25 * t : sqrt(g * hm);
        s1m = uL + 2.0 * cL - 3.0 * cm;
        s2m = uR - 2.0 * cR + 3.0 * cm;
    } else if ((f_max(), d_lez<FAST>(F_max))) { /* 2 shocks, one Newton step on sqrt(h) */
        const double h0 = h_max;
        double gL, gR, dfdh, sh0, rL, rR;
        if (FAST) {
            rL = rhL;
            rR = rhR;
            /* h0 = h_max: the deeper side's root is sqrt(g / h_max) = c_max / h_max
             * and its (h0 - h) terms vanish; the shallower side's root is
             * F_max's, sqrt(g (1/h_min + 1/h_max) / 2) */
            const double r0 = d_min<FAST>(rhL, rhR); /* 1/h_max */
            const double gmx = d_max<FAST>(cL, cR) * r0;
            const bool lmax = d_ge<FAST>(hL, hR);
            gL = lmax ? gmx : s_fm;
            gR = lmax ? s_fm : gmx;
            const double w = 0.25 * (r0 * r0) * g;
            dfdh = gmx + s_fm - (h0 - h_min) * w * q_fm;
            sh0 = d_max<FAST>(cL, cR) * rsg; /* sqrt(h_max) = sqrt(g h_max)/sqrt(g) */
        } else {
            rL = 1.0 / hL;
            rR = 1.0 / hR;
            const double r0 = 1.0 / h0; /* equals rL or rR */
            gL = sqrt(0.5 * g * (r0 + rL));
            gR = sqrt(0.5 * g * (r0 + rR));
            dfdh = gL - g * (h0 - hL) / (4.0 * (h0 * h0) * gL) + gR -
                   g * (h0 - hR) / (4.0 * (h0 * h0) * gR);
            sh0 = sqrt(h0);
        }
        const double F0 = delu + (h0 - hL) * gL + (h0 - hR) * gR;
        const double slope = 2.0 * sh0 * dfdh;
        const double t = sh0 - d_div<FAST>(F0, slope);
        hm = t * t;
        const double rm = d_div<FAST>(1.0, hm);
        const double u1m = uL - (hm - hL) * d_sqrt<FAST>((0.5 * g) * (rm + rL));
        const double u2m = uR + (hm - hR) * d_sqrt<FAST>((0.5 * g) * (rm + rR));
        /* hm = t^2: sqrt(g hm) = sqrt(g) |t| up to rounding in the contracted build */
        const double cm = FAST ? (g * rsg) * fabs(t) : sqrt(g * hm);
        s1m = u1m - cm;
        s2m = u2m + cm;
    } else { /* one shock, one rarefaction, one secant step.
                The first F0 has (h0 - h_min) = 0, so F0 = F_min exactly. */
        const double F0 = F_min;
        if (FAST) {
            hm = h_min - F0 * d_div<FAST>(h_max - h_min, F_max - F0);
        } else {
            const double slope = (F_max - F0) / (h_max - h_min);
            hm = h_min - F0 / slope;
        }
        const double cm = d_sqrt<FAST>(g * hm);
        if (d_gt<FAST>(hL, hR)) {
            s1m = uL + 2.0 * cL - 3.0 * cm;
            s2m = uL + 2.0 * cL - cm;
        } else {
            s2m = uR - 2.0 * cR + 3.0 * cm;
            s1m = uR - 2.0 * cR + cm;
        }
    }
}

/* Normal Riemann problem at one face: rpn2_geoclaw.f:110-315 + aug_JCP.
 * Outputs speeds s[3] and f-waves fw[mw][m] (LOCAL component order). */
template <bool FAST>
__device__ __forceinline__ void gf_rpn2_face(const gf_cell& Lc, const gf_cell& Rc,
                                             double g, double drytol,
                                             double c16g, double rsg, double crit,
                                             double crit2, double s[3],
                                             double fw[3][3])
{
    /* Riemann problem variables (rpn2_geoclaw.f:136-171). */
    double hL, huL, hvL, uL, vL, phiL, cL, rhL = 0.0;
    double hR, huR, hvR, uR, vR, phiR, cR, rhR = 0.0;
    double bL = Lc.b, bR = Rc.b;
    if (Rc.wet) {
        hR = Rc.h; huR = Rc.hun; hvR = Rc.hut; uR = Rc.un; vR = Rc.ut; cR = Rc.c; rhR = Rc.rh;
        /* hu^2/h = hu u: the contracted build reuses the cell quotient */
        phiR = FAST ? 0.0 : 0.5 * g * (hR * hR) + (huR * huR) / hR; /* contracted: delphi below */
    } else {
        hR = 0.0; huR = 0.0; hvR = 0.0; uR = 0.0; vR = 0.0; phiR = 0.0; cR = 0.0;
    }
    if (Lc.wet) {
        hL = Lc.h; huL = Lc.hun; hvL = Lc.hut; uL = Lc.un; vL = Lc.ut; cL = Lc.c; rhL = Lc.rh;
        phiL = FAST ? 0.0 : 0.5 * g * (hL * hL) + (huL * huL) / hL;
    } else {
        hL = 0.0; huL = 0.0; hvL = 0.0; uL = 0.0; vL = 0.0; phiL = 0.0; cL = 0.0;
    }
    (void)hvL; (void)hvR;

    /* Wet/dry interface: wall or overtopping (rpn2_geoclaw.f:185-242). */
    double wall0 = 1.0, wall1 = 1.0, wall2 = 1.0;
    if (!Rc.wet) {
        double hstar, s1x, s2x;
        gf_riemanntype<FAST>(hL, hL, uL, -uL, cL, cL, rhL, rhL, g, drytol, c16g, rsg, hstar, s1x, s2x);
        const double hstartest = d_max<FAST>(hL, hstar);
        if (d_lt<FAST>(hstartest + bL, bR)) {
            wall1 = 0.0; wall2 = 0.0;
            hR = hL; huR = -huL; bR = bL; phiR = phiL; uR = -uL; vR = vL; cR = cL; rhR = rhL;
        } else if (d_lt<FAST>(hL + bL, bR)) {
            bR = hL + bL;
        }
    } else if (!Lc.wet) {
        double hstar, s1x, s2x;
        gf_riemanntype<FAST>(hR, hR, -uR, uR, cR, cR, rhR, rhR, g, drytol, c16g, rsg, hstar, s1x, s2x);
        const double hstartest = d_max<FAST>(hR, hstar);
        if (d_lt<FAST>(hstartest + bR, bL)) {
            wall0 = 0.0; wall1 = 0.0;
            hL = hR; huL = -huR; bL = bR; phiL = phiR; uL = -uR; vL = vR; cL = cR; rhL = rhR;
        } else if (d_lt<FAST>(hR + bR, bL)) {
            bL = hR + bR;
        }
    }

    /* Einfeldt / Roe speeds (rpn2_geoclaw.f:257-266). */
    const double sL = uL - cL;
    const double sR = uR + cR;
    const double uhat = d_div<FAST>(cL * uL + cR * uR, cR + cL);
    /* hbar of the steady-state wave below; g (hL + hR) / 2 = g hbar for the
     * non-negative depths here, so the contracted build shares the product */
    const double hbar = d_max<FAST>(0.5 * (hL + hR), 0.0);
    const double chat = FAST ? d_sqrt<FAST>(g * hbar) : d_sqrt<FAST>(g * 0.5 * (hR + hL));
    double sE1 = d_min<FAST>(sL, uhat - chat);
    double sE2 = d_max<FAST>(sR, uhat + chat);

    /* ---- riemann_aug_JCP (geoclaw_riemann_utils.f:57-306) ---- */
    const double delh = hR - hL;
    const double delhu = huR - huL;
    /* phi = g h^2 / 2 + hu^2 / h: the contracted build forms the jump as
     * (g / 2) (hR - hL) (hR + hL) + (huR uR - huL uL), with hu^2 / h = hu u;
     * both products rounded, so a mirrored wall state gives exactly zero */
    const double delphi = FAST ? fma((0.5 * g) * delh, hR + hL, __dmul_rn(huR, uR) - __dmul_rn(huL, uL))
                               : phiR - phiL;
    const double delb = bR - bL;

    double hm, s1m, s2m;
    gf_riemanntype<FAST>(hL, hR, uL, uR, cL, cR, rhL, rhR, g, drytol, c16g, rsg, hm, s1m, s2m);
    (void)hm;

    const double l1 = d_min<FAST>(sE1, s2m);
    const double l3 = d_max<FAST>(sE2, s1m);
    sE1 = l1;
    sE2 = l3;
    /* One reciprocal serves h*_HLL and Cramer's rule in the contracted
     * build: sE2 - sE1 = l3 - l1 = -(l1 - l3). */
    const double rdet = FAST ? gf_rcp(l1 - l3) : 0.0;
    /* h*_HLL (sE2 - sE1) enters only as hsd: the contracted build takes it as
     * max(numerator, 0) (sE2 - sE1 = l3 - l1 > 0 for a wet face) */
    const double hll_num = huL - huR + sE2 * hR - sE1 * hL;
    const double hstarHLL = FAST ? 0.0 : fmax(hll_num / (sE2 - sE1), 0.0);
    const double l2 = 0.5 * (l1 + l3);

    /* steady-state wave, first (only) iteration: hLstar = hL etc. */
    const double s1s2bar = FAST ? fma(0.25 * (uL + uR), uL + uR, -(g * hbar))
                                : 0.25 * ((uL + uR) * (uL + uR)) - g * hbar;
    const double s1s2tilde = d_max<FAST>(0.0, uL * uR) - g * hbar;
    const double crit_sq = crit * crit;
    bool sonic;
    if (d_le<FAST>(fabs(s1s2bar), crit)) sonic = true;
    else if (d_le<FAST>(s1s2bar * s1s2tilde, crit_sq)) sonic = true;
    else if (d_le<FAST>(s1s2bar * sE1 * sE2, crit_sq)) sonic = true;
    else if (d_lt<FAST>(d_min<FAST>(fabs(sE1), fabs(sE2)), crit2)) sonic = true;
    else if (d_lt<FAST>(sE1, crit2) && d_gt<FAST>(s1m, -crit2)) sonic = true;
    else if (d_gt<FAST>(sE2, -crit2) && d_lt<FAST>(s2m, crit2)) sonic = true;
    else if (FAST ? opposite_signs(uL + cL, uR + cR) : d_ltz<FAST>((uL + cL) * (uR + cR))) sonic = true;
    else if (FAST ? opposite_signs(uL - cL, uR - cR) : d_ltz<FAST>((uL - cL) * (uR - cR))) sonic = true;
    else sonic = false;

    const double rs12 = (FAST && !sonic) ? gf_rcp(s1s2bar) : 0.0;
    /* contracted build: g hbar delb once; deldelphi below is -(g hbar delb /
     * s1s2bar) s1s2tilde, i.e. the unclamped deldelh times -s1s2tilde */
    const double ghd = FAST ? (g * hbar) * delb : 0.0;
    double deldelh = sonic ? -delb : (FAST ? ghd * rs12 : delb * g * hbar / s1s2bar);
    const double deldelh0 = deldelh;
    const double hsd = FAST ? d_max<FAST>(hll_num, 0.0) : hstarHLL * (sE2 - sE1);
    if (FAST) {
        /* The bounds hsd / sE clamp rarely: compare hsd with deldelh * sE (the
         * sign of sE is known in each branch) and divide only to clamp. */
        if (d_lt<FAST>(sE1, -crit) && d_gt<FAST>(sE2, crit)) {
            if (d_lt<FAST>(hsd, deldelh * sE2)) deldelh = d_div<FAST>(hsd, sE2); /* min, sE2 > 0 */
            if (d_lt<FAST>(hsd, deldelh * sE1)) deldelh = d_div<FAST>(hsd, sE1); /* max, sE1 < 0 */
        } else if (d_ge<FAST>(sE1, crit)) {
            if (d_lt<FAST>(hsd, deldelh * sE1)) deldelh = d_div<FAST>(hsd, sE1); /* min, sE1 > 0 */
            deldelh = d_max<FAST>(deldelh, -hL);
        } else if (d_le<FAST>(sE2, -crit)) {
            deldelh = d_min<FAST>(deldelh, hR);
            if (d_lt<FAST>(hsd, deldelh * sE2)) deldelh = d_div<FAST>(hsd, sE2); /* max, sE2 < 0 */
        }
    } else if (d_lt<FAST>(sE1, -crit) && d_gt<FAST>(sE2, crit)) {
        deldelh = d_min<FAST>(deldelh, d_div<FAST>(hsd, sE2));
        deldelh = d_max<FAST>(deldelh, d_div<FAST>(hsd, sE1));
    } else if (d_ge<FAST>(sE1, crit)) {
        deldelh = d_min<FAST>(deldelh, d_div<FAST>(hsd, sE1));
        deldelh = d_max<FAST>(deldelh, -hL);
    } else if (d_le<FAST>(sE2, -crit)) {
        deldelh = d_min<FAST>(deldelh, hR);
        deldelh = d_max<FAST>(deldelh, d_div<FAST>(hsd, sE2));
    }
    double deldelphi;
    if (FAST) {
        deldelphi = sonic ? -ghd : -deldelh0 * s1s2tilde;
        /* g max(-hL delb, -hR delb) = -g delb h_lo and g min(..) = -g delb h_hi,
         * with h_lo the smaller depth when delb > 0 (the larger otherwise) */
        const double mgd = -g * delb;
        const bool pos = d_gtz<FAST>(delb);
        const double hmn = d_min<FAST>(hL, hR), hmx = d_max<FAST>(hL, hR);
        deldelphi = d_min<FAST>(deldelphi, mgd * (pos ? hmn : hmx));
        deldelphi = d_max<FAST>(deldelphi, mgd * (pos ? hmx : hmn));
    } else {
        deldelphi = sonic ? -g * hbar * delb : -delb * g * hbar * s1s2tilde / s1s2bar;
        deldelphi = d_min<FAST>(deldelphi, g * d_max<FAST>(-hL * delb, -hR * delb));
        deldelphi = d_max<FAST>(deldelphi, g * d_min<FAST>(-hL * delb, -hR * delb));
    }

    const double d1 = delh - deldelh;
    const double d2 = delhu;
    const double d3 = delphi - deldelphi;

    /* Cramer's rule with r(:,1) = (1,l1,l1^2), r(:,2) = (0,0,1),
     * r(:,3) = (1,l3,l3^2): determinant = l1 - l3. */
    const double A2 = l1 * l1, C2 = l3 * l3;
    const double det = l1 - l3;
    /* n2 = (l1 - l3) (d3 + d1 l1 l3 - d2 (l1 + l3)): the contracted build
     * takes beta2 = n2 / det as that bracket, without the division */
    const double beta1 = FAST ? (d2 - d1 * l3) * rdet : (d2 - d1 * l3) / det;
    double beta2;
    if (FAST) {
        beta2 = fma(-d2, l1 + l3, fma(d1, l1 * l3, d3));
    } else {
        const double n2 = (d2 * C2 - l3 * d3) - d1 * (l1 * C2 - l3 * A2) + (l1 * d3 - d2 * A2);
        beta2 = n2 / det;
    }
    const double beta3 = FAST ? (d1 * l1 - d2) * rdet : (d1 * l1 - d2) / det;

    /* f-waves (geoclaw_riemann_utils.f:289-306). */
    /* contracted build: l^2 beta = (beta l) l, no squares */
    double f11 = beta1 * l1, f21 = FAST ? f11 * l1 : beta1 * A2, f31 = beta1 * l1 * vL;
    double f13 = beta3 * l3, f23 = FAST ? f13 * l3 : beta3 * C2, f33 = beta3 * l3 * vR;
    /* h u v: the contracted build takes hu v (hu = h u up to rounding) */
    const double corr = FAST ? (huR * vR - huL * vL - f31 - f33) : (hR * uR * vR - hL * uL * vL - f31 - f33);
    if (d_lez<FAST>(huL + f11)) f31 = f31 + corr;
    else f33 = f33 + corr;

    /* Wall masking (rpn2_geoclaw.f:303-309). Without a wall every mask is 1
     * and the products are the values themselves. */
    if (FAST && Lc.wet && Rc.wet) {
        s[0] = l1; s[1] = l2; s[2] = l3;
        fw[0][0] = f11; fw[0][1] = f21; fw[0][2] = f31;
        fw[1][0] = 0.0; fw[1][1] = beta2; fw[1][2] = 0.0;
        fw[2][0] = f13; fw[2][1] = f23; fw[2][2] = f33;
        return;
    }
    s[0] = l1 * wall0; s[1] = l2 * wall1; s[2] = l3 * wall2;
    fw[0][0] = f11 * wall0; fw[0][1] = f21 * wall0; fw[0][2] = f31 * wall0;
    fw[1][0] = 0.0 * wall1; fw[1][1] = beta2 * wall1; fw[1][2] = 0.0 * wall1;
    fw[2][0] = f13 * wall2; fw[2][1] = f23 * wall2; fw[2][2] = f33 * wall2;
}

/* Transverse split of one fluctuation (rpt2_geoclaw.f:63-182), one face.
 * cell: the cell the fluctuation enters; topo_lo / topo_hi: bathymetry of
 * the transverse neighbours below / above it. asdq in LOCAL order (0 = h,
 * 1 = momentum normal to the face, 2 = momentum along the face; "along the
 * face" is the transverse sweep direction). Accumulates into bm / bp. */
template <bool FAST>
__device__ __forceinline__ void gf_rpt2_face(const gf_cell& cl, double topo_lo,
                                             double topo_hi, double tol,
                                             const double asdq[3], double bm[3],
                                             double bp[3])
{
    bm[0] = bm[1] = bm[2] = 0.0;
    bp[0] = bp[1] = bp[2] = 0.0;
    if (d_le<FAST>(cl.h, tol)) return;
    const double eta = cl.h + cl.b;
    if (d_lt<FAST>(eta, d_min<FAST>(topo_lo, topo_hi))) return;
    const bool up_lo = d_ge<FAST>(eta, topo_lo), up_hi = d_ge<FAST>(eta, topo_hi);
    const double u = cl.un;  /* q(mu)/h */
    const double v = cl.ut;  /* q(mv)/h */
    const double s1 = v - cl.c;
    const double s2 = v;
    const double s3 = v + cl.c;
    const double delf1 = asdq[0], delf2 = asdq[1], delf3 = asdq[2];
    /* s3 - s1 = 2 sqrt(g h): the contracted build multiplies by the
     * per-cell reciprocal instead of dividing twice. */
    const double den = s3 - s1;
    const double rden = 0.5 * cl.rc;
    const double beta1 = FAST ? (s3 * delf1 - delf3) * rden : (s3 * delf1 - delf3) / den;
    const double beta2 = -u * delf1 + delf2;
    const double beta3 = FAST ? (delf3 - s1 * delf1) * rden : (delf3 - s1 * delf1) / den;
    /* r(:,1) = (1, u, s1); r(:,2) = (0, 1, 0); r(:,3) = (1, u, s3). The first
     * wave enters zero sums: the contracted build assigns (a zero's sign
     * aside). */
    if (d_ltz<FAST>(s1) && up_lo) {
        const double a = s1 * beta1;
        if (FAST) { bm[0] = a; bm[1] = a * u; bm[2] = a * s1; }
        else { bm[0] += a; bm[1] += a * u; bm[2] += a * s1; }
    } else if (d_gtz<FAST>(s1) && up_hi) {
        const double a = s1 * beta1;
        if (FAST) { bp[0] = a; bp[1] = a * u; bp[2] = a * s1; }
        else { bp[0] += a; bp[1] += a * u; bp[2] += a * s1; }
    }
    if (d_ltz<FAST>(s2) && up_lo) {
        bm[1] += s2 * beta2;
    } else if (d_gtz<FAST>(s2) && up_hi) {
        bp[1] += s2 * beta2;
    }
    if (d_ltz<FAST>(s3) && up_lo) {
        const double a = s3 * beta3;
        bm[0] += a; bm[1] += a * u; bm[2] += a * s3;
    } else if (d_gtz<FAST>(s3) && up_hi) {
        const double a = s3 * beta3;
        bp[0] += a; bp[1] += a * u; bp[2] += a * s3;
    }
}

/* philim (philim.f:4-65): limiter value for wave strengths a (= |w|^2) and
 * b (= projection of the upwind wave). */
template <bool FAST>
__device__ __forceinline__ double gf_philim(double a, double b, int meth)
{
    if (d_eqz<FAST>(a)) return 0.0;
    /* MC with b <= 0: r <= 0 and the limiter is zero; the contracted build
     * skips the division (a zero's sign aside) */
    if (FAST && meth == 4 && d_lez<FAST>(b)) return 0.0;
    const double r = d_div<FAST>(b, a);
    switch (meth) {
    case 2: return d_max<FAST>(d_max<FAST>(0.0, d_min<FAST>(1.0, 2.0 * r)), d_min<FAST>(2.0, r));
    case 3: return (r + fabs(r)) / (1.0 + fabs(r));
    case 4: {
        /* (1 + r) / 2: halving is exact, so the single rounding of the fused
         * form gives the same value */
        const double c = FAST ? fma(r, 0.5, 0.5) : (1.0 + r) * 0.5;
        return d_max<FAST>(0.0, d_min<FAST>(d_min<FAST>(c, 2.0), 2.0 * r));
    }
    case 5: return r;
    default: return d_max<FAST>(0.0, d_min<FAST>(1.0, r));
    }
}

#endif
