/*
 * C entry points around the reference's CUDA Riemann device functions
 * (src/fc2d_cpu_cuda/riemann_source/geoflood_rp2.cu:47-251 cuda_flood_rpn2,
 * :270-384 cuda_flood_rpt2, :408-690 riemann_aug_JCP), compiled for the host
 * by oracle/build_ref.sh. Test infrastructure only: it pins the oracle's
 * restated solver against the reference's own code.
 */
#include "ref_shim.h"
#include "variables.h"

/* The reference declares this as an extern __constant__ symbol; the host
 * build defines it here. */
GeofloodVars d_geofloodVars;

/* Signatures as declared in geoflood_rp2.cu. */
void cuda_flood_rpn2(int idir, int meqn, int mwaves, int maux, double ql[], double qr[],
                     double auxl[], double auxr[], double fwave[], double s[], double amdq[],
                     double apdq[], double drytol, int mcapa);
void cuda_flood_rpt2(int idir, int meqn, int mwaves, int maux, double ql[], double qr[],
                     double aux1[], double aux2[], double aux3[], int imp, double asdq[],
                     double bmasdq[], double bpasdq[], double drytol);

extern "C" {

void ref_set_gravity(double g)
{
    memset(&d_geofloodVars, 0, sizeof d_geofloodVars);
    d_geofloodVars.gravity = g;
    d_geofloodVars.coordinate_system = 1;
}

/* One face: left state ql (h, hu, hv), right state qr, bathymetry bl, br.
 * idir 0 = x, 1 = y. fwave[3*mw + m], s[3], amdq[3], apdq[3]. */
void ref_rpn2_face(int idir, const double* ql, const double* qr, double bl, double br,
                   double drytol, double* fwave, double* s, double* amdq, double* apdq)
{
    double l[3] = {ql[0], ql[1], ql[2]}, r[3] = {qr[0], qr[1], qr[2]};
    double al[1] = {bl}, ar[1] = {br};
    cuda_flood_rpn2(idir, 3, 3, 1, l, r, al, ar, fwave, s, amdq, apdq, drytol, 0);
}

/* Transverse split of asdq: imp 0 uses the left cell, 1 the right cell.
 * aux1/aux2/aux3 hold [left, right] bathymetry of the rows below, on and
 * above the face. */
void ref_rpt2_face(int idir, int imp, const double* ql, const double* qr, const double* aux1,
                   const double* aux2, const double* aux3, const double* asdq, double drytol,
                   double* bmasdq, double* bpasdq)
{
    double l[3] = {ql[0], ql[1], ql[2]}, r[3] = {qr[0], qr[1], qr[2]};
    double a1[2] = {aux1[0], aux1[1]}, a2[2] = {aux2[0], aux2[1]}, a3[2] = {aux3[0], aux3[1]};
    double d[3] = {asdq[0], asdq[1], asdq[2]};
    cuda_flood_rpt2(idir, 3, 3, 1, l, r, a1, a2, a3, imp, d, bmasdq, bpasdq, drytol);
}

} /* extern "C" */
