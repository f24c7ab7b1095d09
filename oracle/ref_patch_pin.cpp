/*
 * C entry point around the reference's CUDA patch update
 * cudaclaw_flux2_and_update (src/fc2d_cpu_cuda/cuda_source/cudaclaw_flux2.cu:
 * 63-1160: b4step2, x and y normal solves with the patch CFL, MC-limited
 * second-order corrections, the eight transverse passes, the
 * flux-difference update and src2), with its limiter
 * (cuda_source/cudaclaw_limiters.cu), Riemann solvers
 * (riemann_source/geoflood_rp2.cu) and friction source
 * (riemann_source/geoflood_src2.cu), all compiled for the host by
 * oracle/build_ref.sh with ref_shim_patch.h (one thread per patch, barriers
 * as no-ops). The reference file is included where it lies so that its
 * file-local kernel body can be called. Test infrastructure only: it pins
 * the oracle's whole patch update against the reference's own code.
 */
#include "cuda_source/cudaclaw_flux2.cu"

#include <stdlib.h>
#include <string.h>

/* The kernel's dynamic shared memory (per-thread work space of mwork doubles). */
double shared_mem[256];

/* Defined for the host build; the reference declares it as an extern
 * __constant__ symbol set by setprob_cuda. */
GeofloodVars d_geofloodVars;

void cuda_flood_rpn2(int idir, int meqn, int mwaves, int maux, double ql[], double qr[],
                     double auxl[], double auxr[], double fwave[], double s[], double amdq[],
                     double apdq[], double drytol, int mcapa);
void cuda_flood_rpt2(int idir, int meqn, int mwaves, int maux, double ql[], double qr[],
                     double aux1[], double aux2[], double aux3[], int imp, double asdq[],
                     double bmasdq[], double bpasdq[], double drytol);
void cuda_flood_src2(int meqn, int maux, double xlower, double ylower, double dx, double dy,
                     double* qr, double* auxr, double t, double dt, int i, int j);

extern "C" {

/* One patch of mx x my cells with mbc = 2, in the reference GPU layout
 * q[m][j][i] (i fastest, (mx+4)(my+4) cells per plane, ghost cells
 * included), updated in place; b is the bathymetry plane. order[2] and
 * mthlim[3] are the [clawpatch] method settings as the CUDA build reads
 * them (order[1] > 0: transverse waves with the second-order correction
 * folded in). src_term > 0 applies the friction source with one Manning
 * coefficient below friction_depth. Returns the patch CFL as the kernel's
 * block reduction leaves it (before the hook's cap). */
double ref_patch_update(int mx, int my, double dx, double dy, double t, double dt,
                        const int* order_in, const int* mthlim_in, int src_term,
                        double drytol, double grav, double manning, double friction_depth,
                        double* q, const double* b)
{
    const int mbc = 2, meqn = 3, maux = 1, mwaves = 3;
    const size_t zs = (size_t)(mx + 2 * mbc) * (my + 2 * mbc);

    memset(&d_geofloodVars, 0, sizeof d_geofloodVars);
    d_geofloodVars.gravity = grav;
    d_geofloodVars.coordinate_system = 1;
    d_geofloodVars.friction_forcing = true;
    d_geofloodVars.friction_depth = friction_depth;
    d_geofloodVars.num_manning = 1;
    d_geofloodVars.manning_coefficent = manning;
    d_geofloodVars.manning_break = 1.0e10;

    int ord[2] = {order_in[0], order_in[1]};
    int lim[3] = {mthlim_in[0], mthlim_in[1], mthlim_in[2]};
    cudaclaw_set_method_parameters(ord, lim, mwaves, 1);

    /* Work arrays with one plane of zeros on either side: with mcapa = 0
     * the kernel still forms aux[I - zs] and dtdx1d[I - 1] (multiplied by
     * zero), and the limiter at the last ghost face reads one row past its
     * plane; those reads land in the zero padding. */
    auto arr = [&](size_t planes) { return (double*)calloc((planes + 2) * zs + 64, sizeof(double)); };
    double* auxb = arr(maux);
    double* fmb = arr(meqn);
    double* fpb = arr(meqn);
    double* gmb = arr(meqn);
    double* gpb = arr(meqn);
    double* amb = arr(meqn);
    double* apb = arr(meqn);
    double* bmb = arr(meqn);
    double* bpb = arr(meqn);
    double* wvb = arr(2 * mwaves * meqn);
    double* spb = arr(2 * mwaves);
    double* dxb = arr(1);
    double* dyb = arr(1);
    double cflblock = 0.0;
    memcpy(auxb + zs, b, zs * sizeof(double));

    const int mwork1 = 4 * meqn + 2 * maux + mwaves + meqn * mwaves;
    const int mwork2 = 5 * meqn + 6 * maux;
    const int mwork = mwork1 > mwork2 ? mwork1 : mwork2;

    cudaclaw_flux2_and_update(mx, my, meqn, mbc, maux, mwaves, mwork, src_term, 0, drytol,
                              0.0, 0.0, dx, dy, q, auxb + zs, fmb + zs, fpb + zs, gmb + zs,
                              gpb + zs, amb + zs, apb + zs, bmb + zs, bpb + zs, wvb + zs,
                              spb + zs, dxb + zs, dyb + zs, &cflblock, cuda_flood_rpn2,
                              cuda_flood_rpt2, nullptr, cuda_flood_src2, t, dt);

    free(auxb); free(fmb); free(fpb); free(gmb); free(gpb); free(amb); free(apb);
    free(bmb); free(bpb); free(wvb); free(spb); free(dxb); free(dyb);
    return cflblock;
}

} /* extern "C" */
