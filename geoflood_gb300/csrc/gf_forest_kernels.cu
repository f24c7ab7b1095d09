/*
 * Raster pyramid, patch fill, sea-level initial state, gauge sampling and
 * the subcycling helpers (time interpolation, patch copies) for
 * multi-level forests.
 *
 * A forest's static fields (bathymetry, optional extra aux fields) and its
 * initial state are given as rasters at the finest level. Level l of the
 * pyramid holds the cell averages over 2^(maxlevel-l) x 2^(maxlevel-l)
 * finest cells, formed level by level as ((a + b) + (c + d)) * 0.25 of the
 * 2 x 2 block below -- the cell-averaged topography the reference's setaux
 * integrates (fortran_source/geoclaw_setaux_fort.f90:107-245) for a raster
 * that is constant on each finest cell. Each level carries a 2-cell halo
 * extended from the edge, so a patch's array (ghost ring included) is one
 * window of the level. Built without FMA contraction.
 */
#include <cuda_runtime.h>

#include "gf_internal.h"

namespace gf {

namespace {

constexpr int H = GF_MBC; /* halo of a pyramid level */

/* interior of one field of one level from the finer level below */
__global__ void pyramid_down_kernel(const double* __restrict__ fine, double* __restrict__ coarse,
                                    int nxc, int nyc)
{
    const int nxf = 2 * nxc;
    const long pf = nxf + 2 * H;  /* padded row length of the finer level */
    const long pc = nxc + 2 * H;
    const long total = (long)nxc * nyc;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
         e += (long)gridDim.x * blockDim.x) {
        const int i = (int)(e % nxc), j = (int)(e / nxc);
        const double* r0 = fine + (long)(2 * j + H) * pf + (2 * i + H);
        const double* r1 = r0 + pf;
        coarse[(long)(j + H) * pc + (i + H)] = ((r0[0] + r0[1]) + (r1[0] + r1[1])) * 0.25;
    }
}

/* halo of one field of one level: copy of the nearest interior cell */
__global__ void pyramid_halo_kernel(double* __restrict__ a, int nx, int ny)
{
    const long p = nx + 2 * H;
    const long total = p * (ny + 2 * H);
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
         e += (long)gridDim.x * blockDim.x) {
        const int i = (int)(e % p), j = (int)(e / p);
        if (i >= H && i < nx + H && j >= H && j < ny + H) continue;
        const int ii = min(max(i, H), nx + H - 1), jj = min(max(j, H), ny + H - 1);
        a[e] = a[(long)jj * p + ii];
    }
}

/* interior of the finest level from a dense (ny, nx) raster */
__global__ void pyramid_top_kernel(const double* __restrict__ src, double* __restrict__ dst, int nx,
                                   int ny)
{
    const long p = nx + 2 * H;
    const long total = (long)nx * ny;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
         e += (long)gridDim.x * blockDim.x) {
        const int i = (int)(e % nx), j = (int)(e / nx);
        dst[(long)(j + H) * p + (i + H)] = src[e];
    }
}

/* one CTA per task: window of a pyramid level into a patch's planes */
template <int M>
__global__ void __launch_bounds__(128) patch_fill_kernel(const gf_fill_task* __restrict__ tasks,
                                                         int ntask)
{
    constexpr int N = M + 2 * H, S = N * N;
    if ((int)blockIdx.x >= ntask) return;
    const gf_fill_task T = tasks[blockIdx.x];
    const long p = T.nx + 2 * H;
    for (int f = 0; f < T.nfield; ++f) {
        const double* src = T.src[f] + (long)T.J * M * p + (long)T.I * M;
        double* dst = T.dst[f];
        for (int k = threadIdx.x; k < S; k += blockDim.x) {
            const int ii = k % N, jj = k / N;
            dst[k] = src[(long)jj * p + ii];
        }
    }
}

/* one thread per gauge: the gauge's value after an accepted step, as
 * fc2d_geoclaw_update_gauge computes it (fortran_source/
 * geoclaw_gauges_fort.f90:19-75): if any of the cell holding the gauge and
 * its +x, +y, +xy neighbours is drier than 0.1 * dry_tolerance, that cell's
 * h, hu, hv and bathymetry; else the bilinear blend of the four, evaluated
 * in the Fortran expression's order (no contraction in this file). Values
 * of h, hu, hv below 1e-99 in magnitude become 0. A gauge outside its
 * window [t1, t2], sampled less than incr ago or already sampled at t
 * writes level -1. Record: level, t, h, hu, hv, bathymetry. */
__global__ void gauge_sample_kernel(const gf_gauge_task* __restrict__ tasks, int n,
                                    const double* __restrict__ qbase,
                                    const double* __restrict__ auxbase, long S, int n4, int maux,
                                    double drytol2, double t, double* __restrict__ last,
                                    double* __restrict__ rec)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const gf_gauge_task T = tasks[g];
    double* r = rec + (long)g * 6;
    const double lt = last[g];
    if (T.slot < 0 || !(t >= T.t1 && t <= T.t2 && t >= lt + T.incr && t > lt)) {
        r[0] = -1.0;
        return;
    }
    const double* q = qbase + (long)T.slot * 3 * S;
    const double* b = auxbase + (long)T.slot * maux * S;
    /* Fortran cell (i, j), 1-based with mbc ghost cells, at plane offset */
    const long c00 = (long)(T.jj + H - 1) * n4 + (T.ii + H - 1);
    const long c10 = c00 + 1, c01 = c00 + n4, c11 = c00 + n4 + 1;
    double v[4];
    if (q[c00] < drytol2 || q[c10] < drytol2 || q[c01] < drytol2 || q[c11] < drytol2) {
        for (int m = 0; m < 3; ++m) v[m] = q[m * S + c00];
        v[3] = b[c00];
    } else {
        const double xo = T.xoff, yo = T.yoff;
        for (int m = 0; m < 3; ++m) {
            const double* p = q + m * S;
            v[m] = (1.0 - xo) * (1.0 - yo) * p[c00] + xo * (1.0 - yo) * p[c10] +
                   (1.0 - xo) * yo * p[c01] + xo * yo * p[c11];
        }
        v[3] = (1.0 - xo) * (1.0 - yo) * b[c00] + xo * (1.0 - yo) * b[c10] + (1.0 - xo) * yo * b[c01] +
               xo * yo * b[c11];
    }
    r[0] = (double)T.level;
    r[1] = t;
    for (int m = 0; m < 3; ++m) r[2 + m] = fabs(v[m]) < 1e-99 ? 0.0 : v[m];
    r[5] = v[3];
    last[g] = t;
}

/* fc2d_geoclaw_qinit without qinit files (fortran_source/
 * geoclaw_qinit_fort.f90:24-27): h = max(0, sea_level - b), hu = hv = 0 */
__global__ void qinit_sea_level_kernel(const double* __restrict__ b, double* __restrict__ h,
                                       double* __restrict__ hu, double* __restrict__ hv, long cells,
                                       double sea_level)
{
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < cells; e += (long)gridDim.x * blockDim.x) {
        h[e] = fmax(0.0, sea_level - b[e]);
        hu[e] = 0.0;
        hv[e] = 0.0;
    }
}

/* Time interpolation of one coarse patch for the ghost cells of finer
 * patches at an intermediate time, as fc2d_geoclaw_fort_timeinterp
 * (fclaw2d_source/fc2d_geoclaw_timeinterp_fort.f:16-58) computes it: the
 * interior cells within two layers of a face take qold + alpha (qnew -
 * qold); the ghost ring takes qold's (exchanged at the old time), so that
 * cells the exchange at the new time does not reach stay defined. */
template <int M>
__global__ void __launch_bounds__(128) tinterp_strip_kernel(const gf_slot_task* __restrict__ tasks, int ntask,
                                                            double alpha)
{
    constexpr int N = M + 2 * H, S = N * N;
    if ((int)blockIdx.x >= ntask) return;
    const gf_slot_task T = tasks[blockIdx.x];
    for (int k = threadIdx.x; k < 3 * S; k += blockDim.x) {
        const int c = k % S, i = c % N - H + 1, j = c / N - H + 1; /* Fortran indices */
        if (i < 1 || i > M || j < 1 || j > M) {
            T.c[k] = T.a[k];
            continue;
        }
        const int d = min(min(i - 1, j - 1), min(M - i, M - j));
        if (d < 2) T.c[k] = T.a[k] + alpha * (T.b[k] - T.a[k]);
    }
}

/* whole-patch copies (3 planes) */
template <int M>
__global__ void __launch_bounds__(128) slot_copy_kernel(const gf_slot_task* __restrict__ tasks, int ntask)
{
    constexpr int N = M + 2 * H, S = N * N;
    if ((int)blockIdx.x >= ntask) return;
    const gf_slot_task T = tasks[blockIdx.x];
    for (int k = threadIdx.x; k < 3 * S; k += blockDim.x) T.c[k] = T.a[k];
}

int grid_for(long total)
{
    long b = (total + 255) / 256;
    if (b > 152L * 16) b = 152L * 16;
    return (int)(b < 1 ? 1 : b);
}

} // namespace

cudaError_t launch_pyramid_top(const double* src, double* dst, int nx, int ny, cudaStream_t st)
{
    pyramid_top_kernel<<<grid_for((long)nx * ny), 256, 0, st>>>(src, dst, nx, ny);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    pyramid_halo_kernel<<<grid_for((long)(nx + 2 * H) * (ny + 2 * H)), 256, 0, st>>>(dst, nx, ny);
    return cudaGetLastError();
}

cudaError_t launch_pyramid_down(const double* fine, double* coarse, int nxc, int nyc,
                                cudaStream_t st)
{
    pyramid_down_kernel<<<grid_for((long)nxc * nyc), 256, 0, st>>>(fine, coarse, nxc, nyc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    pyramid_halo_kernel<<<grid_for((long)(nxc + 2 * H) * (nyc + 2 * H)), 256, 0, st>>>(coarse, nxc,
                                                                                        nyc);
    return cudaGetLastError();
}

cudaError_t launch_patch_fill(int m, const gf_fill_task* tasks, int ntask, cudaStream_t st)
{
    if (ntask <= 0) return cudaSuccess;
    switch (m) {
    case 32: patch_fill_kernel<32><<<ntask, 128, 0, st>>>(tasks, ntask); break;
    case 16: patch_fill_kernel<16><<<ntask, 128, 0, st>>>(tasks, ntask); break;
    case 8: patch_fill_kernel<8><<<ntask, 128, 0, st>>>(tasks, ntask); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_tinterp_strip(int m, const gf_slot_task* tasks, int ntask, double alpha, cudaStream_t st)
{
    if (ntask <= 0) return cudaSuccess;
    switch (m) {
    case 32: tinterp_strip_kernel<32><<<ntask, 128, 0, st>>>(tasks, ntask, alpha); break;
    case 16: tinterp_strip_kernel<16><<<ntask, 128, 0, st>>>(tasks, ntask, alpha); break;
    case 8: tinterp_strip_kernel<8><<<ntask, 128, 0, st>>>(tasks, ntask, alpha); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_slot_copy(int m, const gf_slot_task* tasks, int ntask, cudaStream_t st)
{
    if (ntask <= 0) return cudaSuccess;
    switch (m) {
    case 32: slot_copy_kernel<32><<<ntask, 128, 0, st>>>(tasks, ntask); break;
    case 16: slot_copy_kernel<16><<<ntask, 128, 0, st>>>(tasks, ntask); break;
    case 8: slot_copy_kernel<8><<<ntask, 128, 0, st>>>(tasks, ntask); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_qinit_sea_level(const double* b, double* h, double* hu, double* hv, long cells,
                                   double sea_level, cudaStream_t st)
{
    qinit_sea_level_kernel<<<grid_for(cells), 256, 0, st>>>(b, h, hu, hv, cells, sea_level);
    return cudaGetLastError();
}

cudaError_t launch_gauge_sample(const gf_gauge_task* tasks, int n, const double* qbase,
                                const double* auxbase, int m, int maux, double drytol2, double t,
                                double* last, double* rec, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int n4 = m + 2 * H;
    gauge_sample_kernel<<<(n + 127) / 128, 128, 0, st>>>(tasks, n, qbase, auxbase, (long)n4 * n4, n4,
                                                         maux, drytol2, t, last, rec);
    return cudaGetLastError();
}

} // namespace gf
