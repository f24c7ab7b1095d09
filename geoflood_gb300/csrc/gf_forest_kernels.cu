/*
 * Raster pyramid and patch fill for multi-level forests.
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

} // namespace gf
