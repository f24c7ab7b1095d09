/*
 * Kernel instantiations and launchers for the patch update and the
 * host-layout conversions used at the drop-in boundary.
 *
 * Tile shapes per patch size m (threads per CTA, slices per band):
 *   m = 32: 256 threads, 7 slices  (245 / 231 faces per band stage)
 *   m = 16: 128 threads, 6 slices  (114 / 102)
 *   m =  8:  64 threads, 5 slices  ( 55 /  45)
 * chosen so the flattened face loops of a band fill the CTA.
 */
#include <cuda_runtime.h>

#include "gf_internal.h"
#include "gf_patch_update.cuh"

namespace gf {

template <int M, int NT, int RB, int MINB>
static cudaError_t launch_update(const gf_patch_work* work, int nwork, const gf_phys* phys,
                                 double dt, const double* gdt, const int* gpar, int maux, double* cfl,
                                 unsigned long long* gmax, int* err, int max_ctas, cudaStream_t st)
{
    using L = Smem<M, RB, false>;
    auto kern = patch_update_kernel<M, NT, RB, MINB, false>;
    static bool attr_set = false; /* per process; the attribute is per function */
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)L::BYTES);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    if (nwork <= 0) return cudaSuccess;
    const int grid = (max_ctas > 0 && max_ctas < nwork) ? max_ctas : nwork;
    kern<<<grid, NT, L::BYTES, st>>>(work, nwork, phys, dt, gdt, gpar, maux, cfl, gmax, err);
    return cudaGetLastError();
}

cudaError_t launch_patch_update(int m, const gf_patch_work* work, int nwork, const gf_phys* phys,
                                double dt, const double* gdt, const int* gpar, int maux, double* cfl,
                                unsigned long long* gmax, int* err, cudaStream_t st, int max_ctas)
{
    switch (m) {
    case 32: return launch_update<32, 256, 7, 1>(work, nwork, phys, dt, gdt, gpar, maux, cfl, gmax, err, max_ctas, st);
    case 16: return launch_update<16, 128, 6, 1>(work, nwork, phys, dt, gdt, gpar, maux, cfl, gmax, err, max_ctas, st);
    case 8: return launch_update<8, 64, 5, 1>(work, nwork, phys, dt, gdt, gpar, maux, cfl, gmax, err, max_ctas, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int M, int NT, int RB>
static int occupancy_of()
{
    using L = Smem<M, RB, false>;
    auto kern = patch_update_kernel<M, NT, RB, 1, false>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::BYTES) !=
        cudaSuccess)
        return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, NT, L::BYTES) != cudaSuccess) return 0;
    return n;
}

int patch_update_occupancy(int m)
{
    switch (m) {
    case 32: return occupancy_of<32, 256, 7>();
    case 16: return occupancy_of<16, 128, 6>();
    case 8: return occupancy_of<8, 64, 5>();
    default: return 0;
    }
}

size_t patch_update_smem_bytes(int m)
{
    switch (m) {
    case 32: return Smem<32, 7>::BYTES;
    case 16: return Smem<16, 6>::BYTES;
    case 8: return Smem<8, 5>::BYTES;
    default: return 0;
    }
}

/* ---- layout conversion at the boundary ----
 * Fortran layout a(nf, 0..nx-1, 0..ny-1) of npatch contiguous patches
 * <-> planes [patch][field][cell]. One thread per (patch, cell). */
__global__ void aos_to_soa_kernel(const double* __restrict__ src, double* __restrict__ dst,
                                  long npatch, int ncell, int nf, long src_stride, long dst_stride)
{
    const long total = npatch * (long)ncell;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
         e += (long)gridDim.x * blockDim.x) {
        const long p = e / ncell;
        const int k = (int)(e % ncell);
        const double* s = src + p * src_stride + (long)k * nf;
        double* d = dst + p * dst_stride + k;
        for (int f = 0; f < nf; ++f) d[(long)f * ncell] = s[f];
    }
}

__global__ void soa_to_aos_kernel(const double* __restrict__ src, double* __restrict__ dst,
                                  long npatch, int ncell, int nf, long src_stride, long dst_stride)
{
    const long total = npatch * (long)ncell;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
         e += (long)gridDim.x * blockDim.x) {
        const long p = e / ncell;
        const int k = (int)(e % ncell);
        const double* s = src + p * src_stride + k;
        double* d = dst + p * dst_stride + (long)k * nf;
        for (int f = 0; f < nf; ++f) d[f] = s[(long)f * ncell];
    }
}

static int conv_grid(long total)
{
    long b = (total + 255) / 256;
    if (b > 152L * 16) b = 152L * 16;
    if (b < 1) b = 1;
    return (int)b;
}

cudaError_t launch_aos_to_soa(const double* src, double* dst, long npatch, int ncell, int nf,
                              long src_stride, long dst_stride, cudaStream_t st)
{
    const long total = npatch * (long)ncell;
    if (total == 0) return cudaSuccess;
    aos_to_soa_kernel<<<conv_grid(total), 256, 0, st>>>(src, dst, npatch, ncell, nf, src_stride,
                                                        dst_stride);
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(const double* src, double* dst, long npatch, int ncell, int nf,
                              long src_stride, long dst_stride, cudaStream_t st)
{
    const long total = npatch * (long)ncell;
    if (total == 0) return cudaSuccess;
    soa_to_aos_kernel<<<conv_grid(total), 256, 0, st>>>(src, dst, npatch, ncell, nf, src_stride,
                                                        dst_stride);
    return cudaGetLastError();
}

} // namespace gf
