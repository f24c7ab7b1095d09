/*
 * The patch update compiled with floating-point contraction off
 * (-fmad=false, set by the build for this file) and with the reference's
 * four flux accumulators fm, fp, gm, gp summed in its order. Every FP64
 * operation then rounds as the Fortran expression is written, so the result
 * matches the restated Fortran bit for bit apart from the libm/CUDA pow()
 * in the friction term. Used to prove parity; the production path is the
 * contracted build in gf_kernels.cu.
 */
#include <cuda_runtime.h>

#define GF_KNS gf_exact
#include "gf_internal.h"
#include "gf_patch_update.cuh"

namespace gf {

template <int M, int NT, int RB>
static cudaError_t launch_exact(const gf_patch_work* work, int nwork, const gf_phys* phys,
                                double dt, const double* gdt, const int* gpar, int maux, double* cfl,
                                unsigned long long* gmax, int* err, cudaStream_t st)
{
    using L = gf_exact::Smem<M, RB, true>;
    auto kern = gf_exact::patch_update_kernel<M, NT, RB, 1, true>;
    static std::atomic<unsigned long long> attr_done{0};
    cudaError_t ae = smem_attr_per_device(kern, (int)L::BYTES, attr_done);
    if (ae != cudaSuccess) return ae;
    if (nwork <= 0) return cudaSuccess;
    kern<<<nwork, NT, L::BYTES, st>>>(work, nwork, phys, dt, gdt, gpar, maux, cfl, gmax, err);
    return cudaGetLastError();
}

cudaError_t launch_patch_update_exact(int m, const gf_patch_work* work, int nwork,
                                      const gf_phys* phys, double dt, const double* gdt,
                                      const int* gpar, int maux, double* cfl,
                                      unsigned long long* gmax, int* err, cudaStream_t st)
{
    switch (m) {
    case 32: return launch_exact<32, 256, 4>(work, nwork, phys, dt, gdt, gpar, maux, cfl, gmax, err, st);
    case 16: return launch_exact<16, 128, 6>(work, nwork, phys, dt, gdt, gpar, maux, cfl, gmax, err, st);
    case 8: return launch_exact<8, 64, 5>(work, nwork, phys, dt, gdt, gpar, maux, cfl, gmax, err, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_patch_update_mixed_exact(const gf_patch_work* work, const int n[3],
                                            const gf_phys* phys, double dt, const double* gdt,
                                            const int* gpar, int maux, double* cfl,
                                            unsigned long long* gmax, int* err, unsigned int* sched,
                                            cudaStream_t st, int max_ctas)
{
    /* the per-size exact tiles at 256 threads: mx = 32 keeps 4 slices per band */
    using X = gf_exact::MixedSmem<10, 13, 4, true>;
    auto kern = gf_exact::patch_update_mixed_kernel<256, 10, 13, 4, true>;
    static std::atomic<unsigned long long> attr_done{0};
    cudaError_t ae = smem_attr_per_device(kern, (int)X::BYTES, attr_done);
    if (ae != cudaSuccess) return ae;
    const int nwork = n[0] + n[1] + n[2];
    if (nwork <= 0) return cudaSuccess;
    int grid = sm_count();
    if (max_ctas > 0 && max_ctas < grid) grid = max_ctas;
    if (grid > nwork) grid = nwork;
    kern<<<grid, 256, X::BYTES, st>>>(work, n[0], n[1], n[2], phys, dt, gdt, gpar, maux, cfl, gmax, err, sched);
    return cudaGetLastError();
}

} // namespace gf
