/*
 * Force-included (after ref_shim.h) when the reference's CUDA patch update
 * (src/fc2d_cpu_cuda/cuda_source/cudaclaw_flux2.cu with cudaclaw_limiters.cu,
 * riemann_source/geoflood_src2.cu and geoflood_rp2.cu) is compiled for the
 * host by oracle/build_ref.sh. That kernel runs one patch per CTA, every
 * face loop a block-stride loop over threadIdx.x between __syncthreads()
 * barriers, so with one thread (threadIdx = 0, blockDim = 1) and the
 * barriers as no-ops it runs the same loops one after another, in order.
 * Shared variables become locals of the single thread, the block-wide CFL
 * reduction returns the thread's own value, and the symbol copies become
 * memcpy. Test infrastructure only.
 */
#ifndef GF_REF_SHIM_PATCH_H
#define GF_REF_SHIM_PATCH_H
#include <stdlib.h>

#include "ref_shim.h"

#define __shared__
#define __syncthreads() ((void)0)

struct gf_ref_dim3 {
    unsigned x, y, z;
};
static const gf_ref_dim3 threadIdx = {0, 0, 0};
static const gf_ref_dim3 blockDim = {1, 1, 1};
static const gf_ref_dim3 blockIdx = {0, 0, 0};

#define cudaMemcpyToSymbol(sym, src, n) (memcpy((void*)&(sym), (const void*)(src), (n)), cudaSuccess)

#endif
