/*
 * Force-included when the reference's CUDA Riemann source
 * (src/fc2d_cpu_cuda/riemann_source/geoflood_rp2.cu) is compiled for the host
 * by oracle/build_ref.sh: CUDA qualifiers become plain C++ and the three
 * runtime calls that file makes are given host stand-ins. Test
 * infrastructure only.
 */
#ifndef GF_REF_SHIM_H
#define GF_REF_SHIM_H
#include <math.h>
#include <stdbool.h>
#include <string.h>

#define __device__
#define __host__
#define __global__
#define __constant__

typedef int cudaError_t;
enum { cudaSuccess = 0 };
static inline const char* cudaGetErrorString(cudaError_t) { return "host build"; }
/* ForestClaw's logger, used on the error path of the pointer-assign helpers. */
#define fclaw_global_essentialf(...) ((void)0)
#define cudaMemcpyFromSymbol(dst, sym, n) (memcpy((void*)(dst), (const void*)&(sym), (n)), cudaSuccess)

#endif
