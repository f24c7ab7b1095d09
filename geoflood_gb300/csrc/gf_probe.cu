/*
 * FP64 pipe-rate probe: the denominator of the FP64 roofline the patch
 * update is bound by. Times independent dependency chains of double fma,
 * division and square root (and float fma for comparison) over a full grid
 * with CUDA events and reports operations per second.
 */
#include <cuda_runtime.h>

#include "geoflood_gb300.h"
#include "gf_patch_update.cuh"

namespace {

/* One CTA waits, with the bounded try_wait loop of the patch kernels, on
 * phase 0 of an mbarrier that expects one arrival: thread 0 arrives first
 * (arrive = 1) or nothing ever arrives (arrive = 0). */
__global__ void __launch_bounds__(32) bounded_wait_kernel(int arrive, uint32_t max_iter, int* status)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) gf::mbar_init(&bar, 1);
    __syncthreads();
    if (arrive && threadIdx.x == 0) gf::mbar_expect_tx(&bar, 0);
    const bool ok = __syncthreads_and(gf::mbar_wait(&bar, 0, max_iter));
    if (threadIdx.x == 0) status[0] = ok ? 0 : 1;
}

constexpr int kIters = 2048;

template <int OP>
__global__ void __launch_bounds__(256) rate_kernel(const double* __restrict__ in,
                                                   double* __restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double a[8];
    float f[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        a[k] = in[(t + k) & 255] + k;
        f[k] = (float)a[k];
    }
    const double b = 1.0000001, c = 1e-9;
#pragma unroll 2
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (OP == 0) a[k] = fma(a[k], b, c);
            else if (OP == 1) a[k] = b / a[k];
            else if (OP == 2) a[k] = sqrt(a[k] + c);
            else f[k] = fmaf(f[k], 1.0000001f, 1e-9f);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k] + f[k];
    out[t] = s;
}

template <int OP>
double time_op(const double* in, double* out, int blocks)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    rate_kernel<OP><<<blocks, 256>>>(in, out); /* warm-up */
    cudaEventRecord(e0);
    rate_kernel<OP><<<blocks, 256>>>(in, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double ops = (double)blocks * 256.0 * kIters * 8.0;
    return ms > 0.f ? ops / (ms * 1e-3) : 0.0;
}

} // namespace

extern "C" int gf_measure_fp64_rates(int device, double* rates)
{
    if (!rates) return GF_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return GF_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8;
    double *in = nullptr, *out = nullptr;
    if (cudaMalloc(&in, 256 * sizeof(double)) != cudaSuccess) return GF_ERR_NOMEM;
    if (cudaMalloc(&out, (size_t)blocks * 256 * sizeof(double)) != cudaSuccess) {
        cudaFree(in);
        return GF_ERR_NOMEM;
    }
    double h[256];
    for (int i = 0; i < 256; ++i) h[i] = 1.0 + i * 1e-3;
    cudaMemcpy(in, h, sizeof h, cudaMemcpyHostToDevice);
    rates[0] = time_op<0>(in, out, blocks);
    rates[1] = time_op<1>(in, out, blocks);
    rates[2] = time_op<2>(in, out, blocks);
    rates[3] = time_op<3>(in, out, blocks);
    const cudaError_t e = cudaGetLastError();
    cudaFree(in);
    cudaFree(out);
    return e == cudaSuccess ? GF_OK : GF_ERR_CUDA;
}

extern "C" int gf_probe_bounded_wait(int device, int arrive, unsigned int max_iter, int* timed_out, double* ms)
{
    if (!timed_out || max_iter == 0) return GF_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return GF_ERR_CUDA;
    int* d = nullptr;
    if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return GF_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int h = -1;
    cudaMemset(d, 0xff, sizeof(int));
    cudaEventRecord(e0);
    bounded_wait_kernel<<<1, 32>>>(arrive, max_iter, d);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (e != cudaSuccess) return GF_ERR_CUDA;
    *timed_out = h;
    if (ms) *ms = t;
    return GF_OK;
}
