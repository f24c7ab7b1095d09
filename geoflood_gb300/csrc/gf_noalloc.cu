/*
 * Allocation-free patch update.
 *
 * Some callers cannot allocate device memory when they want a step: a host
 * program whose device memory belongs to another allocator (a framework's
 * caching pool or a fixed budget that a raw cudaMalloc would bypass), a
 * service running at its memory limit where an allocation can fail in the
 * middle of a time step, or code on a latency-critical stream where
 * cudaFree would synchronise the whole device. gf_patch_update_noalloc
 * serves them: the caller passes device buffers it already owns, and the
 * staging space the update needs (structure-of-arrays planes, work entries,
 * physics, status) lives in the file-scope array below, which every GPU that
 * loads this library holds until the process exits.
 *
 * Every call shares that one array and it keeps the last call's contents:
 * the status words are cleared at the start of each call, and two calls
 * whose work overlaps on the GPU (different streams, or different host
 * threads) race on it. Issue them one after another.
 */
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "gf_internal.h"

namespace {

constexpr int kMaxPatches = GF_NOALLOC_MAX_PATCHES;
constexpr int kMaxMaux = GF_NOALLOC_MAX_MAUX;
constexpr long kMaxCells = (32 + 2 * GF_MBC) * (32 + 2 * GF_MBC); /* mx = my = 32 */

struct NoallocStatus {
    unsigned long long gmax;
    int err;
    int pad;
};

/* Byte layout of the scratch array (all offsets multiples of 256). */
constexpr size_t kOffStatus = 0;
constexpr size_t kOffPhys = 256;
constexpr size_t kOffWork = kOffPhys + ((sizeof(gf_phys) + 255) / 256) * 256;
constexpr size_t kOffCfl = kOffWork + ((kMaxPatches * sizeof(gf_patch_work) + 255) / 256) * 256;
constexpr size_t kOffQ = kOffCfl + ((kMaxPatches * sizeof(double) + 255) / 256) * 256;
constexpr size_t kOffAux = kOffQ + (size_t)kMaxPatches * 3 * kMaxCells * sizeof(double);
constexpr size_t kScratchBytes = kOffAux + (size_t)kMaxPatches * kMaxMaux * kMaxCells * sizeof(double);

static_assert(kScratchBytes == GF_NOALLOC_SCRATCH_BYTES, "header and layout disagree");

/* The staging space. Host code must not use this name as a device address:
 * it is a host-side stand-in; the device address comes from
 * cudaGetSymbolAddress, once per device. */
static __device__ __align__(256) unsigned char gf_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
unsigned char* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_setup_mutex;

/* Device address of the scratch array on `device` (current), looked up on
 * the first call per device. */
int scratch_on(int device, unsigned char** out)
{
    if (device < 0 || device >= kMaxDevices) return GF_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, gf_noalloc_scratch);
        if (e != cudaSuccess || !p) return GF_ERR_CUDA;
        g_scratch_addr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_addr[device];
    return GF_OK;
}

int update_on_device(int device, const gf_phys* phys, int npatch, int mx, int my, int maux,
                     const double* dx, const double* dy, double dt, double* q, const double* aux,
                     double* cfl, double* maxcfl, cudaStream_t st);

} // namespace

extern "C" int gf_patch_update_noalloc(int device, const gf_phys* phys, int npatch, int mx, int my,
                                       int mbc, int meqn, int maux, const double* dx,
                                       const double* dy, double dt, double* q, const double* aux,
                                       double* cfl, double* maxcfl, void* stream)
{
    if (!phys || !dx || !dy || !q || !aux || !maxcfl) return GF_ERR_ARG;
    if (mx != my || (mx != 8 && mx != 16 && mx != 32)) return GF_ERR_UNSUPPORTED;
    if (mbc != GF_MBC || meqn != GF_MEQN) return GF_ERR_UNSUPPORTED;
    if (maux < 1 || maux > kMaxMaux) return GF_ERR_ARG;         /* beyond the scratch size */
    if (npatch < 1 || npatch > kMaxPatches) return GF_ERR_ARG;  /* beyond the scratch size */
    /* the same rules as gf_ctx_set_phys, and a variable-friction field that
     * lies inside the maux fields the kernel stages */
    if (gf::phys_problem(phys, maux)) return GF_ERR_ARG;
    for (int k = 0; k < npatch; ++k)
        if (!(dx[k] > 0.0) || !(dy[k] > 0.0)) return GF_ERR_ARG;
    /* the caller's current device is put back on every return below */
    int caller_device = -1;
    if (cudaGetDevice(&caller_device) != cudaSuccess) return GF_ERR_CUDA;
    if (cudaSetDevice(device) != cudaSuccess) return GF_ERR_CUDA;
    const int rc = update_on_device(device, phys, npatch, mx, my, maux, dx, dy, dt, q, aux, cfl,
                                    maxcfl, static_cast<cudaStream_t>(stream));
    if (cudaSetDevice(caller_device) != cudaSuccess && rc == GF_OK) return GF_ERR_CUDA;
    return rc;
}

namespace {

int update_on_device(int device, const gf_phys* phys, int npatch, int mx, int my, int maux,
                     const double* dx, const double* dy, double dt, double* q, const double* aux,
                     double* cfl, double* maxcfl, cudaStream_t st)
{
    unsigned char* base = nullptr;
    int rc = scratch_on(device, &base);
    if (rc) return rc;

    const long S = (long)(mx + 2 * GF_MBC) * (my + 2 * GF_MBC);
    NoallocStatus* d_status = reinterpret_cast<NoallocStatus*>(base + kOffStatus);
    gf_phys* d_phys = reinterpret_cast<gf_phys*>(base + kOffPhys);
    gf_patch_work* d_work = reinterpret_cast<gf_patch_work*>(base + kOffWork);
    double* d_cfl = reinterpret_cast<double*>(base + kOffCfl);
    double* d_q = reinterpret_cast<double*>(base + kOffQ);
    double* d_aux = reinterpret_cast<double*>(base + kOffAux);

    gf_patch_work work[kMaxPatches] = {};
    for (int k = 0; k < npatch; ++k) {
        work[k].q = d_q + (size_t)k * 3 * S;
        work[k].aux = d_aux + (size_t)k * maux * S;
        work[k].dx = dx[k];
        work[k].dy = dy[k];
        work[k].phys = 0;
        work[k].group = 0;
    }
#define GF_NA_CK(call)                                  \
    do {                                                \
        if ((call) != cudaSuccess) return GF_ERR_CUDA;  \
    } while (0)
    GF_NA_CK(cudaMemsetAsync(d_status, 0, sizeof(NoallocStatus), st));
    GF_NA_CK(cudaMemcpyAsync(d_phys, phys, sizeof(gf_phys), cudaMemcpyHostToDevice, st));
    GF_NA_CK(cudaMemcpyAsync(d_work, work, npatch * sizeof(gf_patch_work), cudaMemcpyHostToDevice, st));
    GF_NA_CK(gf::launch_aos_to_soa(q, d_q, npatch, (int)S, 3, 3 * S, 3 * S, st));
    GF_NA_CK(gf::launch_aos_to_soa(aux, d_aux, npatch, (int)S, maux, maux * S, maux * S, st));
    GF_NA_CK(gf::launch_patch_update(mx, d_work, npatch, d_phys, dt, nullptr, nullptr, maux, d_cfl,
                                     &d_status->gmax, &d_status->err, st));
    GF_NA_CK(gf::launch_soa_to_aos(d_q, q, npatch, (int)S, 3, 3 * S, 3 * S, st));
    NoallocStatus hs;
    GF_NA_CK(cudaMemcpyAsync(&hs, d_status, sizeof hs, cudaMemcpyDeviceToHost, st));
    if (cfl) GF_NA_CK(cudaMemcpyAsync(cfl, d_cfl, npatch * sizeof(double), cudaMemcpyDeviceToHost, st));
    GF_NA_CK(cudaStreamSynchronize(st));
#undef GF_NA_CK
    if (hs.err) return GF_ERR_DEVICE;
    double v;
    std::memcpy(&v, &hs.gmax, sizeof v);
    *maxcfl = v;
    return GF_OK;
}

} // namespace
