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

#include <atomic>

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
    static std::atomic<unsigned long long> attr_done{0};
    cudaError_t ae = smem_attr_per_device(kern, (int)L::BYTES, attr_done);
    if (ae != cudaSuccess) return ae;
    if (nwork <= 0) return cudaSuccess;
    const int grid = (max_ctas > 0 && max_ctas < nwork) ? max_ctas : nwork;
    kern<<<grid, NT, L::BYTES, st>>>(work, nwork, phys, dt, gdt, gpar, maux, cfl, gmax, err);
    return cudaGetLastError();
}

/* The latency form: each work item on a cluster of K CTAs (one window of
 * rows each); not persistent, so max_ctas does not apply. */
template <int M, int NT, int RB, int K>
static cudaError_t launch_window(const gf_patch_work* work, int nwork, const gf_phys* phys,
                                 double dt, const double* gdt, const int* gpar, int maux, double* cfl,
                                 unsigned long long* gmax, int* err, int max_ctas, cudaStream_t st)
{
    (void)max_ctas;
    using L = Smem<M, RB, false>;
    auto kern = patch_update_window_kernel<M, NT, RB, K, false>;
    static std::atomic<unsigned long long> attr_done{0};
    cudaError_t ae = smem_attr_per_device(kern, (int)L::BYTES, attr_done);
    if (ae != cudaSuccess) return ae;
    if (nwork <= 0) return cudaSuccess;
    kern<<<nwork * K, NT, L::BYTES, st>>>(work, nwork, phys, dt, gdt, gpar, maux, cfl, gmax, err);
    return cudaGetLastError();
}

/* Patches one launch of the window kernel runs at once: the clusters of K
 * CTAs the device holds resident together (placement inside a GPC counted). */
template <int M, int NT, int RB, int K>
static int window_slots()
{
    using L = Smem<M, RB, false>;
    auto kern = patch_update_window_kernel<M, NT, RB, K, false>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::BYTES) !=
        cudaSuccess)
        return 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(K * sm_count());
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = L::BYTES;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) return 0;
    return n;
}

template <int M, int NT, int RB, int K>
static int window_occupancy()
{
    using L = Smem<M, RB, false>;
    auto kern = patch_update_window_kernel<M, NT, RB, K, false>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::BYTES) !=
        cudaSuccess)
        return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, NT, L::BYTES) != cudaSuccess) return 0;
    return n;
}

/* ---- tile shapes (threads per patch x slices per band) per patch size ----
 * Variant 0 of each size is the default; gf_autotune measures them all and
 * installs the fastest for throughput (whole levels) and for latency (a
 * lone small scenario, where one patch's critical path is the step time). */
using UpdateFn = cudaError_t (*)(const gf_patch_work*, int, const gf_phys*, double, const double*,
                                 const int*, int, double*, unsigned long long*, int*, int, cudaStream_t);
using OccFn = int (*)();

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

template <int M, int NT, int RB>
static int tile_slots() { return occupancy_of<M, NT, RB>() * sm_count(); }

struct Tile {
    int nt, rb, k; /* k > 1: the patch split over a cluster of k CTAs */
    UpdateFn fn;
    OccFn occ;
    OccFn slots; /* patches resident at once in one launch */
};

#define GF_TILE(M, NT, RB) \
    {NT, RB, 1, &launch_update<M, NT, RB, 1>, &occupancy_of<M, NT, RB>, &tile_slots<M, NT, RB>}
#define GF_WTILE(M, NT, RB, K)                                                                \
    {NT, RB, K, &launch_window<M, NT, RB, K>, &window_occupancy<M, NT, RB, K>,                \
     &window_slots<M, NT, RB, K>}
static const Tile kTiles8[] = {GF_TILE(8, 64, 5), GF_TILE(8, 128, 10), GF_TILE(8, 128, 5),
                               GF_WTILE(8, 64, 5, 2), GF_WTILE(8, 64, 5, 4)};
static const Tile kTiles16[] = {GF_TILE(16, 128, 6), GF_TILE(16, 256, 13), GF_TILE(16, 256, 9),
                                GF_WTILE(16, 128, 6, 2), GF_WTILE(16, 128, 6, 4),
                                GF_WTILE(16, 256, 9, 4)};
static const Tile kTiles32[] = {GF_TILE(32, 256, 7), GF_TILE(32, 256, 5), GF_TILE(32, 384, 7),
                                GF_TILE(32, 384, 9), GF_TILE(32, 512, 8), GF_TILE(32, 512, 9),
                                GF_WTILE(32, 256, 7, 4), GF_WTILE(32, 256, 7, 8)};
#undef GF_TILE
#undef GF_WTILE

static const Tile* tiles_of(int m, int* n)
{
    switch (m) {
    case 8: *n = (int)(sizeof kTiles8 / sizeof kTiles8[0]); return kTiles8;
    case 16: *n = (int)(sizeof kTiles16 / sizeof kTiles16[0]); return kTiles16;
    case 32: *n = (int)(sizeof kTiles32 / sizeof kTiles32[0]); return kTiles32;
    default: *n = 0; return nullptr;
    }
}

/* selected variant per goal (0 throughput, 1 latency) and patch size */
static int g_tile[2][3] = {{0, 0, 0}, {0, 0, 0}};
static inline int mcls(int m) { return m == 8 ? 0 : m == 16 ? 1 : 2; }

int tile_count(int m)
{
    int n = 0;
    tiles_of(m, &n);
    return n;
}

int tile_shape(int m, int v, int* nt, int* rb, int* k)
{
    int n = 0;
    const Tile* t = tiles_of(m, &n);
    if (!t || v < 0 || v >= n) return -1;
    *nt = t[v].nt;
    *rb = t[v].rb;
    if (k) *k = t[v].k;
    return 0;
}

int tile_get(int m, int goal) { return g_tile[goal != 0][mcls(m)]; }

/* The latency tile pays for its split only while every patch of the launch
 * is resident at once; past one wave the throughput tile finishes sooner. */
int latency_goal_fits(int m, long npatch)
{
    int n = 0;
    const Tile* t = tiles_of(m, &n);
    if (!t) return 0;
    const int v = g_tile[1][mcls(m)];
    static std::atomic<int> cache[64][3][GF_MAX_TILES] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || v >= GF_MAX_TILES)
        return npatch * t[v].k <= (long)sm_count() ? 1 : 0;
    std::atomic<int>& c = cache[dev][mcls(m)][v];
    int slots = c.load(std::memory_order_relaxed);
    if (!slots) {
        slots = t[v].slots();
        if (slots <= 0) slots = sm_count() / t[v].k;
        if (slots <= 0) slots = 1;
        c.store(slots, std::memory_order_relaxed);
    }
    return npatch <= (long)slots ? 1 : 0;
}

int tile_set(int m, int goal, int v)
{
    int n = 0;
    tiles_of(m, &n);
    if (v < 0 || v >= n) return -1;
    g_tile[goal != 0][mcls(m)] = v;
    return 0;
}

cudaError_t launch_patch_update_tile(int m, int v, const gf_patch_work* work, int nwork,
                                     const gf_phys* phys, double dt, const double* gdt,
                                     const int* gpar, int maux, double* cfl,
                                     unsigned long long* gmax, int* err, cudaStream_t st,
                                     int max_ctas)
{
    int n = 0;
    const Tile* t = tiles_of(m, &n);
    if (!t || v < 0 || v >= n) return cudaErrorInvalidValue;
    return t[v].fn(work, nwork, phys, dt, gdt, gpar, maux, cfl, gmax, err, max_ctas, st);
}

cudaError_t launch_patch_update(int m, const gf_patch_work* work, int nwork, const gf_phys* phys,
                                double dt, const double* gdt, const int* gpar, int maux, double* cfl,
                                unsigned long long* gmax, int* err, cudaStream_t st, int max_ctas,
                                int goal)
{
    if (!(m == 8 || m == 16 || m == 32)) return cudaErrorInvalidValue;
    return launch_patch_update_tile(m, g_tile[goal != 0][mcls(m)], work, nwork, phys, dt, gdt, gpar,
                                    maux, cfl, gmax, err, st, max_ctas);
}

int sm_count()
{
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    if (!cache[dev]) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = n > 0 ? n : 1;
    }
    return cache[dev];
}

/* mixed tile: 256 threads for every size; mx = 8 takes a whole patch per
 * band, mx = 16 its 256-thread variant, mx = 32 the default */
constexpr int kMixNT = 256, kMixRB8 = 10, kMixRB16 = 13, kMixRB32 = 7;

cudaError_t launch_patch_update_mixed(const gf_patch_work* work, const int n[3], const gf_phys* phys,
                                      double dt, const double* gdt, const int* gpar, int maux,
                                      double* cfl, unsigned long long* gmax, int* err,
                                      unsigned int* sched, cudaStream_t st, int max_ctas)
{
    using X = MixedSmem<kMixRB8, kMixRB16, kMixRB32, false>;
    auto kern = patch_update_mixed_kernel<kMixNT, kMixRB8, kMixRB16, kMixRB32, false>;
    static std::atomic<unsigned long long> attr_done{0};
    cudaError_t ae = smem_attr_per_device(kern, (int)X::BYTES, attr_done);
    if (ae != cudaSuccess) return ae;
    const int nwork = n[0] + n[1] + n[2];
    if (nwork <= 0) return cudaSuccess;
    int grid = sm_count();
    if (max_ctas > 0 && max_ctas < grid) grid = max_ctas;
    if (grid > nwork) grid = nwork;
    kern<<<grid, kMixNT, X::BYTES, st>>>(work, n[0], n[1], n[2], phys, dt, gdt, gpar, maux, cfl, gmax, err,
                                         sched);
    return cudaGetLastError();
}

int patch_update_occupancy(int m)
{
    int n = 0;
    const Tile* t = tiles_of(m, &n);
    return t ? t[g_tile[0][mcls(m)]].occ() : 0;
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

/* Two layouts in one launch (a host batch's q and aux): element e of the
 * first npatch * ncell is a cell of set a, the rest cells of set b. */
__global__ void aos_to_soa_pair_kernel(const double* __restrict__ sa, double* __restrict__ da, int nfa,
                                       const double* __restrict__ sb, double* __restrict__ db, int nfb,
                                       long npatch, int ncell)
{
    const long per = npatch * (long)ncell;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < 2 * per;
         e += (long)gridDim.x * blockDim.x) {
        const bool second = e >= per;
        const long ee = second ? e - per : e;
        const int nf = second ? nfb : nfa;
        const long p = ee / ncell;
        const int k = (int)(ee % ncell);
        const double* s = (second ? sb : sa) + p * nf * (long)ncell + (long)k * nf;
        double* d = (second ? db : da) + p * nf * (long)ncell + k;
        for (int f = 0; f < nf; ++f) d[(long)f * ncell] = s[f];
    }
}

cudaError_t launch_aos_to_soa_pair(const double* sa, double* da, int nfa, const double* sb, double* db,
                                   int nfb, long npatch, int ncell, cudaStream_t st)
{
    const long total = 2 * npatch * (long)ncell;
    if (total == 0) return cudaSuccess;
    aos_to_soa_pair_kernel<<<conv_grid(total), 256, 0, st>>>(sa, da, nfa, sb, db, nfb, npatch, ncell);
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
