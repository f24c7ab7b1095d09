/* Internal declarations shared by the kernels and the C-ABI layer. */
#ifndef GF_INTERNAL_H
#define GF_INTERNAL_H

#include <cuda_runtime.h>
#include <stddef.h>

#include <atomic>
#include <functional>

#include "gf_types.h"

namespace gf {

/* Raise a kernel's dynamic shared-memory limit to `bytes` on the current
 * device. The attribute belongs to the kernel in one device's context, so
 * it is set once per device: `done` keeps one bit per device ordinal
 * (ordinals of 64 and above are set on every call). */
template <class Kernel>
inline cudaError_t smem_attr_per_device(Kernel kern, int bytes,
                                        std::atomic<unsigned long long>& done)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    if (bit) done.fetch_or(bit, std::memory_order_release);
    return cudaSuccess;
}

/* What is wrong with a set of physics parameters, or nullptr when they are
 * usable: num_manning within the table, order 1 or 2, transverse 0..2,
 * g > 0, dry tolerance >= 0, and with variable friction a friction_index of
 * at least 1 and, when maux > 0, at most maux (the kernel reads that aux
 * field of every cell). maux = 0 skips the upper bound (not yet known). */
const char* phys_problem(const gf_phys* p, int maux);

/* fn(lo, hi) over shares of [0, n) on a persistent pool of host threads
 * (the caller takes a share); `bytes` is the memory the whole range moves,
 * and small ranges run on the calling thread alone (gf_hostpool.cpp). */
void host_parallel_for(long n, long bytes, const std::function<void(long, long)>& fn);

/* gdt / gpar (nullable): per-group dt (<= 0 skips the group) and state
 * parity (1: the group's state is in the work items' qout buffers). */
/* max_ctas > 0 caps the grid: each CTA then walks the work list with a
 * grid stride, leaving the other SMs to concurrent launches. */
cudaError_t launch_patch_update(int m, const gf_patch_work* work, int nwork, const gf_phys* phys,
                                double dt, const double* gdt, const int* gpar, int maux, double* cfl,
                                unsigned long long* gmax, int* err, cudaStream_t st,
                                int max_ctas = 0, int goal = 0);
size_t patch_update_smem_bytes(int m);
int patch_update_occupancy(int m); /* resident CTAs per SM (throughput tile) */

/* Tile shapes of the production patch kernel: variants per patch size, the
 * selection per goal (0 throughput, 1 latency) used by launch_patch_update. */
int tile_count(int m);
int tile_shape(int m, int v, int* nt, int* rb, int* k = nullptr);
int tile_get(int m, int goal);
/* 1 when npatch patches of size m on the latency tile (each over its
 * cluster of CTAs) are all resident at once on the device, else 0 */
int latency_goal_fits(int m, long npatch);
int tile_set(int m, int goal, int v);
cudaError_t launch_patch_update_tile(int m, int v, const gf_patch_work* work, int nwork,
                                     const gf_phys* phys, double dt, const double* gdt,
                                     const int* gpar, int maux, double* cfl,
                                     unsigned long long* gmax, int* err, cudaStream_t st,
                                     int max_ctas);
cudaError_t launch_patch_update_exact(int m, const gf_patch_work* work, int nwork,
                                      const gf_phys* phys, double dt, const double* gdt,
                                      const int* gpar, int maux, double* cfl,
                                      unsigned long long* gmax, int* err, cudaStream_t st);

/* All patch sizes in one persistent launch. work holds n[0] items of mx =
 * 32, then n[1] of mx = 16, then n[2] of mx = 8; sched is a pair of counters
 * owned by the call site, zero before the first launch and reset by each
 * launch on exit (so launches sharing a pair must not overlap). The grid is
 * one CTA per SM, capped by max_ctas > 0. */
cudaError_t launch_patch_update_mixed(const gf_patch_work* work, const int n[3], const gf_phys* phys,
                                      double dt, const double* gdt, const int* gpar, int maux,
                                      double* cfl, unsigned long long* gmax, int* err,
                                      unsigned int* sched, cudaStream_t st, int max_ctas = 0);
cudaError_t launch_patch_update_mixed_exact(const gf_patch_work* work, const int n[3],
                                            const gf_phys* phys, double dt, const double* gdt,
                                            const int* gpar, int maux, double* cfl,
                                            unsigned long long* gmax, int* err, unsigned int* sched,
                                            cudaStream_t st, int max_ctas = 0);
int sm_count(); /* of the current device */

cudaError_t launch_aos_to_soa(const double* src, double* dst, long npatch, int ncell, int nf,
                              long src_stride, long dst_stride, cudaStream_t st);
cudaError_t launch_soa_to_aos(const double* src, double* dst, long npatch, int ncell, int nf,
                              long src_stride, long dst_stride, cudaStream_t st);
/* both of a host batch's layouts (q with nfa fields, aux with nfb) in one
 * launch; each set is npatch contiguous blocks of nf * ncell doubles */
cudaError_t launch_aos_to_soa_pair(const double* sa, double* da, int nfa, const double* sb, double* db,
                                   int nfb, long npatch, int ncell, cudaStream_t st);

/* Served scenarios: device-side time-step control around a round. */
cudaError_t launch_served_prepare(gf_group_state* gs, gf_ghost_block* blocks, double* gdt, int* gpar,
                                  unsigned long long* gmax, const double* hy_t,
                                  const double* hy_hu, int ng, cudaStream_t st,
                                  long long* qdelta = nullptr);
cudaError_t launch_served_finish(gf_group_state* gs, const double* gdt,
                                 const unsigned long long* gmax, const int* err, int ng,
                                 cudaStream_t st);

/* list (nullable: one block, nlist patches in order) names the patches to
 * fill as (block, local) pairs. */
cudaError_t launch_ghost_fill(int m, const gf_ghost_block* blocks, const gf_ghost_ref* list,
                              int nlist, const gf_phys* phys, cudaStream_t st);

/* qdelta (nullable): per-group offset (in doubles) added to the tasks' q
 * pointers, selecting each group's current state buffer. */
cudaError_t launch_transfer(int m, const gf_xfer_task* tasks, int ntask, const gf_phys* phys,
                            cudaStream_t st, const long long* qdelta = nullptr);
/* qad (geolib_source/qad.f:4-371) over ntask fine-patch sides, svdflx
 * accumulated; built without contraction like the other transfers. */
cudaError_t launch_qad(int m, const gf_qad_dev_task* tasks, int ntask, const gf_phys* phys,
                       double dt, cudaStream_t st);
cudaError_t launch_timeinterp(int m, const gf_tinterp_task* tasks, int ntask, double alpha,
                              cudaStream_t st);
cudaError_t launch_tags(int m, const gf_tag_task* tasks, int ntask, const gf_refine* rf,
                        const gf_phys* phys, int maxlevel, int init_flag, double t, int* tags,
                        cudaStream_t st);

/* Context access from host translation units other than gf_capi.cpp. */
cudaStream_t ctx_stream(gf_ctx* c);
int ctx_device(gf_ctx* c);
bool ctx_exact(gf_ctx* c); /* contraction-free update build selected */
bool ctx_mixed(gf_ctx* c); /* batched forms: one launch for all patch sizes */
const gf_phys* ctx_device_phys(gf_ctx* c);
const gf_phys* ctx_host_phys(gf_ctx* c, int slot);
int ctx_check_phys(gf_ctx* c, int slot, int maux = 0);
int ctx_fail(gf_ctx* c, int code, const char* msg);
int ctx_cuda_fail(gf_ctx* c, cudaError_t e, const char* what);

/* Forest raster pyramid (gf_forest_kernels.cu); levels are padded by 2. */
cudaError_t launch_pyramid_top(const double* src, double* dst, int nx, int ny, cudaStream_t st);
cudaError_t launch_pyramid_down(const double* fine, double* coarse, int nxc, int nyc,
                                cudaStream_t st);
cudaError_t launch_patch_fill(int m, const gf_fill_task* tasks, int ntask, cudaStream_t st);
/* cell averages of topo grids over a raster (interior cells inside the
 * domain, then the cells outside copy the nearest inside); *err = 1 when a
 * cell overlaps no grid */
cudaError_t launch_topo_raster(const gf_topo_grid* grids, const int* order, int n, int nx, int ny,
                               int halo, double xlower, double ylower, double dx, double dy,
                               double xupper, double yupper, double* out, int* err,
                               cudaStream_t st);
int topo_raster_device(gf_ctx* c, gf_topo* t, int nx, int ny, int halo, double xlower,
                       double ylower, double dx, double dy, double xupper, double yupper,
                       double* out, cudaStream_t st);
cudaError_t launch_tinterp_strip(int m, const gf_slot_task* tasks, int ntask, double alpha,
                                 cudaStream_t st);
cudaError_t launch_slot_copy(int m, const gf_slot_task* tasks, int ntask, cudaStream_t st);
cudaError_t launch_qinit_sea_level(const double* b, double* h, double* hu, double* hv, long cells,
                                   double sea_level, cudaStream_t st);
/* one record of 6 doubles per gauge at rec (level -1: not recorded) */
cudaError_t launch_gauge_sample(const gf_gauge_task* tasks, int n, const double* qbase,
                                const double* auxbase, int m, int maux, double drytol2, double t,
                                double* last, double* rec, cudaStream_t st);

/* A batched forest run driven one iteration at a time (gf_forest.cpp):
 * members join between iterations and leave when their run ends (or when
 * dropped); each iteration runs about half a millisecond of rounds, then
 * regrids the members that wait for it. */
struct ForestBatch;
/* stream_priority 0: the context's stream; k >= 1: a stream of its own, k = 1
 * at the greatest priority and each further k lower. max_ctas > 0 caps the
 * update grid. */
int forest_batch_create(gf_ctx* c, ForestBatch** out, int stream_priority = 0, int max_ctas = 0);
void forest_batch_destroy(ForestBatch* b);
/* checks the forest and starts its outstyle-1 run at its current time */
int forest_batch_add(ForestBatch* b, gf_forest* f, double t_final, int nout, double initial_dt,
                     double desired_cfl, double max_cfl);
int forest_batch_iterate(ForestBatch* b, int* live);
/* the same in two halves: launch (members and epoch fixed until the
 * iteration is taken in), then test (wait = 1 blocks) and take it in */
int forest_batch_launch(ForestBatch* b, int* live);
int forest_batch_test(ForestBatch* b, int wait, int* done);
bool forest_batch_inflight(const ForestBatch* b);
/* between iterations: a new update grid cap (the epoch is captured again) */
void forest_batch_set_max_ctas(ForestBatch* b, int max_ctas);
int forest_batch_members(const ForestBatch* b);
/* the forest leaves now (its run ended, or it is cancelled) */
void forest_batch_remove(ForestBatch* b, gf_forest* f);
bool forest_batch_running(const gf_forest* f);
void forest_batch_get_stats(const ForestBatch* b, gf_forest_batch_stats* st);
size_t forest_device_bytes(const gf_forest* f);

/* Subcycled forests side by side (gf_forest.cpp): each coarse step is the
 * forest's captured graph on a stream of a pool; a pass takes in finished
 * steps and launches the next ones without waiting on the device. */
struct SubForests;
int subforests_create(gf_ctx* c, SubForests** out);
void subforests_destroy(SubForests* s);
int subforests_add(SubForests* s, gf_forest* f, double t_final, int nout, double initial_dt,
                   double desired_cfl, double max_cfl);
int subforests_pass(SubForests* s, int* live, int* progress);
bool subforests_pending(const gf_forest* f);   /* a step in flight */
bool subforests_running(const gf_forest* f);   /* in flight or more to run */
void subforests_stop(gf_forest* f);            /* no further step */
void subforests_remove(SubForests* s, gf_forest* f); /* when nothing is in flight */
void subforests_get_stats(const SubForests* s, long long* steps_launched, long long* regrids,
                          long long* cell_updates);

} // namespace gf

#endif
