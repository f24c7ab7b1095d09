/*
 * C ABI of the GB300 patch update: contexts, physics sets, the plain
 * per-patch drop-in, the batched drop-in and device-resident levels.
 *
 * Nothing here computes the solution on the host: every update runs in the
 * sm_103a kernels of gf_kernels.cu. Errors are returned as gf_status codes
 * with a message kept on the context.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gf_internal.h"

namespace {

struct DevStatus {
    unsigned long long gmax; /* order-preserving bits of the max CFL */
    int err;                 /* non-zero: a bounded wait expired     */
    int pad;
};

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t reserve(size_t want)
    {
        if (want <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e == cudaSuccess) n = want;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

template <typename T>
struct HostBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t reserve(size_t want)
    {
        if (want <= n) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMallocHost(&p, want * sizeof(T));
        if (e == cudaSuccess) n = want;
        return e;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
    }
};

inline bool valid_m(int m) { return m == 8 || m == 16 || m == 32; }
inline long cells_of(int mx, int my) { return (long)(mx + 2 * GF_MBC) * (my + 2 * GF_MBC); }

} // namespace

struct gf_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    gf_phys* d_phys = nullptr;
    std::vector<gf_phys> h_phys;
    std::vector<unsigned char> phys_set;
    DevStatus* d_status = nullptr;
    DevStatus* h_status = nullptr; /* pinned */
    double* d_gdt = nullptr;
    double* h_gdt = nullptr; /* pinned */
    std::string last_error;
    bool exact = false; /* run the contraction-free build */
    bool mixed = true;  /* batched forms: one persistent launch for all patch sizes */
    /* scratch for the host-buffer drop-in paths */
    DevBuf<double> q_soa, aux_soa, cfl;
    HostBuf<double> h_cfl;
    /* a host batch's traffic in one block each side (io_layout) */
    DevBuf<char> io_dev;
    HostBuf<char> io_host;
    /* coarse/fine transfers and tags */
    DevBuf<gf_xfer_task> xfer;
    DevBuf<gf_tinterp_task> tint;
    DevBuf<gf_tag_task> tagt;
    DevBuf<int> tags;
    DevBuf<gf_refine> refine;
    /* qad */
    DevBuf<gf_qad_dev_task> qad;
    DevBuf<double> qad_flux;
};

struct gf_level {
    gf_ctx* ctx = nullptr;
    int npatch = 0, mx = 0, my = 0, maux = 0;
    long S = 0;
    double* d_q = nullptr;
    double* d_aux = nullptr;
    double* d_stage = nullptr;
    double* d_cfl = nullptr;
    gf_patch_work* d_work = nullptr;
    DevStatus* d_status = nullptr;
    std::vector<double> dx, dy;
    std::vector<int> phys;
    bool work_dirty = true;
    bool aux_loaded = false;
    /* ghost fill */
    int* d_nbr = nullptr;
    gf_patch_geom* d_geom = nullptr;
    int* d_phys_of = nullptr;
    std::vector<double> xlower, ylower;
    bool layout_set = false;
    bool geom_dirty = true;
    gf_bc_spec bc{};
    gf_ghost_block* d_ghost = nullptr; /* one block, rewritten per fill */
    std::vector<double> hy_time, hy_hu;
    std::vector<int> h_nbr;            /* host copy of the neighbour table */
    /* host-buffer step pipeline: patches in chunks [off[k], off[k+1]) whose
     * copies run on a second stream beside the other chunks' work */
    int pipe_request = 0;              /* 0 auto, else the number of chunks */
    bool pipe_ready = false;
    cudaStream_t cs = nullptr;         /* copies                            */
    cudaStream_t cs2 = nullptr;        /* odd chunks' transposes and updates */
    cudaStream_t cs3 = nullptr;        /* ghost fills and transposes back    */
    std::vector<cudaEvent_t> ev;       /* start, end2, end3, then up[k], upd[k], dn[k] */
    std::vector<int> off, dlo, dhi;    /* chunk j's ghost cells read chunks dlo[j]..dhi[j] */
    gf_ghost_ref* d_refs = nullptr;
};

namespace {

int fail(gf_ctx* c, int code, const std::string& msg)
{
    if (c) c->last_error = msg;
    return code;
}

int cuda_fail(gf_ctx* c, cudaError_t e, const char* what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(c, e == cudaErrorMemoryAllocation ? GF_ERR_NOMEM : GF_ERR_CUDA, m);
}

#define GF_CK(ctx, call)                                   \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

/* maux > 0: the slot must also suit a patch with maux aux fields (a variable
 * friction field inside them). */
int check_phys_slot(gf_ctx* c, int slot, int maux = 0)
{
    if (slot < 0 || slot >= GF_MAX_PHYS) return fail(c, GF_ERR_ARG, "physics slot out of range");
    if (!c->phys_set[slot]) return fail(c, GF_ERR_STATE, "physics slot not set");
    if (const char* why = gf::phys_problem(&c->h_phys[slot], maux)) return fail(c, GF_ERR_ARG, why);
    return GF_OK;
}

/* Tile goal of a batch of nwork patches: the latency tile (goal 1) when
 * even split over its cluster the batch leaves SMs idle, so that a lone patch
 * or a handful of them spread over more SMs; the throughput tile otherwise. */
int small_batch_goal(int m, int nwork) { return gf::latency_goal_fits(m, nwork); }

/* Enqueue one batch on the context stream: clear the status, launch. */
int enqueue_batch(gf_ctx* c, int m, const gf_patch_work* d_work, int nwork, int maux, double dt,
                  double* d_cfl, DevStatus* d_status, int goal = 0)
{
    GF_CK(c, cudaMemsetAsync(d_status, 0, sizeof(DevStatus), c->stream));
    if (c->exact)
        GF_CK(c, gf::launch_patch_update_exact(m, d_work, nwork, c->d_phys, dt, nullptr, nullptr, maux,
                                               d_cfl, &d_status->gmax, &d_status->err, c->stream));
    else
        GF_CK(c, gf::launch_patch_update(m, d_work, nwork, c->d_phys, dt, nullptr, nullptr, maux, d_cfl,
                                         &d_status->gmax, &d_status->err, c->stream, 0, goal));
    return GF_OK;
}

/* Fetch a batch status (waits for the stream). */
int finish_batch(gf_ctx* c, DevStatus* d_status, double* maxcfl)
{
    GF_CK(c, cudaMemcpyAsync(c->h_status, d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost,
                             c->stream));
    GF_CK(c, cudaStreamSynchronize(c->stream));
    if (c->h_status->err) return fail(c, GF_ERR_DEVICE, "patch kernel: bounded wait expired");
    double v;
    std::memcpy(&v, &c->h_status->gmax, sizeof v);
    if (maxcfl) *maxcfl = v;
    return GF_OK;
}

int run_batch(gf_ctx* c, int m, const gf_patch_work* d_work, int nwork, int maux, double dt,
              double* d_cfl, DevStatus* d_status, double* maxcfl, int goal = 0)
{
    int rc = enqueue_batch(c, m, d_work, nwork, maux, dt, d_cfl, d_status, goal);
    if (rc) return rc;
    return finish_batch(c, d_status, maxcfl);
}

int check_shape(gf_ctx* c, int mx, int my, int mbc, int meqn, int maux)
{
    if (mx != my || !valid_m(mx)) return fail(c, GF_ERR_UNSUPPORTED, "patch size must be mx = my in {8,16,32}");
    if (mbc != GF_MBC) return fail(c, GF_ERR_UNSUPPORTED, "mbc must be 2");
    if (meqn != GF_MEQN) return fail(c, GF_ERR_UNSUPPORTED, "meqn must be 3");
    if (maux < 1) return fail(c, GF_ERR_ARG, "maux must be >= 1 (aux(1) = bathymetry)");
    return GF_OK;
}

} // namespace

extern "C" {

void gf_phys_default(gf_phys* p)
{
    std::memset(p, 0, sizeof(*p));
    p->grav = 9.81;
    p->dry_tolerance = 1.0e-3;
    p->sea_level = 0.0;
    p->friction_depth = 1.0e6;
    p->manning_coefficient[0] = 0.035;
    p->manning_break[0] = 1.0e10;
    p->num_manning = 1;
    p->friction_forcing = 1;
    p->variable_friction = 0;
    p->friction_index = 0;
    p->order = 2;
    p->transverse = 2;
    p->mthlim[0] = p->mthlim[1] = p->mthlim[2] = 4;
    p->src_term = 1;
    p->maxcfl_cap = 100.0;
}

int gf_ctx_create(int device, gf_ctx** out)
{
    if (!out) return GF_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GF_ERR_CUDA;
    if (device < 0 || device >= ndev) return GF_ERR_ARG;
    gf_ctx* c = new gf_ctx();
    c->device = device;
    c->h_phys.resize(GF_MAX_PHYS);
    c->phys_set.assign(GF_MAX_PHYS, 0);
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_phys, sizeof(gf_phys) * GF_MAX_PHYS);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_status, sizeof(DevStatus));
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_status, sizeof(DevStatus));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_gdt, sizeof(double) * 64);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_gdt, sizeof(double) * 64);
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(DevStatus));
    if (e != cudaSuccess) {
        gf_ctx_destroy(c);
        return e == cudaErrorMemoryAllocation ? GF_ERR_NOMEM : GF_ERR_CUDA;
    }
    *out = c;
    return GF_OK;
}

void gf_ctx_destroy(gf_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->q_soa.release();
    c->aux_soa.release();
    c->cfl.release();
    c->h_cfl.release();
    c->io_dev.release();
    c->io_host.release();
    c->xfer.release();
    c->tint.release();
    c->tagt.release();
    c->tags.release();
    c->refine.release();
    c->qad.release();
    c->qad_flux.release();
    if (c->d_phys) cudaFree(c->d_phys);
    if (c->d_status) cudaFree(c->d_status);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->d_gdt) cudaFree(c->d_gdt);
    if (c->h_gdt) cudaFreeHost(c->h_gdt);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char* gf_ctx_last_error(const gf_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

int gf_ctx_set_phys(gf_ctx* c, int slot, const gf_phys* p)
{
    if (!c || !p) return GF_ERR_ARG;
    if (slot < 0 || slot >= GF_MAX_PHYS) return fail(c, GF_ERR_ARG, "physics slot out of range");
    if (const char* why = gf::phys_problem(p, 0)) return fail(c, GF_ERR_ARG, why);
    GF_CK(c, cudaSetDevice(c->device));
    c->h_phys[slot] = *p;
    c->phys_set[slot] = 1;
    GF_CK(c, cudaMemcpyAsync(c->d_phys + slot, &c->h_phys[slot], sizeof(gf_phys),
                             cudaMemcpyHostToDevice, c->stream));
    GF_CK(c, cudaStreamSynchronize(c->stream));
    return GF_OK;
}

int gf_patch_update(gf_ctx* c, int mx, int my, int mbc, int meqn, int maux, double dx, double dy,
                    double t, double dt, double* q, const double* aux, double* cfl)
{
    double* qs[1] = {q};
    const double* as[1] = {aux};
    double dxs[1] = {dx}, dys[1] = {dy};
    double maxcfl = 0.0;
    int rc = gf_patch_update_batch(c, 1, mx, my, mbc, meqn, maux, dxs, dys, t, dt, qs, as, nullptr,
                                   &maxcfl);
    if (rc == GF_OK && cfl) *cfl = maxcfl;
    return rc;
}

int gf_patch_update_batch(gf_ctx* c, int npatch, int mx, int my, int mbc, int meqn, int maux,
                          const double* dx, const double* dy, double t, double dt, double* const* q,
                          const double* const* aux, double* cfl, double* maxcfl)
{
    (void)t;
    if (!c) return GF_ERR_ARG;
    int rc = check_shape(c, mx, my, mbc, meqn, maux);
    if (rc) return rc;
    if (npatch < 0 || (npatch > 0 && (!dx || !dy || !q || !aux)))
        return fail(c, GF_ERR_ARG, "null argument");
    if ((rc = check_phys_slot(c, 0, maux))) return rc;
    if (npatch == 0) {
        if (maxcfl) *maxcfl = 0.0;
        return GF_OK;
    }
    GF_CK(c, cudaSetDevice(c->device));
    const long S = cells_of(mx, my);
    const size_t qn = (size_t)npatch * 3 * S, an = (size_t)npatch * maux * S;
    GF_CK(c, c->q_soa.reserve(qn));
    GF_CK(c, c->aux_soa.reserve(an));
    GF_CK(c, c->cfl.reserve(npatch));
    GF_CK(c, c->h_cfl.reserve(npatch));
    /* One block each side, [aux | work | status | q]: one copy carries the
     * batch in (the status zeroed on the host) and one brings the status and
     * q back. */
    auto a256 = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t o_work = a256(an * sizeof(double));
    const size_t o_status = o_work + a256((size_t)npatch * sizeof(gf_patch_work));
    const size_t o_q = o_status + a256(sizeof(DevStatus));
    const size_t io_bytes = o_q + qn * sizeof(double);
    GF_CK(c, c->io_dev.reserve(io_bytes));
    GF_CK(c, c->io_host.reserve(io_bytes));
    char* hio = c->io_host.p;
    char* dio = c->io_dev.p;
    double* hq = reinterpret_cast<double*>(hio + o_q);
    double* ha = reinterpret_cast<double*>(hio);
    gf_patch_work* hw = reinterpret_cast<gf_patch_work*>(hio + o_work);
    DevStatus* hs = reinterpret_cast<DevStatus*>(hio + o_status);
    DevStatus* d_status = reinterpret_cast<DevStatus*>(dio + o_status);
    const gf_patch_work* d_work = reinterpret_cast<const gf_patch_work*>(dio + o_work);

    /* Gather the patches into the pinned block; large batches gather on
     * several host threads. */
    for (int k = 0; k < npatch; ++k)
        if (!q[k] || !aux[k]) return fail(c, GF_ERR_ARG, "null patch pointer");
    gf::host_parallel_for(npatch, (long)((qn + an) * sizeof(double)), [&](long lo, long hi) {
        for (long k = lo; k < hi; ++k) {
            std::memcpy(hq + (size_t)k * 3 * S, q[k], sizeof(double) * 3 * S);
            std::memcpy(ha + (size_t)k * maux * S, aux[k], sizeof(double) * maux * S);
        }
    });
    for (int k = 0; k < npatch; ++k) {
        gf_patch_work w{};
        w.q = c->q_soa.p + (size_t)k * 3 * S;
        w.aux = c->aux_soa.p + (size_t)k * maux * S;
        w.dx = dx[k];
        w.dy = dy[k];
        w.phys = 0;
        w.group = 0;
        hw[k] = w;
    }
    std::memset(hs, 0, sizeof(DevStatus));
    GF_CK(c, cudaMemcpyAsync(dio, hio, io_bytes, cudaMemcpyHostToDevice, c->stream));
    GF_CK(c, gf::launch_aos_to_soa_pair(reinterpret_cast<const double*>(dio + o_q), c->q_soa.p, 3,
                                        reinterpret_cast<const double*>(dio), c->aux_soa.p, maux, npatch,
                                        (int)S, c->stream));
    /* update, layout back, results and status out: one wait at the end */
    if (c->exact)
        GF_CK(c, gf::launch_patch_update_exact(mx, d_work, npatch, c->d_phys, dt, nullptr, nullptr, maux,
                                               c->cfl.p, &d_status->gmax, &d_status->err, c->stream));
    else
        GF_CK(c, gf::launch_patch_update(mx, d_work, npatch, c->d_phys, dt, nullptr, nullptr, maux,
                                         c->cfl.p, &d_status->gmax, &d_status->err, c->stream, 0,
                                         small_batch_goal(mx, npatch)));
    GF_CK(c, gf::launch_soa_to_aos(c->q_soa.p, reinterpret_cast<double*>(dio + o_q), npatch, (int)S, 3,
                                   3 * S, 3 * S, c->stream));
    GF_CK(c, cudaMemcpyAsync(hio + o_status, dio + o_status, io_bytes - o_status, cudaMemcpyDeviceToHost,
                             c->stream));
    if (cfl)
        GF_CK(c, cudaMemcpyAsync(c->h_cfl.p, c->cfl.p, sizeof(double) * npatch,
                                 cudaMemcpyDeviceToHost, c->stream));
    GF_CK(c, cudaStreamSynchronize(c->stream));
    if (hs->err) return fail(c, GF_ERR_DEVICE, "patch kernel: bounded wait expired");
    double mc;
    std::memcpy(&mc, &hs->gmax, sizeof mc);
    gf::host_parallel_for(npatch, (long)(qn * sizeof(double)), [&](long lo, long hi) {
        for (long k = lo; k < hi; ++k)
            std::memcpy(q[k], hq + (size_t)k * 3 * S, sizeof(double) * 3 * S);
    });
    if (cfl) std::memcpy(cfl, c->h_cfl.p, sizeof(double) * npatch);
    if (maxcfl) *maxcfl = mc;
    return GF_OK;
}

/* ------------------------------------------------- buffered per-patch hook */

} /* extern "C" */

struct gf_step_buffer {
    gf_ctx* ctx = nullptr;
    int len = 0;
    int next_iter = 0;               /* the iter the next call must carry */
    int mx = 0, my = 0, maux = 0;
    std::vector<double*> q;
    std::vector<const double*> aux;
    std::vector<double> dx, dy;
};

extern "C" {

int gf_step_buffer_create(gf_ctx* c, int buffer_len, gf_step_buffer** out)
{
    if (!c || !out) return GF_ERR_ARG;
    *out = nullptr;
    if (buffer_len < 1) return fail(c, GF_ERR_ARG, "buffer_len must be >= 1");
    gf_step_buffer* b = new gf_step_buffer();
    b->ctx = c;
    b->len = buffer_len;
    b->q.reserve(buffer_len);
    b->aux.reserve(buffer_len);
    b->dx.reserve(buffer_len);
    b->dy.reserve(buffer_len);
    *out = b;
    return GF_OK;
}

void gf_step_buffer_destroy(gf_step_buffer* b) { delete b; }

int gf_step_buffer_update(gf_step_buffer* b, int iter, int total, int mx, int my, int mbc,
                          int meqn, int maux, double dx, double dy, double t, double dt, double* q,
                          const double* aux, double* maxcfl)
{
    if (!b || !q || !aux || !maxcfl) return GF_ERR_ARG;
    gf_ctx* c = b->ctx;
    *maxcfl = 0.0;
    int rc = check_shape(c, mx, my, mbc, meqn, maux);
    if (rc) return rc;
    if (total < 1 || iter < 0 || iter >= total) return fail(c, GF_ERR_ARG, "need 0 <= iter < total");
    if (iter == 0) { /* a new level step: forget a partial buffer of an abandoned one */
        b->q.clear();
        b->aux.clear();
        b->dx.clear();
        b->dy.clear();
        b->next_iter = 0;
    }
    if (iter != b->next_iter) return fail(c, GF_ERR_STATE, "iter out of sequence");
    if (!b->q.empty() && (mx != b->mx || my != b->my || maux != b->maux))
        return fail(c, GF_ERR_ARG, "patches of one buffer must share mx, my and maux");
    b->mx = mx;
    b->my = my;
    b->maux = maux;
    b->q.push_back(q);
    b->aux.push_back(aux);
    b->dx.push_back(dx);
    b->dy.push_back(dy);
    b->next_iter = iter + 1;
    if ((iter + 1) % b->len != 0 && iter + 1 != total) return GF_OK;
    const int n = (int)b->q.size();
    double mc = 0.0;
    rc = gf_patch_update_batch(c, n, mx, my, mbc, meqn, maux, b->dx.data(), b->dy.data(), t, dt,
                               b->q.data(), b->aux.data(), nullptr, &mc);
    b->q.clear();
    b->aux.clear();
    b->dx.clear();
    b->dy.clear();
    if (rc) return rc;
    *maxcfl = mc;
    return GF_OK;
}

/* ------------------------------------------------------------- levels */

int gf_level_create(gf_ctx* c, int npatch, int mx, int my, int maux, gf_level** out)
{
    if (!c || !out) return GF_ERR_ARG;
    *out = nullptr;
    int rc = check_shape(c, mx, my, GF_MBC, GF_MEQN, maux);
    if (rc) return rc;
    if (npatch <= 0) return fail(c, GF_ERR_ARG, "npatch must be positive");
    GF_CK(c, cudaSetDevice(c->device));
    gf_level* L = new gf_level();
    L->ctx = c;
    L->npatch = npatch;
    L->mx = mx;
    L->my = my;
    L->maux = maux;
    L->S = cells_of(mx, my);
    L->dx.assign(npatch, 1.0);
    L->dy.assign(npatch, 1.0);
    L->phys.assign(npatch, 0);
    L->xlower.assign(npatch, 0.0);
    L->ylower.assign(npatch, 0.0);
    for (int s = 0; s < 4; ++s) L->bc.mthbc[s] = 1;
    const size_t qn = (size_t)npatch * 3 * L->S, an = (size_t)npatch * maux * L->S;
    cudaError_t e = cudaMalloc(&L->d_q, qn * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&L->d_aux, an * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&L->d_stage, std::max(qn, an) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&L->d_cfl, npatch * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&L->d_work, npatch * sizeof(gf_patch_work));
    if (e == cudaSuccess) e = cudaMalloc(&L->d_status, sizeof(DevStatus));
    if (e == cudaSuccess) e = cudaMalloc(&L->d_nbr, (size_t)npatch * 8 * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&L->d_geom, (size_t)npatch * sizeof(gf_patch_geom));
    if (e == cudaSuccess) e = cudaMalloc(&L->d_phys_of, (size_t)npatch * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&L->d_ghost, sizeof(gf_ghost_block));
    if (e == cudaSuccess) e = cudaMemset(L->d_aux, 0, an * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(L->d_q, 0, qn * sizeof(double));
    if (e != cudaSuccess) {
        gf_level_destroy(L);
        return cuda_fail(c, e, "gf_level_create");
    }
    *out = L;
    return GF_OK;
}

void gf_level_destroy(gf_level* L)
{
    if (!L) return;
    cudaSetDevice(L->ctx->device);
    cudaStreamSynchronize(L->ctx->stream);
    if (L->d_q) cudaFree(L->d_q);
    if (L->d_aux) cudaFree(L->d_aux);
    if (L->d_stage) cudaFree(L->d_stage);
    if (L->d_cfl) cudaFree(L->d_cfl);
    if (L->d_work) cudaFree(L->d_work);
    if (L->d_status) cudaFree(L->d_status);
    if (L->d_nbr) cudaFree(L->d_nbr);
    if (L->d_geom) cudaFree(L->d_geom);
    if (L->d_phys_of) cudaFree(L->d_phys_of);
    if (L->d_ghost) cudaFree(L->d_ghost);
    if (L->d_refs) cudaFree(L->d_refs);
    for (cudaEvent_t e : L->ev) cudaEventDestroy(e);
    if (L->cs) cudaStreamDestroy(L->cs);
    if (L->cs2) cudaStreamDestroy(L->cs2);
    if (L->cs3) cudaStreamDestroy(L->cs3);
    delete L;
}

int gf_level_set_geometry(gf_level* L, const double* dx, const double* dy, const int* phys)
{
    if (!L || !dx || !dy) return GF_ERR_ARG;
    for (int k = 0; k < L->npatch; ++k) {
        if (!(dx[k] > 0.0) || !(dy[k] > 0.0)) return fail(L->ctx, GF_ERR_ARG, "dx, dy must be positive");
        if (phys && (phys[k] < 0 || phys[k] >= GF_MAX_PHYS)) return fail(L->ctx, GF_ERR_ARG, "bad physics slot");
    }
    std::copy(dx, dx + L->npatch, L->dx.begin());
    std::copy(dy, dy + L->npatch, L->dy.begin());
    if (phys) std::copy(phys, phys + L->npatch, L->phys.begin());
    else std::fill(L->phys.begin(), L->phys.end(), 0);
    L->work_dirty = true;
    L->geom_dirty = true;
    return GF_OK;
}

int gf_level_set_layout(gf_level* L, const int* nbr, const double* xlower, const double* ylower)
{
    if (!L || !nbr) return GF_ERR_ARG;
    gf_ctx* c = L->ctx;
    for (long k = 0; k < 8L * L->npatch; ++k)
        if (nbr[k] < -1 || nbr[k] >= L->npatch) return fail(c, GF_ERR_ARG, "neighbour index out of range");
    for (int k = 0; k < L->npatch; ++k)
        for (int s = 0; s < 8; ++s)
            if (nbr[8 * k + s] == k) return fail(c, GF_ERR_ARG, "a patch cannot neighbour itself");
    GF_CK(c, cudaSetDevice(c->device));
    if (xlower) std::copy(xlower, xlower + L->npatch, L->xlower.begin());
    if (ylower) std::copy(ylower, ylower + L->npatch, L->ylower.begin());
    GF_CK(c, cudaMemcpyAsync(L->d_nbr, nbr, (size_t)L->npatch * 8 * sizeof(int),
                             cudaMemcpyHostToDevice, c->stream));
    GF_CK(c, cudaStreamSynchronize(c->stream));
    L->h_nbr.assign(nbr, nbr + 8L * L->npatch);
    L->layout_set = true;
    L->geom_dirty = true;
    L->pipe_ready = false;
    return GF_OK;
}

int gf_level_set_bc(gf_level* L, const int* mthbc)
{
    if (!L || !mthbc) return GF_ERR_ARG;
    for (int s = 0; s < 4; ++s) {
        if (mthbc[s] < 0 || mthbc[s] > 3) return fail(L->ctx, GF_ERR_ARG, "mthbc must be 0..3");
        if (mthbc[s] == 0 && !L->bc.hydro_side[s])
            return fail(L->ctx, GF_ERR_ARG,
                        "mthbc = 0 needs a hydrograph on that side (the reference stops here)");
        L->bc.mthbc[s] = mthbc[s];
    }
    return GF_OK;
}

int gf_level_set_hydrograph(gf_level* L, int n, const double* time, const double* hu,
                            const int* side, double width, double x0, double y0)
{
    if (!L || n < 0 || (n > 0 && (!time || !hu || !side))) return GF_ERR_ARG;
    for (int i = 1; i < n; ++i)
        if (!(time[i] >= time[i - 1])) return fail(L->ctx, GF_ERR_ARG, "hydrograph times must increase");
    L->hy_time.assign(time, time + n);
    L->hy_hu.assign(hu, hu + n);
    for (int s = 0; s < 4; ++s) L->bc.hydro_side[s] = n > 0 ? (side[s] != 0) : 0;
    L->bc.width = width;
    L->bc.x0 = x0;
    L->bc.y0 = y0;
    return GF_OK;
}

/* interpolation (hydrograph/hydrograh_module.f90:176-221), discharge type */
static double hydro_interp(const gf_level* L, double t)
{
    const std::vector<double>& tm = L->hy_time;
    const std::vector<double>& hu = L->hy_hu;
    const size_t n = tm.size();
    if (n == 0) return 0.0;
    if (t < tm[0]) return hu[0];
    if (t > tm[n - 1]) return hu[n - 1];
    for (size_t i = 0; i + 1 < n; ++i)
        if (t >= tm[i] && t <= tm[i + 1])
            return hu[i] + (hu[i + 1] - hu[i]) / (tm[i + 1] - tm[i]) * (t - tm[i]);
    return 0.0;
}

/* geometry (if changed) and the ghost block for time t, on the context's stream */
static int level_ghost_prepare(gf_level* L, double t)
{
    gf_ctx* c = L->ctx;
    if (L->geom_dirty) {
        std::vector<gf_patch_geom> g(L->npatch);
        for (int k = 0; k < L->npatch; ++k) g[k] = {L->xlower[k], L->ylower[k], L->dx[k], L->dy[k]};
        GF_CK(c, cudaMemcpyAsync(L->d_geom, g.data(), g.size() * sizeof(gf_patch_geom),
                                 cudaMemcpyHostToDevice, c->stream));
        GF_CK(c, cudaMemcpyAsync(L->d_phys_of, L->phys.data(), L->phys.size() * sizeof(int),
                                 cudaMemcpyHostToDevice, c->stream));
        GF_CK(c, cudaStreamSynchronize(c->stream));
        L->geom_dirty = false;
    }
    gf_ghost_block blk{};
    blk.q = L->d_q;
    blk.aux = L->d_aux;
    blk.nbr = L->d_nbr;
    blk.geom = L->d_geom;
    blk.phys_of = L->d_phys_of;
    blk.bc = L->bc;
    blk.bc.q0hu = hydro_interp(L, t);
    blk.maux = L->maux;
    /* pageable source: the copy is staged before the call returns */
    GF_CK(c, cudaMemcpyAsync(L->d_ghost, &blk, sizeof blk, cudaMemcpyHostToDevice, c->stream));
    return GF_OK;
}

int gf_level_ghost_fill_async(gf_level* L, double t)
{
    if (!L) return GF_ERR_ARG;
    gf_ctx* c = L->ctx;
    if (!L->layout_set) return fail(c, GF_ERR_STATE, "level layout (neighbour table) not set");
    GF_CK(c, cudaSetDevice(c->device));
    int rc = level_ghost_prepare(L, t);
    if (rc) return rc;
    GF_CK(c, gf::launch_ghost_fill(L->mx, L->d_ghost, nullptr, L->npatch, c->d_phys, c->stream));
    return GF_OK;
}

int gf_level_ghost_fill(gf_level* L, double t)
{
    int rc = gf_level_ghost_fill_async(L, t);
    if (rc) return rc;
    GF_CK(L->ctx, cudaStreamSynchronize(L->ctx->stream));
    return GF_OK;
}

static int level_upload_q_async(gf_level* L, const double* q)
{
    gf_ctx* c = L->ctx;
    const size_t qn = (size_t)L->npatch * 3 * L->S;
    GF_CK(c, cudaMemcpyAsync(L->d_stage, q, qn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    GF_CK(c, gf::launch_aos_to_soa(L->d_stage, L->d_q, L->npatch, (int)L->S, 3, 3 * L->S, 3 * L->S,
                                   c->stream));
    return GF_OK;
}

static int level_download_q_async(gf_level* L, double* q)
{
    gf_ctx* c = L->ctx;
    const size_t qn = (size_t)L->npatch * 3 * L->S;
    GF_CK(c, gf::launch_soa_to_aos(L->d_q, L->d_stage, L->npatch, (int)L->S, 3, 3 * L->S, 3 * L->S,
                                   c->stream));
    GF_CK(c, cudaMemcpyAsync(q, L->d_stage, qn * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return GF_OK;
}

int gf_level_upload(gf_level* L, const double* q, const double* aux)
{
    if (!L || !q) return GF_ERR_ARG;
    gf_ctx* c = L->ctx;
    GF_CK(c, cudaSetDevice(c->device));
    if (aux) {
        const size_t an = (size_t)L->npatch * L->maux * L->S;
        GF_CK(c, cudaMemcpyAsync(L->d_stage, aux, an * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        GF_CK(c, gf::launch_aos_to_soa(L->d_stage, L->d_aux, L->npatch, (int)L->S, L->maux,
                                       L->maux * L->S, L->maux * L->S, c->stream));
        L->aux_loaded = true;
    }
    int rc = level_upload_q_async(L, q);
    if (rc) return rc;
    GF_CK(c, cudaStreamSynchronize(c->stream));
    return GF_OK;
}

int gf_level_download(gf_level* L, double* q)
{
    if (!L || !q) return GF_ERR_ARG;
    gf_ctx* c = L->ctx;
    GF_CK(c, cudaSetDevice(c->device));
    int rc = level_download_q_async(L, q);
    if (rc) return rc;
    GF_CK(c, cudaStreamSynchronize(c->stream));
    return GF_OK;
}

int gf_level_download_aux(gf_level* L, double* aux)
{
    if (!L || !aux) return GF_ERR_ARG;
    gf_ctx* c = L->ctx;
    GF_CK(c, cudaSetDevice(c->device));
    const size_t an = (size_t)L->npatch * L->maux * L->S;
    GF_CK(c, gf::launch_soa_to_aos(L->d_aux, L->d_stage, L->npatch, (int)L->S, L->maux,
                                   L->maux * L->S, L->maux * L->S, c->stream));
    GF_CK(c, cudaMemcpyAsync(aux, L->d_stage, an * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    GF_CK(c, cudaStreamSynchronize(c->stream));
    return GF_OK;
}

static int level_prepare(gf_level* L)
{
    gf_ctx* c = L->ctx;
    if (!L->aux_loaded) return fail(c, GF_ERR_STATE, "level aux (bathymetry) not uploaded");
    for (int k = 0; k < L->npatch; ++k) {
        int rc = check_phys_slot(c, L->phys[k], L->maux);
        if (rc) return rc;
    }
    if (!L->work_dirty) return GF_OK;
    std::vector<gf_patch_work> w(L->npatch, gf_patch_work{});
    for (int k = 0; k < L->npatch; ++k) {
        w[k].q = L->d_q + (size_t)k * 3 * L->S;
        w[k].aux = L->d_aux + (size_t)k * L->maux * L->S;
        w[k].dx = L->dx[k];
        w[k].dy = L->dy[k];
        w[k].phys = L->phys[k];
        w[k].group = 0;
    }
    GF_CK(c, cudaMemcpyAsync(L->d_work, w.data(), w.size() * sizeof(gf_patch_work),
                             cudaMemcpyHostToDevice, c->stream));
    GF_CK(c, cudaStreamSynchronize(c->stream));
    L->work_dirty = false;
    return GF_OK;
}

int gf_level_step(gf_level* L, double t, double dt, double* maxcfl)
{
    (void)t;
    if (!L) return GF_ERR_ARG;
    gf_ctx* c = L->ctx;
    GF_CK(c, cudaSetDevice(c->device));
    int rc = level_prepare(L);
    if (rc) return rc;
    return run_batch(c, L->mx, L->d_work, L->npatch, L->maux, dt, L->d_cfl, L->d_status, maxcfl);
}

int gf_level_ghost_fill_async(gf_level* L, double t);

/* Chunks for the host-buffer step: equal whole waves of the update kernel
 * (its resident CTAs on all SMs), about two waves or more each, at most 8. */
static int level_pipe_setup(gf_level* L)
{
    if (L->pipe_ready) return GF_OK;
    gf_ctx* c = L->ctx;
    int sms = 0;
    GF_CK(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    const int wave = std::max(1, gf::patch_update_occupancy(L->mx) * sms);
    int k = L->pipe_request > 0 ? L->pipe_request : std::max(1, std::min(8, L->npatch / (2 * wave)));
    k = std::min(k, L->npatch);
    int chunk = (L->npatch + k - 1) / k;
    if (L->pipe_request <= 0 && k > 1) chunk = (chunk + wave - 1) / wave * wave;
    L->off.clear();
    for (int p = 0; p < L->npatch; p += chunk) L->off.push_back(p);
    L->off.push_back(L->npatch);
    const int nc = (int)L->off.size() - 1;
    L->dlo.assign(nc, 0);
    L->dhi.assign(nc, 0);
    for (int j = 0; j < nc; ++j) {
        int lo = j, hi = j;
        if (L->layout_set)
            for (int p = L->off[j]; p < L->off[j + 1]; ++p)
                for (int s = 0; s < 8; ++s) {
                    const int nb = L->h_nbr[8L * p + s];
                    if (nb >= 0) {
                        lo = std::min(lo, nb / chunk);
                        hi = std::max(hi, nb / chunk);
                    }
                }
        L->dlo[j] = lo;
        L->dhi[j] = hi;
    }
    if (!L->cs) GF_CK(c, cudaStreamCreateWithFlags(&L->cs, cudaStreamNonBlocking));
    if (!L->cs2) GF_CK(c, cudaStreamCreateWithFlags(&L->cs2, cudaStreamNonBlocking));
    if (!L->cs3) GF_CK(c, cudaStreamCreateWithFlags(&L->cs3, cudaStreamNonBlocking));
    while ((int)L->ev.size() < 3 * nc + 3) {
        cudaEvent_t e;
        GF_CK(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        L->ev.push_back(e);
    }
    if (!L->d_refs) {
        std::vector<gf_ghost_ref> r(L->npatch);
        for (int p = 0; p < L->npatch; ++p) r[p] = gf_ghost_ref{0, p};
        GF_CK(c, cudaMalloc(&L->d_refs, r.size() * sizeof(gf_ghost_ref)));
        GF_CK(c, cudaMemcpy(L->d_refs, r.data(), r.size() * sizeof(gf_ghost_ref), cudaMemcpyHostToDevice));
    }
    L->pipe_ready = true;
    return GF_OK;
}

/* One step from host buffers, pipelined over chunks of patches: chunk k's
 * upload runs on a copy stream; its transpose and update run on one of two
 * compute streams (alternating, so one launch's last patches overlap the
 * next launch's first); once every chunk a chunk's ghost cells read is
 * updated, that chunk's ghost fill and transpose back follow on a third
 * stream (so they never hold up an update) and its download on the copy
 * stream. The kernels and data are those of one whole-level pass: the
 * result is identical. */
int gf_level_step_host(gf_level* L, double* q, double t, double dt, double* maxcfl)
{
    if (!L || !q) return GF_ERR_ARG;
    gf_ctx* c = L->ctx;
    GF_CK(c, cudaSetDevice(c->device));
    int rc = level_prepare(L);
    if (rc) return rc;
    if ((rc = level_pipe_setup(L))) return rc;
    if (L->layout_set && (rc = level_ghost_prepare(L, t + dt))) return rc;
    const int nc = (int)L->off.size() - 1;
    cudaEvent_t* up = L->ev.data() + 3;
    cudaEvent_t* upd = up + nc;
    cudaEvent_t* dn = upd + nc;
    const size_t per = 3 * (size_t)L->S;
    cudaStream_t cst[2] = {c->stream, L->cs2};
    GF_CK(c, cudaMemsetAsync(L->d_status, 0, sizeof(DevStatus), c->stream));
    GF_CK(c, cudaEventRecord(L->ev[0], c->stream));
    GF_CK(c, cudaStreamWaitEvent(L->cs, L->ev[0], 0));
    GF_CK(c, cudaStreamWaitEvent(L->cs2, L->ev[0], 0));
    GF_CK(c, cudaStreamWaitEvent(L->cs3, L->ev[0], 0));
    for (int k = 0; k < nc; ++k) {
        const size_t o = L->off[k] * per, n = (size_t)(L->off[k + 1] - L->off[k]) * per;
        GF_CK(c, cudaMemcpyAsync(L->d_stage + o, q + o, n * sizeof(double), cudaMemcpyHostToDevice, L->cs));
        GF_CK(c, cudaEventRecord(up[k], L->cs));
    }
    std::vector<char> done(nc, 0);
    auto finish_chunk = [&](int j) -> int {
        const int p0 = L->off[j], np = L->off[j + 1] - p0;
        cudaStream_t sj = L->cs3;
        for (int i = L->dlo[j]; i <= L->dhi[j]; ++i) GF_CK(c, cudaStreamWaitEvent(sj, upd[i], 0));
        if (L->layout_set)
            GF_CK(c, gf::launch_ghost_fill(L->mx, L->d_ghost, L->d_refs + p0, np, c->d_phys, sj));
        GF_CK(c, gf::launch_soa_to_aos(L->d_q + p0 * per, L->d_stage + p0 * per, np, (int)L->S, 3, per, per, sj));
        GF_CK(c, cudaEventRecord(dn[j], sj));
        GF_CK(c, cudaStreamWaitEvent(L->cs, dn[j], 0));
        GF_CK(c, cudaMemcpyAsync(q + p0 * per, L->d_stage + p0 * per, np * per * sizeof(double),
                                 cudaMemcpyDeviceToHost, L->cs));
        done[j] = 1;
        return GF_OK;
    };
    for (int k = 0; k < nc; ++k) {
        const int p0 = L->off[k], np = L->off[k + 1] - p0;
        cudaStream_t sk = cst[k & 1];
        GF_CK(c, cudaStreamWaitEvent(sk, up[k], 0));
        GF_CK(c, gf::launch_aos_to_soa(L->d_stage + p0 * per, L->d_q + p0 * per, np, (int)L->S, 3, per, per, sk));
        if (c->exact)
            GF_CK(c, gf::launch_patch_update_exact(L->mx, L->d_work + p0, np, c->d_phys, dt, nullptr, nullptr,
                                                   L->maux, L->d_cfl + p0, &L->d_status->gmax,
                                                   &L->d_status->err, sk));
        else
            GF_CK(c, gf::launch_patch_update(L->mx, L->d_work + p0, np, c->d_phys, dt, nullptr, nullptr, L->maux,
                                             L->d_cfl + p0, &L->d_status->gmax, &L->d_status->err, sk));
        GF_CK(c, cudaEventRecord(upd[k], sk));
        /* chunks whose neighbours are all updated now */
        for (int j = 0; j < nc; ++j)
            if (!done[j] && L->dhi[j] <= k && (rc = finish_chunk(j))) return rc;
    }
    GF_CK(c, cudaEventRecord(L->ev[1], L->cs2));
    GF_CK(c, cudaEventRecord(L->ev[2], L->cs3));
    GF_CK(c, cudaStreamWaitEvent(c->stream, L->ev[1], 0));
    GF_CK(c, cudaStreamWaitEvent(c->stream, L->ev[2], 0));
    double mc = 0.0;
    rc = finish_batch(c, L->d_status, &mc);
    GF_CK(c, cudaStreamSynchronize(L->cs));
    if (rc) return rc;
    if (maxcfl) *maxcfl = mc;
    return GF_OK;
}

int gf_level_set_pipeline(gf_level* L, int nchunks)
{
    if (!L || nchunks < 0) return GF_ERR_ARG;
    L->pipe_request = nchunks;
    L->pipe_ready = false;
    return GF_OK;
}

int gf_level_step_async(gf_level* L, double t, double dt)
{
    (void)t;
    if (!L) return GF_ERR_ARG;
    gf_ctx* c = L->ctx;
    GF_CK(c, cudaSetDevice(c->device));
    int rc = level_prepare(L);
    if (rc) return rc;
    return enqueue_batch(c, L->mx, L->d_work, L->npatch, L->maux, dt, L->d_cfl, L->d_status);
}

int gf_level_sync(gf_level* L, double* maxcfl)
{
    if (!L) return GF_ERR_ARG;
    gf_ctx* c = L->ctx;
    GF_CK(c, cudaSetDevice(c->device));
    return finish_batch(c, L->d_status, maxcfl);
}

int gf_ctx_set_fp_contract(gf_ctx* c, int allow)
{
    if (!c) return GF_ERR_ARG;
    c->exact = (allow == 0);
    return GF_OK;
}

int gf_ctx_set_mixed_update(gf_ctx* c, int on)
{
    if (!c) return GF_ERR_ARG;
    c->mixed = (on != 0);
    return GF_OK;
}

int gf_ctx_stream(gf_ctx* c, void** stream)
{
    if (!c || !stream) return GF_ERR_ARG;
    *stream = (void*)c->stream;
    return GF_OK;
}

int gf_level_patch_cfl(gf_level* L, double* cfl)
{
    if (!L || !cfl) return GF_ERR_ARG;
    gf_ctx* c = L->ctx;
    GF_CK(c, cudaSetDevice(c->device));
    GF_CK(c, cudaMemcpyAsync(cfl, L->d_cfl, L->npatch * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    GF_CK(c, cudaStreamSynchronize(c->stream));
    return GF_OK;
}

int gf_level_device_planes(gf_level* L, double** q, double** aux)
{
    if (!L) return GF_ERR_ARG;
    if (q) *q = L->d_q;
    if (aux) *aux = L->d_aux;
    return GF_OK;
}

/* ----------------------------------------------- coarse/fine, regrid */

int gf_level_transfer(gf_level* Cl, gf_level* Fl, int ntask, const gf_transfer* tasks)
{
    if (!Cl || !Fl || (ntask > 0 && !tasks) || ntask < 0) return GF_ERR_ARG;
    gf_ctx* c = Cl->ctx;
    if (Fl->ctx != c) return fail(c, GF_ERR_ARG, "levels belong to different contexts");
    if (Cl->mx != Fl->mx || Cl->maux != Fl->maux)
        return fail(c, GF_ERR_ARG, "coarse and fine levels need the same patch size and maux");
    if (ntask == 0) return GF_OK;
    std::vector<gf_xfer_task> t(ntask);
    for (int k = 0; k < ntask; ++k) {
        const gf_transfer& u = tasks[k];
        if (u.coarse < 0 || u.coarse >= Cl->npatch || u.fine < 0 || u.fine >= Fl->npatch)
            return fail(c, GF_ERR_ARG, "transfer patch index out of range");
        if (u.kind < GF_XFER_AVG_FACE || u.kind > GF_XFER_AVG2COARSE || u.code < 0 || u.code > 3)
            return fail(c, GF_ERR_ARG, "bad transfer kind or code");
        /* (ox, oy) must keep every fine index inside the array (ghosts included) */
        if (u.kind <= GF_XFER_INTERP_CORNER &&
            (u.ox < -2 * Cl->mx - 4 || u.ox > 2 * Cl->mx + 4 || u.oy < -2 * Cl->mx - 4 ||
             u.oy > 2 * Cl->mx + 4))
            return fail(c, GF_ERR_ARG, "transfer offset out of range");
        if (u.kind == GF_XFER_AVG_CORNER || u.kind == GF_XFER_INTERP_CORNER) {
            /* corner kinds touch all four fine cells unconditionally: require them inside */
            const int m = Cl->mx;
            const int i1 = (u.code == 0 || u.code == 2) ? (u.kind == GF_XFER_AVG_CORNER ? -1 : 1)
                                                         : (u.kind == GF_XFER_AVG_CORNER ? m + 2 : m);
            const int j1 = (u.code == 0 || u.code == 1) ? (u.kind == GF_XFER_AVG_CORNER ? -1 : 1)
                                                         : (u.kind == GF_XFER_AVG_CORNER ? m + 2 : m);
            const int lo = u.kind == GF_XFER_AVG_CORNER ? 1 : -1;
            const int hi = u.kind == GF_XFER_AVG_CORNER ? m : m + 2;
            for (int d = 0; d < 2; ++d) {
                /* both ghost layers (avg) or the single corner cell (interp) */
                const int ii = u.kind == GF_XFER_AVG_CORNER ? (i1 < 1 ? i1 + d : i1 - d) : i1;
                const int jj = u.kind == GF_XFER_AVG_CORNER ? (j1 < 1 ? j1 + d : j1 - d) : j1;
                const int fi0 = 2 * ii - 1 + u.ox, fj0 = 2 * jj - 1 + u.oy;
                if (fi0 < lo || fi0 + 1 > hi || fj0 < lo || fj0 + 1 > hi)
                    return fail(c, GF_ERR_ARG, "corner transfer reaches outside the fine patch");
            }
        }
        gf_xfer_task& x = t[k];
        x.qc = Cl->d_q + (size_t)u.coarse * 3 * Cl->S;
        x.ac = Cl->d_aux + (size_t)u.coarse * Cl->maux * Cl->S;
        x.qf = Fl->d_q + (size_t)u.fine * 3 * Fl->S;
        x.af = Fl->d_aux + (size_t)u.fine * Fl->maux * Fl->S;
        x.kind = u.kind;
        x.code = u.code;
        x.ox = u.ox;
        x.oy = u.oy;
        x.phys = Cl->phys[u.coarse];
        int rc = check_phys_slot(c, x.phys);
        if (rc) return rc;
    }
    GF_CK(c, cudaSetDevice(c->device));
    GF_CK(c, c->xfer.reserve(ntask));
    GF_CK(c, cudaMemcpyAsync(c->xfer.p, t.data(), ntask * sizeof(gf_xfer_task),
                             cudaMemcpyHostToDevice, c->stream));
    GF_CK(c, gf::launch_transfer(Cl->mx, c->xfer.p, ntask, c->d_phys, c->stream));
    GF_CK(c, cudaStreamSynchronize(c->stream));
    return GF_OK;
}

int gf_level_qad(gf_level* Cl, gf_level* Fl, int ntask, const gf_qad_task* tasks, double dt,
                 double* svdflx)
{
    if (!Cl || !Fl || ntask < 0 || (ntask > 0 && (!tasks || !svdflx))) return GF_ERR_ARG;
    gf_ctx* c = Cl->ctx;
    if (Fl->ctx != c) return fail(c, GF_ERR_ARG, "levels belong to different contexts");
    if (Cl->mx != Fl->mx || Cl->maux != Fl->maux)
        return fail(c, GF_ERR_ARG, "coarse and fine levels need the same patch size and maux");
    if (!(dt >= 0.0)) return fail(c, GF_ERR_ARG, "dt must be >= 0");
    if (ntask == 0) return GF_OK;
    const int m = Fl->mx, per = 3 * (m / 2);
    auto coarse_of = [](int fi, int o) { /* coarse 1-based index of fine 1-based fi */
        const int v = fi - o + 1;
        return v >= 0 ? v / 2 : -((1 - v) / 2); /* floor(v / 2) */
    };
    std::vector<gf_qad_dev_task> t(ntask);
    for (int k = 0; k < ntask; ++k) {
        const gf_qad_task& u = tasks[k];
        if (u.coarse < 0 || u.coarse >= Cl->npatch || u.fine < 0 || u.fine >= Fl->npatch)
            return fail(c, GF_ERR_ARG, "qad patch index out of range");
        if (u.side < 1 || u.side > 4) return fail(c, GF_ERR_ARG, "qad side must be 1..4");
        /* every coarse cell the side's ghost cells fall in must be interior */
        for (int f : {0, m - 1}) {
            int fi, fj;
            if (u.side == 1) { fi = 0; fj = 1 + f; }
            else if (u.side == 2) { fi = 1 + f; fj = m + 1; }
            else if (u.side == 3) { fi = m + 1; fj = 1 + f; }
            else { fi = 1 + f; fj = 0; }
            const int ci = coarse_of(fi, u.ox), cj = coarse_of(fj, u.oy);
            if (ci < 1 || ci > m || cj < 1 || cj > m)
                return fail(c, GF_ERR_ARG, "qad side's ghost cells are not over the coarse patch");
        }
        gf_qad_dev_task& x = t[k];
        x.qf = Fl->d_q + (size_t)u.fine * 3 * Fl->S;
        x.af = Fl->d_aux + (size_t)u.fine * Fl->maux * Fl->S;
        x.qc = Cl->d_q + (size_t)u.coarse * 3 * Cl->S;
        x.ac = Cl->d_aux + (size_t)u.coarse * Cl->maux * Cl->S;
        x.hx = Fl->dx[u.fine];
        x.hy = Fl->dy[u.fine];
        x.side = u.side;
        x.ox = u.ox;
        x.oy = u.oy;
        x.phys = Fl->phys[u.fine];
        int rc = check_phys_slot(c, x.phys);
        if (rc) return rc;
    }
    GF_CK(c, cudaSetDevice(c->device));
    GF_CK(c, c->qad.reserve(ntask));
    GF_CK(c, c->qad_flux.reserve((size_t)ntask * per));
    for (int k = 0; k < ntask; ++k) t[k].svdflx = c->qad_flux.p + (size_t)k * per;
    GF_CK(c, cudaMemcpyAsync(c->qad_flux.p, svdflx, sizeof(double) * ntask * per,
                             cudaMemcpyHostToDevice, c->stream));
    GF_CK(c, cudaMemcpyAsync(c->qad.p, t.data(), ntask * sizeof(gf_qad_dev_task),
                             cudaMemcpyHostToDevice, c->stream));
    GF_CK(c, gf::launch_qad(m, c->qad.p, ntask, c->d_phys, dt, c->stream));
    GF_CK(c, cudaMemcpyAsync(svdflx, c->qad_flux.p, sizeof(double) * ntask * per,
                             cudaMemcpyDeviceToHost, c->stream));
    GF_CK(c, cudaStreamSynchronize(c->stream));
    return GF_OK;
}

int gf_level_timeinterp(gf_level* D, gf_level* Cu, gf_level* La, double alpha)
{
    if (!D || !Cu || !La) return GF_ERR_ARG;
    gf_ctx* c = D->ctx;
    if (Cu->npatch != D->npatch || La->npatch != D->npatch || Cu->mx != D->mx || La->mx != D->mx)
        return fail(c, GF_ERR_ARG, "time interpolation needs three levels of the same shape");
    std::vector<gf_tinterp_task> t(D->npatch);
    for (int k = 0; k < D->npatch; ++k) {
        t[k].qcurr = Cu->d_q + (size_t)k * 3 * D->S;
        t[k].qlast = La->d_q + (size_t)k * 3 * D->S;
        t[k].qinterp = D->d_q + (size_t)k * 3 * D->S;
    }
    GF_CK(c, cudaSetDevice(c->device));
    GF_CK(c, c->tint.reserve(D->npatch));
    GF_CK(c, cudaMemcpyAsync(c->tint.p, t.data(), t.size() * sizeof(gf_tinterp_task),
                             cudaMemcpyHostToDevice, c->stream));
    GF_CK(c, gf::launch_timeinterp(D->mx, c->tint.p, D->npatch, alpha, c->stream));
    GF_CK(c, cudaStreamSynchronize(c->stream));
    return GF_OK;
}

static int run_tags(gf_level* L, const gf_refine* rf, std::vector<gf_tag_task>& t, int maxlevel,
                    int init_flag, double tm, int* tags)
{
    gf_ctx* c = L->ctx;
    if (rf->num_speed_tolerance < 0 || rf->num_speed_tolerance > GF_MAX_SPEEDS ||
        rf->num_flowgrades < 0 || rf->num_flowgrades > GF_MAX_FLOWGRADES ||
        rf->num_regions < 0 || rf->num_regions > GF_MAX_REGIONS)
        return fail(c, GF_ERR_ARG, "refinement parameter counts out of range");
    const int n = (int)t.size();
    if (n == 0) return GF_OK;
    GF_CK(c, cudaSetDevice(c->device));
    GF_CK(c, c->tagt.reserve(n));
    GF_CK(c, c->tags.reserve(n));
    GF_CK(c, c->refine.reserve(1));
    GF_CK(c, cudaMemcpyAsync(c->refine.p, rf, sizeof(gf_refine), cudaMemcpyHostToDevice, c->stream));
    GF_CK(c, cudaMemcpyAsync(c->tagt.p, t.data(), n * sizeof(gf_tag_task), cudaMemcpyHostToDevice,
                             c->stream));
    GF_CK(c, gf::launch_tags(L->mx, c->tagt.p, n, c->refine.p, c->d_phys, maxlevel, init_flag, tm,
                             c->tags.p, c->stream));
    GF_CK(c, cudaMemcpyAsync(tags, c->tags.p, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    GF_CK(c, cudaStreamSynchronize(c->stream));
    return GF_OK;
}

int gf_level_tag4refinement(gf_level* L, const gf_refine* rf, int level, int maxlevel,
                            int init_flag, double t, int* tags)
{
    if (!L || !rf || !tags) return GF_ERR_ARG;
    std::vector<gf_tag_task> tk(L->npatch);
    for (int k = 0; k < L->npatch; ++k) {
        int rc = check_phys_slot(L->ctx, L->phys[k]);
        if (rc) return rc;
        gf_tag_task& x = tk[k];
        std::memset(&x, 0, sizeof x);
        x.q[0] = L->d_q + (size_t)k * 3 * L->S;
        x.aux[0] = L->d_aux + (size_t)k * L->maux * L->S;
        x.xlower[0] = L->xlower[k];
        x.ylower[0] = L->ylower[k];
        x.dx = L->dx[k];
        x.dy = L->dy[k];
        x.level = level;
        x.nsib = 1;
        x.phys = L->phys[k];
    }
    return run_tags(L, rf, tk, maxlevel, init_flag, t, tags);
}

int gf_level_tag4coarsening(gf_level* L, const gf_refine* rf, int nfam, const int* fam, int level,
                            int maxlevel, int init_flag, double t, int* tags)
{
    if (!L || !rf || !tags || nfam < 0 || (nfam > 0 && !fam)) return GF_ERR_ARG;
    std::vector<gf_tag_task> tk(nfam);
    for (int f = 0; f < nfam; ++f) {
        gf_tag_task& x = tk[f];
        std::memset(&x, 0, sizeof x);
        for (int s = 0; s < 4; ++s) {
            const int k = fam[4 * f + s];
            if (k < 0 || k >= L->npatch) return fail(L->ctx, GF_ERR_ARG, "family index out of range");
            x.q[s] = L->d_q + (size_t)k * 3 * L->S;
            x.aux[s] = L->d_aux + (size_t)k * L->maux * L->S;
            x.xlower[s] = L->xlower[k];
            x.ylower[s] = L->ylower[k];
        }
        x.dx = L->dx[fam[4 * f]];
        x.dy = L->dy[fam[4 * f]];
        x.level = level;
        x.nsib = 4;
        x.phys = L->phys[fam[4 * f]];
        int rc = check_phys_slot(L->ctx, x.phys);
        if (rc) return rc;
    }
    return run_tags(L, rf, tk, maxlevel, init_flag, t, tags);
}

} // extern "C"

/* Context access for the other host translation units (gf_forest.cpp). */
namespace gf {
const char* phys_problem(const gf_phys* p, int maux)
{
    if (!p) return "null physics";
    if (p->num_manning < 0 || p->num_manning > GF_MAX_MANNING) return "num_manning out of range";
    if (p->order != 1 && p->order != 2) return "order must be 1 or 2";
    if (p->transverse < 0 || p->transverse > 2) return "transverse must be 0..2";
    if (!(p->grav > 0.0) || !(p->dry_tolerance >= 0.0)) return "bad grav / dry_tolerance";
    if (p->variable_friction && p->friction_index < 1)
        return "variable friction needs friction_index >= 1";
    if (p->variable_friction && maux > 0 && p->friction_index > maux)
        return "variable friction needs friction_index <= maux";
    return nullptr;
}

cudaStream_t ctx_stream(gf_ctx* c) { return c->stream; }
int ctx_device(gf_ctx* c) { return c->device; }
bool ctx_exact(gf_ctx* c) { return c->exact; }
bool ctx_mixed(gf_ctx* c) { return c->mixed; }
const gf_phys* ctx_device_phys(gf_ctx* c) { return c->d_phys; }
const gf_phys* ctx_host_phys(gf_ctx* c, int slot) { return &c->h_phys[slot]; }
int ctx_check_phys(gf_ctx* c, int slot, int maux) { return check_phys_slot(c, slot, maux); }
int ctx_fail(gf_ctx* c, int code, const char* msg) { return fail(c, code, msg); }
int ctx_cuda_fail(gf_ctx* c, cudaError_t e, const char* what) { return cuda_fail(c, e, what); }
} // namespace gf

/* ------------------------------------------------------------ tiling */
extern "C" int gf_tile_count(int mx)
{
    if (!(mx == 8 || mx == 16 || mx == 32)) return GF_ERR_ARG;
    return gf::tile_count(mx);
}

extern "C" int gf_tile_get(int mx, int goal)
{
    if (!(mx == 8 || mx == 16 || mx == 32)) return GF_ERR_ARG;
    return gf::tile_get(mx, goal);
}

extern "C" int gf_tile_set(int mx, int goal, int variant)
{
    if (!(mx == 8 || mx == 16 || mx == 32)) return GF_ERR_ARG;
    return gf::tile_set(mx, goal, variant) ? GF_ERR_ARG : GF_OK;
}

extern "C" int gf_autotune(gf_ctx* c, int reps, gf_tile_result* out)
{
    if (!c || !out || reps < 1) return GF_ERR_ARG;
    int rc = check_phys_slot(c, 0);
    if (rc) return rc;
    GF_CK(c, cudaSetDevice(c->device));
    static const int ms[3] = {8, 16, 32};
    const long target_cells = 4L << 20;
    const int nsmall = 8;
    cudaEvent_t e0, e1;
    GF_CK(c, cudaEventCreate(&e0));
    GF_CK(c, cudaEventCreate(&e1));
    int result = GF_OK;
    for (int k = 0; k < 3 && result == GF_OK; ++k) {
        const int m = ms[k];
        const long S = cells_of(m, m);
        const int np = (int)(target_cells / ((long)m * m));
        gf_tile_result& R = out[k];
        std::memset(&R, 0, sizeof R);
        R.mx = m;
        R.nvariant = std::min(gf::tile_count(m), GF_MAX_TILES);
        /* synthetic wet state, planes per patch: h, hu, hv then b */
        std::vector<double> hq((size_t)np * 3 * S), hb((size_t)np * S);
        for (int p = 0; p < np; ++p)
            for (long e = 0; e < S; ++e) {
                const int i = (int)(e % (m + 4)), j = (int)(e / (m + 4));
                const double h = 1.5 + 0.5 * std::sin(0.37 * i + 0.11 * p) * std::cos(0.23 * j);
                double* q = &hq[(size_t)p * 3 * S];
                q[e] = h;
                q[S + e] = 0.4 * h * std::sin(0.17 * j + p);
                q[2 * S + e] = 0.3 * h * std::cos(0.19 * i);
                hb[(size_t)p * S + e] = 0.2 * std::sin(0.05 * (i + j));
            }
        double *dq = nullptr, *db = nullptr, *dcfl = nullptr;
        gf_patch_work* dw = nullptr;
        cudaError_t e = cudaMalloc(&dq, hq.size() * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&db, hb.size() * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&dw, (size_t)np * sizeof(gf_patch_work));
        if (e == cudaSuccess) e = cudaMalloc(&dcfl, (size_t)np * sizeof(double));
        std::vector<gf_patch_work> w(np, gf_patch_work{});
        for (int p = 0; p < np; ++p) {
            w[p].q = dq + (size_t)p * 3 * S;
            w[p].aux = db + (size_t)p * S;
            w[p].dx = w[p].dy = 1.0;
        }
        if (e == cudaSuccess) e = cudaMemcpy(dq, hq.data(), hq.size() * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(db, hb.data(), hb.size() * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(dw, w.data(), w.size() * sizeof(gf_patch_work), cudaMemcpyHostToDevice);
        double best_t = -1.0, best_l = 1e300;
        for (int v = 0; v < R.nvariant && e == cudaSuccess; ++v) {
            gf::tile_shape(m, v, &R.threads[v], &R.band[v], &R.cluster[v]);
            for (int pass = 0; pass < 2 && e == cudaSuccess; ++pass) {
                const int n = pass == 0 ? np : nsmall;
                /* a set error flag makes the kernel skip its items */
                e = cudaMemsetAsync(c->d_status, 0, sizeof(DevStatus), c->stream);
                if (e == cudaSuccess)
                    e = gf::launch_patch_update_tile(m, v, dw, n, c->d_phys, 0.02, nullptr, nullptr, 1, dcfl,
                                                 &c->d_status->gmax, &c->d_status->err, c->stream, 0);
                if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
                for (int r = 0; r < reps && e == cudaSuccess; ++r)
                    e = gf::launch_patch_update_tile(m, v, dw, n, c->d_phys, 0.02, nullptr, nullptr, 1,
                                                     dcfl, &c->d_status->gmax, &c->d_status->err,
                                                     c->stream, 0);
                if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float msf = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&msf, e0, e1);
                const double ms1 = (double)msf / reps;
                if (pass == 0) R.throughput[v] = (double)np * m * m / (ms1 * 1e-3);
                else R.latency_us[v] = ms1 * 1e3;
            }
            if (e == cudaSuccess) {
                if (R.throughput[v] > best_t) { best_t = R.throughput[v]; R.best_throughput = v; }
                if (R.latency_us[v] < best_l) { best_l = R.latency_us[v]; R.best_latency = v; }
            }
        }
        if (dq) cudaFree(dq);
        if (db) cudaFree(db);
        if (dw) cudaFree(dw);
        if (dcfl) cudaFree(dcfl);
        if (e != cudaSuccess) {
            result = cuda_fail(c, e, "autotune");
            break;
        }
        gf::tile_set(m, 0, R.best_throughput);
        gf::tile_set(m, 1, R.best_latency);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return result;
}

