/*
 * Multi-level forests on one GPU: the ForestClaw machinery around the
 * patch update (quadtree leaves, 2:1 balance, ghost exchange between
 * levels, regrid, outstyle-1 time stepping), restated for a device-resident
 * slot pool. ForestClaw / p4est are external to the reference tree; the
 * rules below are this file's statement of them, followed equally by the
 * oracle's driver (oracle/forest.py):
 *
 *  - Leaves (level, I, J): I in [0, nbx*2^level), J in [0, nby*2^level).
 *    Canonical order: level, then J, then I.
 *  - Balance: leaves sharing a face or a corner differ by at most one
 *    level. Refinement ripples outward (a leaf next to a split leaf two
 *    levels finer splits too); a family coarsens only if every leaf along
 *    the parent's boundary stays within one level.
 *  - Ghost fill at t: (1) fine->coarse face and corner averages into coarse
 *    ghost cells; (2) same-level copies and physical boundaries on every
 *    leaf; (3) for each level above minlevel, coarse->fine face and corner
 *    interpolation into its leaves, then the physical boundaries again on
 *    those of them with a physical side. A corner that lies inside a
 *    coarser neighbour's face is filled by that face's interpolation.
 *  - Regrid (every regrid_interval accepted steps, after a ghost fill at
 *    the new time): refinement tags on leaves below maxlevel, coarsening
 *    tags on complete families above minlevel; tagged leaves split one
 *    level; balance; families whose four leaves are tagged, unsplit, and
 *    whose parent stays balanced merge; children take interpolate2fine of
 *    their parent, parents average2coarse of their children; every new
 *    patch takes its aux fields from the raster pyramid.
 *  - Initialisation: leaves at minlevel, then initial-refinement passes
 *    (init_flag = 1, no coarsening); every new patch takes the rasters.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "gf_internal.h"

namespace {

template <typename T>
struct DArr {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t reserve(size_t want)
    {
        if (want <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        size_t c = std::max<size_t>(want + want / 2, 16);
        cudaError_t e = cudaMalloc(&p, c * sizeof(T));
        if (e == cudaSuccess) n = c;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct Leaf {
    int level, I, J, slot;
};

inline bool canon_less(const Leaf& a, const Leaf& b)
{
    if (a.level != b.level) return a.level < b.level;
    if (a.J != b.J) return a.J < b.J;
    return a.I < b.I;
}

/* faces: left, right, bottom, top; corners: ll, lr, ul, ur */
const int FDI[4] = {-1, 1, 0, 0}, FDJ[4] = {0, 0, -1, 1};
const int CDI[4] = {-1, 1, -1, 1}, CDJ[4] = {-1, -1, 1, 1};

} // namespace

struct gf_forest {
    gf_ctx* ctx = nullptr;
    int device = 0; /* kept so that destroy does not need the context */
    gf_forest_opts o{};
    int M = 0;
    long S = 0;
    int nf = 0; /* raster fields: maux aux, then h, hu, hv */
    int cap = 0;
    /* raster pyramid: level l, field f at pyr[(l - minlevel) * nf + f] */
    std::vector<double*> pyr;
    /* slot pool */
    double* qbuf[2] = {nullptr, nullptr};
    double* aux = nullptr;
    int par = 0; /* buffer holding the current state */
    std::vector<int> free_slots;
    /* leaves */
    std::vector<Leaf> leaves;
    std::vector<std::vector<int>> grid; /* per level: position in leaves at (I, J), or -1 */
    /* boundary conditions */
    gf_bc_spec bc{};
    std::vector<double> hy_t, hy_hu;
    /* tables of the current leaves (rebuilt after every change) */
    bool dirty = true;
    DArr<int> d_nbr;               /* 8 per slot */
    DArr<gf_patch_geom> d_geom;    /* per slot   */
    DArr<gf_patch_work> d_work;
    DArr<gf_ghost_ref> d_refs_all;
    DArr<gf_ghost_ref> d_refs_lv;  /* refresh lists, concatenated by level */
    DArr<gf_xfer_task> d_avg[2];   /* per parity */
    DArr<gf_xfer_task> d_itp[2];   /* concatenated by level, per parity */
    DArr<gf_ghost_block> d_block;
    DArr<double> d_gdt;
    DArr<int> d_gpar;
    DArr<unsigned long long> d_rb; /* [err][gmax] */
    DArr<gf_tag_task> d_tagt;
    DArr<int> d_tags;
    DArr<gf_refine> d_refine;
    DArr<gf_xfer_task> d_rgx;
    DArr<gf_fill_task> d_fill;
    int n_avg = 0;
    std::vector<int> itp_off, itp_n, ref_off, ref_n; /* per level */
    unsigned long long* h_rb = nullptr;              /* pinned */
    long long cells = 0;                             /* interior cells of all leaves */
    gf_forest_stats st{};
    /* host copies of the tables (buffer-0 pointers), for batched epochs */
    std::vector<gf_patch_work> h_work;
    std::vector<gf_xfer_task> h_avg;
    std::vector<std::vector<gf_xfer_task>> h_itp; /* per level */
    std::vector<std::vector<int>> h_refresh;      /* slots per level */
    gf_group_state gst{};                         /* controller during a batched run */
    /* output: frames and gauges */
    std::string out_dir;
    int out_frames = 0, next_frame = 0;
    bool out_started = false; /* frame 0 and the initial gauge records done */
    std::vector<gf_gauge_task> gauges; /* window per gauge; placement rebuilt */
    std::vector<int> gauge_id;
    std::vector<double> gauge_x, gauge_y;
    bool gauges_placed = false, gauge_ghosts = false;
    DArr<gf_gauge_task> d_gtask;
    DArr<double> d_glast;
    DArr<double> d_grec;
    int grec_rows = 0, grec_cap = 0;
    /* subcycling: time-interpolated coarse patches and the step's start state */
    double* qi = nullptr;
    double* qsave = nullptr;
    bool sub_dirty = true;
    int sub_lo = 0, sub_hi = 0;                 /* levels present            */
    std::vector<int> lev_off, lev_n;             /* canonical range per level */
    std::vector<int> sx_avg_off, sx_avg_n;       /* [l * 6 + bc * 2 + bf]     */
    std::vector<int> sx_itp_off;                 /* [l * 6 + bc * 2 + bf]     */
    DArr<gf_xfer_task> d_sx;
    std::vector<int> ss_ti_off;                  /* [l * 2 + p_old]           */
    int ss_copy_off[3][2] = {{0, 0}, {0, 0}, {0, 0}}; /* save, restore, unify per par */
    int ss_copy_n[3] = {0, 0, 0};
    DArr<gf_slot_task> d_ss;
    DArr<int> d_par01;
    std::vector<gf_xfer_task> h_sx;              /* host copies of d_sx, d_ss */
    std::vector<gf_slot_task> h_ss;
    /* a subcycled step as a CUDA graph: a host-only plan pass writes the
     * step's level dts and ghost blocks (their boundary times) to pinned
     * staging; the graph's first node copies them to the device */
    bool sub_plan = false;
    int sub_nblk = 0;
    std::vector<gf_ghost_block> sub_blocks;
    char* h_sub = nullptr;
    size_t h_sub_cap = 0;
    DArr<char> d_sub_stage;
    cudaGraphExec_t sub_exec = nullptr;
    bool sub_graph_ok = false;
    int sub_graph_par = -1, sub_graph_nblk = -1;
    bool sub_graph_exact = false;
    long long sub_updates = 0; /* cell-updates of the step in flight */
    unsigned long long sub_epoch = 0; /* counts rebuilds of the subcycling tables */
    /* a subcycled run driven step by step among others (concurrent runner):
     * the outstyle-1 state between steps, the step in flight on `sst` */
    struct SubRun {
        double t_curr = 0, dt_minlevel = 0, dt_outer = 0, tend = 0, dt_step = 0;
        double desired_cfl = 0, max_cfl = 0;
        int nout = 0, nint = 0;
        bool took_small = false, active = false, pending = false, cancel = false;
    } sr;
    cudaStream_t sst = nullptr;       /* owned by the runner */
    cudaEvent_t sev_ctx = nullptr, sev_done = nullptr;
};

namespace {

int ffail(gf_forest* f, int code, const char* msg) { return gf::ctx_fail(f->ctx, code, msg); }

#define FK(f, call)                                                               \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) return gf::ctx_cuda_fail((f)->ctx, e_, #call);     \
    } while (0)

inline int nx_at(const gf_forest* f, int l) { return f->o.nbx * f->M << l; }
inline int ny_at(const gf_forest* f, int l) { return f->o.nby * f->M << l; }
inline int npx_at(const gf_forest* f, int l) { return f->o.nbx << l; }
inline int npy_at(const gf_forest* f, int l) { return f->o.nby << l; }
inline double dx_at(const gf_forest* f, int l) { return f->o.dx0 / (double)(1 << l); }
inline double dy_at(const gf_forest* f, int l) { return f->o.dy0 / (double)(1 << l); }

inline double* qslot(gf_forest* f, int b, int slot) { return f->qbuf[b] + (size_t)slot * 3 * f->S; }
inline double* aslot(gf_forest* f, int slot) { return f->aux + (size_t)slot * f->o.maux * f->S; }

int find(const gf_forest* f, int l, int I, int J)
{
    if (l < f->o.minlevel || l > f->o.maxlevel || I < 0 || J < 0) return -1;
    const int nx = f->o.nbx << l;
    if (I >= nx || J >= (f->o.nby << l)) return -1;
    return f->grid[l][(size_t)J * nx + I];
}

/* leaf containing the level-l cell block (I, J) at level <= l, or -1 */
int containing(const gf_forest* f, int l, int I, int J)
{
    for (int k = l; k >= f->o.minlevel; --k) {
        int p = find(f, k, I >> (l - k), J >> (l - k));
        if (p >= 0) return p;
    }
    return -1;
}

inline bool inside(const gf_forest* f, int l, int I, int J)
{
    return I >= 0 && J >= 0 && I < npx_at(f, l) && J < npy_at(f, l);
}

void reindex(gf_forest* f)
{
    std::sort(f->leaves.begin(), f->leaves.end(), canon_less);
    if ((int)f->grid.size() != f->o.maxlevel + 1) {
        f->grid.assign(f->o.maxlevel + 1, {});
        for (int l = f->o.minlevel; l <= f->o.maxlevel; ++l)
            f->grid[l].assign((size_t)(f->o.nbx << l) * (f->o.nby << l), -1);
    } else {
        for (int l = f->o.minlevel; l <= f->o.maxlevel; ++l)
            std::fill(f->grid[l].begin(), f->grid[l].end(), -1);
    }
    f->cells = 0;
    for (size_t k = 0; k < f->leaves.size(); ++k) {
        const Leaf& L = f->leaves[k];
        f->grid[L.level][(size_t)L.J * (f->o.nbx << L.level) + L.I] = (int)k;
        f->cells += (long long)f->M * f->M;
    }
    f->dirty = true;
    f->sub_dirty = true;
    f->gauges_placed = false;
}

int alloc_slot(gf_forest* f)
{
    if (f->free_slots.empty()) return -1;
    int s = f->free_slots.back();
    f->free_slots.pop_back();
    return s;
}

/* build the raster pyramid from the finest-level rasters (host) */
int build_pyramid(gf_forest* f, const double* fields)
{
    const gf_forest_opts& o = f->o;
    cudaStream_t st = gf::ctx_stream(f->ctx);
    const int nlev = o.maxlevel - o.minlevel + 1;
    f->pyr.assign((size_t)nlev * f->nf, nullptr);
    for (int l = o.minlevel; l <= o.maxlevel; ++l)
        for (int k = 0; k < f->nf; ++k) {
            const size_t n = (size_t)(nx_at(f, l) + 2 * GF_MBC) * (ny_at(f, l) + 2 * GF_MBC);
            FK(f, cudaMalloc(&f->pyr[(size_t)(l - o.minlevel) * f->nf + k], n * sizeof(double)));
        }
    if (!fields) {
        /* zero rasters: the caller fills them (gf_forest_set_topo) */
        for (size_t k = 0; k < f->pyr.size(); ++k) {
            const int l = o.minlevel + (int)(k / f->nf);
            const size_t n = (size_t)(nx_at(f, l) + 2 * GF_MBC) * (ny_at(f, l) + 2 * GF_MBC);
            FK(f, cudaMemsetAsync(f->pyr[k], 0, n * sizeof(double), st));
        }
        FK(f, cudaStreamSynchronize(st));
        return GF_OK;
    }
    const int nx = nx_at(f, o.maxlevel), ny = ny_at(f, o.maxlevel);
    double* stage = nullptr;
    FK(f, cudaMalloc(&stage, (size_t)nx * ny * sizeof(double)));
    int rc = GF_OK;
    for (int k = 0; k < f->nf && !rc; ++k) {
        cudaError_t e = cudaMemcpyAsync(stage, fields + (size_t)k * nx * ny,
                                        (size_t)nx * ny * sizeof(double), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = gf::launch_pyramid_top(stage, f->pyr[(size_t)(o.maxlevel - o.minlevel) * f->nf + k], nx,
                                       ny, st);
        for (int l = o.maxlevel - 1; l >= o.minlevel && e == cudaSuccess; --l)
            e = gf::launch_pyramid_down(f->pyr[(size_t)(l + 1 - o.minlevel) * f->nf + k],
                                        f->pyr[(size_t)(l - o.minlevel) * f->nf + k], nx_at(f, l),
                                        ny_at(f, l), st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st); /* the stage is reused */
        if (e != cudaSuccess) rc = gf::ctx_cuda_fail(f->ctx, e, "raster pyramid");
    }
    cudaFree(stage);
    return rc;
}

} // namespace

namespace {

gf_xfer_task xtask(gf_forest* f, int b, int kind, int cslot, int fslot, int code, int ox, int oy)
{
    gf_xfer_task t;
    t.qc = qslot(f, b, cslot);
    t.ac = aslot(f, cslot);
    t.qf = qslot(f, b, fslot);
    t.af = aslot(f, fslot);
    t.kind = kind;
    t.code = code;
    t.ox = ox;
    t.oy = oy;
    t.phys = f->o.phys_slot;
    t.group = 0;
    return t;
}

/* Neighbour tables and transfer lists of the current leaves. */
int build_tables(gf_forest* f)
{
    if (!f->dirty) return GF_OK;
    const gf_forest_opts& o = f->o;
    const int M = f->M;
    const int nlev = o.maxlevel + 1;
    std::vector<int> nbr((size_t)f->cap * 8, -1);
    std::vector<gf_patch_geom> geom(f->cap, gf_patch_geom{0, 0, 1, 1});
    std::vector<gf_patch_work> work(f->leaves.size(), gf_patch_work{});
    std::vector<gf_ghost_ref> refs_all(f->leaves.size());
    std::vector<gf_xfer_task> avg[2];
    std::vector<std::vector<gf_xfer_task>> itp[2];
    std::vector<std::vector<gf_ghost_ref>> refresh(nlev);
    itp[0].resize(nlev);
    itp[1].resize(nlev);
    for (size_t k = 0; k < f->leaves.size(); ++k) {
        const Leaf& P = f->leaves[k];
        const int l = P.level, I = P.I, J = P.J, s = P.slot;
        const double dx = dx_at(f, l), dy = dy_at(f, l);
        geom[s] = {o.x0 + (double)I * M * dx, o.y0 + (double)J * M * dy, dx, dy};
        gf_patch_work& w = work[k];
        w.q = qslot(f, 0, s);
        w.qout = qslot(f, 1, s);
        w.aux = aslot(f, s);
        w.dx = dx;
        w.dy = dy;
        w.phys = o.phys_slot;
        w.group = 0;
        refs_all[k] = gf_ghost_ref{0, s};
        bool interp = false, physical = false;
        for (int fc = 0; fc < 4; ++fc) {
            const int NI = I + FDI[fc], NJ = J + FDJ[fc];
            int& nb = nbr[(size_t)8 * s + fc];
            if (!inside(f, l, NI, NJ)) {
                nb = -1;
                physical = true;
                continue;
            }
            int q = find(f, l, NI, NJ);
            if (q >= 0) {
                nb = f->leaves[q].slot;
                continue;
            }
            nb = -2;
            q = l > o.minlevel ? find(f, l - 1, NI >> 1, NJ >> 1) : -1;
            if (q >= 0) {
                /* coarser neighbour: its face toward P is the opposite one */
                const Leaf& C = f->leaves[q];
                for (int b = 0; b < 2; ++b)
                    itp[b][l].push_back(xtask(f, b, GF_XFER_INTERP_FACE, C.slot, s, fc ^ 1,
                                              M * (2 * C.I - I), M * (2 * C.J - J)));
                interp = true;
                continue;
            }
            /* finer: the two children of the neighbour region next to P */
            for (int c = 0; c < 2; ++c) {
                int FI, FJ;
                if (fc < 2) {
                    FI = 2 * NI + (FDI[fc] < 0 ? 1 : 0);
                    FJ = 2 * J + c;
                } else {
                    FI = 2 * I + c;
                    FJ = 2 * NJ + (FDJ[fc] < 0 ? 1 : 0);
                }
                const int r = find(f, l + 1, FI, FJ);
                if (r < 0) return ffail(f, GF_ERR_STATE, "forest is not 2:1 balanced across a face");
                for (int b = 0; b < 2; ++b)
                    avg[b].push_back(xtask(f, b, GF_XFER_AVG_FACE, s, f->leaves[r].slot, fc,
                                           M * (2 * I - FI), M * (2 * J - FJ)));
            }
        }
        for (int cc = 0; cc < 4; ++cc) {
            const int DI = I + CDI[cc], DJ = J + CDJ[cc];
            int& nb = nbr[(size_t)8 * s + 4 + cc];
            if (!inside(f, l, DI, DJ)) {
                nb = -1;
                continue;
            }
            int q = find(f, l, DI, DJ);
            if (q >= 0) {
                nb = f->leaves[q].slot;
                continue;
            }
            nb = -2;
            q = l > o.minlevel ? find(f, l - 1, DI >> 1, DJ >> 1) : -1;
            if (q >= 0) {
                const Leaf& C = f->leaves[q];
                const bool dxok = CDI[cc] > 0 ? 2 * C.I == DI : 2 * C.I + 1 == DI;
                const bool dyok = CDJ[cc] > 0 ? 2 * C.J == DJ : 2 * C.J + 1 == DJ;
                if (dxok && dyok) {
                    /* diagonal coarser neighbour: its corner toward P is 3 - cc */
                    for (int b = 0; b < 2; ++b)
                        itp[b][l].push_back(xtask(f, b, GF_XFER_INTERP_CORNER, C.slot, s, 3 - cc,
                                                  M * (2 * C.I - I), M * (2 * C.J - J)));
                    interp = true;
                }
                /* otherwise the corner lies inside C's face: face interpolation fills it */
                continue;
            }
            if (containing(f, l, DI, DJ) >= 0)
                return ffail(f, GF_ERR_STATE, "forest is not 2:1 balanced across a corner");
            const int FI = 2 * DI + (CDI[cc] < 0 ? 1 : 0), FJ = 2 * DJ + (CDJ[cc] < 0 ? 1 : 0);
            const int r = find(f, l + 1, FI, FJ);
            if (r < 0) return ffail(f, GF_ERR_STATE, "forest is not 2:1 balanced across a corner");
            for (int b = 0; b < 2; ++b)
                avg[b].push_back(xtask(f, b, GF_XFER_AVG_CORNER, s, f->leaves[r].slot, cc,
                                       M * (2 * I - FI), M * (2 * J - FJ)));
        }
        if (interp && physical) refresh[l].push_back(gf_ghost_ref{0, s});
    }
    cudaStream_t st = gf::ctx_stream(f->ctx);
    FK(f, f->d_nbr.reserve(nbr.size()));
    FK(f, f->d_geom.reserve(geom.size()));
    FK(f, f->d_work.reserve(work.size()));
    FK(f, f->d_refs_all.reserve(refs_all.size()));
    FK(f, cudaMemcpyAsync(f->d_nbr.p, nbr.data(), nbr.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    FK(f, cudaMemcpyAsync(f->d_geom.p, geom.data(), geom.size() * sizeof(gf_patch_geom),
                          cudaMemcpyHostToDevice, st));
    FK(f, cudaMemcpyAsync(f->d_work.p, work.data(), work.size() * sizeof(gf_patch_work),
                          cudaMemcpyHostToDevice, st));
    FK(f, cudaMemcpyAsync(f->d_refs_all.p, refs_all.data(), refs_all.size() * sizeof(gf_ghost_ref),
                          cudaMemcpyHostToDevice, st));
    f->n_avg = (int)avg[0].size();
    f->itp_off.assign(nlev, 0);
    f->itp_n.assign(nlev, 0);
    f->ref_off.assign(nlev, 0);
    f->ref_n.assign(nlev, 0);
    std::vector<gf_xfer_task> itp_all[2];
    std::vector<gf_ghost_ref> ref_all;
    for (int l = 0; l < nlev; ++l) {
        f->itp_off[l] = (int)itp_all[0].size();
        f->itp_n[l] = (int)itp[0][l].size();
        for (int b = 0; b < 2; ++b) itp_all[b].insert(itp_all[b].end(), itp[b][l].begin(), itp[b][l].end());
        f->ref_off[l] = (int)ref_all.size();
        f->ref_n[l] = (int)refresh[l].size();
        ref_all.insert(ref_all.end(), refresh[l].begin(), refresh[l].end());
    }
    for (int b = 0; b < 2; ++b) {
        FK(f, f->d_avg[b].reserve(avg[b].size() + 1));
        FK(f, f->d_itp[b].reserve(itp_all[b].size() + 1));
        if (!avg[b].empty())
            FK(f, cudaMemcpyAsync(f->d_avg[b].p, avg[b].data(), avg[b].size() * sizeof(gf_xfer_task),
                                  cudaMemcpyHostToDevice, st));
        if (!itp_all[b].empty())
            FK(f, cudaMemcpyAsync(f->d_itp[b].p, itp_all[b].data(),
                                  itp_all[b].size() * sizeof(gf_xfer_task), cudaMemcpyHostToDevice, st));
    }
    FK(f, f->d_refs_lv.reserve(ref_all.size() + 1));
    if (!ref_all.empty())
        FK(f, cudaMemcpyAsync(f->d_refs_lv.p, ref_all.data(), ref_all.size() * sizeof(gf_ghost_ref),
                              cudaMemcpyHostToDevice, st));
    /* pageable sources are staged before each copy call returns */
    f->h_work.swap(work);
    f->h_avg.swap(avg[0]);
    f->h_itp.assign(nlev, {});
    f->h_refresh.assign(nlev, {});
    for (int l = 0; l < nlev; ++l) {
        f->h_itp[l].swap(itp[0][l]);
        for (const gf_ghost_ref& r : refresh[l]) f->h_refresh[l].push_back(r.local);
    }
    f->dirty = false;
    return GF_OK;
}

/* hydrograph/hydrograh_module.f90:176-221, discharge type */
double hydro_at(const gf_forest* f, double t)
{
    const size_t n = f->hy_t.size();
    if (n == 0) return 0.0;
    if (t < f->hy_t[0]) return f->hy_hu[0];
    if (t > f->hy_t[n - 1]) return f->hy_hu[n - 1];
    for (size_t i = 0; i + 1 < n; ++i)
        if (t >= f->hy_t[i] && t <= f->hy_t[i + 1])
            return f->hy_hu[i] + (f->hy_hu[i + 1] - f->hy_hu[i]) / (f->hy_t[i + 1] - f->hy_t[i]) *
                                     (t - f->hy_t[i]);
    return 0.0;
}

int ghost_fill(gf_forest* f, double t)
{
    int rc = build_tables(f);
    if (rc) return rc;
    cudaStream_t st = gf::ctx_stream(f->ctx);
    const gf_phys* phys = gf::ctx_device_phys(f->ctx);
    gf_ghost_block blk{};
    blk.q = f->qbuf[f->par];
    blk.aux = f->aux;
    blk.nbr = f->d_nbr.p;
    blk.geom = f->d_geom.p;
    blk.phys_of = nullptr;
    blk.bc = f->bc;
    blk.bc.q0hu = hydro_at(f, t);
    blk.phys = f->o.phys_slot;
    blk.maux = f->o.maux;
    blk.skip = 0;
    FK(f, f->d_block.reserve(1));
    /* pageable source: staged before the call returns */
    FK(f, cudaMemcpyAsync(f->d_block.p, &blk, sizeof blk, cudaMemcpyHostToDevice, st));
    if (f->n_avg) FK(f, gf::launch_transfer(f->M, f->d_avg[f->par].p, f->n_avg, phys, st));
    FK(f, gf::launch_ghost_fill(f->M, f->d_block.p, f->d_refs_all.p, (int)f->leaves.size(), phys, st));
    for (int l = f->o.minlevel + 1; l <= f->o.maxlevel; ++l) {
        if (f->itp_n[l])
            FK(f, gf::launch_transfer(f->M, f->d_itp[f->par].p + f->itp_off[l], f->itp_n[l], phys, st));
        if (f->ref_n[l])
            FK(f, gf::launch_ghost_fill(f->M, f->d_block.p, f->d_refs_lv.p + f->ref_off[l], f->ref_n[l],
                                        phys, st));
    }
    return GF_OK;
}

int step(gf_forest* f, double t, double dt, double* cfl)
{
    int rc = ghost_fill(f, t);
    if (rc) return rc;
    cudaStream_t st = gf::ctx_stream(f->ctx);
    FK(f, f->d_gdt.reserve(1));
    FK(f, f->d_gpar.reserve(1));
    FK(f, f->d_rb.reserve(2));
    FK(f, cudaMemcpyAsync(f->d_gdt.p, &dt, sizeof dt, cudaMemcpyHostToDevice, st));
    FK(f, cudaMemcpyAsync(f->d_gpar.p, &f->par, sizeof(int), cudaMemcpyHostToDevice, st));
    FK(f, cudaMemsetAsync(f->d_rb.p, 0, 2 * sizeof(unsigned long long), st));
    const gf_phys* phys = gf::ctx_device_phys(f->ctx);
    int* err = reinterpret_cast<int*>(f->d_rb.p);
    if (gf::ctx_exact(f->ctx))
        FK(f, gf::launch_patch_update_exact(f->M, f->d_work.p, (int)f->leaves.size(), phys, 0.0,
                                            f->d_gdt.p, f->d_gpar.p, f->o.maux, nullptr, f->d_rb.p + 1,
                                            err, st));
    else
        FK(f, gf::launch_patch_update(f->M, f->d_work.p, (int)f->leaves.size(), phys, 0.0, f->d_gdt.p,
                                      f->d_gpar.p, f->o.maux, nullptr, f->d_rb.p + 1, err, st));
    FK(f, cudaMemcpyAsync(f->h_rb, f->d_rb.p, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    FK(f, cudaStreamSynchronize(st));
    if ((int)f->h_rb[0]) return ffail(f, GF_ERR_DEVICE, "a patch-update copy wait timed out");
    double c;
    std::memcpy(&c, &f->h_rb[1], sizeof c);
    if (cfl) *cfl = c;
    return GF_OK;
}

} // namespace

namespace {

/* One forest's regrid in flight: tags, then the new leaves. */
struct Regrid {
    gf_forest* f = nullptr;
    double t = 0.0;
    int init_flag = 0;
    std::vector<int> who;                   /* leaf of each refinement-tag task */
    std::vector<std::array<int, 4>> fams;   /* complete families (ll, lr, ul, ur) */
    std::vector<char> refine, coarsen;
    size_t base = 0;                        /* first tag of this forest in its class */
    bool changed = false;
};

inline int mclass_of(int mx) { return mx == 8 ? 0 : mx == 16 ? 1 : 2; }
const int kMx[3] = {8, 16, 32};

gf_tag_task tag_task(gf_forest* f, const Regrid& R, int level, int nsib)
{
    gf_tag_task x;
    std::memset(&x, 0, sizeof x);
    x.dx = dx_at(f, level);
    x.dy = dy_at(f, level);
    x.level = level;
    x.nsib = nsib;
    x.phys = f->o.phys_slot;
    x.rf = f->d_refine.p;
    x.t = R.t;
    x.maxlevel = f->o.maxlevel;
    x.init_flag = R.init_flag;
    return x;
}

/* Refinement tags (leaves below maxlevel) and coarsening tags (complete
 * families above minlevel) of several forests: one launch per patch size. */
int run_tags(gf_ctx* ctx, std::vector<Regrid>& W)
{
    std::vector<gf_tag_task> tk[3];
    for (Regrid& R : W) {
        gf_forest* f = R.f;
        const gf_forest_opts& o = f->o;
        const int c = mclass_of(f->M);
        R.base = tk[c].size();
        R.who.clear();
        R.fams.clear();
        for (size_t k = 0; k < f->leaves.size(); ++k) {
            const Leaf& L = f->leaves[k];
            if (L.level >= o.maxlevel) continue;
            gf_tag_task x = tag_task(f, R, L.level, 1);
            x.q[0] = qslot(f, f->par, L.slot);
            x.aux[0] = aslot(f, L.slot);
            x.xlower[0] = o.x0 + (double)L.I * f->M * dx_at(f, L.level);
            x.ylower[0] = o.y0 + (double)L.J * f->M * dy_at(f, L.level);
            tk[c].push_back(x);
            R.who.push_back((int)k);
        }
        if (!R.init_flag) {
            for (size_t k = 0; k < f->leaves.size(); ++k) {
                const Leaf& L = f->leaves[k];
                if (L.level <= o.minlevel || (L.I & 1) || (L.J & 1)) continue;
                std::array<int, 4> fam;
                bool full = true;
                for (int cc = 0; cc < 4 && full; ++cc) {
                    fam[cc] = find(f, L.level, L.I + (cc & 1), L.J + (cc >> 1));
                    full = fam[cc] >= 0;
                }
                if (!full) continue;
                gf_tag_task x = tag_task(f, R, L.level, 4);
                for (int cc = 0; cc < 4; ++cc) {
                    const Leaf& C = f->leaves[fam[cc]];
                    x.q[cc] = qslot(f, f->par, C.slot);
                    x.aux[cc] = aslot(f, C.slot);
                    x.xlower[cc] = o.x0 + (double)C.I * f->M * dx_at(f, C.level);
                    x.ylower[cc] = o.y0 + (double)C.J * f->M * dy_at(f, C.level);
                }
                tk[c].push_back(x);
                R.fams.push_back(fam);
            }
        }
        R.refine.assign(f->leaves.size(), 0);
        R.coarsen.assign(R.fams.size(), 0);
    }
    size_t total = tk[0].size() + tk[1].size() + tk[2].size();
    if (total == 0) return GF_OK;
    cudaStream_t st = gf::ctx_stream(ctx);
    gf_tag_task* d_t = nullptr;
    int* d_tags = nullptr;
    std::vector<int> tags(total);
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&d_t), total * sizeof(gf_tag_task), st);
    if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&d_tags), total * sizeof(int), st);
    size_t off = 0;
    for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
        if (tk[c].empty()) continue;
        e = cudaMemcpyAsync(d_t + off, tk[c].data(), tk[c].size() * sizeof(gf_tag_task),
                            cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = gf::launch_tags(kMx[c], d_t + off, (int)tk[c].size(), nullptr, gf::ctx_device_phys(ctx), 0,
                                0, 0.0, d_tags + off, st);
        off += tk[c].size();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(tags.data(), d_tags, total * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (d_t) cudaFreeAsync(d_t, st);
    if (d_tags) cudaFreeAsync(d_tags, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return gf::ctx_cuda_fail(ctx, e, "refinement tags");
    size_t cbase[3] = {0, tk[0].size(), tk[0].size() + tk[1].size()};
    for (Regrid& R : W) {
        const int* tg = tags.data() + cbase[mclass_of(R.f->M)] + R.base;
        for (size_t k = 0; k < R.who.size(); ++k) R.refine[R.who[k]] = tg[k] != 0;
        for (size_t m = 0; m < R.fams.size(); ++m) R.coarsen[m] = tg[R.who.size() + m] != 0;
    }
    return GF_OK;
}

/* Grow the split set until the refined forest is 2:1 balanced. */
void balance_splits(const gf_forest* f, std::vector<char>& split)
{
    std::vector<int> work;
    for (size_t k = 0; k < split.size(); ++k)
        if (split[k]) work.push_back((int)k);
    while (!work.empty()) {
        const int k = work.back();
        work.pop_back();
        const Leaf& P = f->leaves[k];
        const int l = P.level;
        for (int d = 0; d < 8; ++d) {
            const int di = d < 4 ? FDI[d] : CDI[d - 4], dj = d < 4 ? FDJ[d] : CDJ[d - 4];
            const int NI = P.I + di, NJ = P.J + dj;
            if (!inside(f, l, NI, NJ)) continue;
            const int q = containing(f, l, NI, NJ);
            if (q < 0) continue; /* finer there */
            if (f->leaves[q].level <= l - 1 && !split[q]) {
                split[q] = 1; /* P's children at l + 1 would touch a leaf at <= l - 1 */
                work.push_back(q);
            }
        }
    }
}

/* May the family under parent (l - 1, PI, PJ) merge, given the splits? */
bool family_can_merge(const gf_forest* f, int l, int PI, int PJ, const std::vector<char>& split)
{
    /* leaves along the parent's boundary, as level-l cell blocks */
    for (int a = -1; a <= 2; ++a)
        for (int b = -1; b <= 2; ++b) {
            if (a >= 0 && a <= 1 && b >= 0 && b <= 1) continue;
            const int I = 2 * PI + a, J = 2 * PJ + b;
            if (!inside(f, l, I, J)) continue;
            const int q = containing(f, l, I, J);
            if (q < 0) return false;                               /* finer than l */
            if (f->leaves[q].level == l && split[q]) return false; /* will be l + 1 */
        }
    return true;
}

gf_fill_task fill_task(gf_forest* f, const Leaf& L, bool with_q)
{
    gf_fill_task x;
    std::memset(&x, 0, sizeof x);
    int n = 0;
    const size_t base = (size_t)(L.level - f->o.minlevel) * f->nf;
    for (int a = 0; a < f->o.maux; ++a, ++n) {
        x.src[n] = f->pyr[base + a];
        x.dst[n] = aslot(f, L.slot) + (size_t)a * f->S;
    }
    if (with_q)
        for (int m = 0; m < 3; ++m, ++n) {
            x.src[n] = f->pyr[base + f->o.maux + m];
            x.dst[n] = qslot(f, f->par, L.slot) + (size_t)m * f->S;
        }
    x.nfield = n;
    x.nx = nx_at(f, L.level);
    x.I = L.I;
    x.J = L.J;
    return x;
}

/* Fill tasks and transfer tasks, one launch of each per patch size. */
int launch_fills_and_transfers(gf_ctx* ctx, std::vector<gf_fill_task>* fill,
                               std::vector<gf_xfer_task>* xfer)
{
    size_t nf = 0, nx = 0;
    for (int c = 0; c < 3; ++c) {
        nf += fill[c].size();
        nx += xfer[c].size();
    }
    if (nf + nx == 0) return GF_OK;
    cudaStream_t st = gf::ctx_stream(ctx);
    gf_fill_task* d_f = nullptr;
    gf_xfer_task* d_x = nullptr;
    cudaError_t e = cudaSuccess;
    if (nf) e = cudaMallocAsync(reinterpret_cast<void**>(&d_f), nf * sizeof(gf_fill_task), st);
    if (e == cudaSuccess && nx) e = cudaMallocAsync(reinterpret_cast<void**>(&d_x), nx * sizeof(gf_xfer_task), st);
    size_t of = 0, ox = 0;
    /* fills first: interpolate2fine reads the children's bathymetry */
    for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
        if (fill[c].empty()) continue;
        e = cudaMemcpyAsync(d_f + of, fill[c].data(), fill[c].size() * sizeof(gf_fill_task),
                            cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = gf::launch_patch_fill(kMx[c], d_f + of, (int)fill[c].size(), st);
        of += fill[c].size();
    }
    for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
        if (xfer[c].empty()) continue;
        e = cudaMemcpyAsync(d_x + ox, xfer[c].data(), xfer[c].size() * sizeof(gf_xfer_task),
                            cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = gf::launch_transfer(kMx[c], d_x + ox, (int)xfer[c].size(), gf::ctx_device_phys(ctx), st);
        ox += xfer[c].size();
    }
    if (d_f) cudaFreeAsync(d_f, st);
    if (d_x) cudaFreeAsync(d_x, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st); /* old slots are read before reuse */
    if (e != cudaSuccess) return gf::ctx_cuda_fail(ctx, e, "regrid transfers");
    return GF_OK;
}

/* Decide splits and merges from the tags and replace the leaves of every
 * forest; children / parents take interpolate2fine / average2coarse of the
 * current state (at initialisation: the rasters); new patches take their aux
 * fields from the pyramid. */
int apply_regrids(gf_ctx* ctx, std::vector<Regrid>& W, bool init)
{
    std::vector<gf_fill_task> fill[3];
    std::vector<gf_xfer_task> xfer[3];
    std::vector<std::vector<Leaf>> next(W.size());
    std::vector<std::vector<int>> freed(W.size());
    for (size_t w = 0; w < W.size(); ++w) {
        Regrid& R = W[w];
        gf_forest* f = R.f;
        const int c = mclass_of(f->M);
        std::vector<char> split = R.refine;
        balance_splits(f, split);
        std::vector<char> merge(R.fams.size(), 0);
        for (size_t m = 0; m < R.fams.size(); ++m) {
            if (!R.coarsen[m]) continue;
            bool any_split = false;
            for (int cc = 0; cc < 4; ++cc) any_split |= split[R.fams[m][cc]] != 0;
            const Leaf& C0 = f->leaves[R.fams[m][0]];
            merge[m] = !any_split && family_can_merge(f, C0.level, C0.I >> 1, C0.J >> 1, split);
        }
        size_t need = 0;
        std::vector<char> in_merge(f->leaves.size(), 0);
        for (size_t k = 0; k < split.size(); ++k) need += split[k] ? 4 : 0;
        for (size_t m = 0; m < R.fams.size(); ++m)
            if (merge[m]) {
                need += 1;
                for (int cc = 0; cc < 4; ++cc) in_merge[R.fams[m][cc]] = 1;
            }
        R.changed = need > 0;
        if (!R.changed) continue;
        if (need > f->free_slots.size())
            return ffail(f, GF_ERR_NOMEM, "forest slot pool exhausted (raise max_patches)");
        const int b = f->par;
        std::vector<Leaf>& nx = next[w];
        for (size_t k = 0; k < f->leaves.size(); ++k) {
            const Leaf& P = f->leaves[k];
            if (in_merge[k]) continue;
            if (!split[k]) {
                nx.push_back(P);
                continue;
            }
            for (int cc = 0; cc < 4; ++cc) {
                Leaf C{P.level + 1, 2 * P.I + (cc & 1), 2 * P.J + (cc >> 1), alloc_slot(f)};
                nx.push_back(C);
                fill[c].push_back(fill_task(f, C, init));
                if (!init) xfer[c].push_back(xtask(f, b, GF_XFER_INTERP2FINE, P.slot, C.slot, cc, 0, 0));
            }
            freed[w].push_back(P.slot);
        }
        for (size_t m = 0; m < R.fams.size(); ++m) {
            if (!merge[m]) continue;
            const Leaf& C0 = f->leaves[R.fams[m][0]];
            Leaf Pn{C0.level - 1, C0.I >> 1, C0.J >> 1, alloc_slot(f)};
            nx.push_back(Pn);
            fill[c].push_back(fill_task(f, Pn, false));
            for (int cc = 0; cc < 4; ++cc) {
                const Leaf& C = f->leaves[R.fams[m][cc]];
                xfer[c].push_back(xtask(f, b, GF_XFER_AVG2COARSE, Pn.slot, C.slot, cc, 0, 0));
                freed[w].push_back(C.slot);
            }
        }
    }
    int rc = launch_fills_and_transfers(ctx, fill, xfer);
    if (rc) return rc;
    for (size_t w = 0; w < W.size(); ++w) {
        Regrid& R = W[w];
        if (!R.changed) continue;
        gf_forest* f = R.f;
        for (int sl : freed[w]) f->free_slots.push_back(sl);
        f->leaves.swap(next[w]);
        reindex(f);
        f->st.npatch = (int)f->leaves.size();
        f->st.npatch_max = std::max(f->st.npatch_max, f->st.npatch);
    }
    return GF_OK;
}

/* Regrid several forests, each at its own time, with shared launches. */
int regrid_many(gf_ctx* ctx, std::vector<gf_forest*>& fs, const std::vector<double>& ts)
{
    std::vector<Regrid> W(fs.size());
    for (size_t k = 0; k < fs.size(); ++k) {
        int rc = ghost_fill(fs[k], ts[k]); /* interpolate2fine reads the parents' ghost cells */
        if (rc) return rc;
        W[k].f = fs[k];
        W[k].t = ts[k];
        W[k].init_flag = 0;
    }
    int rc = run_tags(ctx, W);
    if (!rc) rc = apply_regrids(ctx, W, false);
    if (!rc)
        for (gf_forest* f : fs) f->st.regrids++;
    return rc;
}

int regrid(gf_forest* f, double t, bool* changed)
{
    std::vector<gf_forest*> fs{f};
    std::vector<double> ts{t};
    const size_t n0 = f->leaves.size();
    std::vector<Leaf> before = f->leaves;
    int rc = regrid_many(f->ctx, fs, ts);
    if (changed) {
        bool ch = f->leaves.size() != n0;
        for (size_t k = 0; !ch && k < n0; ++k)
            ch = f->leaves[k].level != before[k].level || f->leaves[k].I != before[k].I ||
                 f->leaves[k].J != before[k].J;
        *changed = ch;
    }
    return rc;
}

int init_forest(gf_forest* f)
{
    const gf_forest_opts& o = f->o;
    f->free_slots.clear();
    for (int s2 = f->cap - 1; s2 >= 0; --s2) f->free_slots.push_back(s2);
    f->leaves.clear();
    const size_t n0 = (size_t)npx_at(f, o.minlevel) * npy_at(f, o.minlevel);
    if (n0 > f->free_slots.size()) return ffail(f, GF_ERR_NOMEM, "max_patches below the minlevel patch count");
    for (int J = 0; J < npy_at(f, o.minlevel); ++J)
        for (int I = 0; I < npx_at(f, o.minlevel); ++I)
            f->leaves.push_back(Leaf{o.minlevel, I, J, alloc_slot(f)});
    f->par = 0;
    reindex(f);
    {
        std::vector<gf_fill_task> fill[3];
        std::vector<gf_xfer_task> none[3];
        for (const Leaf& L : f->leaves) fill[mclass_of(f->M)].push_back(fill_task(f, L, true));
        int rc = launch_fills_and_transfers(f->ctx, fill, none);
        if (rc) return rc;
    }
    f->st = gf_forest_stats{};
    for (int pass = o.minlevel; pass < o.maxlevel; ++pass) {
        std::vector<Regrid> W(1);
        W[0].f = f;
        W[0].t = 0.0;
        W[0].init_flag = 1;
        int rc = run_tags(f->ctx, W);
        if (!rc) rc = apply_regrids(f->ctx, W, true);
        if (rc) return rc;
        if (!W[0].changed) break;
    }
    f->st.npatch = (int)f->leaves.size();
    f->st.npatch_max = std::max(f->st.npatch_max, f->st.npatch);
    return build_tables(f);
}

/* ---- gauges ---------------------------------------------------------
 * Each gauge lives in the leaf holding it: the finest-level patch index of
 * the point (half-open cells, the domain's upper edges closed) selects the
 * leaf through the level grids. Inside the leaf the cell and the offsets
 * follow fc2d_geoclaw_update_gauge (fortran_source/geoclaw_gauges_fort.f90:
 * 19-25); rounding at a patch edge is clamped to the cells the stencil can
 * reach. The placement is rebuilt whenever the leaves change. */
int place_gauges(gf_forest* f)
{
    const gf_forest_opts& o = f->o;
    const int L = o.maxlevel, M = f->M;
    const int nxL = npx_at(f, L), nyL = npy_at(f, L);
    const double pxL = M * dx_at(f, L), pyL = M * dy_at(f, L);
    f->gauge_ghosts = false;
    for (size_t g = 0; g < f->gauges.size(); ++g) {
        gf_gauge_task& T = f->gauges[g];
        T.slot = -1;
        const double x = f->gauge_x[g], y = f->gauge_y[g];
        const double ux = (x - o.x0) / pxL, uy = (y - o.y0) / pyL;
        if (!(ux >= 0.0) || !(uy >= 0.0) || ux > nxL || uy > nyL) continue;
        const int IF = std::min((int)std::floor(ux), nxL - 1), JF = std::min((int)std::floor(uy), nyL - 1);
        const int p = containing(f, L, IF, JF);
        if (p < 0) continue;
        const Leaf& lf = f->leaves[p];
        const double dx = dx_at(f, lf.level), dy = dy_at(f, lf.level);
        const double xl = o.x0 + lf.I * M * dx, yl = o.y0 + lf.J * M * dy;
        const int ii = std::min(std::max((int)((x - xl) / dx) + 1, 1), M + 1);
        const int jj = std::min(std::max((int)((y - yl) / dy) + 1, 1), M + 1);
        T.xoff = (x - (xl + (ii - .5) * dx)) / dx;
        T.yoff = (y - (yl + (jj - .5) * dy)) / dy;
        T.slot = lf.slot;
        T.level = lf.level;
        T.ii = ii;
        T.jj = jj;
        if (ii >= M || jj >= M) f->gauge_ghosts = true;
    }
    FK(f, f->d_gtask.reserve(f->gauges.size()));
    FK(f, cudaMemcpy(f->d_gtask.p, f->gauges.data(), f->gauges.size() * sizeof(gf_gauge_task),
                     cudaMemcpyHostToDevice));
    f->gauges_placed = true;
    return GF_OK;
}

/* buffered records -> gaugeXXXXX.txt rows, each gauge's rows in time order */
int flush_gauges(gf_forest* f)
{
    const int n = (int)f->gauges.size();
    if (n == 0 || f->grec_rows == 0) return GF_OK;
    std::vector<double> rec((size_t)f->grec_rows * n * 6);
    cudaStream_t st = gf::ctx_stream(f->ctx);
    FK(f, cudaMemcpyAsync(rec.data(), f->d_grec.p, rec.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    FK(f, cudaStreamSynchronize(st));
    std::vector<int> lev;
    std::vector<double> tt, qv;
    for (int g = 0; g < n; ++g) {
        lev.clear();
        tt.clear();
        qv.clear();
        for (int r = 0; r < f->grec_rows; ++r) {
            const double* x = &rec[((size_t)r * n + g) * 6];
            if (x[0] < 0) continue;
            lev.push_back((int)x[0]);
            tt.push_back(x[1]);
            qv.insert(qv.end(), x + 2, x + 6);
        }
        if (lev.empty()) continue;
        int rc = gf_write_gauge_rows(f->out_dir.c_str(), f->gauge_id[g], (int)lev.size(), lev.data(), tt.data(),
                                     qv.data());
        if (rc) return ffail(f, rc, "cannot append to a gauge file");
    }
    f->grec_rows = 0;
    return GF_OK;
}

/* one record per gauge at time t from the current state */
int sample_gauges(gf_forest* f, double t)
{
    const int n = (int)f->gauges.size();
    if (n == 0) return GF_OK;
    int rc;
    if (f->dirty && (rc = build_tables(f))) return rc;
    if (!f->gauges_placed && (rc = place_gauges(f))) return rc;
    if (f->gauge_ghosts) {
        /* a stencil reaches ghost cells: exchange them at t first (the
         * exchange leaves the interiors unchanged) */
        bool any = false;
        for (const gf_gauge_task& T : f->gauges) any |= T.slot >= 0 && t >= T.t1 && t <= T.t2;
        if (any && (rc = ghost_fill(f, t))) return rc;
    }
    if (f->grec_rows == f->grec_cap && (rc = flush_gauges(f))) return rc;
    const double drytol2 = 0.1 * gf::ctx_host_phys(f->ctx, f->o.phys_slot)->dry_tolerance;
    FK(f, gf::launch_gauge_sample(f->d_gtask.p, n, f->qbuf[f->par], f->aux, f->M, f->o.maux, drytol2, t,
                                  f->d_glast.p, f->d_grec.p + (size_t)f->grec_rows * n * 6,
                                  gf::ctx_stream(f->ctx)));
    f->grec_rows++;
    return GF_OK;
}

int write_frame(gf_forest* f, const char* dir, int iframe);

/* ---- subcycling -----------------------------------------------------
 * ForestClaw's fclaw2d_advance_all_levels with subcycle = T (an external
 * library; the schedule below is this project's statement of it): over one
 * coarse step dt, level l takes 2^(l - lo) steps of dt / 2^(l - lo), coarse
 * before fine (Berger-Oliger order). Before the first of its two sub-steps
 * inside a parent step, a level's ghost cells come from the parent's state
 * at the parent's start time; before the second, from the parent time-
 * interpolated to the midpoint (fc2d_geoclaw_fort_timeinterp, alpha =
 * 1/2) in a separate buffer whose own ghost cells are exchanged at that
 * time. Each level keeps its own parity in the two state buffers; the
 * step's start state is saved for a retake, and on acceptance the coarsest
 * level (one step, odd parity) is copied back so all levels share one
 * buffer again. Buffers: 0, 1 = state, 2 = time-interpolated patches. */
inline double* qslot_b(gf_forest* f, int b, int slot)
{
    double* base = b < 2 ? f->qbuf[b] : f->qi;
    return base + (size_t)slot * 3 * f->S;
}

int build_sub_tables(gf_forest* f)
{
    int rc = build_tables(f);
    if (rc) return rc;
    if (!f->sub_dirty) return GF_OK;
    f->sub_graph_ok = false;
    const size_t pool = (size_t)f->cap * 3 * f->S * sizeof(double);
    if (!f->qi) FK(f, cudaMalloc(&f->qi, pool));
    if (!f->qsave) FK(f, cudaMalloc(&f->qsave, pool));
    const int nlev = f->o.maxlevel + 1;
    f->lev_off.assign(nlev + 1, 0);
    f->lev_n.assign(nlev + 1, 0);
    f->sub_lo = nlev;
    f->sub_hi = -1;
    for (size_t k = 0; k < f->leaves.size(); ++k) {
        const int l = f->leaves[k].level;
        if (f->lev_n[l]++ == 0) f->lev_off[l] = (int)k;
        f->sub_lo = std::min(f->sub_lo, l);
        f->sub_hi = std::max(f->sub_hi, l);
    }
    std::vector<int> slot_level(f->cap, -1);
    for (const Leaf& L : f->leaves) slot_level[L.slot] = L.level;
    const size_t per = 3 * (size_t)f->S;
    auto slot_of = [&](const double* q) { return (int)((q - f->qbuf[0]) / (long)per); };
    /* transfer lists by level and buffer pair (coarse bc in 0..2, fine bf in 0..1) */
    std::vector<gf_xfer_task> x;
    f->sx_avg_off.assign((size_t)nlev * 6, 0);
    f->sx_avg_n.assign(nlev, 0);
    f->sx_itp_off.assign((size_t)nlev * 6, 0);
    std::vector<std::vector<gf_xfer_task>> avg_l(nlev);
    for (const gf_xfer_task& t : f->h_avg) avg_l[slot_level[slot_of(t.qc)]].push_back(t);
    for (int l = 0; l < nlev; ++l) {
        f->sx_avg_n[l] = (int)avg_l[l].size();
        for (int bc = 0; bc < 3; ++bc)
            for (int bf = 0; bf < 2; ++bf) {
                f->sx_avg_off[(size_t)l * 6 + bc * 2 + bf] = (int)x.size();
                for (gf_xfer_task t : avg_l[l]) {
                    t.qc = qslot_b(f, bc, slot_of(t.qc));
                    t.qf = qslot_b(f, bf, slot_of(t.qf));
                    x.push_back(t);
                }
                f->sx_itp_off[(size_t)l * 6 + bc * 2 + bf] = (int)x.size();
                for (gf_xfer_task t : f->h_itp[l]) {
                    t.qc = qslot_b(f, bc, slot_of(t.qc));
                    t.qf = qslot_b(f, bf, slot_of(t.qf));
                    x.push_back(t);
                }
            }
    }
    /* time interpolation per level and old parity; save / restore / unify per parity */
    std::vector<gf_slot_task> sl;
    f->ss_ti_off.assign((size_t)nlev * 2, 0);
    for (int l = 0; l < nlev; ++l)
        for (int po = 0; po < 2; ++po) {
            f->ss_ti_off[(size_t)l * 2 + po] = (int)sl.size();
            for (int k = 0; k < f->lev_n[l]; ++k) {
                const int s = f->leaves[f->lev_off[l] + k].slot;
                sl.push_back(gf_slot_task{qslot(f, po, s), qslot(f, po ^ 1, s), f->qi + (size_t)s * per});
            }
        }
    for (int kind = 0; kind < 3; ++kind)
        for (int par = 0; par < 2; ++par) {
            f->ss_copy_off[kind][par] = (int)sl.size();
            int n = 0;
            for (const Leaf& L : f->leaves) {
                const bool fine = L.level > f->sub_lo;
                const double* save = f->qsave + (size_t)L.slot * per;
                if (kind == 0 && fine) sl.push_back(gf_slot_task{qslot(f, par, L.slot), nullptr, const_cast<double*>(save)});
                else if (kind == 1 && fine) sl.push_back(gf_slot_task{save, nullptr, qslot(f, par, L.slot)});
                else if (kind == 2 && !fine)
                    sl.push_back(gf_slot_task{qslot(f, par ^ 1, L.slot), nullptr, qslot(f, par, L.slot)});
                else continue;
                ++n;
            }
            f->ss_copy_n[kind] = n;
        }
    cudaStream_t st = gf::ctx_stream(f->ctx);
    FK(f, f->d_sx.reserve(x.size() + 1));
    FK(f, f->d_ss.reserve(sl.size() + 1));
    if (!x.empty())
        FK(f, cudaMemcpyAsync(f->d_sx.p, x.data(), x.size() * sizeof(gf_xfer_task), cudaMemcpyHostToDevice, st));
    if (!sl.empty())
        FK(f, cudaMemcpyAsync(f->d_ss.p, sl.data(), sl.size() * sizeof(gf_slot_task), cudaMemcpyHostToDevice, st));
    FK(f, f->d_par01.reserve(2));
    const int p01[2] = {0, 1};
    FK(f, cudaMemcpyAsync(f->d_par01.p, p01, sizeof p01, cudaMemcpyHostToDevice, st));
    f->h_sx.swap(x);
    f->h_ss.swap(sl);
    f->sub_dirty = false;
    ++f->sub_epoch;
    return GF_OK;
}

/* same-level copies and physical sides of level l's leaves in buffer b at
 * t. Ghost block i of the step: the plan pass writes it, the launch pass
 * points the fill at its device copy. */
constexpr size_t kSubBlkOff = 256 * sizeof(double); /* staging: dts, then blocks */

int sub_ghost(gf_forest* f, int l, int b, double t, const gf_ghost_ref* refs, int n)
{
    (void)l;
    if (n <= 0) return GF_OK;
    const int i = f->sub_nblk++;
    if (f->sub_plan) {
        gf_ghost_block blk{};
        blk.q = b < 2 ? f->qbuf[b] : f->qi;
        blk.aux = f->aux;
        blk.nbr = f->d_nbr.p;
        blk.geom = f->d_geom.p;
        blk.phys_of = nullptr;
        blk.bc = f->bc;
        blk.bc.q0hu = hydro_at(f, t);
        blk.phys = f->o.phys_slot;
        blk.maux = f->o.maux;
        blk.skip = 0;
        if ((int)f->sub_blocks.size() <= i) f->sub_blocks.resize(i + 1);
        f->sub_blocks[i] = blk;
        return GF_OK;
    }
    const gf_ghost_block* d_blk = reinterpret_cast<const gf_ghost_block*>(f->d_sub_stage.p + kSubBlkOff) + i;
    FK(f, gf::launch_ghost_fill(f->M, d_blk, refs, n, gf::ctx_device_phys(f->ctx), gf::ctx_stream(f->ctx)));
    return GF_OK;
}

/* ghost cells of level l at t: averages from level l + 1, copies and
 * physical sides, then (cbuf >= 0) interpolation from level l - 1's
 * patches in buffer cbuf and the physical sides again */
int sub_fill_level(gf_forest* f, int l, double t, const int* p, int cbuf)
{
    cudaStream_t st = gf::ctx_stream(f->ctx);
    const gf_phys* phys = gf::ctx_device_phys(f->ctx);
    int rc;
    const bool go = !f->sub_plan;
    if (go && l < f->sub_hi && f->sx_avg_n[l])
        FK(f, gf::launch_transfer(f->M, f->d_sx.p + f->sx_avg_off[(size_t)l * 6 + p[l] * 2 + p[l + 1]],
                                  f->sx_avg_n[l], phys, st));
    if ((rc = sub_ghost(f, l, p[l], t, f->d_refs_all.p + f->lev_off[l], f->lev_n[l]))) return rc;
    if (cbuf >= 0 && f->itp_n[l]) {
        if (go)
            FK(f, gf::launch_transfer(f->M, f->d_sx.p + f->sx_itp_off[(size_t)l * 6 + cbuf * 2 + p[l]],
                                      f->itp_n[l], phys, st));
        if ((rc = sub_ghost(f, l, p[l], t, f->d_refs_lv.p + f->ref_off[l], f->ref_n[l]))) return rc;
    }
    return GF_OK;
}

int sub_update(gf_forest* f, int l, int* p)
{
    cudaStream_t st = gf::ctx_stream(f->ctx);
    const gf_phys* phys = gf::ctx_device_phys(f->ctx);
    int* err = reinterpret_cast<int*>(f->d_rb.p);
    const gf_patch_work* w = f->d_work.p + f->lev_off[l];
    const double* dts = reinterpret_cast<const double*>(f->d_sub_stage.p);
    if (f->sub_plan) {
        /* the plan pass only tracks the parities */
    } else if (gf::ctx_exact(f->ctx))
        FK(f, gf::launch_patch_update_exact(f->M, w, f->lev_n[l], phys, 0.0, dts + l, f->d_par01.p + p[l],
                                            f->o.maux, nullptr, f->d_rb.p + 1, err, st));
    else
        FK(f, gf::launch_patch_update(f->M, w, f->lev_n[l], phys, 0.0, dts + l, f->d_par01.p + p[l],
                                      f->o.maux, nullptr, f->d_rb.p + 1, err, st));
    p[l] ^= 1;
    return GF_OK;
}

int sub_level(gf_forest* f, int l, double tl, double dtl, int* p)
{
    int rc;
    if ((rc = sub_update(f, l, p))) return rc;
    if (l >= f->sub_hi) return GF_OK;
    const int po = p[l] ^ 1; /* level l's state at tl */
    cudaStream_t st = gf::ctx_stream(f->ctx);
    const gf_phys* phys = gf::ctx_device_phys(f->ctx);
    for (int k = 0; k < 2; ++k) {
        const double tf = k ? tl + dtl * 0.5 : tl;
        int cbuf = po;
        if (k == 1) {
            /* level l at the midpoint, with its ghost cells exchanged there */
            if (!f->sub_plan) {
                FK(f, gf::launch_tinterp_strip(f->M, f->d_ss.p + f->ss_ti_off[(size_t)l * 2 + po], f->lev_n[l],
                                               0.5, st));
                if (f->sx_avg_n[l])
                    FK(f, gf::launch_transfer(f->M, f->d_sx.p + f->sx_avg_off[(size_t)l * 6 + 2 * 2 + p[l + 1]],
                                              f->sx_avg_n[l], phys, st));
            }
            if ((rc = sub_ghost(f, l, 2, tf, f->d_refs_all.p + f->lev_off[l], f->lev_n[l]))) return rc;
            cbuf = 2;
        }
        if ((rc = sub_fill_level(f, l + 1, tf, p, cbuf))) return rc;
        if ((rc = sub_level(f, l + 1, tf, dtl * 0.5, p))) return rc;
    }
    return GF_OK;
}

/* one subcycled coarse step; the result is pending until sub_finish.
 * The step's launches (a few per level and sub-step) run as one CUDA graph:
 * captured on the first step after the leaves change, replayed after a
 * host-only plan pass has written this step's level dts and ghost blocks
 * (whose boundary times move with t and dt) to the pinned staging the
 * graph's first node copies. */
int sub_launch(gf_forest* f, double t, double dt, cudaStream_t ls)
{
    int rc = build_sub_tables(f);
    if (rc) return rc;
    cudaStream_t st = gf::ctx_stream(f->ctx);
    const int nlev = f->o.maxlevel + 1;
    long long cu = 0;
    for (int l = f->sub_lo; l <= f->sub_hi; ++l) cu += (long long)f->lev_n[l] * f->M * f->M << (l - f->sub_lo);
    /* plan pass */
    std::vector<int> p(nlev + 1, f->par);
    f->sub_plan = true;
    f->sub_nblk = 0;
    rc = sub_fill_level(f, f->sub_lo, t, p.data(), -1);
    if (!rc) rc = sub_level(f, f->sub_lo, t, dt, p.data());
    f->sub_plan = false;
    if (rc) return rc;
    const int nblk = f->sub_nblk;
    const size_t bytes = kSubBlkOff + (size_t)nblk * sizeof(gf_ghost_block);
    if (bytes > f->h_sub_cap) {
        if (f->h_sub) cudaFreeHost(f->h_sub);
        f->h_sub = nullptr;
        f->h_sub_cap = 0;
        FK(f, cudaMallocHost(reinterpret_cast<void**>(&f->h_sub), bytes + bytes / 2));
        f->h_sub_cap = bytes + bytes / 2;
        f->sub_graph_ok = false;
    }
    double* hdt = reinterpret_cast<double*>(f->h_sub);
    double d = dt;
    for (int l = 0; l < nlev; ++l) hdt[l] = 0.0;
    for (int l = f->sub_lo; l <= f->sub_hi; ++l, d *= 0.5) hdt[l] = d;
    std::memcpy(f->h_sub + kSubBlkOff, f->sub_blocks.data(), (size_t)nblk * sizeof(gf_ghost_block));
    const bool exact = gf::ctx_exact(f->ctx);
    if (!f->sub_graph_ok || f->sub_graph_par != f->par || f->sub_graph_nblk != nblk || f->sub_graph_exact != exact) {
        f->sub_graph_ok = false;
        FK(f, f->d_sub_stage.reserve(bytes));
        FK(f, f->d_rb.reserve(2));
        FK(f, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int crc = GF_OK;
        auto cap = [&](cudaError_t e) { if (e != cudaSuccess && crc == GF_OK) crc = gf::ctx_cuda_fail(f->ctx, e, "subcycled step capture"); };
        cap(cudaMemcpyAsync(f->d_sub_stage.p, f->h_sub, bytes, cudaMemcpyHostToDevice, st));
        cap(cudaMemsetAsync(f->d_rb.p, 0, 2 * sizeof(unsigned long long), st));
        cap(gf::launch_slot_copy(f->M, f->d_ss.p + f->ss_copy_off[0][f->par], f->ss_copy_n[0], st));
        std::vector<int> q(nlev + 1, f->par);
        f->sub_nblk = 0;
        if (crc == GF_OK) crc = sub_fill_level(f, f->sub_lo, t, q.data(), -1);
        if (crc == GF_OK) crc = sub_level(f, f->sub_lo, t, dt, q.data());
        cudaGraph_t graph = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(st, &graph);
        if (crc) {
            if (graph) cudaGraphDestroy(graph);
            return crc;
        }
        FK(f, ee);
        /* same shape as the last capture (the usual regrid): update in place */
        bool updated = false;
        if (f->sub_exec) {
            cudaGraphExecUpdateResultInfo info;
            updated = cudaGraphExecUpdate(f->sub_exec, graph, &info) == cudaSuccess;
            if (!updated) {
                cudaGetLastError();
                cudaGraphExecDestroy(f->sub_exec);
                f->sub_exec = nullptr;
            }
        }
        cudaError_t ei = cudaSuccess;
        if (!updated) ei = cudaGraphInstantiate(&f->sub_exec, graph, 0);
        cudaGraphDestroy(graph);
        FK(f, ei);
        f->sub_graph_ok = true;
        f->sub_graph_par = f->par;
        f->sub_graph_nblk = nblk;
        f->sub_graph_exact = exact;
    }
    f->sub_updates = cu;
    if (ls && ls != st) {
        /* on the runner's stream, after this forest's tables, transfers and
         * slot copies on the context's stream */
        if (!f->sev_ctx) FK(f, cudaEventCreateWithFlags(&f->sev_ctx, cudaEventDisableTiming));
        if (!f->sev_done) FK(f, cudaEventCreateWithFlags(&f->sev_done, cudaEventDisableTiming));
        FK(f, cudaEventRecord(f->sev_ctx, st));
        FK(f, cudaStreamWaitEvent(ls, f->sev_ctx, 0));
        st = ls;
    }
    FK(f, cudaGraphLaunch(f->sub_exec, st));
    FK(f, cudaMemcpyAsync(f->h_rb, f->d_rb.p, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    if (f->sev_done && st == ls) FK(f, cudaEventRecord(f->sev_done, st));
    return GF_OK;
}

/* the launched step's CFL (its readback has landed) */
int sub_collect(gf_forest* f, double* cfl, long long* updates)
{
    if ((int)f->h_rb[0]) return ffail(f, GF_ERR_DEVICE, "a patch-update copy wait timed out");
    std::memcpy(cfl, &f->h_rb[1], sizeof *cfl);
    *updates = f->sub_updates;
    return GF_OK;
}

int sub_step(gf_forest* f, double t, double dt, double* cfl, long long* updates)
{
    int rc = sub_launch(f, t, dt, nullptr);
    if (rc) return rc;
    FK(f, cudaStreamSynchronize(gf::ctx_stream(f->ctx)));
    return sub_collect(f, cfl, updates);
}

/* accept: the coarsest level back into the shared buffer; retake: the
 * finer levels' start state back */
int sub_finish(gf_forest* f, bool accept)
{
    cudaStream_t st = gf::ctx_stream(f->ctx);
    const int kind = accept ? 2 : 1;
    FK(f, gf::launch_slot_copy(f->M, f->d_ss.p + f->ss_copy_off[kind][f->par], f->ss_copy_n[kind], st));
    return GF_OK;
}

/* ForestClaw outstyle 1 (fc2d_geoclaw_run.c:190-395) with variable dt and
 * reduce_cfl: with advance-one-step (subcycle = 0) every level takes the
 * minlevel dt over 2^(maxlevel - minlevel); with subcycle = 1 the step is
 * the minlevel dt and the levels subcycle (sub_step). */
int run_outstyle1(gf_forest* f, double t_final, int nout, double initial_dt, double desired_cfl,
                  double max_cfl, int max_steps)
{
    const gf_forest_opts& o = f->o;
    const double level_factor = (double)(1 << (o.maxlevel - o.minlevel));
    const double dt_outer = t_final / nout;
    double t_curr = f->st.t;
    double dt_minlevel = initial_dt;
    long long taken = 0;
    int rc;
    if (!f->out_started) {
        /* frame 0 and the initial gauge records (fc2d_geoclaw_run.c:195-210) */
        if (f->out_frames && (rc = write_frame(f, f->out_dir.c_str(), f->next_frame++))) return rc;
        if ((rc = sample_gauges(f, t_curr))) return rc;
        f->out_started = true;
    }
    for (int n = 0; n < nout; ++n) {
        const double tend = t_curr + dt_outer;
        while (t_curr < tend) {
            if (max_steps > 0 && taken >= max_steps) goto out;
            double dt_step = o.subcycle ? dt_minlevel : dt_minlevel / level_factor;
            const double tol = 1e-2 * dt_step;
            bool took_small = false;
            const double small_step = tend - (t_curr + dt_step);
            if (small_step < tol) {
                dt_step = tend - t_curr;
                if (small_step < 0) took_small = true;
            }
            double cfl = 0.0;
            long long updates = f->cells;
            if (o.subcycle) rc = sub_step(f, t_curr, dt_step, &cfl, &updates);
            else rc = step(f, t_curr, dt_step, &cfl);
            if (rc) return rc;
            ++taken;
            f->st.max_cfl_seen = std::max(f->st.max_cfl_seen, cfl);
            if (cfl > max_cfl) {
                if (o.subcycle && (rc = sub_finish(f, false))) return rc;
                dt_minlevel = dt_minlevel * desired_cfl / cfl;
                f->st.rejects++;
                continue;
            }
            if (o.subcycle) {
                if ((rc = sub_finish(f, true))) return rc;
            } else {
                f->par ^= 1;
            }
            f->st.steps++;
            f->st.cell_updates += updates;
            t_curr += dt_step;
            const double dt_new = dt_minlevel * desired_cfl / cfl;
            if (!took_small) dt_minlevel = dt_new;
            f->st.t = t_curr;
            f->st.dt = dt_minlevel;
            /* gauges after every step, before a regrid (fc2d_geoclaw_run.c:380-393) */
            if ((rc = sample_gauges(f, t_curr))) return rc;
            if (o.regrid_interval > 0 && f->st.steps % o.regrid_interval == 0) {
                bool changed = false;
                if ((rc = regrid(f, t_curr, &changed))) return rc;
            }
        }
        /* a frame at every output time (fc2d_geoclaw_run.c:396-401) */
        if (f->out_frames) {
            if ((rc = flush_gauges(f))) return rc;
            if ((rc = write_frame(f, f->out_dir.c_str(), f->next_frame++))) return rc;
        }
    }
out:
    f->st.t = t_curr;
    f->st.dt = dt_minlevel;
    return flush_gauges(f);
}

} // namespace

extern "C" {

void gf_forest_opts_default(gf_forest_opts* o)
{
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->mx = 16;
    o->maux = 1;
    o->nbx = o->nby = 1;
    o->minlevel = 0;
    o->maxlevel = 0;
    o->dx0 = o->dy0 = 1.0;
    for (int s = 0; s < 4; ++s) o->mthbc[s] = 1;
    o->regrid_interval = 0;
    o->refine.wave_tolerance = 0.1;
    o->refine.speed_tolerance[0] = 1e12;
    o->refine.num_speed_tolerance = 1;
    o->refine.deep_depth = 1e10;
    o->refine.max_level_deep = 0;
    o->refine.max_velocity_depth_product = 1e20;
}

void gf_forest_destroy(gf_forest* f)
{
    if (!f) return;
    /* the caller destroys forests before their context; the frees below
     * synchronise the device, so no stream of the context is needed */
    cudaSetDevice(f->device);
    for (double* p : f->pyr)
        if (p) cudaFree(p);
    for (int b = 0; b < 2; ++b)
        if (f->qbuf[b]) cudaFree(f->qbuf[b]);
    if (f->aux) cudaFree(f->aux);
    f->d_nbr.release();
    f->d_geom.release();
    f->d_work.release();
    f->d_refs_all.release();
    f->d_refs_lv.release();
    for (int b = 0; b < 2; ++b) {
        f->d_avg[b].release();
        f->d_itp[b].release();
    }
    f->d_block.release();
    f->d_gdt.release();
    f->d_gpar.release();
    f->d_rb.release();
    f->d_tagt.release();
    f->d_tags.release();
    f->d_refine.release();
    f->d_rgx.release();
    f->d_fill.release();
    f->d_gtask.release();
    f->d_glast.release();
    f->d_grec.release();
    if (f->qi) cudaFree(f->qi);
    if (f->qsave) cudaFree(f->qsave);
    f->d_sx.release();
    f->d_ss.release();
    f->d_par01.release();
    if (f->sub_exec) cudaGraphExecDestroy(f->sub_exec);
    f->d_sub_stage.release();
    if (f->h_sub) cudaFreeHost(f->h_sub);
    if (f->h_rb) cudaFreeHost(f->h_rb);
    if (f->sev_ctx) cudaEventDestroy(f->sev_ctx);
    if (f->sev_done) cudaEventDestroy(f->sev_done);
    delete f;
}

int gf_forest_create(gf_ctx* c, const gf_forest_opts* o, const double* fields, gf_forest** out)
{
    if (!c || !o || !out) return GF_ERR_ARG;
    *out = nullptr;
    if (!(o->mx == 8 || o->mx == 16 || o->mx == 32)) return gf::ctx_fail(c, GF_ERR_ARG, "mx must be 8, 16 or 32");
    if (o->maux < 1 || o->maux > 3) return gf::ctx_fail(c, GF_ERR_ARG, "maux must be 1..3");
    if (o->nbx < 1 || o->nby < 1) return gf::ctx_fail(c, GF_ERR_ARG, "nbx, nby must be positive");
    if (o->minlevel < 0 || o->maxlevel < o->minlevel || o->maxlevel > 10)
        return gf::ctx_fail(c, GF_ERR_ARG, "need 0 <= minlevel <= maxlevel <= 10");
    if (!(o->dx0 > 0) || !(o->dy0 > 0)) return gf::ctx_fail(c, GF_ERR_ARG, "dx0, dy0 must be positive");
    for (int s = 0; s < 4; ++s)
        if (!(o->mthbc[s] == 0 || o->mthbc[s] == 1 || o->mthbc[s] == 3))
            return gf::ctx_fail(c, GF_ERR_ARG, "forest mthbc must be 0, 1 or 3");
    if (o->regrid_interval < 0) return gf::ctx_fail(c, GF_ERR_ARG, "regrid_interval must be >= 0");
    if (o->refine.num_speed_tolerance < 0 || o->refine.num_speed_tolerance > GF_MAX_SPEEDS ||
        o->refine.num_flowgrades < 0 || o->refine.num_flowgrades > GF_MAX_FLOWGRADES ||
        o->refine.num_regions < 0 || o->refine.num_regions > GF_MAX_REGIONS)
        return gf::ctx_fail(c, GF_ERR_ARG, "refinement parameter counts out of range");
    int rc = gf::ctx_check_phys(c, o->phys_slot, o->maux);
    if (rc) return rc;
    /* a regrid holds the new patches and the ones they replace at once: at
     * most full refinement plus the parents being split (a quarter of it) */
    const long long full = (long long)o->nbx * o->nby << (2 * o->maxlevel);
    const long long peak = full + (full + 3) / 4;
    long long cap = o->max_patches > 0 ? std::min<long long>(o->max_patches, peak) : peak;
    if (cap > (1LL << 22)) return gf::ctx_fail(c, GF_ERR_ARG, "set max_patches (full refinement is too large)");
    gf_forest* f = new gf_forest;
    f->ctx = c;
    f->device = gf::ctx_device(c);
    f->o = *o;
    f->M = o->mx;
    f->S = (long)(o->mx + 2 * GF_MBC) * (o->mx + 2 * GF_MBC);
    f->nf = o->maux + 3;
    f->cap = (int)cap;
    for (int s = 0; s < 4; ++s) f->bc.mthbc[s] = o->mthbc[s];
    cudaError_t e = cudaSetDevice(gf::ctx_device(c));
    for (int b = 0; b < 2 && e == cudaSuccess; ++b)
        e = cudaMalloc(&f->qbuf[b], (size_t)cap * 3 * f->S * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&f->aux, (size_t)cap * o->maux * f->S * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&f->h_rb, 2 * sizeof(unsigned long long));
    if (e != cudaSuccess) {
        gf_forest_destroy(f);
        return gf::ctx_cuda_fail(c, e, "forest pool allocation");
    }
    if ((rc = build_pyramid(f, fields))) {
        gf_forest_destroy(f);
        return rc;
    }
    /* the refinement criteria live on the device for the tag launches */
    e = f->d_refine.reserve(1);
    if (e == cudaSuccess)
        e = cudaMemcpy(f->d_refine.p, &o->refine, sizeof(gf_refine), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        gf_forest_destroy(f);
        return gf::ctx_cuda_fail(c, e, "forest refinement criteria");
    }
    *out = f;
    return GF_OK;
}

size_t gf_forest_footprint(const gf_forest_opts* o)
{
    if (!o || !(o->mx == 8 || o->mx == 16 || o->mx == 32) || o->maux < 1 || o->maux > 3 || o->nbx < 1 ||
        o->nby < 1 || o->minlevel < 0 || o->maxlevel < o->minlevel || o->maxlevel > 10)
        return 0;
    const long long full = (long long)o->nbx * o->nby << (2 * o->maxlevel);
    const long long peak = full + (full + 3) / 4;
    const long long cap = o->max_patches > 0 ? std::min<long long>(o->max_patches, peak) : peak;
    if (cap > (1LL << 22)) return 0;
    const size_t S = (size_t)(o->mx + 2 * GF_MBC) * (o->mx + 2 * GF_MBC);
    const int nf = o->maux + 3;
    size_t n = 0;
    for (int l = o->minlevel; l <= o->maxlevel; ++l)
        n += (size_t)nf * ((size_t)(o->nbx * o->mx << l) + 2 * GF_MBC) * ((size_t)(o->nby * o->mx << l) + 2 * GF_MBC) *
             sizeof(double);
    n += (size_t)(o->nbx * o->mx << o->maxlevel) * (size_t)(o->nby * o->mx << o->maxlevel) * sizeof(double);
    n += (size_t)cap * (6 + o->maux) * S * sizeof(double);
    /* leaf tables (grown by half again when they grow): neighbours, geometry,
     * work item, ghost references, coarse/fine transfers of both parities,
     * tagging and regrid transfers */
    const size_t per_slot = 8 * sizeof(int) + sizeof(gf_patch_geom) + sizeof(gf_patch_work) + 2 * sizeof(gf_ghost_ref) +
                            20 * sizeof(gf_xfer_task) + sizeof(gf_tag_task) + sizeof(int) + sizeof(gf_fill_task);
    n += (size_t)cap * per_slot * 3 / 2;
    return n + ((size_t)1 << 20);
}

int gf_forest_set_hydrograph(gf_forest* f, int n, const double* time, const double* hu,
                             const int* side, double width, double x0, double y0)
{
    if (!f || n < 0 || (n > 0 && (!time || !hu || !side))) return GF_ERR_ARG;
    for (int i = 1; i < n; ++i)
        if (!(time[i] >= time[i - 1])) return ffail(f, GF_ERR_ARG, "hydrograph times must increase");
    f->hy_t.assign(time, time + n);
    f->hy_hu.assign(hu, hu + n);
    for (int s = 0; s < 4; ++s) f->bc.hydro_side[s] = n > 0 ? (side[s] != 0) : 0;
    f->bc.width = width;
    f->bc.x0 = x0;
    f->bc.y0 = y0;
    return GF_OK;
}

int gf_forest_set_topo(gf_forest* f, gf_topo* t, int qinit)
{
    if (!f || !t) return GF_ERR_ARG;
    if (!f->leaves.empty()) return ffail(f, GF_ERR_STATE, "set the topography before gf_forest_init");
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    const gf_forest_opts& o = f->o;
    cudaStream_t st = gf::ctx_stream(f->ctx);
    const double xupper = o.x0 + (o.nbx * f->M) * o.dx0, yupper = o.y0 + (o.nby * f->M) * o.dy0;
    const double sea_level = gf::ctx_host_phys(f->ctx, o.phys_slot)->sea_level;
    for (int l = o.minlevel; l <= o.maxlevel; ++l) {
        double* const* lv = &f->pyr[(size_t)(l - o.minlevel) * f->nf];
        int rc = gf::topo_raster_device(f->ctx, t, nx_at(f, l), ny_at(f, l), GF_MBC, o.x0, o.y0, dx_at(f, l),
                                        dy_at(f, l), xupper, yupper, lv[0], st);
        if (rc) return rc;
        if (qinit) {
            const long cells = (long)(nx_at(f, l) + 2 * GF_MBC) * (ny_at(f, l) + 2 * GF_MBC);
            FK(f, gf::launch_qinit_sea_level(lv[0], lv[o.maux], lv[o.maux + 1], lv[o.maux + 2], cells, sea_level, st));
        }
    }
    FK(f, cudaStreamSynchronize(st));
    return GF_OK;
}

int gf_forest_init(gf_forest* f)
{
    if (!f) return GF_ERR_ARG;
    for (int s = 0; s < 4; ++s)
        if (f->o.mthbc[s] == 0 && !f->bc.hydro_side[s])
            return ffail(f, GF_ERR_ARG, "mthbc = 0 needs a hydrograph on that side (the reference stops here)");
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    return init_forest(f);
}

int gf_forest_ghost_fill(gf_forest* f, double t)
{
    if (!f) return GF_ERR_ARG;
    if (f->leaves.empty()) return ffail(f, GF_ERR_STATE, "forest not initialised");
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    int rc = ghost_fill(f, t);
    if (rc) return rc;
    FK(f, cudaStreamSynchronize(gf::ctx_stream(f->ctx)));
    return GF_OK;
}

int gf_forest_step(gf_forest* f, double t, double dt, double* cfl)
{
    if (!f || !(dt > 0)) return GF_ERR_ARG;
    if (f->leaves.empty()) return ffail(f, GF_ERR_STATE, "forest not initialised");
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    return step(f, t, dt, cfl);
}

int gf_forest_accept(gf_forest* f, int accept)
{
    if (!f) return GF_ERR_ARG;
    if (accept) {
        f->par ^= 1;
        f->st.steps++;
        f->st.cell_updates += f->cells;
    } else {
        f->st.rejects++;
    }
    return GF_OK;
}

int gf_forest_regrid(gf_forest* f, double t, int* changed)
{
    if (!f) return GF_ERR_ARG;
    if (f->leaves.empty()) return ffail(f, GF_ERR_STATE, "forest not initialised");
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    bool ch = false;
    int rc = regrid(f, t, &ch);
    if (changed) *changed = ch;
    return rc;
}

int gf_forest_run(gf_forest* f, double t_final, int nout, double initial_dt, double desired_cfl,
                  double max_cfl, int max_steps, gf_forest_stats* st)
{
    if (!f || !(t_final > 0) || nout < 1 || !(initial_dt > 0) || !(desired_cfl > 0) || !(max_cfl > 0))
        return GF_ERR_ARG;
    if (f->leaves.empty()) return ffail(f, GF_ERR_STATE, "forest not initialised");
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    int rc = run_outstyle1(f, t_final, nout, initial_dt, desired_cfl, max_cfl, max_steps);
    if (st) gf_forest_get_stats(f, st);
    return rc;
}

int gf_forest_get_stats(gf_forest* f, gf_forest_stats* st)
{
    if (!f || !st) return GF_ERR_ARG;
    *st = f->st;
    st->npatch = (int)f->leaves.size();
    st->levels_used = 0;
    for (const Leaf& L : f->leaves) st->levels_used = std::max(st->levels_used, L.level);
    return GF_OK;
}

int gf_forest_npatch(const gf_forest* f) { return f ? (int)f->leaves.size() : -1; }

int gf_forest_patches(const gf_forest* f, int* level, int* I, int* J)
{
    if (!f) return GF_ERR_ARG;
    for (size_t k = 0; k < f->leaves.size(); ++k) {
        if (level) level[k] = f->leaves[k].level;
        if (I) I[k] = f->leaves[k].I;
        if (J) J[k] = f->leaves[k].J;
    }
    return GF_OK;
}

} // extern "C"

namespace {

/* planes of the leaves' slots <-> Fortran layout in canonical order */
int move_leaves(gf_forest* f, double* host, int nfield, bool to_host, bool aux)
{
    const size_t per = (size_t)nfield * f->S;
    const size_t n = f->leaves.size();
    std::vector<double> tmp(per);
    cudaStream_t st = gf::ctx_stream(f->ctx);
    for (size_t k = 0; k < n; ++k) {
        const int s = f->leaves[k].slot;
        double* dev = aux ? aslot(f, s) : qslot(f, f->par, s);
        double* h = host + k * per;
        if (to_host) {
            FK(f, cudaMemcpyAsync(tmp.data(), dev, per * sizeof(double), cudaMemcpyDeviceToHost, st));
            FK(f, cudaStreamSynchronize(st));
            for (long c = 0; c < f->S; ++c)
                for (int m = 0; m < nfield; ++m) h[(size_t)c * nfield + m] = tmp[(size_t)m * f->S + c];
        } else {
            for (long c = 0; c < f->S; ++c)
                for (int m = 0; m < nfield; ++m) tmp[(size_t)m * f->S + c] = h[(size_t)c * nfield + m];
            FK(f, cudaMemcpyAsync(dev, tmp.data(), per * sizeof(double), cudaMemcpyHostToDevice, st));
            FK(f, cudaStreamSynchronize(st));
        }
    }
    return GF_OK;
}

/* p4est numbers the trees of an mi x mj brick along the Morton curve of
 * the smallest power-of-two box holding it (x bit first at each rank, a
 * direction with no bits left skipped), leaving out positions outside the
 * brick (p4est_connectivity_new_brick; p4est is not part of the reference
 * tree). id[by * mi + bx] = tree number. */
std::vector<int> brick_tree_ids(int mi, int mj)
{
    auto bits = [](int m) {
        int b = 0;
        while ((1 << b) < m) ++b;
        return b;
    };
    const int lx = bits(mi), ly = bits(mj), rank = std::max(lx, ly);
    std::vector<int> id((size_t)mi * mj, -1);
    int next = 0;
    for (long ti = 0; ti < (1L << (lx + ly)); ++ti) {
        int x = 0, y = 0, c = 0;
        for (int i = 0; i < rank; ++i) {
            if (i < lx) x |= (int)((ti >> c++) & 1) << i;
            if (i < ly) y |= (int)((ti >> c++) & 1) << i;
        }
        if (x < mi && y < mj) id[(size_t)y * mi + x] = next++;
    }
    return id;
}

inline uint64_t morton2(uint32_t x, uint32_t y)
{
    uint64_t k = 0;
    for (int b = 0; b < 32; ++b)
        k |= (uint64_t)((x >> b) & 1) << (2 * b) | (uint64_t)((y >> b) & 1) << (2 * b + 1);
    return k;
}

/* the leaves in p4est order: tree, then the Morton index of the leaf's
 * lower-left corner at maxlevel within the tree */
std::vector<size_t> p4est_order(const gf_forest* f, std::vector<int>* block)
{
    const std::vector<int> tid = brick_tree_ids(f->o.nbx, f->o.nby);
    const size_t n = f->leaves.size();
    std::vector<std::pair<uint64_t, size_t>> key(n);
    block->assign(n, 0);
    for (size_t k = 0; k < n; ++k) {
        const Leaf& L = f->leaves[k];
        const int bx = L.I >> L.level, by = L.J >> L.level;
        const uint32_t sx = (uint32_t)(L.I - (bx << L.level)) << (f->o.maxlevel - L.level);
        const uint32_t sy = (uint32_t)(L.J - (by << L.level)) << (f->o.maxlevel - L.level);
        const int t = tid[(size_t)by * f->o.nbx + bx];
        (*block)[k] = t;
        key[k] = {((uint64_t)t << 44) | morton2(sx, sy), k};
    }
    std::sort(key.begin(), key.end());
    std::vector<size_t> ord(n);
    for (size_t r = 0; r < n; ++r) ord[r] = key[r].second;
    return ord;
}

int write_frame(gf_forest* f, const char* dir, int iframe)
{
    const size_t n = f->leaves.size();
    const int M = f->M, maux = f->o.maux;
    const size_t qper = 3 * (size_t)f->S, aper = (size_t)maux * f->S;
    std::vector<double> q(n * qper), a(n * aper);
    int rc = move_leaves(f, q.data(), 3, true, false);
    if (!rc) rc = move_leaves(f, a.data(), maux, true, true);
    if (rc) return rc;
    std::vector<int> block;
    const std::vector<size_t> ord = p4est_order(f, &block);
    std::vector<double> qo(n * qper), ao(n * aper), xl(n), yl(n), dxv(n), dyv(n);
    std::vector<int> gn(n), lv(n), bk(n);
    for (size_t r = 0; r < n; ++r) {
        const size_t k = ord[r];
        const Leaf& L = f->leaves[k];
        std::copy(q.begin() + k * qper, q.begin() + (k + 1) * qper, qo.begin() + r * qper);
        std::copy(a.begin() + k * aper, a.begin() + (k + 1) * aper, ao.begin() + r * aper);
        gn[r] = (int)r;
        lv[r] = L.level;
        bk[r] = block[k];
        dxv[r] = dx_at(f, L.level);
        dyv[r] = dy_at(f, L.level);
        xl[r] = f->o.x0 + L.I * M * dxv[r];
        yl[r] = f->o.y0 + L.J * M * dyv[r];
    }
    rc = gf_write_ascii_frame(dir, iframe, f->st.t, (int)n, M, maux, qo.data(), ao.data(), gn.data(), lv.data(),
                              bk.data(), xl.data(), yl.data(), dxv.data(), dyv.data());
    if (rc) return ffail(f, rc, "cannot write the frame files");
    return GF_OK;
}

} // namespace

extern "C" {

int gf_forest_write_ascii(gf_forest* f, const char* dir, int iframe)
{
    if (!f || iframe < 0) return GF_ERR_ARG;
    if (f->leaves.empty()) return ffail(f, GF_ERR_STATE, "forest not initialised");
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    return write_frame(f, dir, iframe);
}

int gf_forest_set_output(gf_forest* f, const char* dir, int frames)
{
    if (!f) return GF_ERR_ARG;
    f->out_dir = dir ? dir : "";
    f->out_frames = frames != 0;
    return GF_OK;
}

int gf_forest_set_gauges(gf_forest* f, int n, const int* id, const double* xc, const double* yc,
                         const double* t1, const double* t2, const double* min_time_increment)
{
    if (!f || n < 0 || (n > 0 && (!id || !xc || !yc || !t1 || !t2 || !min_time_increment))) return GF_ERR_ARG;
    for (int g = 0; g < n; ++g)
        if (id[g] < 0 || id[g] > 99999 || !std::isfinite(xc[g]) || !std::isfinite(yc[g]) || !(min_time_increment[g] >= 0))
            return ffail(f, GF_ERR_ARG, "gauge ids must be 0..99999 with finite positions and increments >= 0");
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    int rc = flush_gauges(f);
    if (rc) return rc;
    f->gauges.assign(n, gf_gauge_task{});
    f->gauge_id.assign(id, id + n);
    f->gauge_x.assign(xc, xc + n);
    f->gauge_y.assign(yc, yc + n);
    for (int g = 0; g < n; ++g) {
        f->gauges[g].slot = -1;
        f->gauges[g].t1 = t1[g];
        f->gauges[g].t2 = t2[g];
        f->gauges[g].incr = min_time_increment[g];
        if ((rc = gf_write_gauge_header(f->out_dir.c_str(), id[g], xc[g], yc[g])))
            return ffail(f, rc, "cannot create a gauge file");
    }
    f->gauges_placed = false;
    f->grec_rows = 0;
    f->grec_cap = n > 0 ? std::max(1, std::min(4096, (1 << 21) / (6 * n))) : 0;
    if (n > 0) {
        FK(f, f->d_glast.reserve(n));
        FK(f, f->d_grec.reserve((size_t)f->grec_cap * n * 6));
        const std::vector<double> never(n, -INFINITY);
        FK(f, cudaMemcpy(f->d_glast.p, never.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    }
    return GF_OK;
}

int gf_forest_sample_gauges(gf_forest* f, double t)
{
    if (!f) return GF_ERR_ARG;
    if (f->leaves.empty()) return ffail(f, GF_ERR_STATE, "forest not initialised");
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    return sample_gauges(f, t);
}

int gf_forest_flush_gauges(gf_forest* f)
{
    if (!f) return GF_ERR_ARG;
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    return flush_gauges(f);
}

int gf_forest_download(gf_forest* f, double* q)
{
    if (!f || !q) return GF_ERR_ARG;
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    return move_leaves(f, q, 3, true, false);
}

int gf_forest_download_aux(gf_forest* f, double* aux)
{
    if (!f || !aux) return GF_ERR_ARG;
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    return move_leaves(f, aux, f->o.maux, true, true);
}

int gf_forest_upload(gf_forest* f, const double* q)
{
    if (!f || !q) return GF_ERR_ARG;
    FK(f, cudaSetDevice(gf::ctx_device(f->ctx)));
    return move_leaves(f, const_cast<double*>(q), 3, false, false);
}

} // extern "C"

/* ------------------------------------------------------------------------
 * Batched form: many forests in shared launches, device-side time-step
 * control, one captured round per epoch.
 * --------------------------------------------------------------------- */
namespace {

inline int cls_of(int mx) { return mx == 8 ? 0 : mx == 16 ? 1 : 2; }
inline size_t align_up(size_t b) { return (b + 255) & ~(size_t)255; }
const int kCls[3] = {8, 16, 32};
constexpr int kBatchLevels = 11;

struct Batch {
    gf_ctx* ctx = nullptr;
    std::vector<gf_forest*> fs;     /* members: group g = fs[g] */
    cudaStream_t st = nullptr;
    /* epoch area (pinned mirror + device) */
    char* h = nullptr;
    char* d = nullptr;
    size_t cap = 0;
    size_t off_blk = 0, off_gs = 0, off_dt = 0, off_par = 0, off_dl = 0, off_rb = 0, off_hyt = 0,
           off_hyu = 0, off_sched = 0;
    size_t off_refs[3] = {}, off_avg[3] = {}, off_work[3] = {};
    size_t off_itp[3][kBatchLevels] = {}, off_ref[3][kBatchLevels] = {};
    int n_refs[3] = {}, n_avg[3] = {}, n_work[3] = {};
    int n_itp[3][kBatchLevels] = {}, n_ref[3][kBatchLevels] = {};
    char* h_rb = nullptr;           /* readback: [err 8 B][states] */
    size_t rb_cap = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int launches_per_round = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_ctx = nullptr; /* context-stream work (tables, regrids) before the rounds */
    bool own_stream = false;
    int max_ctas = 0;             /* grid cap of the mixed update (0: one CTA per SM) */
    ~Batch()
    {
        if (ev_ctx) cudaEventDestroy(ev_ctx);
        if (own_stream && st) cudaStreamDestroy(st);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (d) cudaFree(d);
        if (h) cudaFreeHost(h);
        if (h_rb) cudaFreeHost(h_rb);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
    }
};

#define BK(b, call)                                                               \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) return gf::ctx_cuda_fail((b).ctx, e_, #call);      \
    } while (0)

/* one round of the epoch on the batch stream (captured) */
int enqueue_batch_round(Batch& B)
{
    const int ng = (int)B.fs.size();
    char* d = B.d;
    const gf_phys* phys = gf::ctx_device_phys(B.ctx);
    gf_ghost_block* blk = reinterpret_cast<gf_ghost_block*>(d + B.off_blk);
    gf_group_state* gs = reinterpret_cast<gf_group_state*>(d + B.off_gs);
    double* gdt = reinterpret_cast<double*>(d + B.off_dt);
    int* gpar = reinterpret_cast<int*>(d + B.off_par);
    long long* dl = reinterpret_cast<long long*>(d + B.off_dl);
    unsigned long long* rb = reinterpret_cast<unsigned long long*>(d + B.off_rb);
    int* err = reinterpret_cast<int*>(rb);
    const double* hyt = reinterpret_cast<const double*>(d + B.off_hyt);
    const double* hyu = reinterpret_cast<const double*>(d + B.off_hyu);
    int n = 0;
    BK(B, gf::launch_served_prepare(gs, blk, gdt, gpar, rb + 1, hyt, hyu, ng, B.st, dl));
    ++n;
    for (int c = 0; c < 3; ++c) {
        const int m = kCls[c];
        if (!B.n_refs[c]) continue;
        if (B.n_avg[c]) {
            BK(B, gf::launch_transfer(m, reinterpret_cast<gf_xfer_task*>(d + B.off_avg[c]), B.n_avg[c],
                                      phys, B.st, dl));
            ++n;
        }
        BK(B, gf::launch_ghost_fill(m, blk, reinterpret_cast<gf_ghost_ref*>(d + B.off_refs[c]),
                                    B.n_refs[c], phys, B.st));
        ++n;
        for (int l = 0; l < kBatchLevels; ++l) {
            if (B.n_itp[c][l]) {
                BK(B, gf::launch_transfer(m, reinterpret_cast<gf_xfer_task*>(d + B.off_itp[c][l]),
                                          B.n_itp[c][l], phys, B.st, dl));
                ++n;
            }
            if (B.n_ref[c][l]) {
                BK(B, gf::launch_ghost_fill(m, blk, reinterpret_cast<gf_ghost_ref*>(d + B.off_ref[c][l]),
                                            B.n_ref[c][l], phys, B.st));
                ++n;
            }
        }
    }
    const bool exact = gf::ctx_exact(B.ctx);
    if (gf::ctx_mixed(B.ctx)) {
        /* one persistent launch: the work lists lie contiguous, mx 32 first */
        const int nw[3] = {B.n_work[2], B.n_work[1], B.n_work[0]};
        const gf_patch_work* w = reinterpret_cast<gf_patch_work*>(d + B.off_work[2]);
        unsigned int* sched = reinterpret_cast<unsigned int*>(d + B.off_sched);
        if (nw[0] + nw[1] + nw[2]) {
            if (exact)
                BK(B, gf::launch_patch_update_mixed_exact(w, nw, phys, 0.0, gdt, gpar, 3, nullptr, rb + 1, err,
                                                          sched, B.st, B.max_ctas));
            else
                BK(B, gf::launch_patch_update_mixed(w, nw, phys, 0.0, gdt, gpar, 3, nullptr, rb + 1, err, sched,
                                                    B.st, B.max_ctas));
            ++n;
        }
    }
    for (int c = 0; c < 3 && !gf::ctx_mixed(B.ctx); ++c) {
        if (!B.n_work[c]) continue;
        const gf_patch_work* w = reinterpret_cast<gf_patch_work*>(d + B.off_work[c]);
        if (exact)
            BK(B, gf::launch_patch_update_exact(kCls[c], w, B.n_work[c], phys, 0.0, gdt, gpar, 3, nullptr,
                                                rb + 1, err, B.st));
        else
            BK(B, gf::launch_patch_update(kCls[c], w, B.n_work[c], phys, 0.0, gdt, gpar, 3, nullptr,
                                          rb + 1, err, B.st));
        ++n;
    }
    BK(B, gf::launch_served_finish(gs, gdt, rb + 1, err, ng, B.st));
    ++n;
    B.launches_per_round = n;
    return GF_OK;
}

/* Concatenate the members' tables into a new epoch and capture its round. */
int build_epoch(Batch& B)
{
    const int ng = (int)B.fs.size();
    for (gf_forest* f : B.fs) {
        int rc = build_tables(f);
        if (rc) return rc;
    }
    /* sizes */
    size_t nhy = 0;
    std::memset(B.n_refs, 0, sizeof B.n_refs);
    std::memset(B.n_avg, 0, sizeof B.n_avg);
    std::memset(B.n_work, 0, sizeof B.n_work);
    std::memset(B.n_itp, 0, sizeof B.n_itp);
    std::memset(B.n_ref, 0, sizeof B.n_ref);
    for (gf_forest* f : B.fs) {
        const int c = cls_of(f->M);
        nhy += f->hy_t.size();
        B.n_refs[c] += (int)f->leaves.size();
        B.n_work[c] += (int)f->h_work.size();
        B.n_avg[c] += (int)f->h_avg.size();
        for (size_t l = 0; l < f->h_itp.size(); ++l) {
            B.n_itp[c][l] += (int)f->h_itp[l].size();
            B.n_ref[c][l] += (int)f->h_refresh[l].size();
        }
    }
    size_t off = 0;
    auto take = [&off](size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes);
        return o;
    };
    B.off_blk = take(ng * sizeof(gf_ghost_block));
    B.off_gs = take(ng * sizeof(gf_group_state));
    B.off_dt = take(ng * sizeof(double));
    B.off_par = take(ng * sizeof(int));
    B.off_dl = take(ng * sizeof(long long));
    B.off_rb = take((ng + 1) * sizeof(unsigned long long));
    B.off_hyt = take(std::max<size_t>(nhy, 1) * sizeof(double));
    B.off_hyu = take(std::max<size_t>(nhy, 1) * sizeof(double));
    /* work items of all sizes contiguous, mx 32 first (the mixed launch's list) */
    B.off_work[2] = take((size_t)(B.n_work[0] + B.n_work[1] + B.n_work[2]) * sizeof(gf_patch_work));
    B.off_work[1] = B.off_work[2] + (size_t)B.n_work[2] * sizeof(gf_patch_work);
    B.off_work[0] = B.off_work[1] + (size_t)B.n_work[1] * sizeof(gf_patch_work);
    B.off_sched = take(2 * sizeof(unsigned int));
    for (int c = 0; c < 3; ++c) {
        B.off_refs[c] = take(B.n_refs[c] * sizeof(gf_ghost_ref));
        B.off_avg[c] = take(B.n_avg[c] * sizeof(gf_xfer_task));
        for (int l = 0; l < kBatchLevels; ++l) {
            B.off_itp[c][l] = take(B.n_itp[c][l] * sizeof(gf_xfer_task));
            B.off_ref[c][l] = take(B.n_ref[c][l] * sizeof(gf_ghost_ref));
        }
    }
    const size_t need = off;
    if (need > B.cap) {
        if (B.d) cudaFree(B.d);
        if (B.h) cudaFreeHost(B.h);
        B.d = nullptr;
        B.h = nullptr;
        B.cap = 0;
        const size_t c2 = need + need / 2;
        BK(B, cudaMalloc(reinterpret_cast<void**>(&B.d), c2));
        BK(B, cudaMallocHost(reinterpret_cast<void**>(&B.h), c2));
        B.cap = c2;
    }
    const size_t rbn = 8 + ng * sizeof(gf_group_state);
    if (rbn > B.rb_cap) {
        if (B.h_rb) cudaFreeHost(B.h_rb);
        B.h_rb = nullptr;
        BK(B, cudaMallocHost(reinterpret_cast<void**>(&B.h_rb), rbn * 2));
        B.rb_cap = rbn * 2;
    }
    char* h = B.h;
    /* every per-group table starts defined: the round's prepare kernel
     * rewrites them, but only for groups that step */
    std::memset(h, 0, need);
    int fill_refs[3] = {}, fill_avg[3] = {}, fill_work[3] = {};
    int fill_itp[3][kBatchLevels] = {}, fill_ref[3][kBatchLevels] = {};
    size_t hoff = 0;
    for (int g = 0; g < ng; ++g) {
        gf_forest* f = B.fs[g];
        const int c = cls_of(f->M);
        gf_ghost_block blk{};
        blk.q = f->qbuf[f->gst.cur];
        blk.aux = f->aux;
        blk.nbr = f->d_nbr.p;
        blk.geom = f->d_geom.p;
        blk.phys_of = nullptr;
        blk.bc = f->bc;
        blk.phys = f->o.phys_slot;
        blk.maux = f->o.maux;
        blk.skip = 1;
        reinterpret_cast<gf_ghost_block*>(h + B.off_blk)[g] = blk;
        f->gst.hydro_off = (int)hoff;
        f->gst.nhydro = (int)f->hy_t.size();
        std::copy(f->hy_t.begin(), f->hy_t.end(), reinterpret_cast<double*>(h + B.off_hyt) + hoff);
        std::copy(f->hy_hu.begin(), f->hy_hu.end(), reinterpret_cast<double*>(h + B.off_hyu) + hoff);
        hoff += f->hy_t.size();
        reinterpret_cast<gf_group_state*>(h + B.off_gs)[g] = f->gst;
        gf_ghost_ref* refs = reinterpret_cast<gf_ghost_ref*>(h + B.off_refs[c]);
        for (const Leaf& L : f->leaves) refs[fill_refs[c]++] = gf_ghost_ref{g, L.slot};
        gf_xfer_task* av = reinterpret_cast<gf_xfer_task*>(h + B.off_avg[c]);
        for (gf_xfer_task t : f->h_avg) {
            t.group = g;
            av[fill_avg[c]++] = t;
        }
        gf_patch_work* wk = reinterpret_cast<gf_patch_work*>(h + B.off_work[c]);
        for (gf_patch_work w : f->h_work) {
            w.group = g;
            wk[fill_work[c]++] = w;
        }
        for (size_t l = 0; l < f->h_itp.size(); ++l) {
            gf_xfer_task* it = reinterpret_cast<gf_xfer_task*>(h + B.off_itp[c][l]);
            for (gf_xfer_task t : f->h_itp[l]) {
                t.group = g;
                it[fill_itp[c][l]++] = t;
            }
            gf_ghost_ref* rr = reinterpret_cast<gf_ghost_ref*>(h + B.off_ref[c][l]);
            for (int slot : f->h_refresh[l]) rr[fill_ref[c][l]++] = gf_ghost_ref{g, slot};
        }
    }
    BK(B, cudaMemcpyAsync(B.d, B.h, need, cudaMemcpyHostToDevice, B.st));
    /* capture one round */
    if (B.exec) cudaGraphExecDestroy(B.exec);
    if (B.graph) cudaGraphDestroy(B.graph);
    B.exec = nullptr;
    B.graph = nullptr;
    BK(B, cudaStreamBeginCapture(B.st, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_batch_round(B);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(B.st, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    BK(B, e);
    B.graph = g;
    BK(B, cudaGraphInstantiate(&B.exec, B.graph, 0));
    return GF_OK;
}

} // namespace

namespace {

/* A batched run in progress: the members' rounds, their regrids and the
 * epoch rebuilds, one iteration at a time (gf_forest_batch_run drives it to
 * the end; the forest server adds and retires members between iterations). */
struct BatchRun {
    Batch B;
    gf_forest_batch_stats S{};
    double round_ms = 0.05;
    int rounds_paused = 0;
    bool rebuild = true;
    bool inflight = false; /* rounds and their readback enqueued, not yet taken in */
    int rounds_inflight = 0;
    std::chrono::steady_clock::time_point t_launch;
};

/* stream_priority: 0 runs the rounds on the context's stream; k >= 1 on a
 * stream of their own, k = 1 at the greatest priority the device offers and
 * each further k a step lower, so that batches can overlap on the device. */
int batch_begin(BatchRun& R, gf_ctx* ctx, int stream_priority = 0, int max_ctas = 0)
{
    Batch& B = R.B;
    if (cudaSetDevice(gf::ctx_device(ctx)) != cudaSuccess) return GF_ERR_CUDA;
    B.ctx = ctx;
    B.st = gf::ctx_stream(ctx);
    B.max_ctas = max_ctas;
    if (stream_priority) {
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi); /* hi: the numerically lowest, greatest priority */
        const int step = std::max(1, (lo - hi) / 2);
        BK(B, cudaStreamCreateWithPriority(&B.st, cudaStreamNonBlocking,
                                           std::min(lo, hi + (stream_priority - 1) * step)));
        B.own_stream = true;
    }
    BK(B, cudaEventCreateWithFlags(&B.ev_ctx, cudaEventDisableTiming));
    BK(B, cudaEventCreate(&B.ev0));
    BK(B, cudaEventCreate(&B.ev1));
    /* kernel attributes are set outside stream capture */
    for (int c = 0; c < 3; ++c) {
        gf::launch_patch_update(kCls[c], nullptr, 0, nullptr, 0.0, nullptr, nullptr, 0, nullptr, nullptr,
                                nullptr, B.st);
        gf::launch_patch_update_exact(kCls[c], nullptr, 0, nullptr, 0.0, nullptr, nullptr, 0, nullptr,
                                      nullptr, nullptr, B.st);
    }
    const int none[3] = {0, 0, 0};
    gf::launch_patch_update_mixed(nullptr, none, nullptr, 0.0, nullptr, nullptr, 0, nullptr, nullptr, nullptr,
                                  nullptr, B.st);
    gf::launch_patch_update_mixed_exact(nullptr, none, nullptr, 0.0, nullptr, nullptr, 0, nullptr, nullptr,
                                        nullptr, nullptr, B.st);
    return GF_OK;
}

/* controller at the start of a member's run (fc2d_geoclaw_run.c:197-225) */
void batch_add(BatchRun& R, gf_forest* f, double t_final, int nout, double initial_dt, double desired_cfl,
               double max_cfl)
{
    gf_group_state& g = f->gst;
    std::memset(&g, 0, sizeof g);
    g.qb[0] = f->qbuf[0];
    g.qb[1] = f->qbuf[1];
    g.dt_outer = t_final / nout;
    g.t_curr = f->st.t;
    g.tend = g.t_curr + g.dt_outer;
    g.dt_minlevel = initial_dt;
    g.desired_cfl = desired_cfl;
    g.max_cfl = max_cfl;
    g.max_cfl_seen = f->st.max_cfl_seen;
    g.level_factor = (double)(1 << (f->o.maxlevel - f->o.minlevel));
    g.steps = f->st.steps;
    g.rejects = f->st.rejects;
    g.nout = nout;
    g.active = 1;
    g.cur = f->par;
    g.regrid_interval = f->o.regrid_interval;
    g.since_regrid = f->o.regrid_interval > 0 ? (int)(f->st.steps % f->o.regrid_interval) : 0;
    R.B.fs.push_back(f);
    R.rebuild = true;
}

/* Launch one iteration: drop finished members, rebuild the epoch if needed,
 * enqueue ~0.5 ms of rounds and the controllers' readback. *live = members
 * (0: nothing was launched). */
int batch_launch(BatchRun& R, int* live_out)
{
    Batch& B = R.B;
    gf_forest_batch_stats& S = R.S;
    if (R.inflight) return gf::ctx_fail(B.ctx, GF_ERR_STATE, "batch iteration already in flight");
    std::vector<gf_forest*> live;
    for (gf_forest* f : B.fs)
        if (f->gst.active) live.push_back(f);
    if (live.size() != B.fs.size()) {
        B.fs.swap(live);
        R.rebuild = true;
    }
    *live_out = (int)B.fs.size();
    if (B.fs.empty()) return GF_OK;
    using clk = std::chrono::steady_clock;
    auto secs = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
    if (R.rebuild) {
        const auto te = clk::now();
        int rc = build_epoch(B);
        S.s_epoch += secs(te);
        if (rc) return rc;
        S.epochs++;
        R.rebuild = false;
        R.rounds_paused = 0;
    }
    const int ng = (int)B.fs.size();
    int rounds = (int)std::ceil(0.5 / std::max(R.round_ms, 1e-3));
    rounds = std::max(1, std::min(64, rounds));
    R.t_launch = clk::now();
    const cudaStream_t cst = gf::ctx_stream(B.ctx);
    if (B.st != cst) {
        /* tables and regrids of the members went to the context's stream */
        BK(B, cudaEventRecord(B.ev_ctx, cst));
        BK(B, cudaStreamWaitEvent(B.st, B.ev_ctx, 0));
    }
    BK(B, cudaEventRecord(B.ev0, B.st));
    for (int r = 0; r < rounds; ++r) BK(B, cudaGraphLaunch(B.exec, B.st));
    BK(B, cudaMemcpyAsync(B.h_rb, B.d + B.off_rb, 8, cudaMemcpyDeviceToHost, B.st));
    BK(B, cudaMemcpyAsync(B.h_rb + 8, B.d + B.off_gs, ng * sizeof(gf_group_state), cudaMemcpyDeviceToHost,
                          B.st));
    BK(B, cudaEventRecord(B.ev1, B.st));
    R.inflight = true;
    R.rounds_inflight = rounds;
    return GF_OK;
}

/* Take in a finished iteration (its readback has landed): the members'
 * controllers, then the regrids of the waiting members. */
int batch_complete(BatchRun& R)
{
    Batch& B = R.B;
    gf_forest_batch_stats& S = R.S;
    using clk = std::chrono::steady_clock;
    auto secs = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
    R.inflight = false;
    const int ng = (int)B.fs.size();
    const int rounds = R.rounds_inflight;
    S.s_rounds += secs(R.t_launch);
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, B.ev0, B.ev1) == cudaSuccess) R.round_ms = std::max(1e-3, (double)ms / rounds);
    S.rounds += rounds;
    S.launches += (long long)rounds * B.launches_per_round;
    int err;
    std::memcpy(&err, B.h_rb, sizeof err);
    if (err) return ffail(B.fs[0], GF_ERR_DEVICE, "a patch-update copy wait timed out");
    const gf_group_state* gs = reinterpret_cast<const gf_group_state*>(B.h_rb + 8);
    int npaused = 0, nactive = 0;
    for (int g = 0; g < ng; ++g) {
        gf_forest* f = B.fs[g];
        const long long before = f->gst.steps;
        const int hoff = f->gst.hydro_off;
        f->gst = gs[g];
        f->gst.hydro_off = hoff;
        f->par = f->gst.cur;
        f->st.cell_updates += (f->gst.steps - before) * f->cells;
        S.cell_updates += (f->gst.steps - before) * f->cells;
        f->st.steps = f->gst.steps;
        f->st.rejects = f->gst.rejects;
        f->st.t = f->gst.t_curr;
        f->st.dt = f->gst.dt_minlevel;
        f->st.max_cfl_seen = f->gst.max_cfl_seen;
        if (f->gst.active) {
            ++nactive;
            npaused += f->gst.paused != 0;
        } else {
            f->st.npatch = (int)f->leaves.size();
            f->st.npatch_max = std::max(f->st.npatch_max, f->st.npatch);
        }
    }
    if (npaused) R.rounds_paused += rounds;
    /* regrid the waiting members together once all live ones wait, or
     * after a while (the others keep stepping meanwhile) */
    if (npaused && (npaused == nactive || R.rounds_paused >= 16)) {
        std::vector<gf_forest*> due;
        std::vector<double> ts;
        for (gf_forest* f : B.fs)
            if (f->gst.active && f->gst.paused) {
                due.push_back(f);
                ts.push_back(f->gst.t_curr);
            }
        const auto tg = clk::now();
        int rc = regrid_many(B.ctx, due, ts);
        S.s_regrid += secs(tg);
        if (rc) return rc;
        for (gf_forest* f : due) {
            f->gst.paused = 0;
            f->gst.since_regrid = 0;
            f->st.npatch_max = std::max(f->st.npatch_max, (int)f->leaves.size());
            S.regrids++;
        }
        R.rebuild = true;
    } else if (nactive < ng) {
        R.rebuild = true; /* finished members leave the epoch */
    }
    return GF_OK;
}

/* one iteration, waited for */
int batch_iterate(BatchRun& R, int* live_out)
{
    int rc = batch_launch(R, live_out);
    if (rc || !*live_out) return rc;
    BK(R.B, cudaEventSynchronize(R.B.ev1));
    return batch_complete(R);
}

int batch_check(gf_forest* f, gf_ctx* ctx)
{
    if (!f || f->ctx != ctx) return GF_ERR_ARG;
    if (f->leaves.empty()) return ffail(f, GF_ERR_STATE, "forest not initialised");
    if (f->o.maxlevel >= kBatchLevels) return ffail(f, GF_ERR_ARG, "maxlevel too deep");
    if (f->o.subcycle)
        return ffail(f, GF_ERR_UNSUPPORTED, "shared rounds take every level's step together (subcycle = 0)");
    return GF_OK;
}

/* ---- subcycled forests side by side ----
 * A subcycled coarse step is one captured graph per forest (sub_launch), so
 * subcycled forests batch by running side by side: each forest's steps go
 * to one of a pool of streams and the host drives every forest's outstyle-1
 * loop (fc2d_geoclaw_run.c:190-395, as run_outstyle1 with subcycle = 1)
 * without waiting on the device: a pass takes in the steps whose readback
 * has landed (accept or retake, next dt, regrid when due) and launches each
 * idle forest's next step. Each forest's launches keep their order, so its
 * result equals its own gf_forest_run. */
struct SubRunner {
    gf_ctx* ctx = nullptr;
    std::vector<cudaStream_t> streams;
    std::vector<gf_forest*> fs;
    size_t next = 0;
    long long launched = 0, regrids = 0, cell_updates = 0;
    ~SubRunner()
    {
        for (cudaStream_t st : streams) cudaStreamDestroy(st);
    }
};
constexpr int kSubStreams = 16;

int sub_run_add(SubRunner& R, gf_forest* f, double t_final, int nout, double initial_dt, double desired_cfl,
                double max_cfl)
{
    if (!f || f->ctx != R.ctx) return GF_ERR_ARG;
    if (f->leaves.empty()) return ffail(f, GF_ERR_STATE, "forest not initialised");
    if (!f->o.subcycle) return ffail(f, GF_ERR_ARG, "not a subcycled forest");
    if ((int)R.streams.size() < kSubStreams) {
        cudaStream_t st;
        FK(f, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        R.streams.push_back(st);
    }
    f->sst = R.streams[R.next++ % R.streams.size()];
    gf_forest::SubRun& r = f->sr;
    r = gf_forest::SubRun{};
    r.t_curr = f->st.t;
    r.dt_minlevel = initial_dt;
    r.dt_outer = t_final / nout;
    r.tend = r.t_curr + r.dt_outer;
    r.nout = nout;
    r.desired_cfl = desired_cfl;
    r.max_cfl = max_cfl;
    r.active = true;
    R.fs.push_back(f);
    return GF_OK;
}

/* the next step: the outstyle-1 dt clipping to the output time, then launch */
int sub_run_launch(SubRunner& R, gf_forest* f)
{
    gf_forest::SubRun& r = f->sr;
    while (!(r.t_curr < r.tend)) {
        if (++r.nint >= r.nout) {
            r.active = false;
            f->st.t = r.t_curr;
            f->st.dt = r.dt_minlevel;
            f->st.npatch = (int)f->leaves.size();
            f->st.npatch_max = std::max(f->st.npatch_max, f->st.npatch);
            return GF_OK;
        }
        r.tend = r.t_curr + r.dt_outer;
    }
    double dt_step = r.dt_minlevel;
    const double tol = 1e-2 * dt_step;
    r.took_small = false;
    const double small_step = r.tend - (r.t_curr + dt_step);
    if (small_step < tol) {
        dt_step = r.tend - r.t_curr;
        if (small_step < 0) r.took_small = true;
    }
    r.dt_step = dt_step;
    int rc = sub_launch(f, r.t_curr, dt_step, f->sst);
    if (rc) return rc;
    r.pending = true;
    R.launched++;
    return GF_OK;
}

/* take in the step in flight: accept or retake, next dt, regrid when due */
int sub_run_complete(SubRunner& R, gf_forest* f)
{
    gf_forest::SubRun& r = f->sr;
    r.pending = false;
    double cfl = 0.0;
    long long updates = 0;
    int rc = sub_collect(f, &cfl, &updates);
    if (rc) return rc;
    f->st.max_cfl_seen = std::max(f->st.max_cfl_seen, cfl);
    if (cfl > r.max_cfl) {
        if ((rc = sub_finish(f, false))) return rc;
        r.dt_minlevel = r.dt_minlevel * r.desired_cfl / cfl;
        f->st.rejects++;
        return GF_OK;
    }
    if ((rc = sub_finish(f, true))) return rc;
    f->st.steps++;
    f->st.cell_updates += updates;
    R.cell_updates += updates;
    r.t_curr += r.dt_step;
    const double dt_new = r.dt_minlevel * r.desired_cfl / cfl;
    if (!r.took_small) r.dt_minlevel = dt_new;
    f->st.t = r.t_curr;
    f->st.dt = r.dt_minlevel;
    if (f->o.regrid_interval > 0 && f->st.steps % f->o.regrid_interval == 0) {
        bool changed = false;
        if ((rc = regrid(f, r.t_curr, &changed))) return rc;
        R.regrids++;
        f->st.npatch_max = std::max(f->st.npatch_max, (int)f->leaves.size());
    }
    return GF_OK;
}

/* One pass; never waits on the device (wait = 1: block on one step in
 * flight when nothing else could move). *live = forests still running. */
int sub_run_pass(SubRunner& R, int wait, int* live, int* progress)
{
    int moved = 0;
    for (gf_forest* f : R.fs) {
        if (!f->sr.pending) continue;
        const cudaError_t e = cudaEventQuery(f->sev_done);
        if (e == cudaErrorNotReady) continue;
        if (e != cudaSuccess) return gf::ctx_cuda_fail(R.ctx, e, "subcycled step");
        int rc = sub_run_complete(R, f);
        if (rc) return rc;
        moved = 1;
    }
    for (gf_forest* f : R.fs) {
        if (f->sr.pending || !f->sr.active || f->sr.cancel) continue;
        int rc = sub_run_launch(R, f);
        if (rc) return rc;
        moved = 1;
    }
    int n = 0;
    gf_forest* first = nullptr;
    for (gf_forest* f : R.fs) {
        n += f->sr.active || f->sr.pending;
        if (!first && f->sr.pending) first = f;
    }
    if (wait && !moved && first) {
        const cudaError_t e = cudaEventSynchronize(first->sev_done);
        if (e != cudaSuccess) return gf::ctx_cuda_fail(R.ctx, e, "subcycled step");
    }
    *live = n;
    if (progress) *progress = moved;
    return GF_OK;
}


/* ---- subcycled forests in shared launches ----
 * Forests whose leaves span the same levels and that share the patch size,
 * the aux count, the state buffer parity and the update build step
 * together: every launch of the subcycled schedule (the order of
 * sub_fill_level / sub_level above) carries the tasks of every member, with
 * each member's own level dts (group = member in the update's work items),
 * boundary times (one ghost block per member and call), buffers and CFL
 * slot. Each member's arithmetic is the same as in its own step, so its run
 * is the same bits; the launches per coarse step no longer grow with the
 * number of forests. The merged lists are the concatenation of the members'
 * own lists (build_sub_tables), rebuilt when a member's tables change
 * (regrid) or the membership does. */
struct SubGroup {
    gf_ctx* ctx = nullptr;
    int M = 0, lo = 0, hi = 0, par = 0, maux = 0;
    bool exact = false;
    std::vector<gf_forest*> mem;
    std::vector<unsigned long long> epochs; /* the members' table epochs merged */
    bool built = false;
    DArr<gf_patch_work> d_work;
    std::vector<int> w_off, w_n;             /* per level */
    DArr<gf_ghost_ref> d_refs;
    std::vector<int> ra_off, ra_n, rr_off, rr_n;
    DArr<gf_xfer_task> d_x;
    std::vector<int> xa_off, xi_off;         /* [l * 6 + bc * 2 + bf] */
    std::vector<int> xa_n, xi_n;             /* per level */
    DArr<gf_slot_task> d_s;
    std::vector<int> ti_off, ti_n;           /* [l * 2 + po], per level */
    int save_off = 0, save_n = 0;
    DArr<int> d_par;                         /* K zeros, then K ones */
    DArr<unsigned long long> d_rb;           /* [err][gmax of member k] */
    unsigned long long* h_rb = nullptr;      /* pinned, 1 + K */
    size_t h_rb_cap = 0;
    DArr<char> d_stage;                      /* level dts [nlev * K], then the blocks */
    char* h_stage = nullptr;
    size_t h_stage_cap = 0;
    std::vector<gf_ghost_block> blocks;      /* the step's ghost blocks, K per call */
    std::vector<double> tl, dtl;             /* per member during the plan pass */
    bool plan = false;
    int ncall = 0;
    size_t blk_off = 0;                      /* byte offset of the blocks in the staging */
    /* the step's launches as a CUDA graph, captured after a rebuild and
     * replayed while the tables stand; the plan pass rewrites the staging
     * (level dts, ghost blocks) that the graph's first node copies */
    cudaGraphExec_t exec = nullptr;
    bool graph_ok = false;
    size_t graph_bytes = 0;
    ~SubGroup()
    {
        if (exec) cudaGraphExecDestroy(exec);
        d_work.release();
        d_refs.release();
        d_x.release();
        d_s.release();
        d_par.release();
        d_rb.release();
        d_stage.release();
        if (h_rb) cudaFreeHost(h_rb);
        if (h_stage) cudaFreeHost(h_stage);
    }
};

int sg_fail(SubGroup& G, cudaError_t e, const char* what) { return gf::ctx_cuda_fail(G.ctx, e, what); }
#define GK(G, call)                                      \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return sg_fail((G), e_, #call); \
    } while (0)

/* merged tables of the group's members (their sub tables are current) */
int sg_build(SubGroup& G)
{
    const int K = (int)G.mem.size();
    const int nlev = G.hi + 1;
    std::vector<gf_patch_work> work;
    std::vector<gf_ghost_ref> refs;
    std::vector<gf_xfer_task> x;
    std::vector<gf_slot_task> sl;
    G.w_off.assign(nlev, 0);
    G.w_n.assign(nlev, 0);
    G.ra_off.assign(nlev, 0);
    G.ra_n.assign(nlev, 0);
    G.rr_off.assign(nlev, 0);
    G.rr_n.assign(nlev, 0);
    G.xa_off.assign((size_t)nlev * 6, 0);
    G.xi_off.assign((size_t)nlev * 6, 0);
    G.xa_n.assign(nlev, 0);
    G.xi_n.assign(nlev, 0);
    G.ti_off.assign((size_t)nlev * 2, 0);
    G.ti_n.assign(nlev, 0);
    for (int l = G.lo; l <= G.hi; ++l) {
        G.w_off[l] = (int)work.size();
        G.ra_off[l] = (int)refs.size();
        for (int k = 0; k < K; ++k) {
            const gf_forest* f = G.mem[k];
            for (int i = 0; i < f->lev_n[l]; ++i) {
                gf_patch_work w = f->h_work[f->lev_off[l] + i];
                w.group = k;
                work.push_back(w);
                refs.push_back(gf_ghost_ref{k, f->leaves[f->lev_off[l] + i].slot});
            }
        }
        G.w_n[l] = (int)work.size() - G.w_off[l];
        G.ra_n[l] = (int)refs.size() - G.ra_off[l];
    }
    for (int l = G.lo; l <= G.hi; ++l) {
        G.rr_off[l] = (int)refs.size();
        for (int k = 0; k < K; ++k)
            for (int s : G.mem[k]->h_refresh[l]) refs.push_back(gf_ghost_ref{k, s});
        G.rr_n[l] = (int)refs.size() - G.rr_off[l];
    }
    for (int l = G.lo; l <= G.hi; ++l)
        for (int c = 0; c < 6; ++c) {
            G.xa_off[(size_t)l * 6 + c] = (int)x.size();
            for (int k = 0; k < K; ++k) {
                const gf_forest* f = G.mem[k];
                const int o = f->sx_avg_off[(size_t)l * 6 + c];
                x.insert(x.end(), f->h_sx.begin() + o, f->h_sx.begin() + o + f->sx_avg_n[l]);
            }
            G.xa_n[l] = (int)x.size() - G.xa_off[(size_t)l * 6 + c];
            G.xi_off[(size_t)l * 6 + c] = (int)x.size();
            for (int k = 0; k < K; ++k) {
                const gf_forest* f = G.mem[k];
                const int o = f->sx_itp_off[(size_t)l * 6 + c];
                x.insert(x.end(), f->h_sx.begin() + o, f->h_sx.begin() + o + f->itp_n[l]);
            }
            G.xi_n[l] = (int)x.size() - G.xi_off[(size_t)l * 6 + c];
        }
    for (int l = G.lo; l <= G.hi; ++l)
        for (int po = 0; po < 2; ++po) {
            G.ti_off[(size_t)l * 2 + po] = (int)sl.size();
            for (int k = 0; k < K; ++k) {
                const gf_forest* f = G.mem[k];
                const int o = f->ss_ti_off[(size_t)l * 2 + po];
                sl.insert(sl.end(), f->h_ss.begin() + o, f->h_ss.begin() + o + f->lev_n[l]);
            }
            G.ti_n[l] = (int)sl.size() - G.ti_off[(size_t)l * 2 + po];
        }
    G.save_off = (int)sl.size();
    for (int k = 0; k < K; ++k) {
        const gf_forest* f = G.mem[k];
        const int o = f->ss_copy_off[0][G.par];
        sl.insert(sl.end(), f->h_ss.begin() + o, f->h_ss.begin() + o + f->ss_copy_n[0]);
    }
    G.save_n = (int)sl.size() - G.save_off;
    cudaStream_t st = gf::ctx_stream(G.ctx);
    GK(G, G.d_work.reserve(work.size() + 1));
    GK(G, G.d_refs.reserve(refs.size() + 1));
    GK(G, G.d_x.reserve(x.size() + 1));
    GK(G, G.d_s.reserve(sl.size() + 1));
    if (!work.empty())
        GK(G, cudaMemcpyAsync(G.d_work.p, work.data(), work.size() * sizeof(gf_patch_work), cudaMemcpyHostToDevice, st));
    if (!refs.empty())
        GK(G, cudaMemcpyAsync(G.d_refs.p, refs.data(), refs.size() * sizeof(gf_ghost_ref), cudaMemcpyHostToDevice, st));
    if (!x.empty())
        GK(G, cudaMemcpyAsync(G.d_x.p, x.data(), x.size() * sizeof(gf_xfer_task), cudaMemcpyHostToDevice, st));
    if (!sl.empty())
        GK(G, cudaMemcpyAsync(G.d_s.p, sl.data(), sl.size() * sizeof(gf_slot_task), cudaMemcpyHostToDevice, st));
    std::vector<int> pars((size_t)2 * K, 0);
    for (int k = 0; k < K; ++k) pars[(size_t)K + k] = 1;
    GK(G, G.d_par.reserve(pars.size()));
    GK(G, cudaMemcpyAsync(G.d_par.p, pars.data(), pars.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    GK(G, G.d_rb.reserve((size_t)K + 1));
    if (G.h_rb_cap < (size_t)K + 1) {
        if (G.h_rb) cudaFreeHost(G.h_rb);
        G.h_rb = nullptr;
        G.h_rb_cap = 0;
        GK(G, cudaMallocHost(reinterpret_cast<void**>(&G.h_rb), ((size_t)K + 1) * 2 * sizeof(unsigned long long)));
        G.h_rb_cap = ((size_t)K + 1) * 2;
    }
    G.epochs.clear();
    for (gf_forest* f : G.mem) G.epochs.push_back(f->sub_epoch);
    G.built = true;
    G.graph_ok = false;
    return GF_OK;
}

/* one ghost fill of level l's leaves (refs at roff, n) in buffer b of every
 * member, at each member's time tt[k] */
int sg_ghost(SubGroup& G, int b, const std::vector<double>& tt, int roff, int n)
{
    const int K = (int)G.mem.size();
    if (n <= 0) return GF_OK;
    const int i = G.ncall++;
    if (G.plan) {
        if ((int)G.blocks.size() < (i + 1) * K) G.blocks.resize((size_t)(i + 1) * K);
        for (int k = 0; k < K; ++k) {
            gf_forest* f = G.mem[k];
            gf_ghost_block blk{};
            blk.q = b < 2 ? f->qbuf[b] : f->qi;
            blk.aux = f->aux;
            blk.nbr = f->d_nbr.p;
            blk.geom = f->d_geom.p;
            blk.phys_of = nullptr;
            blk.bc = f->bc;
            blk.bc.q0hu = hydro_at(f, tt[k]);
            blk.phys = f->o.phys_slot;
            blk.maux = f->o.maux;
            blk.skip = 0;
            G.blocks[(size_t)i * K + k] = blk;
        }
        return GF_OK;
    }
    const gf_ghost_block* d_blk =
        reinterpret_cast<const gf_ghost_block*>(G.d_stage.p + G.blk_off) + (size_t)i * K;
    GK(G, gf::launch_ghost_fill(G.M, d_blk, G.d_refs.p + roff, n, gf::ctx_device_phys(G.ctx),
                                gf::ctx_stream(G.ctx)));
    return GF_OK;
}

/* sub_fill_level for the group */
int sg_fill_level(SubGroup& G, int l, const std::vector<double>& tt, const int* p, int cbuf)
{
    cudaStream_t st = gf::ctx_stream(G.ctx);
    const gf_phys* phys = gf::ctx_device_phys(G.ctx);
    const bool go = !G.plan;
    int rc;
    if (go && l < G.hi && G.xa_n[l])
        GK(G, gf::launch_transfer(G.M, G.d_x.p + G.xa_off[(size_t)l * 6 + p[l] * 2 + p[l + 1]], G.xa_n[l],
                                  phys, st));
    if ((rc = sg_ghost(G, p[l], tt, G.ra_off[l], G.ra_n[l]))) return rc;
    if (cbuf >= 0 && G.xi_n[l]) {
        if (go)
            GK(G, gf::launch_transfer(G.M, G.d_x.p + G.xi_off[(size_t)l * 6 + cbuf * 2 + p[l]], G.xi_n[l],
                                      phys, st));
        if ((rc = sg_ghost(G, p[l], tt, G.rr_off[l], G.rr_n[l]))) return rc;
    }
    return GF_OK;
}

int sg_update(SubGroup& G, int l, int* p)
{
    const int K = (int)G.mem.size();
    if (!G.plan && G.w_n[l]) {
        cudaStream_t st = gf::ctx_stream(G.ctx);
        const gf_phys* phys = gf::ctx_device_phys(G.ctx);
        int* err = reinterpret_cast<int*>(G.d_rb.p);
        const double* dts = reinterpret_cast<const double*>(G.d_stage.p) + (size_t)l * K;
        const gf_patch_work* w = G.d_work.p + G.w_off[l];
        const int* gpar = G.d_par.p + (size_t)p[l] * K;
        if (G.exact)
            GK(G, gf::launch_patch_update_exact(G.M, w, G.w_n[l], phys, 0.0, dts, gpar, G.maux, nullptr,
                                                G.d_rb.p + 1, err, st));
        else
            GK(G, gf::launch_patch_update(G.M, w, G.w_n[l], phys, 0.0, dts, gpar, G.maux, nullptr,
                                          G.d_rb.p + 1, err, st));
    }
    p[l] ^= 1;
    return GF_OK;
}

/* sub_level for the group: tl / dtl per member as in the member's own step */
int sg_level(SubGroup& G, int l, const std::vector<double>& tl, const std::vector<double>& dtl, int* p)
{
    int rc;
    if ((rc = sg_update(G, l, p))) return rc;
    if (l >= G.hi) return GF_OK;
    const int K = (int)G.mem.size();
    const int po = p[l] ^ 1;
    cudaStream_t st = gf::ctx_stream(G.ctx);
    const gf_phys* phys = gf::ctx_device_phys(G.ctx);
    std::vector<double> tf(K), dth(K);
    for (int k = 0; k < K; ++k) dth[k] = dtl[k] * 0.5;
    for (int s = 0; s < 2; ++s) {
        for (int k = 0; k < K; ++k) tf[k] = s ? tl[k] + dtl[k] * 0.5 : tl[k];
        int cbuf = po;
        if (s == 1) {
            if (!G.plan) {
                if (G.ti_n[l])
                    GK(G, gf::launch_tinterp_strip(G.M, G.d_s.p + G.ti_off[(size_t)l * 2 + po], G.ti_n[l], 0.5, st));
                if (G.xa_n[l])
                    GK(G, gf::launch_transfer(G.M, G.d_x.p + G.xa_off[(size_t)l * 6 + 2 * 2 + p[l + 1]],
                                              G.xa_n[l], phys, st));
            }
            if ((rc = sg_ghost(G, 2, tf, G.ra_off[l], G.ra_n[l]))) return rc;
            cbuf = 2;
        }
        if ((rc = sg_fill_level(G, l + 1, tf, p, cbuf))) return rc;
        if ((rc = sg_level(G, l + 1, tf, dth, p))) return rc;
    }
    return GF_OK;
}

/* one coarse step of every member (t[k], dt[k]), launched on the context's
 * stream with the per-member CFL readback into G.h_rb */
int sg_launch(SubGroup& G, const std::vector<double>& t, const std::vector<double>& dt)
{
    const int K = (int)G.mem.size();
    const int nlev = G.hi + 1;
    cudaStream_t st = gf::ctx_stream(G.ctx);
    std::vector<int> p(nlev + 1, G.par);
    /* plan: the step's ghost blocks */
    G.plan = true;
    G.ncall = 0;
    int rc = sg_fill_level(G, G.lo, t, p.data(), -1);
    if (!rc) rc = sg_level(G, G.lo, t, dt, p.data());
    G.plan = false;
    if (rc) return rc;
    const int ncall = G.ncall;
    G.blk_off = ((size_t)nlev * K * sizeof(double) + 255) / 256 * 256;
    const size_t bytes = G.blk_off + (size_t)ncall * K * sizeof(gf_ghost_block);
    if (bytes > G.h_stage_cap) {
        if (G.h_stage) cudaFreeHost(G.h_stage);
        G.h_stage = nullptr;
        G.h_stage_cap = 0;
        GK(G, cudaMallocHost(reinterpret_cast<void**>(&G.h_stage), bytes + bytes / 2));
        G.h_stage_cap = bytes + bytes / 2;
        G.graph_ok = false; /* the graph's first node reads the old staging */
    }
    double* hdt = reinterpret_cast<double*>(G.h_stage);
    for (size_t e = 0; e < (size_t)nlev * K; ++e) hdt[e] = 0.0;
    for (int k = 0; k < K; ++k) {
        double d = dt[k];
        for (int l = G.lo; l <= G.hi; ++l, d *= 0.5) hdt[(size_t)l * K + k] = d;
    }
    std::memcpy(G.h_stage + G.blk_off, G.blocks.data(), (size_t)ncall * K * sizeof(gf_ghost_block));
    if (!G.graph_ok || G.graph_bytes != bytes) {
        G.graph_ok = false;
        GK(G, G.d_stage.reserve(bytes));
        GK(G, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int crc = GF_OK;
        auto cap = [&](cudaError_t e) {
            if (e != cudaSuccess && crc == GF_OK) crc = sg_fail(G, e, "subcycled group step capture");
        };
        cap(cudaMemcpyAsync(G.d_stage.p, G.h_stage, bytes, cudaMemcpyHostToDevice, st));
        cap(cudaMemsetAsync(G.d_rb.p, 0, ((size_t)K + 1) * sizeof(unsigned long long), st));
        if (G.save_n) cap(gf::launch_slot_copy(G.M, G.d_s.p + G.save_off, G.save_n, st));
        std::vector<int> q(nlev + 1, G.par);
        G.ncall = 0;
        if (crc == GF_OK) crc = sg_fill_level(G, G.lo, t, q.data(), -1);
        if (crc == GF_OK) crc = sg_level(G, G.lo, t, dt, q.data());
        cap(cudaMemcpyAsync(G.h_rb, G.d_rb.p, ((size_t)K + 1) * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, st));
        cudaGraph_t graph = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(st, &graph);
        if (crc) {
            if (graph) cudaGraphDestroy(graph);
            return crc;
        }
        GK(G, ee);
        /* the same launch sequence as the last capture: update in place */
        bool updated = false;
        if (G.exec) {
            cudaGraphExecUpdateResultInfo info;
            updated = cudaGraphExecUpdate(G.exec, graph, &info) == cudaSuccess;
            if (!updated) {
                cudaGetLastError();
                cudaGraphExecDestroy(G.exec);
                G.exec = nullptr;
            }
        }
        cudaError_t ei = cudaSuccess;
        if (!updated) ei = cudaGraphInstantiate(&G.exec, graph, 0);
        cudaGraphDestroy(graph);
        GK(G, ei);
        G.graph_ok = true;
        G.graph_bytes = bytes;
    }
    GK(G, cudaGraphLaunch(G.exec, st));
    return GF_OK;
}

/* Subcycled forests in shared launches, each with its own outstyle-1
 * control (as sub_run_launch / sub_run_complete); forests that match
 * (same level range, patch size, aux count, parity, build) share a group. */
struct SubBatch {
    gf_ctx* ctx = nullptr;
    std::vector<gf_forest*> fs;
    std::vector<std::unique_ptr<SubGroup>> groups;
    long long regrids = 0, cell_updates = 0, steps_launched = 0;
    /* the step's end for every member in one launch: restore copies of
     * retaken steps, unify copies of accepted ones */
    DArr<gf_slot_task> d_fin;
    gf_slot_task* h_fin = nullptr; /* pinned */
    size_t h_fin_cap = 0;
    ~SubBatch()
    {
        d_fin.release();
        if (h_fin) cudaFreeHost(h_fin);
    }
};

int sb_add(SubBatch& B, gf_forest* f, double t_final, int nout, double initial_dt, double desired_cfl,
           double max_cfl)
{
    if (!f || f->ctx != B.ctx) return GF_ERR_ARG;
    if (f->leaves.empty()) return ffail(f, GF_ERR_STATE, "forest not initialised");
    if (!f->o.subcycle) return ffail(f, GF_ERR_ARG, "not a subcycled forest");
    gf_forest::SubRun& r = f->sr;
    r = gf_forest::SubRun{};
    r.t_curr = f->st.t;
    r.dt_minlevel = initial_dt;
    r.dt_outer = t_final / nout;
    r.tend = r.t_curr + r.dt_outer;
    r.nout = nout;
    r.desired_cfl = desired_cfl;
    r.max_cfl = max_cfl;
    r.active = true;
    B.fs.push_back(f);
    return GF_OK;
}

/* the outstyle-1 clipping of the member's next step; false when its run is over */
bool sb_next(gf_forest* f)
{
    gf_forest::SubRun& r = f->sr;
    while (!(r.t_curr < r.tend)) {
        if (++r.nint >= r.nout) {
            r.active = false;
            f->st.t = r.t_curr;
            f->st.dt = r.dt_minlevel;
            f->st.npatch = (int)f->leaves.size();
            f->st.npatch_max = std::max(f->st.npatch_max, f->st.npatch);
            return false;
        }
        r.tend = r.t_curr + r.dt_outer;
    }
    double dt_step = r.dt_minlevel;
    const double tol = 1e-2 * dt_step;
    r.took_small = false;
    const double small_step = r.tend - (r.t_curr + dt_step);
    if (small_step < tol) {
        dt_step = r.tend - r.t_curr;
        if (small_step < 0) r.took_small = true;
    }
    r.dt_step = dt_step;
    return true;
}

/* One iteration: every running forest takes one coarse step (accepted or
 * retaken), group by group; *live = forests still running. */
int sb_iterate(SubBatch& B, int* live)
{
    std::vector<gf_forest*> run;
    for (gf_forest* f : B.fs)
        if (f->sr.active && !f->sr.cancel && sb_next(f)) run.push_back(f);
    for (gf_forest* f : run) {
        int rc = build_sub_tables(f);
        if (rc) return rc;
    }
    /* regroup: key (patch size, levels present, aux count, parity, build) */
    const bool exact = gf::ctx_exact(B.ctx);
    std::vector<std::unique_ptr<SubGroup>> next;
    for (gf_forest* f : run) {
        SubGroup* g = nullptr;
        for (auto& h : next)
            if (h->M == f->M && h->lo == f->sub_lo && h->hi == f->sub_hi && h->maux == f->o.maux &&
                h->par == f->par)
                g = h.get();
        if (!g) {
            next.emplace_back(new SubGroup());
            g = next.back().get();
            g->ctx = B.ctx;
            g->M = f->M;
            g->lo = f->sub_lo;
            g->hi = f->sub_hi;
            g->maux = f->o.maux;
            g->par = f->par;
            g->exact = exact;
        }
        g->mem.push_back(f);
    }
    /* keep the built tables of groups whose members and epochs are unchanged */
    for (auto& g : next)
        for (auto& old : B.groups)
            if (old && old->M == g->M && old->lo == g->lo && old->hi == g->hi && old->maux == g->maux &&
                old->par == g->par && old->exact == g->exact && old->mem == g->mem) {
                bool same = old->built;
                for (size_t k = 0; same && k < g->mem.size(); ++k)
                    same = old->epochs[k] == g->mem[k]->sub_epoch;
                if (same) std::swap(g, old);
                break;
            }
    /* a rebuilt group takes over the graph of the group it replaces, which
     * is updated in place when the launch sequence is unchanged */
    for (auto& g : next)
        if (!g->built && !g->exec)
            for (auto& old : B.groups)
                if (old && old->exec && old->M == g->M && old->lo == g->lo && old->hi == g->hi &&
                    old->maux == g->maux && old->par == g->par && old->exact == g->exact) {
                    g->exec = old->exec;
                    old->exec = nullptr;
                    break;
                }
    B.groups.swap(next);
    for (auto& g : B.groups) {
        if (!g->built) {
            int rc = sg_build(*g);
            if (rc) return rc;
        }
        const int K = (int)g->mem.size();
        std::vector<double> t(K), dt(K);
        for (int k = 0; k < K; ++k) {
            t[k] = g->mem[k]->sr.t_curr;
            dt[k] = g->mem[k]->sr.dt_step;
        }
        int rc = sg_launch(*g, t, dt);
        if (rc) return rc;
        B.steps_launched += K;
    }
    cudaStream_t st = gf::ctx_stream(B.ctx);
    const cudaError_t se = cudaStreamSynchronize(st);
    if (se != cudaSuccess) return gf::ctx_cuda_fail(B.ctx, se, "subcycled group step");
    /* take in each member's step: accept or retake, next dt; the restore /
     * unify copies of all members in one launch, then the due regrids
     * together (one tag launch and one transfer launch per patch size) */
    std::vector<gf_slot_task> fin[3]; /* per patch size 8, 16, 32 */
    std::vector<gf_forest*> due;
    std::vector<double> due_t;
    for (auto& g : B.groups) {
        const int K = (int)g->mem.size();
        if ((int)g->h_rb[0]) return gf::ctx_fail(B.ctx, GF_ERR_DEVICE, "a patch-update copy wait timed out");
        for (int k = 0; k < K; ++k) {
            gf_forest* f = g->mem[k];
            gf_forest::SubRun& r = f->sr;
            double cfl;
            std::memcpy(&cfl, &g->h_rb[1 + k], sizeof cfl);
            long long cu = 0;
            for (int l = f->sub_lo; l <= f->sub_hi; ++l)
                cu += (long long)f->lev_n[l] * f->M * f->M << (l - f->sub_lo);
            f->st.max_cfl_seen = std::max(f->st.max_cfl_seen, cfl);
            const bool accept = !(cfl > r.max_cfl);
            const int kind = accept ? 2 : 1; /* sub_finish's copy lists */
            std::vector<gf_slot_task>& fl = fin[f->M == 8 ? 0 : f->M == 16 ? 1 : 2];
            const int o = f->ss_copy_off[kind][f->par];
            fl.insert(fl.end(), f->h_ss.begin() + o, f->h_ss.begin() + o + f->ss_copy_n[kind]);
            if (!accept) {
                r.dt_minlevel = r.dt_minlevel * r.desired_cfl / cfl;
                f->st.rejects++;
                continue;
            }
            f->st.steps++;
            f->st.cell_updates += cu;
            B.cell_updates += cu;
            r.t_curr += r.dt_step;
            const double dt_new = r.dt_minlevel * r.desired_cfl / cfl;
            if (!r.took_small) r.dt_minlevel = dt_new;
            f->st.t = r.t_curr;
            f->st.dt = r.dt_minlevel;
            if (f->o.regrid_interval > 0 && f->st.steps % f->o.regrid_interval == 0) {
                due.push_back(f);
                due_t.push_back(r.t_curr);
            }
        }
    }
    const size_t nfin = fin[0].size() + fin[1].size() + fin[2].size();
    if (nfin) {
        if (B.h_fin_cap < nfin) {
            if (B.h_fin) cudaFreeHost(B.h_fin);
            B.h_fin = nullptr;
            B.h_fin_cap = 0;
            const cudaError_t e =
                cudaMallocHost(reinterpret_cast<void**>(&B.h_fin), (nfin + nfin / 2) * sizeof(gf_slot_task));
            if (e != cudaSuccess) return gf::ctx_cuda_fail(B.ctx, e, "subcycled step end");
            B.h_fin_cap = nfin + nfin / 2;
        }
        size_t off[3], o = 0;
        for (int c = 0; c < 3; ++c) {
            off[c] = o;
            if (!fin[c].empty()) std::memcpy(B.h_fin + o, fin[c].data(), fin[c].size() * sizeof(gf_slot_task));
            o += fin[c].size();
        }
        cudaError_t e = B.d_fin.reserve(nfin);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(B.d_fin.p, B.h_fin, nfin * sizeof(gf_slot_task), cudaMemcpyHostToDevice, st);
        static const int ms[3] = {8, 16, 32};
        for (int c = 0; c < 3 && e == cudaSuccess; ++c)
            if (!fin[c].empty()) e = gf::launch_slot_copy(ms[c], B.d_fin.p + off[c], (int)fin[c].size(), st);
        if (e != cudaSuccess) return gf::ctx_cuda_fail(B.ctx, e, "subcycled step end");
        /* the pinned list is reused next iteration: its copy must have landed */
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return gf::ctx_cuda_fail(B.ctx, e, "subcycled step end");
    }
    if (!due.empty()) {
        int rc = regrid_many(B.ctx, due, due_t);
        if (rc) return rc;
        B.regrids += (long long)due.size();
        for (gf_forest* f : due) f->st.npatch_max = std::max(f->st.npatch_max, (int)f->leaves.size());
    }
    int n = 0;
    for (gf_forest* f : B.fs) n += f->sr.active && !f->sr.cancel;
    *live = n;
    return GF_OK;
}
#undef GK

} // namespace

extern "C" int gf_forest_batch_run(gf_forest** forests, int n, double t_final, int nout,
                                   double initial_dt, double desired_cfl, double max_cfl,
                                   gf_forest_batch_stats* bst)
{
    if (!forests || n < 1 || !(t_final > 0) || nout < 1 || !(initial_dt > 0) || !(desired_cfl > 0) ||
        !(max_cfl > 0))
        return GF_ERR_ARG;
    gf_ctx* ctx = forests[0] ? forests[0]->ctx : nullptr;
    for (int k = 0; k < n; ++k) {
        if (!forests[k] || forests[k]->ctx != ctx) return GF_ERR_ARG;
        int rc = forests[k]->o.subcycle ? (forests[k]->leaves.empty()
                                               ? ffail(forests[k], GF_ERR_STATE, "forest not initialised")
                                               : GF_OK)
                                        : batch_check(forests[k], ctx);
        if (rc) return rc;
        for (int j = 0; j < k; ++j)
            if (forests[j] == forests[k]) return ffail(forests[k], GF_ERR_ARG, "a forest appears twice");
    }
    /* forests that take every level's step together share rounds;
     * subcycled forests share the launches of their coarse steps, grouped
     * by the levels they span */
    BatchRun R;
    SubBatch U;
    U.ctx = ctx;
    int rc = batch_begin(R, ctx);
    if (rc) return rc;
    int nb = 0, ns = 0;
    for (int k = 0; k < n; ++k) {
        if (forests[k]->o.subcycle) {
            if ((rc = sb_add(U, forests[k], t_final, nout, initial_dt, desired_cfl, max_cfl))) return rc;
            ++ns;
        } else {
            batch_add(R, forests[k], t_final, nout, initial_dt, desired_cfl, max_cfl);
            ++nb;
        }
    }
    int live_b = nb, live_s = ns;
    while (live_b || live_s) {
        if (live_s && (rc = sb_iterate(U, &live_s))) return rc;
        if (live_b && (rc = batch_iterate(R, &live_b))) return rc;
    }
    if (bst) {
        *bst = R.S;
        bst->regrids += U.regrids;
        bst->cell_updates += U.cell_updates;
    }
    return GF_OK;
}

struct gf::ForestBatch {
    BatchRun R;
};

struct gf::SubForests {
    SubRunner U;
};

int gf::subforests_create(gf_ctx* c, SubForests** out)
{
    if (!c || !out) return GF_ERR_ARG;
    SubForests* s = new SubForests;
    s->U.ctx = c;
    *out = s;
    return GF_OK;
}

void gf::subforests_destroy(SubForests* s) { delete s; }

int gf::subforests_add(SubForests* s, gf_forest* f, double t_final, int nout, double initial_dt,
                       double desired_cfl, double max_cfl)
{
    if (!s || !(t_final > 0) || nout < 1 || !(initial_dt > 0) || !(desired_cfl > 0) || !(max_cfl > 0))
        return GF_ERR_ARG;
    return sub_run_add(s->U, f, t_final, nout, initial_dt, desired_cfl, max_cfl);
}

int gf::subforests_pass(SubForests* s, int* live, int* progress) { return sub_run_pass(s->U, 0, live, progress); }

bool gf::subforests_pending(const gf_forest* f) { return f->sr.pending; }

bool gf::subforests_running(const gf_forest* f) { return f->sr.pending || (f->sr.active && !f->sr.cancel); }

void gf::subforests_stop(gf_forest* f) { f->sr.cancel = true; }

void gf::subforests_remove(SubForests* s, gf_forest* f)
{
    std::vector<gf_forest*>& fs = s->U.fs;
    auto it = std::find(fs.begin(), fs.end(), f);
    if (it != fs.end()) fs.erase(it);
}

void gf::subforests_get_stats(const SubForests* s, long long* steps_launched, long long* regrids,
                              long long* cell_updates)
{
    *steps_launched = s->U.launched;
    *regrids = s->U.regrids;
    *cell_updates = s->U.cell_updates;
}

int gf::forest_batch_create(gf_ctx* c, ForestBatch** out, int stream_priority, int max_ctas)
{
    if (!c || !out) return GF_ERR_ARG;
    ForestBatch* b = new ForestBatch;
    int rc = batch_begin(b->R, c, stream_priority, max_ctas);
    if (rc) {
        delete b;
        return rc;
    }
    *out = b;
    return GF_OK;
}

void gf::forest_batch_destroy(ForestBatch* b) { delete b; }

int gf::forest_batch_add(ForestBatch* b, gf_forest* f, double t_final, int nout, double initial_dt,
                         double desired_cfl, double max_cfl)
{
    if (!b || !(t_final > 0) || nout < 1 || !(initial_dt > 0) || !(desired_cfl > 0) || !(max_cfl > 0))
        return GF_ERR_ARG;
    int rc = batch_check(f, b->R.B.ctx);
    if (rc) return rc;
    if (b->R.inflight) return ffail(f, GF_ERR_STATE, "members join between iterations");
    for (gf_forest* g : b->R.B.fs)
        if (g == f) return ffail(f, GF_ERR_ARG, "the forest is already a member");
    batch_add(b->R, f, t_final, nout, initial_dt, desired_cfl, max_cfl);
    return GF_OK;
}

int gf::forest_batch_iterate(ForestBatch* b, int* live) { return batch_iterate(b->R, live); }

int gf::forest_batch_launch(ForestBatch* b, int* live) { return batch_launch(b->R, live); }

int gf::forest_batch_test(ForestBatch* b, int wait, int* done)
{
    *done = 1;
    if (!b->R.inflight) return GF_OK;
    cudaError_t e = wait ? cudaEventSynchronize(b->R.B.ev1) : cudaEventQuery(b->R.B.ev1);
    if (e == cudaErrorNotReady) {
        *done = 0;
        return GF_OK;
    }
    if (e != cudaSuccess) return gf::ctx_cuda_fail(b->R.B.ctx, e, "batch iteration");
    return batch_complete(b->R);
}

bool gf::forest_batch_inflight(const ForestBatch* b) { return b->R.inflight; }

void gf::forest_batch_set_max_ctas(ForestBatch* b, int max_ctas)
{
    if (b->R.B.max_ctas == max_ctas) return;
    b->R.B.max_ctas = max_ctas;
    b->R.rebuild = true;
}

int gf::forest_batch_members(const ForestBatch* b) { return (int)b->R.B.fs.size(); }

void gf::forest_batch_remove(ForestBatch* b, gf_forest* f)
{
    /* callers remove members only between iterations */
    std::vector<gf_forest*>& fs = b->R.B.fs;
    auto it = std::find(fs.begin(), fs.end(), f);
    if (it == fs.end()) return;
    fs.erase(it);
    f->gst.active = 0;
    b->R.rebuild = true;
}

bool gf::forest_batch_running(const gf_forest* f) { return f->gst.active != 0; }

void gf::forest_batch_get_stats(const ForestBatch* b, gf_forest_batch_stats* st) { *st = b->R.S; }

size_t gf::forest_device_bytes(const gf_forest* f)
{
    size_t n = 0;
    for (int l = f->o.minlevel; l <= f->o.maxlevel; ++l)
        n += (size_t)f->nf * (nx_at(f, l) + 2 * GF_MBC) * (ny_at(f, l) + 2 * GF_MBC) * sizeof(double);
    n += (size_t)f->cap * (6 + f->o.maux) * f->S * sizeof(double);
    n += f->d_nbr.n * sizeof(int) + f->d_geom.n * sizeof(gf_patch_geom) + f->d_work.n * sizeof(gf_patch_work) +
         (f->d_refs_all.n + f->d_refs_lv.n) * sizeof(gf_ghost_ref) + f->d_block.n * sizeof(gf_ghost_block) +
         f->d_gdt.n * sizeof(double) + f->d_gpar.n * sizeof(int) + f->d_rb.n * 8 +
         f->d_tagt.n * sizeof(gf_tag_task) + f->d_tags.n * sizeof(int) + f->d_refine.n * sizeof(gf_refine) +
         f->d_rgx.n * sizeof(gf_xfer_task) + f->d_fill.n * sizeof(gf_fill_task) +
         f->d_gtask.n * sizeof(gf_gauge_task) + (f->d_glast.n + f->d_grec.n) * sizeof(double);
    for (int b = 0; b < 2; ++b) n += (f->d_avg[b].n + f->d_itp[b].n) * sizeof(gf_xfer_task);
    return n;
}
