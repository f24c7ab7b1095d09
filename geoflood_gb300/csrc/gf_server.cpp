/*
 * Served form: a continuous-batching request loop over flood scenarios.
 *
 * Scenarios are single-level forests (a brick of npx x npy patches of one
 * mx). On admission a scenario gets one stream-ordered device allocation
 * (two state buffers, aux, neighbour table, geometry) and a physics slot;
 * its state then stays on the device until it finishes.
 *
 * Scenarios are sorted into size lanes; each lane has its own stream and a
 * fixed membership (an epoch) between admissions and completions. A round
 * of a lane steps every member once:
 *
 *   prepare (1 thread / scenario: dt, buffer parity, inflow state)
 *   -> ghost fill (one launch per mx present)
 *   -> patch update (one launch per mx present, each scenario its own
 *      dt and CFL group)
 *   -> finish (1 thread / scenario: accept or retake, next dt).
 *
 * The time-step control runs on the device (gf_served.cu), so rounds of a
 * lane are enqueued back to back in chunks sized to about half a
 * millisecond, two chunks in flight; the host reads the controllers back at
 * each chunk end to notice finished scenarios, and changes the membership
 * only when the lane has drained. Lanes overlap on the device, and smaller
 * lanes run on higher-priority streams so that their short rounds are not
 * held behind the large scenarios' launches.
 *
 * A rejected step costs no copy: the update writes into the second state
 * buffer and the controller flips the current buffer only on acceptance
 * (ForestClaw's save/restore, src/fc2d_geoclaw/fc2d_geoclaw_run.c:239-243,
 * :326-340).
 */
#include <cuda_runtime.h>
#include <sys/prctl.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gf_internal.h"

namespace {

constexpr int kMaxSlots = 1024; /* physics slots = active scenarios */
constexpr int kLaneMaux = 3;     /* largest maux a served scenario may have */
constexpr int kMaxRounds = 64;   /* rounds per chunk */
constexpr double kChunkTargetMs = 0.5;

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
inline int mclass(int mx) { return mx == 8 ? 0 : mx == 16 ? 1 : 2; }

using Clock = std::chrono::steady_clock;

struct Scen {
    long long id = 0;
    gf_scenario sc{};
    std::vector<double> hy_t, hy_hu;
    gf_scenario_info info{};
    gf_group_state gst{}; /* host copy of the device controller */
    int lane = -1, slot = -1;
    int queue = -1; /* the round queue: lane x patch size */
    int np = 0;
    long S = 0;          /* cells per patch incl. halo */
    long long cells = 0; /* interior cells */
    size_t bytes = 0;
    char* dev = nullptr;
    double* qbuf[2] = {nullptr, nullptr};
    double* aux = nullptr;
    int* nbr = nullptr;
    gf_patch_geom* geom = nullptr;
    gf_patch_flags* fl = nullptr; /* dry-patch culling flags, zero at admission */
    bool cancel_req = false;
    bool failed = false;
    cudaEvent_t ev_fin = nullptr;
};

struct Chunk {
    int slot = 0;
    int rounds = 0;
};

/* One queue of shared rounds: the scenarios of one size lane and one patch
 * size (all sizes of a lane when its update is the one-launch form). Queues
 * step independently, so a small scenario's round never waits for a larger
 * patch size's update in the same lane. */
struct Lane {
    int idx = 0; /* the size lane: stream priority, tile goal, grid caps */
    cudaStream_t st = nullptr;
    /* two more streams of the lane's priority: a round's patch sizes run as
     * parallel branches of its graph (fork after the controllers' prepare,
     * join before their finish) */
    cudaStream_t side[2] = {nullptr, nullptr};
    cudaEvent_t ev_fork = nullptr, ev_join[2] = {nullptr, nullptr};
    int goal[3] = {0, 0, 0}; /* update tile goal per patch size of the epoch */
    std::vector<Scen*> members; /* group g of the epoch = members[g] */
    std::vector<Scen*> joining; /* admitted, enter at the next epoch */
    std::vector<Scen*> fin;     /* final download in flight */
    std::deque<Chunk> inflight; /* at most two */
    cudaEvent_t ev_start[2] = {nullptr, nullptr}, ev_end[2] = {nullptr, nullptr};
    int next_slot = 0;
    double round_ms = 0.05;
    /* epoch area: pinned mirror and device copy */
    char* h_ep = nullptr;
    char* d_ep = nullptr;
    size_t ep_cap = 0;
    size_t off_blk = 0, off_gs = 0, off_dt = 0, off_par = 0, off_rb = 0, off_hyt = 0, off_hyu = 0;
    size_t off_ref[3] = {0, 0, 0}, off_work[3] = {0, 0, 0}, off_sched = 0;
    int npm[3] = {0, 0, 0};
    /* two readback slots: [err (8 B)][states] */
    char* h_rb[2] = {nullptr, nullptr};
    size_t rb_cap = 0;
    /* one round of the epoch, captured once and replayed per round */
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int launches_per_round = 0;
};

} // namespace

struct gf_server {
    int device = 0;
    gf_server_opts o{};
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv;
    std::string last_error;
    bool broken = false;
    long long next_id = 1;
    std::map<long long, Scen*> all;
    std::deque<Scen*> queue;
    Lane lanes[GF_SERVER_MAX_LANES * 3]; /* queue lane * 3 + size class */
    int nqueues() const { return o.nlanes * 3; }
    gf_phys* d_phys = nullptr;
    std::vector<gf_phys> h_phys;
    std::vector<int> free_slots;
    gf_server_stats stats{};
    int cta_cap[GF_SERVER_MAX_LANES][3] = {}; /* update-kernel grid caps per lane and mx */
    int mix_cap[GF_SERVER_MAX_LANES] = {};    /* the one-launch update's grid cap per lane */
    std::thread loop;
    std::atomic<bool> running{false};

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

int sfail(gf_server* s, int code, const std::string& msg)
{
    s->last_error = msg;
    return code;
}

int scuda(gf_server* s, cudaError_t e, const char* where)
{
    s->last_error = std::string(where) + ": " + cudaGetErrorString(e);
    s->broken = true;
    return GF_ERR_CUDA;
}

#define SV_CK(s, call)                                       \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return scuda((s), e_, #call); \
    } while (0)

size_t footprint_of(const gf_scenario& sc)
{
    const long S = (long)(sc.mx + 2 * GF_MBC) * (sc.mx + 2 * GF_MBC);
    const size_t np = (size_t)sc.npx * sc.npy;
    return 2 * align256(np * 3 * S * sizeof(double)) + align256(np * sc.maux * S * sizeof(double)) +
           align256(np * 8 * sizeof(int)) + align256(np * sizeof(gf_patch_geom)) +
           align256(np * sizeof(gf_patch_flags));
}

const char* validate(const gf_scenario& sc)
{
    if (!(sc.mx == 8 || sc.mx == 16 || sc.mx == 32)) return "mx must be 8, 16 or 32";
    if (sc.npx < 1 || sc.npy < 1) return "npx, npy must be positive";
    if ((long long)sc.npx * sc.npy > (1LL << 24)) return "too many patches";
    if (sc.maux < 1 || sc.maux > kLaneMaux) return "maux must be 1..3";
    if (!(sc.dx > 0) || !(sc.dy > 0)) return "dx, dy must be positive";
    if (!sc.q || !sc.aux) return "q and aux are required";
    if (!(sc.t_final > 0) || sc.nout < 1) return "t_final > 0 and nout >= 1 required";
    if (!(sc.initial_dt > 0) || !(sc.desired_cfl > 0) || !(sc.max_cfl > 0))
        return "initial_dt, desired_cfl, max_cfl must be positive";
    if (sc.phys.variable_friction &&
        (sc.phys.friction_index < 1 || sc.phys.friction_index > sc.maux))
        return "variable friction needs 1 <= friction_index <= maux";
    for (int s = 0; s < 4; ++s) {
        if (sc.mthbc[s] < 0 || sc.mthbc[s] > 3 || sc.mthbc[s] == 2)
            return "mthbc must be 0, 1 or 3 (no periodic sides in a served scenario)";
        if (sc.mthbc[s] == 0 && !(sc.hydro_side[s] && sc.nhydro > 0))
            return "mthbc = 0 needs a hydrograph on that side (the reference stops here)";
    }
    if (sc.nhydro < 0 || (sc.nhydro > 0 && (!sc.hydro_time || !sc.hydro_hu)))
        return "bad hydrograph";
    for (int i = 1; i < sc.nhydro; ++i)
        if (!(sc.hydro_time[i] >= sc.hydro_time[i - 1])) return "hydrograph times must increase";
    return nullptr;
}

int lane_of(const gf_server* s, long long cells)
{
    for (int k = 0; k < s->o.nlanes - 1; ++k)
        if (cells < s->o.lane_cells[k]) return k;
    return s->o.nlanes - 1;
}

int queue_of(const gf_server* s, int lane, int mx)
{
    const bool one_queue = !s->o.split_sizes || (s->o.mixed_update && lane > 0);
    return lane * 3 + (one_queue ? 0 : mclass(mx));
}

void sync_info(Scen* s)
{
    s->info.t = s->gst.t_curr;
    s->info.dt = s->gst.dt_minlevel;
    s->info.steps = s->gst.steps;
    s->info.rejects = s->gst.rejects;
    s->info.cell_updates = s->gst.steps * s->cells;
    s->info.max_cfl_seen = s->gst.max_cfl_seen;
}

void release_device(gf_server* srv, Scen* s, cudaStream_t st)
{
    if (s->dev) {
        cudaFreeAsync(s->dev, st);
        s->dev = nullptr;
        srv->stats.bytes_in_use -= s->bytes;
    }
    if (s->slot >= 0) {
        srv->free_slots.push_back(s->slot);
        s->slot = -1;
    }
    if (s->ev_fin) {
        cudaEventDestroy(s->ev_fin);
        s->ev_fin = nullptr;
    }
}

void end_scenario(gf_server* srv, Scen* s, int state)
{
    s->info.state = state;
    s->info.t_done = srv->now();
    srv->stats.active--;
    if (state == GF_SCEN_DONE) srv->stats.done++;
    srv->cv.notify_all();
}

int admit(gf_server* srv, Scen* s)
{
    Lane& L = srv->lanes[s->queue];
    const gf_scenario& sc = s->sc;
    const int np = s->np;
    const long S = s->S;
    SV_CK(srv, cudaMallocAsync(reinterpret_cast<void**>(&s->dev), s->bytes, L.st));
    char* p = s->dev;
    s->qbuf[0] = reinterpret_cast<double*>(p);
    p += align256((size_t)np * 3 * S * sizeof(double));
    s->qbuf[1] = reinterpret_cast<double*>(p);
    p += align256((size_t)np * 3 * S * sizeof(double));
    s->aux = reinterpret_cast<double*>(p);
    p += align256((size_t)np * sc.maux * S * sizeof(double));
    s->nbr = reinterpret_cast<int*>(p);
    p += align256((size_t)np * 8 * sizeof(int));
    s->geom = reinterpret_cast<gf_patch_geom*>(p);
    p += align256((size_t)np * sizeof(gf_patch_geom));
    s->fl = reinterpret_cast<gf_patch_flags*>(p);
    /* no update has run: no patch is known to be idle */
    SV_CK(srv, cudaMemsetAsync(s->fl, 0, (size_t)np * sizeof(gf_patch_flags), L.st));
    srv->stats.bytes_in_use += s->bytes;
    srv->stats.bytes_peak = std::max(srv->stats.bytes_peak, srv->stats.bytes_in_use);

    /* brick layout with physical sides all round (block-local indices) */
    std::vector<int> nbr((size_t)np * 8);
    std::vector<gf_patch_geom> geom(np);
    for (int py = 0; py < sc.npy; ++py)
        for (int px = 0; px < sc.npx; ++px) {
            const int k = py * sc.npx + px;
            const bool l = px > 0, r = px < sc.npx - 1, b = py > 0, t = py < sc.npy - 1;
            int* n = &nbr[(size_t)8 * k];
            n[0] = l ? k - 1 : -1;
            n[1] = r ? k + 1 : -1;
            n[2] = b ? k - sc.npx : -1;
            n[3] = t ? k + sc.npx : -1;
            n[4] = (l && b) ? k - sc.npx - 1 : -1;
            n[5] = (r && b) ? k - sc.npx + 1 : -1;
            n[6] = (l && t) ? k + sc.npx - 1 : -1;
            n[7] = (r && t) ? k + sc.npx + 1 : -1;
            geom[k] = {sc.xlower + px * sc.mx * sc.dx, sc.ylower + py * sc.mx * sc.dy, sc.dx, sc.dy};
        }
    /* pageable sources are staged before cudaMemcpyAsync returns */
    SV_CK(srv, cudaMemcpyAsync(s->nbr, nbr.data(), nbr.size() * sizeof(int), cudaMemcpyHostToDevice, L.st));
    SV_CK(srv, cudaMemcpyAsync(s->geom, geom.data(), geom.size() * sizeof(gf_patch_geom),
                               cudaMemcpyHostToDevice, L.st));
    s->slot = srv->free_slots.back();
    srv->free_slots.pop_back();
    srv->h_phys[s->slot] = sc.phys;
    SV_CK(srv, cudaMemcpyAsync(srv->d_phys + s->slot, &srv->h_phys[s->slot], sizeof(gf_phys),
                               cudaMemcpyHostToDevice, L.st));
    /* Fortran layout in through the spare buffer, transposed to planes */
    double* spare = s->qbuf[1];
    SV_CK(srv, cudaMemcpyAsync(spare, sc.q, (size_t)np * 3 * S * sizeof(double), cudaMemcpyHostToDevice, L.st));
    SV_CK(srv, gf::launch_aos_to_soa(spare, s->qbuf[0], np, (int)S, 3, 3 * S, 3 * S, L.st));
    SV_CK(srv, cudaMemcpyAsync(spare, sc.aux, (size_t)np * sc.maux * S * sizeof(double),
                               cudaMemcpyHostToDevice, L.st));
    SV_CK(srv, gf::launch_aos_to_soa(spare, s->aux, np, (int)S, sc.maux, sc.maux * S, sc.maux * S, L.st));
    srv->stats.launches += 2;
    /* controller at t = 0 (fc2d_geoclaw_run.c:197-225) */
    gf_group_state& g = s->gst;
    std::memset(&g, 0, sizeof g);
    g.qb[0] = s->qbuf[0];
    g.qb[1] = s->qbuf[1];
    g.dt_outer = sc.t_final / sc.nout;
    g.t_curr = 0.0;
    g.tend = g.dt_outer;
    g.dt_minlevel = sc.initial_dt;
    g.desired_cfl = sc.desired_cfl;
    g.max_cfl = sc.max_cfl;
    g.nout = sc.nout;
    g.level_factor = 1.0; /* one level */
    g.active = 1;
    g.cur = 0;
    g.nhydro = (int)s->hy_t.size();
    s->info.state = GF_SCEN_ACTIVE;
    s->info.t_admit = srv->now();
    s->info.device_bytes = s->bytes;
    sync_info(s);
    L.joining.push_back(s);
    srv->stats.admitted++;
    srv->stats.active++;
    return GF_OK;
}

int admit_queued(gf_server* srv)
{
    for (auto it = srv->queue.begin(); it != srv->queue.end();) {
        Scen* s = *it;
        const bool fits = srv->stats.bytes_in_use + s->bytes <= srv->o.hbm_budget &&
                          srv->stats.active < srv->o.max_active && !srv->free_slots.empty();
        if (!fits) {
            if (!srv->o.backfill) break;
            ++it;
            continue;
        }
        it = srv->queue.erase(it);
        int rc = admit(srv, s);
        if (rc) return rc;
    }
    return GF_OK;
}

template <typename T>
int grow_pinned(gf_server* srv, T** p, size_t& cap, size_t need)
{
    if (need <= cap) return GF_OK;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    cap = 0;
    const size_t c = std::max(need * 2, (size_t)1 << 16);
    SV_CK(srv, cudaMallocHost(reinterpret_cast<void**>(p), c));
    cap = c;
    return GF_OK;
}

int capture_round(gf_server* srv, Lane& L);
void drop_graph(Lane& L);

/* New epoch of a drained lane: drop finished / cancelled / failed members,
 * start their final downloads, take in the joining scenarios, and upload
 * the round tables. */
int rebuild_epoch(gf_server* srv, Lane& L)
{
    std::vector<Scen*> keep;
    for (Scen* s : L.members) {
        if (s->failed) {
            release_device(srv, s, L.st);
            end_scenario(srv, s, GF_SCEN_FAILED);
        } else if (s->cancel_req) {
            release_device(srv, s, L.st);
            end_scenario(srv, s, GF_SCEN_CANCELLED);
        } else if (!s->gst.active) {
            const long S = s->S;
            double* curq = s->qbuf[s->gst.cur];
            double* spare = s->qbuf[s->gst.cur ^ 1];
            if (s->sc.q_out) {
                SV_CK(srv, gf::launch_soa_to_aos(curq, spare, s->np, (int)S, 3, 3 * S, 3 * S, L.st));
                SV_CK(srv, cudaMemcpyAsync(s->sc.q_out, spare, (size_t)s->np * 3 * S * sizeof(double),
                                           cudaMemcpyDeviceToHost, L.st));
                srv->stats.launches++;
            }
            SV_CK(srv, cudaEventCreateWithFlags(&s->ev_fin, cudaEventDisableTiming));
            SV_CK(srv, cudaEventRecord(s->ev_fin, L.st));
            L.fin.push_back(s);
        } else {
            keep.push_back(s);
        }
    }
    for (Scen* s : L.joining) {
        if (s->cancel_req) {
            release_device(srv, s, L.st);
            end_scenario(srv, s, GF_SCEN_CANCELLED);
        } else {
            keep.push_back(s);
        }
    }
    L.joining.clear();
    L.members.swap(keep);
    const int nm = (int)L.members.size();
    if (nm == 0) {
        drop_graph(L);
        return GF_OK;
    }

    int npm[3] = {0, 0, 0};
    size_t nhy = 0;
    for (Scen* s : L.members) {
        npm[mclass(s->sc.mx)] += s->np;
        nhy += s->hy_t.size();
    }
    size_t off = 0;
    L.off_blk = off;
    off = align256(off + nm * sizeof(gf_ghost_block));
    L.off_gs = off;
    off = align256(off + nm * sizeof(gf_group_state));
    L.off_dt = off;
    off = align256(off + nm * sizeof(double));
    L.off_par = off;
    off = align256(off + nm * sizeof(int));
    L.off_rb = off; /* [err][gmax per group] */
    off = align256(off + (nm + 1) * sizeof(unsigned long long));
    L.off_hyt = off;
    off = align256(off + std::max<size_t>(nhy, 1) * sizeof(double));
    L.off_hyu = off;
    off = align256(off + std::max<size_t>(nhy, 1) * sizeof(double));
    for (int c = 0; c < 3; ++c) {
        L.off_ref[c] = off;
        off = align256(off + npm[c] * sizeof(gf_ghost_ref));
        L.npm[c] = npm[c];
    }
    /* work items of all sizes contiguous, mx 32 first (the one-launch update's list) */
    L.off_work[2] = off;
    L.off_work[1] = L.off_work[2] + (size_t)npm[2] * sizeof(gf_patch_work);
    L.off_work[0] = L.off_work[1] + (size_t)npm[1] * sizeof(gf_patch_work);
    off = align256(off + (size_t)(npm[0] + npm[1] + npm[2]) * sizeof(gf_patch_work));
    L.off_sched = off;
    off = align256(off + 2 * sizeof(unsigned int));
    const size_t need = off;
    if (need > L.ep_cap) {
        if (L.d_ep) cudaFreeAsync(L.d_ep, L.st);
        L.d_ep = nullptr;
        size_t cap = L.ep_cap;
        int rc = grow_pinned(srv, &L.h_ep, cap, need);
        if (rc) return rc;
        SV_CK(srv, cudaMallocAsync(reinterpret_cast<void**>(&L.d_ep), cap, L.st));
        L.ep_cap = cap;
    }
    const size_t rb_need = 8 + nm * sizeof(gf_group_state);
    if (rb_need > L.rb_cap) {
        size_t c0 = L.rb_cap, c1 = L.rb_cap;
        int rc = grow_pinned(srv, &L.h_rb[0], c0, rb_need);
        if (!rc) rc = grow_pinned(srv, &L.h_rb[1], c1, rb_need);
        if (rc) return rc;
        L.rb_cap = std::min(c0, c1);
    }
    char* h = L.h_ep;
    std::memset(h + L.off_rb, 0, (nm + 1) * sizeof(unsigned long long));
    std::memset(h + L.off_sched, 0, 2 * sizeof(unsigned int));
    gf_ghost_block* hb = reinterpret_cast<gf_ghost_block*>(h + L.off_blk);
    gf_group_state* hg = reinterpret_cast<gf_group_state*>(h + L.off_gs);
    double* hyt = reinterpret_cast<double*>(h + L.off_hyt);
    double* hyu = reinterpret_cast<double*>(h + L.off_hyu);
    gf_ghost_ref* href[3];
    gf_patch_work* hwork[3];
    int fill[3] = {0, 0, 0};
    for (int c = 0; c < 3; ++c) {
        href[c] = reinterpret_cast<gf_ghost_ref*>(h + L.off_ref[c]);
        hwork[c] = reinterpret_cast<gf_patch_work*>(h + L.off_work[c]);
    }
    size_t hoff = 0;
    for (int g = 0; g < nm; ++g) {
        Scen* s = L.members[g];
        const long S = s->S;
        gf_ghost_block blk{};
        blk.q = s->qbuf[s->gst.cur];
        blk.aux = s->aux;
        blk.nbr = s->nbr;
        blk.geom = s->geom;
        blk.phys_of = nullptr;
        blk.fl = srv->o.cull_dry ? s->fl : nullptr;
        for (int k = 0; k < 4; ++k) {
            blk.bc.mthbc[k] = s->sc.mthbc[k];
            blk.bc.hydro_side[k] = s->sc.nhydro > 0 ? (s->sc.hydro_side[k] != 0) : 0;
        }
        blk.bc.width = s->sc.hydro_width;
        blk.bc.x0 = s->sc.hydro_x0;
        blk.bc.y0 = s->sc.hydro_y0;
        blk.phys = s->slot;
        blk.maux = s->sc.maux;
        blk.skip = 1;
        hb[g] = blk;
        s->gst.hydro_off = (int)hoff;
        s->gst.nhydro = (int)s->hy_t.size();
        std::copy(s->hy_t.begin(), s->hy_t.end(), hyt + hoff);
        std::copy(s->hy_hu.begin(), s->hy_hu.end(), hyu + hoff);
        hoff += s->hy_t.size();
        hg[g] = s->gst;
        const int c = mclass(s->sc.mx);
        for (int p = 0; p < s->np; ++p) {
            href[c][fill[c]] = gf_ghost_ref{g, p};
            gf_patch_work w{};
            w.q = s->qbuf[0] + (size_t)p * 3 * S;
            w.qout = s->qbuf[1] + (size_t)p * 3 * S;
            w.aux = s->aux + (size_t)p * s->sc.maux * S;
            w.dx = s->sc.dx;
            w.dy = s->sc.dy;
            w.phys = s->slot;
            w.group = g;
            w.fl = srv->o.cull_dry ? s->fl + p : nullptr;
            hwork[c][fill[c]] = w;
            ++fill[c];
        }
    }
    SV_CK(srv, cudaMemcpyAsync(L.d_ep, L.h_ep, need, cudaMemcpyHostToDevice, L.st));
    /* the smallest lane's step time is one patch's critical path: the
     * latency tile, while its patches (split over their clusters) all run in
     * one wave; decided here, outside the capture */
    static const int ms[3] = {8, 16, 32};
    for (int c = 0; c < 3; ++c)
        L.goal[c] = (L.idx == 0 && srv->o.nlanes > 1 && npm[c] && gf::latency_goal_fits(ms[c], npm[c])) ? 1 : 0;
    return capture_round(srv, L);
}

/* Enqueue one round of the lane's epoch on its stream (used once per epoch,
 * under stream capture). */
int enqueue_round(gf_server* srv, Lane& L)
{
    static const int ms[3] = {8, 16, 32};
    const int nm = (int)L.members.size();
    char* d = L.d_ep;
    gf_ghost_block* blk = reinterpret_cast<gf_ghost_block*>(d + L.off_blk);
    gf_group_state* gs = reinterpret_cast<gf_group_state*>(d + L.off_gs);
    double* gdt = reinterpret_cast<double*>(d + L.off_dt);
    int* gpar = reinterpret_cast<int*>(d + L.off_par);
    unsigned long long* rb = reinterpret_cast<unsigned long long*>(d + L.off_rb);
    int* err = reinterpret_cast<int*>(rb);
    const double* hyt = reinterpret_cast<const double*>(d + L.off_hyt);
    const double* hyu = reinterpret_cast<const double*>(d + L.off_hyu);
    int n = 0;
    SV_CK(srv, gf::launch_served_prepare(gs, blk, gdt, gpar, rb + 1, hyt, hyu, nm, L.st));
    ++n;
    if (srv->o.mixed_update && L.idx > 0) {
        for (int c = 0; c < 3; ++c)
            if (L.npm[c]) {
                SV_CK(srv, gf::launch_ghost_fill(ms[c], blk, reinterpret_cast<const gf_ghost_ref*>(d + L.off_ref[c]),
                                                 L.npm[c], srv->d_phys, L.st));
                ++n;
            }
        /* later lanes: every size in one persistent launch (a device cursor
         * over the contiguous work list), on the lane's capped grid */
        const int nw[3] = {L.npm[2], L.npm[1], L.npm[0]};
        if (nw[0] + nw[1] + nw[2]) {
            SV_CK(srv, gf::launch_patch_update_mixed(reinterpret_cast<const gf_patch_work*>(d + L.off_work[2]), nw,
                                                     srv->d_phys, 0.0, gdt, gpar, kLaneMaux, nullptr, rb + 1, err,
                                                     reinterpret_cast<unsigned int*>(d + L.off_sched), L.st,
                                                     srv->mix_cap[L.idx]));
            ++n;
        }
    } else {
        /* Each patch size's ghost fill and update form one branch; the sizes
         * touch disjoint patches and meet only in the atomic maxima, so the
         * branches run concurrently with the same results. */
        int nb = 0;
        cudaStream_t bst[3];
        for (int c = 2; c >= 0; --c)
            if (L.npm[c]) {
                bst[nb] = nb == 0 ? L.st : L.side[nb - 1];
                ++nb;
            }
        if (nb > 1) {
            SV_CK(srv, cudaEventRecord(L.ev_fork, L.st));
            for (int b = 1; b < nb; ++b) SV_CK(srv, cudaStreamWaitEvent(bst[b], L.ev_fork, 0));
        }
        int b = 0;
        for (int c = 2; c >= 0; --c)
            if (L.npm[c]) {
                cudaStream_t st = bst[b++];
                SV_CK(srv, gf::launch_ghost_fill(ms[c], blk, reinterpret_cast<const gf_ghost_ref*>(d + L.off_ref[c]),
                                                 L.npm[c], srv->d_phys, st));
                SV_CK(srv, gf::launch_patch_update(ms[c], reinterpret_cast<const gf_patch_work*>(d + L.off_work[c]),
                                                   L.npm[c], srv->d_phys, 0.0, gdt, gpar, kLaneMaux, nullptr,
                                                   rb + 1, err, st, srv->cta_cap[L.idx][c], L.goal[c]));
                n += 2;
            }
        for (int j = 1; j < nb; ++j) {
            SV_CK(srv, cudaEventRecord(L.ev_join[j - 1], bst[j]));
            SV_CK(srv, cudaStreamWaitEvent(L.st, L.ev_join[j - 1], 0));
        }
    }
    SV_CK(srv, gf::launch_served_finish(gs, gdt, rb + 1, err, nm, L.st));
    ++n;
    L.launches_per_round = n;
    return GF_OK;
}

void drop_graph(Lane& L)
{
    if (L.exec) cudaGraphExecDestroy(L.exec);
    if (L.graph) cudaGraphDestroy(L.graph);
    L.exec = nullptr;
    L.graph = nullptr;
}

/* Capture the epoch's round as a graph (one graph launch per round). */
int capture_round(gf_server* srv, Lane& L)
{
    drop_graph(L);
    SV_CK(srv, cudaStreamBeginCapture(L.st, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_round(srv, L);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(L.st, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    SV_CK(srv, e);
    L.graph = g;
    SV_CK(srv, cudaGraphInstantiate(&L.exec, L.graph, 0));
    return GF_OK;
}

/* Enqueue a chunk of rounds (epoch unchanged) and the controllers' readback. */
int launch_chunk(gf_server* srv, Lane& L)
{
    const int nm = (int)L.members.size();
    char* d = L.d_ep;
    const gf_group_state* gs = reinterpret_cast<const gf_group_state*>(d + L.off_gs);
    const unsigned long long* rb = reinterpret_cast<const unsigned long long*>(d + L.off_rb);
    int rounds = (int)std::ceil(kChunkTargetMs / std::max(L.round_ms, 1e-3));
    rounds = std::max(1, std::min(kMaxRounds, rounds));
    const int slot = L.next_slot;
    L.next_slot ^= 1;
    SV_CK(srv, cudaEventRecord(L.ev_start[slot], L.st));
    for (int r = 0; r < rounds; ++r) SV_CK(srv, cudaGraphLaunch(L.exec, L.st));
    srv->stats.launches += (long long)rounds * L.launches_per_round;
    SV_CK(srv, cudaMemcpyAsync(L.h_rb[slot], rb, 8, cudaMemcpyDeviceToHost, L.st));
    SV_CK(srv, cudaMemcpyAsync(L.h_rb[slot] + 8, gs, nm * sizeof(gf_group_state),
                               cudaMemcpyDeviceToHost, L.st));
    SV_CK(srv, cudaEventRecord(L.ev_end[slot], L.st));
    L.inflight.push_back(Chunk{slot, rounds});
    srv->stats.rounds += rounds;
    return GF_OK;
}

/* A chunk has completed: copy the controllers back to the scenarios. */
void finish_chunk(gf_server* srv, Lane& L, const Chunk& ch)
{
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, L.ev_start[ch.slot], L.ev_end[ch.slot]) == cudaSuccess && ch.rounds > 0)
        L.round_ms = std::max(1e-3, (double)ms / ch.rounds);
    const char* rb = L.h_rb[ch.slot];
    int err;
    std::memcpy(&err, rb, sizeof err);
    const gf_group_state* st = reinterpret_cast<const gf_group_state*>(rb + 8);
    for (size_t g = 0; g < L.members.size(); ++g) {
        Scen* s = L.members[g];
        const long long before = s->gst.steps;
        s->gst = st[g];
        srv->stats.cell_updates += (s->gst.steps - before) * s->cells;
        sync_info(s);
        if (err) s->failed = true;
    }
    if (err) srv->last_error = "a patch-update copy wait timed out; the lane's scenarios failed";
}

bool lane_needs_epoch(const Lane& L)
{
    if (!L.joining.empty()) return true;
    for (const Scen* s : L.members)
        if (!s->gst.active || s->cancel_req || s->failed) return true;
    return false;
}

int pump_locked(gf_server* srv, int* busy)
{
    if (srv->broken) return GF_ERR_STATE;
    SV_CK(srv, cudaSetDevice(srv->device));
    for (int k = 0; k < srv->nqueues(); ++k) {
        Lane& L = srv->lanes[k];
        for (size_t i = 0; i < L.fin.size();) {
            Scen* s = L.fin[i];
            cudaError_t e = cudaEventQuery(s->ev_fin);
            if (e == cudaErrorNotReady) { ++i; continue; }
            if (e != cudaSuccess) return scuda(srv, e, "final download");
            release_device(srv, s, L.st);
            end_scenario(srv, s, GF_SCEN_DONE);
            L.fin.erase(L.fin.begin() + i);
        }
        while (!L.inflight.empty()) {
            const Chunk ch = L.inflight.front();
            cudaError_t e = cudaEventQuery(L.ev_end[ch.slot]);
            if (e == cudaErrorNotReady) break;
            if (e != cudaSuccess) return scuda(srv, e, "round chunk");
            finish_chunk(srv, L, ch);
            L.inflight.pop_front();
        }
    }
    int rc = admit_queued(srv);
    if (rc) return rc;
    for (int k = 0; k < srv->nqueues(); ++k) {
        Lane& L = srv->lanes[k];
        if (lane_needs_epoch(L)) {
            if (!L.inflight.empty()) continue; /* drain first */
            rc = rebuild_epoch(srv, L);
            if (rc) return rc;
        }
        if (L.members.empty()) continue;
        while (L.inflight.size() < 2) {
            rc = launch_chunk(srv, L);
            if (rc) return rc;
        }
    }
    int b = !srv->queue.empty();
    for (int k = 0; k < srv->nqueues(); ++k) {
        const Lane& L = srv->lanes[k];
        b |= !L.inflight.empty() || !L.members.empty() || !L.joining.empty() || !L.fin.empty();
    }
    if (busy) *busy = b;
    return GF_OK;
}

void loop_main(gf_server* srv)
{
    /* short sleeps between passes: ask for fine timer slack on this thread */
    prctl(PR_SET_TIMERSLACK, 1000UL, 0, 0, 0);
    while (srv->running.load()) {
        int busy = 0;
        int rc;
        {
            std::lock_guard<std::mutex> g(srv->mu);
            rc = pump_locked(srv, &busy);
            if (rc == GF_ERR_CUDA || rc == GF_ERR_STATE) {
                srv->cv.notify_all();
                break;
            }
        }
        /* outside the lock, so that submitters and pollers get their turn */
        std::this_thread::sleep_for(std::chrono::microseconds(busy ? 10 : 200));
    }
}

} // namespace

extern "C" {

void gf_server_opts_default(gf_server_opts* o)
{
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->hbm_budget = (size_t)64 << 30;
    o->max_active = 256;
    o->nlanes = 3;
    o->lane_cells[0] = 100000;
    o->lane_cells[1] = 1000000;
    o->lane_cells[2] = 0;
    o->priority = 1;
    o->backfill = 1;
    o->reserve_sms = 0; /* one CTA per patch: priority hands freed SMs to smaller lanes */
    o->mixed_update = 0; /* per-size launches: measured faster for served scenarios */
    o->cull_dry = 1;
    o->split_sizes = 1;
}

int gf_server_create(int device, const gf_server_opts* opts, gf_server** out)
{
    if (!out) return GF_ERR_ARG;
    *out = nullptr;
    gf_server_opts o;
    if (opts) o = *opts;
    else gf_server_opts_default(&o);
    if (o.nlanes < 1 || o.nlanes > GF_SERVER_MAX_LANES || o.max_active < 1 || o.max_active > kMaxSlots)
        return GF_ERR_ARG;
    for (int k = 0; k + 1 < o.nlanes; ++k)
        if (o.lane_cells[k] <= 0 || (k > 0 && o.lane_cells[k] <= o.lane_cells[k - 1])) return GF_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return GF_ERR_CUDA;
    if (cudaSetDevice(device) != cudaSuccess) return GF_ERR_CUDA;
    gf_server* s = new gf_server;
    s->device = device;
    s->o = o;
    s->t0 = Clock::now();
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi); /* hi is the numerically lowest (greatest) */
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < s->nqueues() && e == cudaSuccess; ++k) {
        Lane& L = s->lanes[k];
        L.idx = k / 3;
        int prio = lo;
        if (o.priority && o.nlanes > 1) prio = hi + (lo - hi) * L.idx / (o.nlanes - 1);
        e = cudaStreamCreateWithPriority(&L.st, cudaStreamNonBlocking, prio);
        for (int j = 0; j < 2 && e == cudaSuccess; ++j) {
            e = cudaEventCreate(&L.ev_start[j]);
            if (e == cudaSuccess) e = cudaEventCreate(&L.ev_end[j]);
            if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&L.side[j], cudaStreamNonBlocking, prio);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L.ev_join[j], cudaEventDisableTiming);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L.ev_fork, cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaMalloc(&s->d_phys, kMaxSlots * sizeof(gf_phys));
    if (e == cudaSuccess) {
        /* keep freed scenario memory in the pool for the next admission */
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            unsigned long long thr = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    }
    if (e != cudaSuccess) {
        gf_server_destroy(s);
        return GF_ERR_CUDA;
    }
    /* with reserve_sms > 0 later lanes run persistent update grids that
     * leave that many SMs to the first lane; with 0 (the default) every lane
     * launches one CTA per patch, each resident for about a tenth of a
     * millisecond, and the higher priority of the smaller lanes' streams
     * gives them the SMs those CTAs free */
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    static const int ms[3] = {8, 16, 32};
    for (int c = 0; c < 3; ++c) /* sets the kernels' shared-memory attribute outside capture */
        gf::launch_patch_update(ms[c], nullptr, 0, nullptr, 0.0, nullptr, nullptr, 0, nullptr,
                                nullptr, nullptr, nullptr);
    const int none[3] = {0, 0, 0};
    gf::launch_patch_update_mixed(nullptr, none, nullptr, 0.0, nullptr, nullptr, 0, nullptr, nullptr, nullptr,
                                  nullptr, nullptr);
    for (int k = 1; k < o.nlanes; ++k) {
        const int sms = nsm - o.reserve_sms;
        for (int c = 0; c < 3; ++c) {
            const int occ = gf::patch_update_occupancy(ms[c]);
            s->cta_cap[k][c] = (o.reserve_sms > 0 && sms > 0 && occ > 0) ? sms * occ : 0;
        }
        s->mix_cap[k] = (o.reserve_sms > 0 && sms > 0) ? sms : 0; /* one CTA per SM */
    }
    s->h_phys.resize(kMaxSlots);
    for (int k = kMaxSlots - 1; k >= 0; --k) s->free_slots.push_back(k);
    *out = s;
    return GF_OK;
}

void gf_server_destroy(gf_server* s)
{
    if (!s) return;
    gf_server_stop(s);
    cudaSetDevice(s->device);
    for (int k = 0; k < GF_SERVER_MAX_LANES * 3; ++k) {
        Lane& L = s->lanes[k];
        if (L.st) cudaStreamSynchronize(L.st);
    }
    for (auto& kv : s->all) {
        Scen* sc = kv.second;
        if (sc->dev) cudaFree(sc->dev);
        if (sc->ev_fin) cudaEventDestroy(sc->ev_fin);
        delete sc;
    }
    for (int k = 0; k < GF_SERVER_MAX_LANES * 3; ++k) {
        Lane& L = s->lanes[k];
        if (L.d_ep) cudaFree(L.d_ep);
        if (L.h_ep) cudaFreeHost(L.h_ep);
        for (int j = 0; j < 2; ++j) {
            if (L.h_rb[j]) cudaFreeHost(L.h_rb[j]);
            if (L.ev_start[j]) cudaEventDestroy(L.ev_start[j]);
            if (L.ev_end[j]) cudaEventDestroy(L.ev_end[j]);
            if (L.ev_join[j]) cudaEventDestroy(L.ev_join[j]);
            if (L.side[j]) cudaStreamDestroy(L.side[j]);
        }
        if (L.ev_fork) cudaEventDestroy(L.ev_fork);
        drop_graph(L);
        if (L.st) cudaStreamDestroy(L.st);
    }
    if (s->d_phys) cudaFree(s->d_phys);
    delete s;
}

const char* gf_server_last_error(const gf_server* s) { return s ? s->last_error.c_str() : "null server"; }

size_t gf_scenario_footprint(const gf_scenario* sc)
{
    if (!sc || validate(*sc)) return 0;
    return footprint_of(*sc);
}

int gf_server_submit(gf_server* s, const gf_scenario* sc, long long* id)
{
    if (!s || !sc) return GF_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    if (const char* why = validate(*sc)) return sfail(s, GF_ERR_ARG, why);
    const size_t bytes = footprint_of(*sc);
    if (bytes > s->o.hbm_budget) return sfail(s, GF_ERR_NOMEM, "scenario exceeds the server's HBM budget");
    Scen* x = new Scen;
    x->id = s->next_id++;
    x->sc = *sc;
    x->hy_t.assign(sc->hydro_time, sc->hydro_time + sc->nhydro);
    x->hy_hu.assign(sc->hydro_hu, sc->hydro_hu + sc->nhydro);
    x->sc.hydro_time = nullptr;
    x->sc.hydro_hu = nullptr;
    x->np = sc->npx * sc->npy;
    x->S = (long)(sc->mx + 2 * GF_MBC) * (sc->mx + 2 * GF_MBC);
    x->cells = (long long)x->np * sc->mx * sc->mx;
    x->bytes = bytes;
    x->lane = lane_of(s, x->cells);
    x->queue = queue_of(s, x->lane, sc->mx);
    x->info.state = GF_SCEN_QUEUED;
    x->info.lane = x->lane;
    x->info.t_submit = s->now();
    x->info.t_admit = -1;
    x->info.t_done = -1;
    x->info.dt = sc->initial_dt;
    s->all[x->id] = x;
    s->queue.push_back(x);
    s->stats.submitted++;
    if (id) *id = x->id;
    return GF_OK;
}

int gf_server_pump(gf_server* s, int* busy)
{
    if (!s) return GF_ERR_ARG;
    if (s->running.load()) return sfail(s, GF_ERR_STATE, "the request loop thread is running");
    std::lock_guard<std::mutex> g(s->mu);
    return pump_locked(s, busy);
}

int gf_server_start(gf_server* s)
{
    if (!s) return GF_ERR_ARG;
    if (s->running.exchange(true)) return GF_OK;
    s->loop = std::thread(loop_main, s);
    return GF_OK;
}

int gf_server_stop(gf_server* s)
{
    if (!s) return GF_ERR_ARG;
    if (!s->running.exchange(false)) return GF_OK;
    if (s->loop.joinable()) s->loop.join();
    return GF_OK;
}

int gf_server_wait(gf_server* s, long long id, double timeout_s)
{
    if (!s) return GF_ERR_ARG;
    const double t_end = s->now() + timeout_s;
    std::unique_lock<std::mutex> g(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return sfail(s, GF_ERR_ARG, "unknown scenario id");
    Scen* x = it->second;
    while (x->info.state == GF_SCEN_QUEUED || x->info.state == GF_SCEN_ACTIVE) {
        if (s->broken) return GF_ERR_STATE;
        if (s->now() > t_end) return sfail(s, GF_ERR_STATE, "wait timed out");
        if (s->running.load()) {
            s->cv.wait_for(g, std::chrono::milliseconds(2));
        } else {
            int busy = 0;
            int rc = pump_locked(s, &busy);
            if (rc) return rc;
            if (busy) {
                g.unlock();
                std::this_thread::sleep_for(std::chrono::microseconds(20));
                g.lock();
            }
        }
    }
    return GF_OK;
}

int gf_server_poll(gf_server* s, long long id, gf_scenario_info* info)
{
    if (!s || !info) return GF_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return sfail(s, GF_ERR_ARG, "unknown scenario id");
    *info = it->second->info;
    return GF_OK;
}

int gf_server_cancel(gf_server* s, long long id)
{
    if (!s) return GF_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return sfail(s, GF_ERR_ARG, "unknown scenario id");
    Scen* x = it->second;
    if (x->info.state == GF_SCEN_QUEUED) {
        s->queue.erase(std::find(s->queue.begin(), s->queue.end(), x));
        x->info.state = GF_SCEN_CANCELLED;
        x->info.t_done = s->now();
        s->cv.notify_all();
    } else if (x->info.state == GF_SCEN_ACTIVE) {
        x->cancel_req = true; /* taken out at the lane's next epoch */
    }
    return GF_OK;
}

int gf_server_stats_get(gf_server* s, gf_server_stats* st)
{
    if (!s || !st) return GF_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    *st = s->stats;
    st->queued = (int)s->queue.size();
    return GF_OK;
}

double gf_server_clock(const gf_server* s) { return s ? s->now() : -1.0; }

} // extern "C"
