/*
 * Served form: a continuous-batching request loop over flood scenarios.
 *
 * Scenarios are single-level forests (a brick of npx x npy patches of one
 * mx). On admission a scenario gets one stream-ordered device allocation
 * (two state buffers, aux, neighbour table, geometry) and a physics slot;
 * its state then stays on the device until it finishes. Scenarios are
 * sorted into size lanes; each lane has its own stream and runs rounds: a
 * round steps every active scenario of the lane once, with one ghost-fill
 * launch and one patch-update launch per mx present, each scenario in its
 * own dt / CFL group. The host reads the group maxima back at the end of a
 * round and runs each scenario's time-step controller. Lanes overlap on the
 * device, and small lanes can run on higher-priority streams so that their
 * short rounds are not held behind the large scenarios' launches.
 *
 * Time stepping follows ForestClaw's outstyle 1 loop
 * (src/fc2d_geoclaw/fc2d_geoclaw_run.c:190-395) with variable dt and
 * reduce_cfl on: save / restore around a rejected step (:239-243, :326-340)
 * becomes a flip between the two state buffers.
 */
#include <cuda_runtime.h>

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

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

using Clock = std::chrono::steady_clock;

struct Scen {
    long long id = 0;
    gf_scenario sc{};
    std::vector<double> hy_t, hy_hu;
    gf_scenario_info info{};
    int lane = -1, slot = -1;
    int np = 0;
    long S = 0;         /* cells per patch incl. halo */
    long long cells = 0; /* interior cells */
    size_t bytes = 0;
    /* device */
    char* dev = nullptr;
    double* qbuf[2] = {nullptr, nullptr};
    double* aux = nullptr;
    int* nbr = nullptr;
    gf_patch_geom* geom = nullptr;
    int cur = 0;
    /* outstyle-1 controller */
    double dt_outer = 0, t_curr = 0, tend = 0, dt_minlevel = 0;
    double dt_step = 0;
    int nint = 0;           /* output interval in progress */
    bool took_small = false;
    bool cancel_req = false;
    bool finishing = false;
    cudaEvent_t ev_fin = nullptr;
};

struct Lane {
    int idx = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    bool in_flight = false;
    std::vector<Scen*> act;     /* admitted, not finishing */
    std::vector<Scen*> members; /* stepped by the round in flight */
    std::vector<Scen*> fin;     /* final download in flight */
    /* one pinned upload area and its device twin, one readback area */
    char* h_up = nullptr;
    char* d_up = nullptr;
    size_t up_cap = 0;
    unsigned long long* h_rb = nullptr; /* [0] err, [1..] group maxima */
    unsigned long long* d_rb = nullptr;
    size_t rb_cap = 0;
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
    Lane lanes[GF_SERVER_MAX_LANES];
    gf_phys* d_phys = nullptr;
    std::vector<gf_phys> h_phys;
    std::vector<int> free_slots;
    gf_server_stats stats{};
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

#define SV_CK(s, call)                                        \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return scuda((s), e_, #call);  \
    } while (0)

size_t footprint_of(const gf_scenario& sc)
{
    const long S = (long)(sc.mx + 2 * GF_MBC) * (sc.mx + 2 * GF_MBC);
    const size_t np = (size_t)sc.npx * sc.npy;
    return 2 * align256(np * 3 * S * sizeof(double)) + align256(np * sc.maux * S * sizeof(double)) +
           align256(np * 8 * sizeof(int)) + align256(np * sizeof(gf_patch_geom));
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

/* hydrograph/hydrograh_module.f90:176-221, discharge type */
double hydro_at(const Scen& s, double t)
{
    const size_t n = s.hy_t.size();
    if (n == 0) return 0.0;
    if (t < s.hy_t[0]) return s.hy_hu[0];
    if (t > s.hy_t[n - 1]) return s.hy_hu[n - 1];
    for (size_t i = 0; i + 1 < n; ++i)
        if (t >= s.hy_t[i] && t <= s.hy_t[i + 1])
            return s.hy_hu[i] +
                   (s.hy_hu[i + 1] - s.hy_hu[i]) / (s.hy_t[i + 1] - s.hy_t[i]) * (t - s.hy_t[i]);
    return 0.0;
}

int lane_of(const gf_server* s, long long cells)
{
    for (int k = 0; k < s->o.nlanes - 1; ++k)
        if (cells < s->o.lane_cells[k]) return k;
    return s->o.nlanes - 1;
}

/* Advance the controller to the next step; false when the run is over
 * (the outer loop over output intervals, fc2d_geoclaw_run.c:229-236). */
bool prepare_step(Scen* s)
{
    while (!(s->t_curr < s->tend)) {
        if (++s->nint >= s->sc.nout) return false;
        s->tend = s->t_curr + s->dt_outer;
    }
    /* fc2d_geoclaw_run.c:251-278: hit tend without a tiny trailing step */
    double dt_step = s->dt_minlevel;
    const double tol = 1e-2 * dt_step;
    s->took_small = false;
    const double small_step = s->tend - (s->t_curr + dt_step);
    if (small_step < tol) {
        dt_step = s->tend - s->t_curr;
        if (small_step < 0) s->took_small = true;
    }
    s->dt_step = dt_step;
    return true;
}

/* fc2d_geoclaw_run.c:326-376: reject and retake, or accept and set dt. */
void finish_step(Scen* s, double cfl)
{
    s->info.max_cfl_seen = std::max(s->info.max_cfl_seen, cfl);
    if (cfl > s->sc.max_cfl) {
        s->dt_minlevel = s->dt_minlevel * s->sc.desired_cfl / cfl;
        s->info.rejects++;
    } else {
        s->info.steps++;
        s->info.cell_updates += s->cells;
        s->t_curr += s->dt_step;
        s->cur ^= 1;
        const double dt_new = s->dt_minlevel * s->sc.desired_cfl / cfl;
        if (!s->took_small) s->dt_minlevel = dt_new;
    }
    s->info.t = s->t_curr;
    s->info.dt = s->dt_minlevel;
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
    Lane& L = srv->lanes[s->lane];
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
    s->cur = 0;
    /* controller state (fc2d_geoclaw_run.c:197-225) */
    s->dt_outer = sc.t_final / sc.nout;
    s->t_curr = 0.0;
    s->nint = 0;
    s->tend = s->dt_outer;
    s->dt_minlevel = sc.initial_dt;
    s->info.state = GF_SCEN_ACTIVE;
    s->info.t_admit = srv->now();
    s->info.dt = s->dt_minlevel;
    s->info.device_bytes = s->bytes;
    L.act.push_back(s);
    srv->stats.admitted++;
    srv->stats.active++;
    srv->stats.queued--;
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

/* Launch the next round of a lane (lane idle on entry). */
int launch_round(gf_server* srv, Lane& L)
{
    L.members.clear();
    for (size_t k = 0; k < L.act.size();) {
        Scen* s = L.act[k];
        if (s->cancel_req) {
            release_device(srv, s, L.st);
            end_scenario(srv, s, GF_SCEN_CANCELLED);
            L.act.erase(L.act.begin() + k);
            continue;
        }
        if (!prepare_step(s)) {
            /* run over: final state out through the spare buffer */
            const long S = s->S;
            double* curq = s->qbuf[s->cur];
            double* spare = s->qbuf[s->cur ^ 1];
            if (s->sc.q_out) {
                SV_CK(srv, gf::launch_soa_to_aos(curq, spare, s->np, (int)S, 3, 3 * S, 3 * S, L.st));
                SV_CK(srv, cudaMemcpyAsync(s->sc.q_out, spare, (size_t)s->np * 3 * S * sizeof(double),
                                           cudaMemcpyDeviceToHost, L.st));
                srv->stats.launches++;
            }
            SV_CK(srv, cudaEventCreateWithFlags(&s->ev_fin, cudaEventDisableTiming));
            SV_CK(srv, cudaEventRecord(s->ev_fin, L.st));
            s->finishing = true;
            L.fin.push_back(s);
            L.act.erase(L.act.begin() + k);
            continue;
        }
        L.members.push_back(s);
        ++k;
    }
    const int nm = (int)L.members.size();
    if (nm == 0) return GF_OK;

    /* upload area: [blocks][group dt][refs m=8][work m=8][refs 16][work 16][refs 32][work 32] */
    static const int ms[3] = {8, 16, 32};
    int npm[3] = {0, 0, 0};
    for (Scen* s : L.members) npm[s->sc.mx == 8 ? 0 : s->sc.mx == 16 ? 1 : 2] += s->np;
    size_t off_blk = 0;
    size_t off_dt = align256(off_blk + nm * sizeof(gf_ghost_block));
    size_t off = align256(off_dt + nm * sizeof(double));
    size_t off_ref[3], off_work[3];
    for (int c = 0; c < 3; ++c) {
        off_ref[c] = off;
        off = align256(off + npm[c] * sizeof(gf_ghost_ref));
        off_work[c] = off;
        off = align256(off + npm[c] * sizeof(gf_patch_work));
    }
    const size_t need = off;
    if (need > L.up_cap) {
        if (L.h_up) cudaFreeHost(L.h_up);
        if (L.d_up) cudaFreeAsync(L.d_up, L.st);
        L.h_up = nullptr;
        L.d_up = nullptr;
        L.up_cap = 0;
        const size_t cap = std::max(need * 2, (size_t)1 << 20);
        SV_CK(srv, cudaMallocHost(reinterpret_cast<void**>(&L.h_up), cap));
        SV_CK(srv, cudaMallocAsync(reinterpret_cast<void**>(&L.d_up), cap, L.st));
        L.up_cap = cap;
    }
    if ((size_t)nm + 1 > L.rb_cap) {
        if (L.h_rb) cudaFreeHost(L.h_rb);
        if (L.d_rb) cudaFreeAsync(L.d_rb, L.st);
        L.h_rb = nullptr;
        L.d_rb = nullptr;
        L.rb_cap = 0;
        const size_t cap = std::max<size_t>(2 * (nm + 1), 64);
        SV_CK(srv, cudaMallocHost(reinterpret_cast<void**>(&L.h_rb), cap * sizeof(unsigned long long)));
        SV_CK(srv, cudaMallocAsync(reinterpret_cast<void**>(&L.d_rb), cap * sizeof(unsigned long long), L.st));
        L.rb_cap = cap;
    }
    gf_ghost_block* hb = reinterpret_cast<gf_ghost_block*>(L.h_up + off_blk);
    double* hdt = reinterpret_cast<double*>(L.h_up + off_dt);
    gf_ghost_ref* href[3];
    gf_patch_work* hwork[3];
    int fill[3] = {0, 0, 0};
    for (int c = 0; c < 3; ++c) {
        href[c] = reinterpret_cast<gf_ghost_ref*>(L.h_up + off_ref[c]);
        hwork[c] = reinterpret_cast<gf_patch_work*>(L.h_up + off_work[c]);
    }
    for (int g = 0; g < nm; ++g) {
        Scen* s = L.members[g];
        const long S = s->S;
        double* qc = s->qbuf[s->cur];
        double* qn = s->qbuf[s->cur ^ 1];
        gf_ghost_block blk{};
        blk.q = qc;
        blk.aux = s->aux;
        blk.nbr = s->nbr;
        blk.geom = s->geom;
        blk.phys_of = nullptr;
        for (int k = 0; k < 4; ++k) {
            blk.bc.mthbc[k] = s->sc.mthbc[k];
            blk.bc.hydro_side[k] = s->sc.nhydro > 0 ? (s->sc.hydro_side[k] != 0) : 0;
        }
        blk.bc.width = s->sc.hydro_width;
        blk.bc.x0 = s->sc.hydro_x0;
        blk.bc.y0 = s->sc.hydro_y0;
        blk.bc.q0hu = hydro_at(*s, s->t_curr);
        blk.phys = s->slot;
        blk.maux = s->sc.maux;
        hb[g] = blk;
        hdt[g] = s->dt_step;
        const int c = s->sc.mx == 8 ? 0 : s->sc.mx == 16 ? 1 : 2;
        for (int p = 0; p < s->np; ++p) {
            href[c][fill[c]] = gf_ghost_ref{g, p};
            gf_patch_work w{};
            w.q = qc + (size_t)p * 3 * S;
            w.qout = qn + (size_t)p * 3 * S;
            w.aux = s->aux + (size_t)p * s->sc.maux * S;
            w.dx = s->sc.dx;
            w.dy = s->sc.dy;
            w.phys = s->slot;
            w.group = g;
            hwork[c][fill[c]] = w;
            ++fill[c];
        }
    }
    SV_CK(srv, cudaMemcpyAsync(L.d_up, L.h_up, need, cudaMemcpyHostToDevice, L.st));
    SV_CK(srv, cudaMemsetAsync(L.d_rb, 0, (nm + 1) * sizeof(unsigned long long), L.st));
    const gf_ghost_block* db = reinterpret_cast<const gf_ghost_block*>(L.d_up + off_blk);
    const double* ddt = reinterpret_cast<const double*>(L.d_up + off_dt);
    for (int c = 0; c < 3; ++c) {
        if (!npm[c]) continue;
        SV_CK(srv, gf::launch_ghost_fill(ms[c], db, reinterpret_cast<const gf_ghost_ref*>(L.d_up + off_ref[c]),
                                         npm[c], srv->d_phys, L.st));
        srv->stats.launches++;
    }
    for (int c = 0; c < 3; ++c) {
        if (!npm[c]) continue;
        SV_CK(srv, gf::launch_patch_update(ms[c], reinterpret_cast<const gf_patch_work*>(L.d_up + off_work[c]),
                                           npm[c], srv->d_phys, 0.0, ddt, kLaneMaux, nullptr, L.d_rb + 1,
                                           reinterpret_cast<int*>(L.d_rb), L.st));
        srv->stats.launches++;
    }
    SV_CK(srv, cudaMemcpyAsync(L.h_rb, L.d_rb, (nm + 1) * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, L.st));
    SV_CK(srv, cudaEventRecord(L.ev, L.st));
    L.in_flight = true;
    srv->stats.rounds++;
    return GF_OK;
}

/* A lane's round has completed: run the controllers. */
int finish_round(gf_server* srv, Lane& L)
{
    L.in_flight = false;
    const int err = (int)L.h_rb[0];
    for (size_t g = 0; g < L.members.size(); ++g) {
        Scen* s = L.members[g];
        if (err) {
            continue;
        }
        double cfl;
        std::memcpy(&cfl, &L.h_rb[1 + g], sizeof cfl);
        const long long before = s->info.cell_updates;
        finish_step(s, cfl);
        srv->stats.cell_updates += s->info.cell_updates - before;
    }
    if (err) {
        /* a bounded wait in the kernel expired: the round is void */
        for (Scen* s : L.members) {
            auto it = std::find(L.act.begin(), L.act.end(), s);
            if (it != L.act.end()) L.act.erase(it);
            release_device(srv, s, L.st);
            end_scenario(srv, s, GF_SCEN_FAILED);
        }
        L.members.clear();
        return sfail(srv, GF_ERR_DEVICE, "a patch-update copy wait timed out; scenarios failed");
    }
    L.members.clear();
    return GF_OK;
}

int pump_locked(gf_server* srv, int* busy)
{
    if (srv->broken) return GF_ERR_STATE;
    SV_CK(srv, cudaSetDevice(srv->device));
    int rc = GF_OK;
    for (int k = 0; k < srv->o.nlanes; ++k) {
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
        if (L.in_flight) {
            cudaError_t e = cudaEventQuery(L.ev);
            if (e == cudaErrorNotReady) continue;
            if (e != cudaSuccess) return scuda(srv, e, "round");
            int r = finish_round(srv, L);
            if (r && !rc) rc = r;
        }
    }
    int r = admit_queued(srv);
    if (r) return r;
    for (int k = 0; k < srv->o.nlanes; ++k) {
        Lane& L = srv->lanes[k];
        if (!L.in_flight) {
            r = launch_round(srv, L);
            if (r) return r;
        }
    }
    int b = !srv->queue.empty();
    for (int k = 0; k < srv->o.nlanes; ++k) {
        const Lane& L = srv->lanes[k];
        b |= L.in_flight || !L.act.empty() || !L.fin.empty();
    }
    if (busy) *busy = b;
    return rc;
}

void loop_main(gf_server* srv)
{
    while (srv->running.load()) {
        int busy = 0;
        int rc;
        {
            std::lock_guard<std::mutex> g(srv->mu);
            rc = pump_locked(srv, &busy);
        }
        if (rc == GF_ERR_CUDA || rc == GF_ERR_STATE) {
            std::lock_guard<std::mutex> g(srv->mu);
            srv->cv.notify_all();
            break;
        }
        if (!busy) std::this_thread::sleep_for(std::chrono::microseconds(200));
        else std::this_thread::yield();
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
    for (int k = 0; k < o.nlanes && e == cudaSuccess; ++k) {
        Lane& L = s->lanes[k];
        L.idx = k;
        int prio = lo;
        if (o.priority && o.nlanes > 1) prio = hi + (lo - hi) * k / (o.nlanes - 1);
        e = cudaStreamCreateWithPriority(&L.st, cudaStreamNonBlocking, prio);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L.ev, cudaEventDisableTiming);
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
    for (int k = 0; k < GF_SERVER_MAX_LANES; ++k) {
        Lane& L = s->lanes[k];
        if (L.st) cudaStreamSynchronize(L.st);
    }
    for (auto& kv : s->all) {
        Scen* sc = kv.second;
        if (sc->dev) cudaFree(sc->dev);
        if (sc->ev_fin) cudaEventDestroy(sc->ev_fin);
        delete sc;
    }
    for (int k = 0; k < GF_SERVER_MAX_LANES; ++k) {
        Lane& L = s->lanes[k];
        if (L.d_up) cudaFree(L.d_up);
        if (L.d_rb) cudaFree(L.d_rb);
        if (L.h_up) cudaFreeHost(L.h_up);
        if (L.h_rb) cudaFreeHost(L.h_rb);
        if (L.ev) cudaEventDestroy(L.ev);
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
    x->info.state = GF_SCEN_QUEUED;
    x->info.lane = x->lane;
    x->info.t_submit = s->now();
    x->info.t_admit = -1;
    x->info.t_done = -1;
    x->info.dt = sc->initial_dt;
    s->all[x->id] = x;
    s->queue.push_back(x);
    s->stats.submitted++;
    s->stats.queued++;
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
                std::this_thread::yield();
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
        s->stats.queued--;
        x->info.state = GF_SCEN_CANCELLED;
        x->info.t_done = s->now();
        s->cv.notify_all();
    } else if (x->info.state == GF_SCEN_ACTIVE && !x->finishing) {
        x->cancel_req = true;
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
