/*
 * Served AMR forests: a request loop over adaptive flood scenarios.
 *
 * Each request is a forest built on admission (raster pyramid or DEM
 * rasters, hydrograph, initial refinement) that then runs ForestClaw's
 * outstyle-1 loop (src/fc2d_geoclaw/fc2d_geoclaw_run.c:190-395) as a member
 * of one batched run (gf_forest.cpp): all members' leaves, of any patch
 * size, step in the same graph-replayed rounds, each forest with its own
 * time-step controller on the device and its own regrid cadence. The loop
 * alternates
 *
 *   admit (queued requests that fit the budget: create, init, join)
 *   -> one batch iteration (about half a millisecond of rounds; regrids of
 *      the members that wait for one; graph re-capture on any change)
 *   -> retire (members whose run ended: DONE, forest kept for the caller).
 *
 * The admitted and finished-but-unreleased forests together stay within the
 * HBM budget, by the footprint bound of their options; each active forest
 * has its own physics slot of the server's context.
 *
 * The loop keeps one batch per lane in flight at once. Forests go to up to
 * three lanes by their cells after the initial refinement (lane_cells),
 * each on its own stream, smaller lanes at higher priority; a lane's update
 * grid leaves reserve_sms SMs per smaller lane that has forests running.
 * Subcycled forests form a fourth lane that steps each forest's own graphs
 * side by side. A pass takes in the iterations that have finished, lets
 * members leave and join the idle lanes, admits, and launches the idle lanes
 * again; it never waits on the device.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
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

using Clock = std::chrono::steady_clock;
constexpr int kSubLane = GF_FSERVER_LANES; /* subcycled forests, side by side */

struct Req {
    long long id = 0;
    gf_forest_request r{};
    std::vector<double> hy_t, hy_hu;
    gf_forest_request_info info{};
    gf_forest* f = nullptr;
    int slot = -1;
    int lane = -1;
    size_t held = 0; /* bytes counted against the budget */
    bool cancel_req = false;
};

} // namespace

struct gf_fserver {
    int device = 0;
    gf_fserver_opts o{};
    gf_ctx* ctx = nullptr;
    int nlanes = 1;   /* lanes of shared rounds (subcycled forests are lane kSubLane) */
    int nsm = 0;
    gf::SubForests* sub = nullptr; /* lane 2: subcycled forests side by side */
    gf::ForestBatch* lanes[GF_FSERVER_LANES] = {};
    std::vector<Req*> joining[GF_FSERVER_LANES]; /* built forests waiting for their lane to be idle */
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv;
    std::thread loop;
    std::atomic<bool> running{false};
    bool broken = false;
    std::string last_error;
    std::map<long long, Req*> all;
    std::deque<Req*> queue;
    std::vector<Req*> active;
    std::vector<int> free_slots;
    long long next_id = 1;
    size_t bytes_in_use = 0, bytes_peak = 0;
    gf_fserver_stats stats{};
    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

int sfail(gf_fserver* s, int code, const char* msg)
{
    s->last_error = msg;
    return code;
}

const char* validate(const gf_forest_request& r)
{
    const gf_forest_opts& o = r.opts;
    if (!(o.mx == 8 || o.mx == 16 || o.mx == 32)) return "mx must be 8, 16 or 32";
    if (o.maux < 1 || o.maux > 3) return "maux must be 1..3";
    if (o.nbx < 1 || o.nby < 1) return "nbx, nby must be positive";
    if (o.minlevel < 0 || o.maxlevel < o.minlevel || o.maxlevel > 10) return "need 0 <= minlevel <= maxlevel <= 10";
    if (!(o.dx0 > 0) || !(o.dy0 > 0)) return "dx0, dy0 must be positive";
    if (!(r.t_final > 0) || r.nout < 1 || !(r.initial_dt > 0) || !(r.desired_cfl > 0) || !(r.max_cfl > 0))
        return "bad time-stepping parameters";
    if (r.nhydro < 0 || (r.nhydro > 0 && (!r.hydro_time || !r.hydro_hu))) return "bad hydrograph";
    for (int k = 1; k < r.nhydro; ++k)
        if (!(r.hydro_time[k] >= r.hydro_time[k - 1])) return "hydrograph times must increase";
    for (int s = 0; s < 4; ++s)
        if (o.mthbc[s] == 0 && !(r.nhydro > 0 && r.hydro_side[s]))
            return "mthbc = 0 needs a hydrograph on that side";
    if (!gf_forest_footprint(&o)) return "forest too large (set max_patches)";
    return nullptr;
}

void finish(gf_fserver* s, Req* x, int state)
{
    x->info.state = state;
    x->info.t_done = s->now();
    if (x->f) {
        gf_forest_stats st;
        gf_forest_get_stats(x->f, &st);
        x->info.steps = st.steps;
        x->info.rejects = st.rejects;
        x->info.regrids = st.regrids;
        x->info.cell_updates = st.cell_updates;
        x->info.t = st.t;
        x->info.dt = st.dt;
        x->info.max_cfl_seen = st.max_cfl_seen;
        x->info.npatch = st.npatch;
        x->info.npatch_max = std::max(st.npatch_max, st.npatch);
        x->info.device_bytes = gf::forest_device_bytes(x->f);
    }
    if (state == GF_SCEN_DONE) s->stats.done++;
    else if (state == GF_SCEN_FAILED) s->stats.failed++;
    s->cv.notify_all();
}

/* give back what a request holds (forest, slot, bytes) */
void drop(gf_fserver* s, Req* x)
{
    if (x->f) {
        gf_forest_destroy(x->f);
        x->f = nullptr;
    }
    if (x->slot >= 0) {
        s->free_slots.push_back(x->slot);
        x->slot = -1;
    }
    s->bytes_in_use -= x->held;
    x->held = 0;
}

/* build the request's forest; on failure the request is FAILED */
int admit(gf_fserver* s, Req* x)
{
    x->slot = s->free_slots.back();
    s->free_slots.pop_back();
    x->held = x->info.footprint;
    s->bytes_in_use += x->held;
    s->bytes_peak = std::max(s->bytes_peak, s->bytes_in_use);
    x->info.state = GF_SCEN_ACTIVE;
    x->info.t_admit = s->now();
    s->stats.admitted++;
    gf_forest_opts o = x->r.opts;
    o.phys_slot = x->slot;
    int rc = gf_ctx_set_phys(s->ctx, x->slot, &x->r.phys);
    if (!rc) rc = gf_forest_create(s->ctx, &o, x->r.fields, &x->f);
    if (!rc && x->r.nhydro > 0)
        rc = gf_forest_set_hydrograph(x->f, x->r.nhydro, x->hy_t.data(), x->hy_hu.data(), x->r.hydro_side,
                                      x->r.hydro_width, x->r.hydro_x0, x->r.hydro_y0);
    if (!rc && x->r.topo) rc = gf_forest_set_topo(x->f, x->r.topo, x->r.qinit);
    if (!rc) rc = gf_forest_init(x->f);
    x->r.fields = nullptr;
    x->r.topo = nullptr;
    if (rc) {
        s->last_error = gf_ctx_last_error(s->ctx);
        finish(s, x, GF_SCEN_FAILED);
        drop(s, x);
        return rc;
    }
    if (x->r.opts.subcycle) {
        /* subcycled: its own graph per coarse step, side by side with the
         * other subcycled forests; it joins at once */
        x->lane = kSubLane;
        x->info.lane = kSubLane;
        s->stats.lane_admitted[kSubLane]++;
        rc = gf::subforests_add(s->sub, x->f, x->r.t_final, x->r.nout, x->r.initial_dt, x->r.desired_cfl,
                                x->r.max_cfl);
        if (rc) {
            s->last_error = gf_ctx_last_error(s->ctx);
            finish(s, x, GF_SCEN_FAILED);
            drop(s, x);
            return rc;
        }
        s->active.push_back(x);
        return GF_OK;
    }
    const long long cells = (long long)gf_forest_npatch(x->f) * x->r.opts.mx * x->r.opts.mx;
    x->lane = 0;
    while (x->lane + 1 < s->nlanes && cells >= s->o.lane_cells[x->lane]) ++x->lane;
    x->info.lane = x->lane;
    s->stats.lane_admitted[x->lane]++;
    s->joining[x->lane].push_back(x);
    return GF_OK;
}

/* members join a lane between its iterations */
void join(gf_fserver* s, int k)
{
    for (Req* x : s->joining[k]) {
        if (x->cancel_req) {
            finish(s, x, GF_SCEN_CANCELLED);
            drop(s, x);
            continue;
        }
        int rc = gf::forest_batch_add(s->lanes[k], x->f, x->r.t_final, x->r.nout, x->r.initial_dt,
                                      x->r.desired_cfl, x->r.max_cfl);
        if (rc) {
            s->last_error = gf_ctx_last_error(s->ctx);
            finish(s, x, GF_SCEN_FAILED);
            drop(s, x);
            continue;
        }
        s->active.push_back(x);
    }
    s->joining[k].clear();
}

int fail_all(gf_fserver* s, int rc)
{
    s->broken = true;
    s->last_error = gf_ctx_last_error(s->ctx);
    for (Req* x : s->active) finish(s, x, GF_SCEN_FAILED);
    s->active.clear();
    for (int k = 0; k < GF_FSERVER_LANES; ++k) {
        for (Req* x : s->joining[k]) finish(s, x, GF_SCEN_FAILED);
        s->joining[k].clear();
    }
    return rc;
}

bool fits(const gf_fserver* s, const Req* x)
{
    size_t running = s->active.size();
    for (int k = 0; k < GF_FSERVER_LANES; ++k) running += s->joining[k].size();
    return (int)running < s->o.max_active && !s->free_slots.empty() &&
           s->bytes_in_use + x->info.footprint <= s->o.hbm_budget;
}

/* One pass of the loop; never waits on the device. *progress = 1 when an
 * iteration was taken in or launched, or a request changed state. */
int pump_locked(gf_fserver* s, int* busy, int* progress = nullptr)
{
    if (s->broken) return sfail(s, GF_ERR_STATE, "the batch failed; destroy the server");
    int moved = 0;
    /* take in the iterations that have finished */
    for (int k = 0; k < s->nlanes; ++k) {
        if (!gf::forest_batch_inflight(s->lanes[k])) continue;
        int done = 0;
        int rc = gf::forest_batch_test(s->lanes[k], 0, &done);
        if (rc) return fail_all(s, rc);
        if (done) {
            s->stats.iterations++;
            moved = 1;
        }
    }
    /* subcycled forests: take in finished steps, launch the next ones */
    {
        int live = 0, prog = 0;
        int rc = gf::subforests_pass(s->sub, &live, &prog);
        if (rc) return fail_all(s, rc);
        moved |= prog;
    }
    /* idle lanes: cancelled and finished members leave (a finished forest
     * stays resident for the caller; its physics slot is free again) */
    std::vector<Req*> still;
    for (Req* x : s->active) {
        if (x->lane == kSubLane) {
            if (x->cancel_req) gf::subforests_stop(x->f);
            if (gf::subforests_running(x->f)) {
                still.push_back(x);
                continue;
            }
            gf::subforests_remove(s->sub, x->f);
            if (x->cancel_req) {
                finish(s, x, GF_SCEN_CANCELLED);
                drop(s, x);
            } else {
                finish(s, x, GF_SCEN_DONE);
                s->free_slots.push_back(x->slot);
                x->slot = -1;
            }
            moved = 1;
            continue;
        }
        gf::ForestBatch* b = s->lanes[x->lane];
        if (gf::forest_batch_inflight(b)) {
            still.push_back(x);
            continue;
        }
        if (x->cancel_req) {
            gf::forest_batch_remove(b, x->f);
            finish(s, x, GF_SCEN_CANCELLED);
            drop(s, x);
            moved = 1;
        } else if (!gf::forest_batch_running(x->f)) {
            gf::forest_batch_remove(b, x->f);
            finish(s, x, GF_SCEN_DONE);
            s->free_slots.push_back(x->slot);
            x->slot = -1;
            moved = 1;
        } else {
            still.push_back(x);
        }
    }
    s->active.swap(still);
    /* admission, first come first served (backfill: later requests that
     * fit may pass a head that does not); built forests join their lane
     * when it is idle */
    const auto ta = Clock::now();
    for (auto it = s->queue.begin(); it != s->queue.end();) {
        Req* x = *it;
        if (!fits(s, x)) {
            if (!s->o.backfill) break;
            ++it;
            continue;
        }
        it = s->queue.erase(it);
        admit(s, x); /* a failed build fails only this request */
        moved = 1;
    }
    s->stats.s_admit += std::chrono::duration<double>(Clock::now() - ta).count();
    for (int k = 0; k < s->nlanes; ++k) {
        if (gf::forest_batch_inflight(s->lanes[k])) continue;
        if (!s->joining[k].empty()) join(s, k);
        if (!gf::forest_batch_members(s->lanes[k])) continue;
        if (k > 0) {
            /* a lane leaves reserve_sms SMs free per smaller lane with forests running */
            int smaller = 0;
            for (int j = 0; j < k; ++j)
                smaller += gf::forest_batch_members(s->lanes[j]) > 0 || !s->joining[j].empty();
            int cap = 0;
            if (smaller && s->o.reserve_sms > 0)
                cap = std::max(s->nsm / 4, s->nsm - s->o.reserve_sms * smaller);
            gf::forest_batch_set_max_ctas(s->lanes[k], cap);
        }
        int live = 0;
        int rc = gf::forest_batch_launch(s->lanes[k], &live);
        if (rc) return fail_all(s, rc);
        moved |= live > 0;
    }
    gf_forest_batch_stats sum{};
    for (int k = 0; k < s->nlanes; ++k) {
        gf_forest_batch_stats b;
        gf::forest_batch_get_stats(s->lanes[k], &b);
        sum.epochs += b.epochs;
        sum.rounds += b.rounds;
        sum.launches += b.launches;
        sum.regrids += b.regrids;
        sum.cell_updates += b.cell_updates;
        sum.s_epoch += b.s_epoch;
        sum.s_rounds += b.s_rounds;
        sum.s_regrid += b.s_regrid;
    }
    long long sub_steps = 0, sub_regrids = 0, sub_cu = 0;
    gf::subforests_get_stats(s->sub, &sub_steps, &sub_regrids, &sub_cu);
    s->stats.epochs = sum.epochs;
    s->stats.rounds = sum.rounds;
    s->stats.launches = sum.launches;
    s->stats.regrids = sum.regrids + sub_regrids;
    s->stats.cell_updates = sum.cell_updates + sub_cu;
    s->stats.sub_steps = sub_steps;
    s->stats.s_epoch = sum.s_epoch;
    s->stats.s_rounds = sum.s_rounds;
    s->stats.s_regrid = sum.s_regrid;
    bool joining = false;
    for (int k = 0; k < GF_FSERVER_LANES; ++k) joining |= !s->joining[k].empty();
    if (busy) *busy = !s->queue.empty() || !s->active.empty() || joining;
    if (progress) *progress = moved;
    return GF_OK;
}

/* wait for every lane's iteration in flight (before forests are freed) */
void drain(gf_fserver* s)
{
    for (int k = 0; k < s->nlanes; ++k) {
        int done = 0;
        if (s->lanes[k] && gf::forest_batch_inflight(s->lanes[k])) gf::forest_batch_test(s->lanes[k], 1, &done);
    }
    cudaSetDevice(s->device);
    cudaDeviceSynchronize(); /* subcycled steps on the runner's streams */
}

void loop_main(gf_fserver* s)
{
    cudaSetDevice(s->device);
    while (s->running.load()) {
        int busy = 0, moved = 0;
        {
            std::lock_guard<std::mutex> g(s->mu);
            if (pump_locked(s, &busy, &moved)) busy = 0;
        }
        if (!busy) std::this_thread::sleep_for(std::chrono::microseconds(200));
        else if (!moved) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

Req* find_req(gf_fserver* s, long long id)
{
    auto it = s->all.find(id);
    return it == s->all.end() ? nullptr : it->second;
}

} // namespace

extern "C" {

void gf_fserver_opts_default(gf_fserver_opts* o)
{
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->hbm_budget = (size_t)64 << 30;
    o->max_active = 256;
    o->backfill = 1;
    o->lane_cells[0] = 1 << 18;
    o->lane_cells[1] = 1 << 20;
    o->reserve_sms = 40;
}

int gf_fserver_create(int device, const gf_fserver_opts* opts, gf_fserver** out)
{
    if (!out) return GF_ERR_ARG;
    *out = nullptr;
    gf_fserver_opts o;
    if (opts) o = *opts;
    else gf_fserver_opts_default(&o);
    if (o.max_active < 1 || o.max_active > GF_MAX_PHYS || o.hbm_budget == 0 || o.reserve_sms < 0)
        return GF_ERR_ARG;
    int nl = 1;
    for (int k = 0; k < GF_FSERVER_LANES - 1 && o.lane_cells[k] > 0; ++k) {
        if (k > 0 && o.lane_cells[k] <= o.lane_cells[k - 1]) return GF_ERR_ARG;
        ++nl;
    }
    gf_fserver* s = new gf_fserver;
    s->device = device;
    s->o = o;
    s->t0 = Clock::now();
    int rc = gf_ctx_create(device, &s->ctx);
    if (!rc) {
        cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, device);
        s->nlanes = nl;
        /* one lane: the context's stream; several: a stream each, smaller
         * lanes at higher priority */
        for (int k = 0; k < nl && !rc; ++k)
            rc = gf::forest_batch_create(s->ctx, &s->lanes[k], nl > 1 ? k + 1 : 0, 0);
    }
    if (!rc) rc = gf::subforests_create(s->ctx, &s->sub);
    if (rc) {
        gf_fserver_destroy(s);
        return rc;
    }
    for (int k = GF_MAX_PHYS - 1; k >= 0; --k) s->free_slots.push_back(k);
    *out = s;
    return GF_OK;
}

void gf_fserver_destroy(gf_fserver* s)
{
    if (!s) return;
    gf_fserver_stop(s);
    drain(s);
    for (auto& kv : s->all) {
        if (kv.second->f) gf_forest_destroy(kv.second->f);
        delete kv.second;
    }
    for (int k = 0; k < GF_FSERVER_LANES; ++k)
        if (s->lanes[k]) gf::forest_batch_destroy(s->lanes[k]);
    if (s->sub) gf::subforests_destroy(s->sub);
    if (s->ctx) gf_ctx_destroy(s->ctx);
    delete s;
}

const char* gf_fserver_last_error(const gf_fserver* s) { return s ? s->last_error.c_str() : "null server"; }

gf_ctx* gf_fserver_ctx(gf_fserver* s) { return s ? s->ctx : nullptr; }

int gf_fserver_submit(gf_fserver* s, const gf_forest_request* r, long long* id)
{
    if (!s || !r) return GF_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    if (const char* why = validate(*r)) return sfail(s, GF_ERR_ARG, why);
    const size_t bytes = gf_forest_footprint(&r->opts);
    if (bytes > s->o.hbm_budget) return sfail(s, GF_ERR_NOMEM, "forest exceeds the server's HBM budget");
    Req* x = new Req;
    x->id = s->next_id++;
    x->r = *r;
    x->hy_t.assign(r->hydro_time, r->hydro_time + r->nhydro);
    x->hy_hu.assign(r->hydro_hu, r->hydro_hu + r->nhydro);
    x->r.hydro_time = nullptr;
    x->r.hydro_hu = nullptr;
    x->info.state = GF_SCEN_QUEUED;
    x->info.t_submit = s->now();
    x->info.t_admit = -1;
    x->info.t_done = -1;
    x->info.dt = r->initial_dt;
    x->info.footprint = bytes;
    x->info.lane = -1;
    s->all[x->id] = x;
    s->queue.push_back(x);
    s->stats.submitted++;
    if (id) *id = x->id;
    return GF_OK;
}

int gf_fserver_pump(gf_fserver* s, int* busy)
{
    if (!s) return GF_ERR_ARG;
    if (s->running.load()) return sfail(s, GF_ERR_STATE, "the request loop thread is running");
    std::lock_guard<std::mutex> g(s->mu);
    return pump_locked(s, busy);
}

int gf_fserver_start(gf_fserver* s)
{
    if (!s) return GF_ERR_ARG;
    if (s->running.exchange(true)) return GF_OK;
    s->loop = std::thread(loop_main, s);
    return GF_OK;
}

int gf_fserver_stop(gf_fserver* s)
{
    if (!s) return GF_ERR_ARG;
    if (!s->running.exchange(false)) return GF_OK;
    if (s->loop.joinable()) s->loop.join();
    return GF_OK;
}

int gf_fserver_wait(gf_fserver* s, long long id, double timeout_s)
{
    if (!s) return GF_ERR_ARG;
    const double t_end = s->now() + timeout_s;
    std::unique_lock<std::mutex> g(s->mu);
    Req* x = find_req(s, id);
    if (!x) return sfail(s, GF_ERR_ARG, "unknown request id");
    while (x->info.state == GF_SCEN_QUEUED || x->info.state == GF_SCEN_ACTIVE) {
        if (s->broken) return GF_ERR_STATE;
        if (s->now() > t_end) return sfail(s, GF_ERR_STATE, "wait timed out");
        if (s->running.load()) {
            s->cv.wait_for(g, std::chrono::milliseconds(2));
        } else {
            int busy = 0, moved = 0;
            int rc = pump_locked(s, &busy, &moved);
            if (rc) return rc;
            if (!moved) {
                g.unlock();
                std::this_thread::sleep_for(std::chrono::microseconds(20));
                g.lock();
            }
        }
    }
    return x->info.state == GF_SCEN_FAILED ? GF_ERR_STATE : GF_OK;
}

int gf_fserver_poll(gf_fserver* s, long long id, gf_forest_request_info* info)
{
    if (!s || !info) return GF_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    Req* x = find_req(s, id);
    if (!x) return sfail(s, GF_ERR_ARG, "unknown request id");
    *info = x->info;
    if (x->info.state == GF_SCEN_ACTIVE && x->f) {
        gf_forest_stats st;
        gf_forest_get_stats(x->f, &st);
        info->steps = st.steps;
        info->rejects = st.rejects;
        info->regrids = st.regrids;
        info->cell_updates = st.cell_updates;
        info->t = st.t;
        info->dt = st.dt;
        info->max_cfl_seen = st.max_cfl_seen;
        info->npatch = st.npatch;
        info->npatch_max = std::max(st.npatch_max, st.npatch);
    }
    return GF_OK;
}

int gf_fserver_cancel(gf_fserver* s, long long id)
{
    if (!s) return GF_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    Req* x = find_req(s, id);
    if (!x) return sfail(s, GF_ERR_ARG, "unknown request id");
    if (x->info.state == GF_SCEN_QUEUED) {
        s->queue.erase(std::find(s->queue.begin(), s->queue.end(), x));
        x->info.state = GF_SCEN_CANCELLED;
        x->info.t_done = s->now();
        x->info.footprint = 0;
        s->cv.notify_all();
    } else if (x->info.state == GF_SCEN_ACTIVE) {
        x->cancel_req = true; /* leaves the batch before the next iteration */
    }
    return GF_OK;
}

int gf_fserver_forest(gf_fserver* s, long long id, gf_forest** f)
{
    if (!s || !f) return GF_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    Req* x = find_req(s, id);
    if (!x) return sfail(s, GF_ERR_ARG, "unknown request id");
    if (x->info.state != GF_SCEN_DONE || !x->f) return sfail(s, GF_ERR_STATE, "the request is not done");
    *f = x->f;
    return GF_OK;
}

int gf_fserver_download(gf_fserver* s, long long id, int* npatch, int* level, int* I, int* J, double* q,
                        double* aux)
{
    if (!s) return GF_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    Req* x = find_req(s, id);
    if (!x) return sfail(s, GF_ERR_ARG, "unknown request id");
    if (x->info.state != GF_SCEN_DONE || !x->f) return sfail(s, GF_ERR_STATE, "the request is not done");
    if (npatch) *npatch = gf_forest_npatch(x->f);
    int rc = gf_forest_patches(x->f, level, I, J);
    if (!rc && q) rc = gf_forest_download(x->f, q);
    if (!rc && aux) rc = gf_forest_download_aux(x->f, aux);
    if (rc) s->last_error = gf_ctx_last_error(s->ctx);
    return rc;
}

int gf_fserver_release(gf_fserver* s, long long id)
{
    if (!s) return GF_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    Req* x = find_req(s, id);
    if (!x) return sfail(s, GF_ERR_ARG, "unknown request id");
    if (x->info.state == GF_SCEN_QUEUED || x->info.state == GF_SCEN_ACTIVE)
        return sfail(s, GF_ERR_STATE, "the request is still running (cancel it first)");
    drop(s, x); /* a finished forest is no member of any lane: nothing in flight reads it */
    return GF_OK;
}

int gf_fserver_stats_get(gf_fserver* s, gf_fserver_stats* st)
{
    if (!s || !st) return GF_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    *st = s->stats;
    st->bytes_in_use = s->bytes_in_use;
    st->bytes_peak = s->bytes_peak;
    st->active = (int)s->active.size();
    st->queued = (int)s->queue.size();
    int held = 0;
    for (auto& kv : s->all) held += kv.second->info.state == GF_SCEN_DONE && kv.second->f;
    st->held = held;
    return GF_OK;
}

double gf_fserver_clock(const gf_fserver* s) { return s ? s->now() : -1.0; }

} // extern "C"
