/*
 * Device-side time-step control of served scenarios (one thread per
 * scenario). Compiled without FMA contraction, so the controller's
 * arithmetic is the same IEEE sequence as the host restatement of
 * ForestClaw's outstyle 1 loop (src/fc2d_geoclaw/fc2d_geoclaw_run.c:190-395):
 *
 *   prepare: hold the group for a due regrid, close finished output
 *            intervals (:229-236), stop after the last one, pick
 *            dt_step = dt_minlevel / level_factor clipped to land on the
 *            interval end with the 1 % tolerance (:251-278), select the
 *            current state buffer and the hydrograph inflow at t_curr
 *            (hydrograph/hydrograh_module.f90:176-221).
 *   finish : CFL over max_cfl -> retake with dt_minlevel *= desired/cfl
 *            (:326-343); else accept, advance t, flip the state buffer,
 *            and set dt_minlevel = dt_minlevel * desired / cfl unless the
 *            step was a small one (:346-376).
 */
#include <cuda_runtime.h>

#include "gf_internal.h"

namespace gf {

namespace {

__device__ double hydro_at(const double* __restrict__ tm, const double* __restrict__ hu, int n,
                           double t)
{
    if (n == 0) return 0.0;
    if (t < tm[0]) return hu[0];
    if (t > tm[n - 1]) return hu[n - 1];
    for (int i = 0; i + 1 < n; ++i)
        if (t >= tm[i] && t <= tm[i + 1])
            return hu[i] + (hu[i + 1] - hu[i]) / (tm[i + 1] - tm[i]) * (t - tm[i]);
    return 0.0;
}

__global__ void served_prepare_kernel(gf_group_state* __restrict__ gs,
                                      gf_ghost_block* __restrict__ blocks,
                                      double* __restrict__ gdt, int* __restrict__ gpar,
                                      unsigned long long* __restrict__ gmax,
                                      const double* __restrict__ hy_t,
                                      const double* __restrict__ hy_hu, int ng,
                                      long long* __restrict__ qdelta)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    gf_group_state s = gs[g];
    gmax[g] = 0ull;
    bool go = s.active != 0;
    /* a regrid is due right after the accepted step that completes the
     * interval (fc2d_geoclaw_run.c:388-395): wait for the host */
    if (go && s.regrid_interval > 0 && s.since_regrid >= s.regrid_interval) {
        s.paused = 1;
        go = false;
    }
    while (go && !(s.t_curr < s.tend)) {
        if (++s.nint >= s.nout) {
            s.active = 0;
            go = false;
        } else {
            s.tend = s.t_curr + s.dt_outer;
        }
    }
    if (!go) {
        gdt[g] = 0.0;
        blocks[g].skip = 1;
        if (qdelta) qdelta[g] = GF_QDELTA_SKIP;
        gs[g] = s;
        return;
    }
    /* advance-one-step: the step is the minlevel dt over 2^(maxlevel-minlevel) */
    double dt_step = s.dt_minlevel / s.level_factor;
    const double tol = 1e-2 * dt_step;
    s.took_small = 0;
    const double small_step = s.tend - (s.t_curr + dt_step);
    if (small_step < tol) {
        dt_step = s.tend - s.t_curr;
        if (small_step < 0) s.took_small = 1;
    }
    s.dt_step = dt_step;
    gdt[g] = dt_step;
    gpar[g] = s.cur;
    if (qdelta) qdelta[g] = s.cur ? (long long)(s.qb[1] - s.qb[0]) : 0ll;
    blocks[g].q = s.qb[s.cur];
    blocks[g].skip = 0;
    blocks[g].bc.q0hu = hydro_at(hy_t + s.hydro_off, hy_hu + s.hydro_off, s.nhydro, s.t_curr);
    gs[g] = s;
}

__global__ void served_finish_kernel(gf_group_state* __restrict__ gs,
                                     const double* __restrict__ gdt,
                                     const unsigned long long* __restrict__ gmax,
                                     const int* __restrict__ err, int ng)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    if (!(gdt[g] > 0.0)) return; /* no step this round */
    gf_group_state s = gs[g];
    if (*err) {
        /* a bounded copy wait expired somewhere in the round: stop */
        s.active = 0;
        gs[g] = s;
        return;
    }
    const double cfl = __longlong_as_double((long long)gmax[g]);
    s.max_cfl_seen = fmax(s.max_cfl_seen, cfl);
    if (cfl > s.max_cfl) {
        s.dt_minlevel = s.dt_minlevel * s.desired_cfl / cfl;
        s.rejects++;
    } else {
        s.steps++;
        s.since_regrid++;
        s.t_curr += s.dt_step;
        s.cur ^= 1;
        const double dt_new = s.dt_minlevel * s.desired_cfl / cfl;
        if (!s.took_small) s.dt_minlevel = dt_new;
    }
    gs[g] = s;
}

} // namespace

cudaError_t launch_served_prepare(gf_group_state* gs, gf_ghost_block* blocks, double* gdt, int* gpar,
                                  unsigned long long* gmax, const double* hy_t,
                                  const double* hy_hu, int ng, cudaStream_t st, long long* qdelta)
{
    if (ng <= 0) return cudaSuccess;
    served_prepare_kernel<<<(ng + 127) / 128, 128, 0, st>>>(gs, blocks, gdt, gpar, gmax, hy_t, hy_hu,
                                                            ng, qdelta);
    return cudaGetLastError();
}

cudaError_t launch_served_finish(gf_group_state* gs, const double* gdt,
                                 const unsigned long long* gmax, const int* err, int ng,
                                 cudaStream_t st)
{
    if (ng <= 0) return cudaSuccess;
    served_finish_kernel<<<(ng + 127) / 128, 128, 0, st>>>(gs, gdt, gmax, err, ng);
    return cudaGetLastError();
}

} // namespace gf
