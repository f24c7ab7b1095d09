/*
 * Coarse/fine transfers, time interpolation and refinement tags on the
 * device (paths relative to the GeoFlood source tree):
 *
 *   average_face / _corner / _average2coarse
 *       fclaw2d_source/fc2d_geoclaw_average_fort.f:33, 323, 482-602
 *   interpolate_face / _corner / _interpolate2fine
 *       fclaw2d_source/fc2d_geoclaw_interpolate_fort.f:24, 261, 405-579
 *   timeinterp      fclaw2d_source/fc2d_geoclaw_timeinterp_fort.f:1-69
 *   tag4refinement / flag2refine / tag4coarsening / test_regions
 *       fclaw2d_source/fc2d_geoclaw_tag4refinement_fort.f90,
 *       fc2d_geoflood_flag2refine.f90, fc2d_geoclaw_tag4coarsening_fort.f90,
 *       fc2d_geoclaw_test_regions.f90 (called from fc2d_geoclaw.cpp:405-506)
 *
 * The fine cells under a coarse cell are the aligned-brick restatement of
 * ForestClaw's transform_face_half / transform_corner_half (lower-left
 * first, x fastest); slopes are minmod (mth = 5, the reference's own
 * comment at interpolate_fort.f:430). Each task is one CTA; a launch holds
 * tasks whose destinations are disjoint from their sources.
 */
#include <cuda_runtime.h>

#include "gf_internal.h"

namespace gf {

namespace {

template <int M>
struct AmrGeo {
    static constexpr int N = M + 4;
    static constexpr int S = N * N;
    __device__ static int at(int i, int j) { return (j + 1) * N + (i + 1); }
};

__device__ __forceinline__ double slope_minmod(double sl, double sr)
{
    if (sl * sr <= 0.0) return 0.0;
    return fabs(sl) < fabs(sr) ? sl : sr;
}

/* wet-weighted average of 4 fine cells (average_fort.f:154-198) */
template <int M>
__device__ void avg4(double drytol, const double* qf, const double* bf, const int* k4, double bc,
                     double& h, double& hu, double& hv)
{
    using G = AmrGeo<M>;
    double etasum = 0.0, hsum = 0.0, husum = 0.0, hvsum = 0.0;
    int nwet = 0;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const double hf = qf[k4[m]];
        const double b = bf[k4[m]];
        double huf = qf[G::S + k4[m]];
        double hvf = qf[2 * G::S + k4[m]];
        double etaf;
        if (hf > drytol) {
            etaf = hf + b;
            nwet = nwet + 1;
        } else {
            etaf = 0.0;
            huf = 0.0;
            hvf = 0.0;
        }
        hsum = hsum + hf;
        husum = husum + huf;
        hvsum = hvsum + hvf;
        etasum = etasum + etaf;
    }
    if (nwet > 0) {
        const double etaav = etasum / (double)nwet;
        const double hav = hsum / (double)nwet;
        const double hc = fmin(hav, fmax(etaav - bc, 0.0));
        h = hc;
        hu = (hc / hsum) * husum;
        hv = (hc / hsum) * hvsum;
    } else {
        h = hu = hv = 0.0;
    }
}

/* limited reconstruction of coarse cell (ic, jc) into its 4 fine cells
 * (interpolate_fort.f:122-176) */
template <int M>
__device__ void interp_cell(double drytol, double sea, const double* qc, const double* bcp,
                            double* qf, const double* bfp, int ic, int jc, const int* k4, bool clip)
{
    using G = AmrGeo<M>;
    for (int mq = 0; mq < 3; ++mq) {
        double qcv, gx, gy;
        if (mq == 0) {
            double eb[3][3];
#pragma unroll
            for (int ii = -1; ii <= 1; ++ii)
#pragma unroll
                for (int jj = -1; jj <= 1; ++jj) {
                    const int k = G::at(ic + ii, jc + jj);
                    const double h = qc[k];
                    eb[ii + 1][jj + 1] = (h < drytol) ? sea : h + bcp[k];
                }
            qcv = eb[1][1];
            gx = slope_minmod(qcv - eb[0][1], eb[2][1] - qcv);
            gy = slope_minmod(qcv - eb[1][0], eb[1][2] - qcv);
        } else {
            const double* p = qc + mq * G::S;
            qcv = p[G::at(ic, jc)];
            gx = slope_minmod(qcv - p[G::at(ic - 1, jc)], p[G::at(ic + 1, jc)] - qcv);
            gy = slope_minmod(qcv - p[G::at(ic, jc - 1)], p[G::at(ic, jc + 1)] - qcv);
        }
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const double sx = ((m & 1) - 0.5) / 2.0, sy = ((m >> 1) - 0.5) / 2.0;
            double v = qcv + gx * sx + gy * sy;
            if (mq == 0) {
                v = v - bfp[k4[m]];
                if (clip) v = fmax(v, 0.0);
            }
            qf[mq * G::S + k4[m]] = v;
        }
    }
}

template <int M>
__device__ __forceinline__ void under(int ic, int jc, int ox, int oy, int* i2, int* j2)
{
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        i2[m] = 2 * ic - 1 + ox + (m & 1);
        j2[m] = 2 * jc - 1 + oy + (m >> 1);
    }
}

template <int M>
__global__ void __launch_bounds__(128) transfer_kernel(const gf_xfer_task* __restrict__ tasks,
                                                       int ntask,
                                                       const gf_phys* __restrict__ phys_table,
                                                       const long long* __restrict__ qdelta)
{
    using G = AmrGeo<M>;
    constexpr int MBC = 2;
    const int ti = blockIdx.x;
    if (ti >= ntask) return;
    gf_xfer_task T = tasks[ti];
    if (qdelta) {
        const long long d = qdelta[T.group];
        if (d == GF_QDELTA_SKIP) return; /* the group does not step this round */
        /* shift to the buffer holding the group's current state */
        T.qc += d;
        T.qf += d;
    }
    const double drytol = phys_table[T.phys].dry_tolerance;
    const double sea = phys_table[T.phys].sea_level;
    const double* bc = T.ac; /* aux field 0 = bathymetry */
    const double* bf = T.af;
    switch (T.kind) {
    case GF_XFER_AVG_FACE: {
        const int idir = T.code / 2;
        for (int e = threadIdx.x; e < M * MBC; e += blockDim.x) {
            int ic, jc;
            if (idir == 0) {
                jc = 1 + e / MBC;
                const int ibc = 1 + e % MBC;
                ic = (T.code == 0) ? 1 - ibc : M + ibc;
            } else {
                const int jbc = 1 + e / M;
                ic = 1 + e % M;
                jc = (T.code == 2) ? 1 - jbc : M + jbc;
            }
            int i2[4], j2[4], k4[4];
            under<M>(ic, jc, T.ox, T.oy, i2, j2);
            bool ok = true;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                ok = ok && i2[m] >= 1 && i2[m] <= M && j2[m] >= 1 && j2[m] <= M;
                k4[m] = G::at(i2[m], j2[m]);
            }
            if (!ok) continue;
            double h, hu, hv;
            const int kc = G::at(ic, jc);
            avg4<M>(drytol, T.qf, bf, k4, bc[kc], h, hu, hv);
            T.qc[kc] = h;
            T.qc[G::S + kc] = hu;
            T.qc[2 * G::S + kc] = hv;
        }
        break;
    }
    case GF_XFER_AVG_CORNER: {
        for (int e = threadIdx.x; e < MBC * MBC; e += blockDim.x) {
            const int ibc = 1 + e / MBC, jbc = 1 + e % MBC;
            const int i1 = (T.code == 0 || T.code == 2) ? 1 - ibc : M + ibc;
            const int j1 = (T.code == 0 || T.code == 1) ? 1 - jbc : M + jbc;
            int i2[4], j2[4], k4[4];
            under<M>(i1, j1, T.ox, T.oy, i2, j2);
#pragma unroll
            for (int m = 0; m < 4; ++m) k4[m] = G::at(i2[m], j2[m]);
            double h, hu, hv;
            const int kc = G::at(i1, j1);
            avg4<M>(drytol, T.qf, bf, k4, bc[kc], h, hu, hv);
            T.qc[kc] = h;
            T.qc[G::S + kc] = hu;
            T.qc[2 * G::S + kc] = hv;
        }
        break;
    }
    case GF_XFER_INTERP_FACE: {
        const int idir = T.code / 2;
        for (int e = threadIdx.x; e < M; e += blockDim.x) {
            const int k = 1 + e;
            const int ic = idir == 0 ? ((T.code == 0) ? 1 : M) : k;
            const int jc = idir == 0 ? k : ((T.code == 2) ? 1 : M);
            int i2[4], j2[4], k4[4];
            under<M>(ic, jc, T.ox, T.oy, i2, j2);
            bool ok = true;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                ok = ok && i2[m] >= 1 - MBC && i2[m] <= M + MBC && j2[m] >= 1 - MBC &&
                     j2[m] <= M + MBC;
                k4[m] = G::at(i2[m], j2[m]);
            }
            if (!ok) continue;
            interp_cell<M>(drytol, sea, T.qc, bc, T.qf, bf, ic, jc, k4, true);
        }
        break;
    }
    case GF_XFER_INTERP_CORNER: {
        if (threadIdx.x == 0) {
            const int ic = (T.code == 0 || T.code == 2) ? 1 : M;
            const int jc = (T.code == 0 || T.code == 1) ? 1 : M;
            int i2[4], j2[4], k4[4];
            under<M>(ic, jc, T.ox, T.oy, i2, j2);
            bool ok = true;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                ok = ok && i2[m] >= 1 - MBC && i2[m] <= M + MBC && j2[m] >= 1 - MBC &&
                     j2[m] <= M + MBC;
                k4[m] = G::at(i2[m], j2[m]);
            }
            if (ok) interp_cell<M>(drytol, sea, T.qc, bc, T.qf, bf, ic, jc, k4, true);
        }
        break;
    }
    case GF_XFER_INTERP2FINE: {
        const int ig = T.code % 2, jg = T.code / 2;
        const int i1 = 1 - ig, j1 = 1 - jg, ic_add = ig * M / 2, jc_add = jg * M / 2;
        const int ni = M / 2 + 1;
        for (int e = threadIdx.x; e < ni * ni; e += blockDim.x) {
            const int i = i1 + e % ni, j = j1 + e / ni;
            int k4[4];
#pragma unroll
            for (int m = 0; m < 4; ++m) k4[m] = G::at((i - 1) * 2 + 1 + (m & 1), (j - 1) * 2 + 1 + (m >> 1));
            interp_cell<M>(drytol, sea, T.qc, bc, T.qf, bf, i + ic_add, j + jc_add, k4, false);
        }
        break;
    }
    case GF_XFER_AVG2COARSE: {
        const int ig = T.code % 2, jg = T.code / 2;
        const int ic_add = ig * M / 2, jc_add = jg * M / 2;
        for (int e = threadIdx.x; e < (M / 2) * (M / 2); e += blockDim.x) {
            const int i = 1 + e % (M / 2), j = 1 + e / (M / 2);
            int k4[4];
#pragma unroll
            for (int m = 0; m < 4; ++m) k4[m] = G::at((i - 1) * 2 + 1 + (m & 1), (j - 1) * 2 + 1 + (m >> 1));
            const int kc = G::at(i + ic_add, j + jc_add);
            double h, hu, hv;
            avg4<M>(drytol, T.qf, bf, k4, bc[kc], h, hu, hv);
            T.qc[kc] = h;
            T.qc[G::S + kc] = hu;
            T.qc[2 * G::S + kc] = hv;
        }
        break;
    }
    default:
        break;
    }
}

/* q_interp = q_last + alpha (q_curr - q_last) on the 2-cell interior strip
 * (timeinterp_fort.f:23-56, mint = 2, ng = 0). */
template <int M>
__global__ void __launch_bounds__(128) timeinterp_kernel(const gf_tinterp_task* __restrict__ tasks,
                                                         int ntask, double alpha)
{
    using G = AmrGeo<M>;
    const int ti = blockIdx.x;
    if (ti >= ntask) return;
    const gf_tinterp_task T = tasks[ti];
    constexpr int MINT = 2;
    for (int e = threadIdx.x; e < M * M; e += blockDim.x) {
        const int i = 1 + e % M, j = 1 + e / M;
        const bool strip = i <= MINT || i > M - MINT || j <= MINT || j > M - MINT;
        if (!strip) continue;
        const int k = G::at(i, j);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const double last = T.qlast[f * G::S + k];
            T.qinterp[f * G::S + k] = last + alpha * (T.qcurr[f * G::S + k] - last);
        }
    }
}

/* ------------------------------ tags ------------------------------ */
__device__ int test_regions(const gf_refine& rf, int level, double xl, double yl, double xu,
                            double yu, double t, int refine)
{
    bool found = false;
    int min_level = 100, max_level = 0;
    for (int m = 0; m < rf.num_regions; ++m) {
        const gf_region& r = rf.regions[m];
        const bool in = !(t < r.t_low || t > r.t_hi) && !(xu < r.x_low || xl > r.x_hi) &&
                        !(yu < r.y_low || yl > r.y_hi);
        if (in) {
            found = true;
            min_level = min(min_level, r.min_level);
            max_level = max(max_level, r.max_level);
        }
    }
    if (!found) return -1;
    if (refine) {
        if (level < min_level) return 1;
        if (level >= max_level) return 0;
    } else {
        if (level <= min_level) return 0;
        if (level > max_level) return 1;
    }
    return -1;
}

/* fc2d_geoflood_flag2refine.f90:7-130 for one interior cell (allowflag is
 * always true; the legacy regions.i block is never filled). */
__device__ int flag2refine(double drytol, double sea, const gf_refine& rf, double h, double hu,
                           double hv, double b, int level, int maxlevel, int init_flag,
                           bool coarsening)
{
    if (init_flag != 0 && coarsening) return 0;
    const int max_num_speeds = min(rf.num_speed_tolerance, maxlevel);
    const double momentum = sqrt(hu * hu + hv * hv);
    const double depth = h;
    const double eta = depth + b;
    const int th_factor = coarsening ? 0 : 1; /* integer variable assigned 0.5 */
    for (int m = 0; m < rf.num_flowgrades; ++m) {
        bool needed = false;
        const int var = rf.flowgradevariable[m];
        if (var == 1) needed = depth > rf.flowgradevalue[m];
        else if (var == 2) needed = momentum > rf.flowgradevalue[m];
        else if (var == 3 && depth > drytol) needed = fabs(eta) > rf.flowgradevalue[m];
        if (needed && level < rf.flowgrademinlevel[m]) return 1;
    }
    double speed = 0.0;
    if (depth > drytol) {
        speed = momentum / depth;
        for (int n = 1; n <= max_num_speeds; ++n)
            if (speed > th_factor * rf.speed_tolerance[n - 1] && level <= n) return 1;
    }
    if (rf.num_flowgrades == 0 && depth > drytol) {
        if (fabs(eta - sea) > th_factor * rf.wave_tolerance) {
            if (level < rf.max_level_deep) return 1;
            if (fabs(b) < rf.deep_depth) return 1;
        }
        if (fabs(b) > rf.deep_depth && speed < rf.speed_tolerance[0]) return 0;
        if (speed / depth > rf.max_velocity_depth_product) return 1;
    }
    return 0;
}

/* One CTA per tag task; refine tasks cover one patch, coarsen tasks the
 * four siblings of a family. */
template <int M>
__global__ void __launch_bounds__(128) tag_kernel(const gf_tag_task* __restrict__ tasks, int ntask,
                                                  const gf_refine* __restrict__ rfp,
                                                  const gf_phys* __restrict__ phys_table,
                                                  int maxlevel, int init_flag, double t,
                                                  int* __restrict__ tags)
{
    using G = AmrGeo<M>;
    const int ti = blockIdx.x;
    if (ti >= ntask) return;
    const gf_tag_task T = tasks[ti];
    const gf_refine& rf = T.rf ? *T.rf : *rfp;
    if (T.rf) {
        maxlevel = T.maxlevel;
        init_flag = T.init_flag;
        t = T.t;
    }
    const gf_phys& P = phys_table[T.phys];
    const bool coarsen = T.nsib == 4;
    __shared__ int verdict;
    if (threadIdx.x == 0) {
        /* parent box for a family from siblings 0 (ll), 1 (lr), 2 (ul) */
        const double xu = coarsen ? T.xlower[1] + M * T.dx : T.xlower[0] + M * T.dx;
        const double yu = coarsen ? T.ylower[2] + M * T.dy : T.ylower[0] + M * T.dy;
        verdict = test_regions(rf, T.level, T.xlower[0], T.ylower[0], xu, yu, t, coarsen ? 0 : 1);
    }
    __syncthreads();
    if (verdict >= 0) {
        if (threadIdx.x == 0) tags[ti] = verdict;
        return;
    }
    int hit = 0;
    for (int s = 0; s < T.nsib; ++s) {
        const double* q = T.q[s];
        const double* a = T.aux[s];
        for (int e = threadIdx.x; e < M * M && !hit; e += blockDim.x) {
            const int k = G::at(1 + e % M, 1 + e / M);
            hit |= flag2refine(P.dry_tolerance, P.sea_level, rf, q[k], q[G::S + k], q[2 * G::S + k],
                               a[k], T.level, maxlevel, init_flag, coarsen) > 0;
        }
    }
    hit = __syncthreads_or(hit);
    if (threadIdx.x == 0) tags[ti] = coarsen ? (hit ? 0 : 1) : (hit ? 1 : 0);
}

} // namespace

cudaError_t launch_transfer(int m, const gf_xfer_task* tasks, int ntask, const gf_phys* phys,
                            cudaStream_t st, const long long* qdelta)
{
    if (ntask <= 0) return cudaSuccess;
    switch (m) {
    case 32: transfer_kernel<32><<<ntask, 128, 0, st>>>(tasks, ntask, phys, qdelta); break;
    case 16: transfer_kernel<16><<<ntask, 128, 0, st>>>(tasks, ntask, phys, qdelta); break;
    case 8: transfer_kernel<8><<<ntask, 128, 0, st>>>(tasks, ntask, phys, qdelta); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_timeinterp(int m, const gf_tinterp_task* tasks, int ntask, double alpha,
                              cudaStream_t st)
{
    if (ntask <= 0) return cudaSuccess;
    switch (m) {
    case 32: timeinterp_kernel<32><<<ntask, 128, 0, st>>>(tasks, ntask, alpha); break;
    case 16: timeinterp_kernel<16><<<ntask, 128, 0, st>>>(tasks, ntask, alpha); break;
    case 8: timeinterp_kernel<8><<<ntask, 128, 0, st>>>(tasks, ntask, alpha); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_tags(int m, const gf_tag_task* tasks, int ntask, const gf_refine* rf,
                        const gf_phys* phys, int maxlevel, int init_flag, double t, int* tags,
                        cudaStream_t st)
{
    if (ntask <= 0) return cudaSuccess;
    switch (m) {
    case 32: tag_kernel<32><<<ntask, 128, 0, st>>>(tasks, ntask, rf, phys, maxlevel, init_flag, t, tags); break;
    case 16: tag_kernel<16><<<ntask, 128, 0, st>>>(tasks, ntask, rf, phys, maxlevel, init_flag, t, tags); break;
    case 8: tag_kernel<8><<<ntask, 128, 0, st>>>(tasks, ntask, rf, phys, maxlevel, init_flag, t, tags); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

} // namespace gf
