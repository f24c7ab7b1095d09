/*
 * Fused GeoClaw patch update for sm_103a: b4step2 + step2 + CFL + src2 on a
 * batch of patches, one CTA per patch.
 *
 * Reference behaviour (paths relative to the GeoFlood source tree):
 *   geoclaw_update              src/fc2d_geoclaw/fc2d_geoclaw.cpp:352-387
 *   b4step2                     fortran_source/geoclaw_b4step2_fort.f90:183-186
 *   step2 sweeps                fortran_source/geoclaw_step2_fort.f90:80-250
 *   flux2 (f-wave form)         fortran_source/geoclaw_flux2fw_fort.f:113-267
 *   limiter / philim            fortran_source/geoclaw_limiter_fort.f:34-58, philim.f
 *   flux-difference update      fortran_source/geoclaw_step2_wrap_fort.f:95-115
 *   src2 (Manning friction)     fortran_source/geoclaw_src2_fort.f90:41-71
 *
 * The kernel computes exactly the faces the interior update depends on:
 * normal solves on faces 0..m+2 of slices 0..m+1, limiting / transverse
 * splitting on faces 1..m+1 (the Fortran's own ranges), and writes the
 * interior cells only. Ghost cells are refilled by the ghost-fill step
 * before they are read again, so their post-step values are not part of
 * the state.
 *
 * The update is FP64-issue bound on GB300 (the FP64 pipe, not HBM, is the
 * ceiling), so the layout of the work aims at few FP64 instructions and
 * uniform warps:
 *   - per-cell quotients computed once (hu/h, hv/h, sqrt(g h), and in the
 *     contracted build 1/h and 1/sqrt(g h));
 *   - the faces of each band are listed by class (both cells wet, grouped
 *     by the wave structure riemanntype will find; one wet; both dry) so a
 *     warp runs one code path; dry faces only store zeros;
 *   - the per-face outputs of a band go to shared memory and each interior
 *     cell gathers its six contributing faces in slice order, so every cell
 *     is written by one thread per band, in a fixed order: deterministic and
 *     independent of launch shape (no atomics on the data).
 *
 * EXACT = true is the parity build: the reference's four flux accumulators
 * fm, fp, gm, gp summed in its order and every division as written; compiled
 * with floating-point contraction off it reproduces the Fortran's rounding.
 */
#ifndef GF_PATCH_UPDATE_CUH
#define GF_PATCH_UPDATE_CUH

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "gf_riemann.cuh"
#include "gf_types.h"

#ifndef GF_KNS
#define GF_KNS gf
#endif

namespace GF_KNS {

/* ---- bulk-async (TMA) copy + mbarrier helpers (inline PTX, sm_90+) ---- */
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
/* Polls of a wait before it gives up: a poll of a phase that does not
 * complete suspends about 3.8 us on GB300 (gf_probe_bounded_wait), so the
 * limit is about half a second, far above any staging copy. */
constexpr uint32_t kWaitPolls = 1u << 17;

/* Bounded wait on phase `parity`; returns false if the limit ran out. */
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_iter)
{
    for (uint32_t it = 0; it < max_iter; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

/* sign(s) * x for the limiter's factor: x with its sign bit flipped when s
 * is negative (-0 included), on the integer pipe instead of a product */
__device__ __forceinline__ double with_sign_of(double x, double s)
{
    const unsigned long long ux = static_cast<unsigned long long>(__double_as_longlong(x));
    const unsigned long long us = static_cast<unsigned long long>(__double_as_longlong(s));
    return __longlong_as_double(static_cast<long long>(ux ^ (us & 0x8000000000000000ull)));
}

/* Order-preserving key of a non-negative double (for atomicMax). */
__device__ __forceinline__ unsigned long long dkey(double v)
{
    return static_cast<unsigned long long>(__double_as_longlong(v));
}

template <int M>
struct Geo {
    static constexpr int N = M + 2 * GF_MBC; /* cells per row incl. halo */
    static constexpr int S = N * N;          /* cells per plane          */
    static constexpr int FA = M + 3;         /* normal-solve faces/slice */
    static constexpr int FB = M + 1;         /* limited faces / slice    */
    static constexpr int NSLICE = M + 2;     /* slices 0..m+1            */
};

/* Shared-memory layout (doubles unless noted). NACC flux accumulators of 3
 * components per interior cell: 2 (DX, DY) in the contracted build, 4 (fm,
 * fp, gm, gp) in the exact build. The contracted build also keeps 1/h and
 * 1/sqrt(g h) planes. */
template <int M, int RB, bool EXACT = false>
struct Smem {
    using G = Geo<M>;
    static constexpr int NACC = EXACT ? 4 : 2;
    static constexpr int NBAND = (G::NSLICE + RB - 1) / RB;
    /* Odd strides (in doubles) spread a warp's accesses to face records and
     * accumulator rows over the shared-memory banks. */
    static constexpr int W_STRIDE = 13; /* s[3] + fw[3][3], 1 pad            */
    /* limited-face records: exact build faddm faddp A B C D (3 comps each, 1
     * pad); contracted build amdq apdq cq (local order) */
    static constexpr int O_STRIDE = EXACT ? 19 : 9;
    /* per-cell records of the contracted build: N (flux difference), U (up-going
     * and Dn (down-going transverse parts), global order, one slot per face slot */
    static constexpr int C_STRIDE = 9;
    static constexpr int MS = M + 1;    /* accumulator row stride            */
    static constexpr int PLANE = M * MS; /* one accumulator component        */
    static constexpr int OFF_H = 0;
    static constexpr int OFF_HU = OFF_H + G::S;
    static constexpr int OFF_HV = OFF_HU + G::S;
    static constexpr int OFF_B = OFF_HV + G::S;
    static constexpr int OFF_U = OFF_B + G::S;
    static constexpr int OFF_V = OFF_U + G::S;
    static constexpr int OFF_C = OFF_V + G::S;
    static constexpr int OFF_RH = OFF_C + G::S;                     /* contracted only */
    static constexpr int OFF_RC = OFF_RH + (EXACT ? 0 : G::S);      /* contracted only */
    static constexpr int OFF_ACC = OFF_RC + (EXACT ? 0 : G::S);     /* NACC x [3][M*M] */
    static constexpr int OFF_W = OFF_ACC + NACC * 3 * PLANE;
    static constexpr int OFF_O = OFF_W + RB * G::FA * W_STRIDE;
    static constexpr int OFF_C2 = OFF_O + RB * G::FB * O_STRIDE;   /* contracted only */
    static constexpr int OFF_RED = OFF_C2 + (EXACT ? 0 : RB * G::FB * C_STRIDE); /* 2*32 doubles */
    static constexpr int OFF_BAR = OFF_RED + 64;                    /* 1 x u64     */
    /* integer region: class counts per band and face lists (u16) */
    static constexpr int OFF_INT = OFF_BAR + 2;
    static constexpr int NCLS = 5;                                  /* face classes, see build_lists */
    static constexpr int CNT_INTS = NBAND * 2 * NCLS * 2;           /* [band][A|B][class][count|pos] */
    static constexpr int LIST_A = G::NSLICE * G::FA;
    static constexpr int LIST_B = G::NSLICE * G::FB;
    static constexpr size_t INT_BYTES = ((CNT_INTS * 4 + (LIST_A + LIST_B) * 2) + 15) / 16 * 16;
    static constexpr size_t OFF_WET_BYTES = (size_t)OFF_INT * 8 + INT_BYTES;
    /* class of each normal-solve face of the sweep (u8), kept between the
     * count and place passes */
    static constexpr size_t OFF_FCLS_BYTES = OFF_WET_BYTES + ((G::S + 15) / 16) * 16;
    static constexpr size_t BYTES = OFF_FCLS_BYTES + ((LIST_A + 15) / 16) * 16;
};

/* Load the cell view for a face sweep in direction DIR (0 = x, 1 = y). */
template <int DIR, bool EXACT, class L>
__device__ __forceinline__ gf_cell load_cell(const double* sm, const unsigned char* wet, int k)
{
    gf_cell c;
    c.h = sm[L::OFF_H + k];
    c.b = sm[L::OFF_B + k];
    c.c = sm[L::OFF_C + k];
    c.wet = wet[k] != 0;
    if (DIR == 0) {
        c.hun = sm[L::OFF_HU + k]; c.hut = sm[L::OFF_HV + k];
        c.un = sm[L::OFF_U + k];   c.ut = sm[L::OFF_V + k];
    } else {
        c.hun = sm[L::OFF_HV + k]; c.hut = sm[L::OFF_HU + k];
        c.un = sm[L::OFF_V + k];   c.ut = sm[L::OFF_U + k];
    }
    if (!EXACT) {
        c.rh = sm[L::OFF_RH + k];
        c.rc = sm[L::OFF_RC + k];
    } else {
        c.rh = 0.0;
        c.rc = 0.0;
    }
    return c;
}

/* The faces one sweep computes when a work item updates only the interior
 * rows rlo..rhi of its patch (the whole patch: rlo = 1, rhi = M). The x
 * sweep takes the slices (rows) rlo-1..rhi+1 with all their faces; the y
 * sweep takes every slice (column) with the normal-solve faces rlo-1..rhi+2
 * and the limited faces rlo..rhi+1, which are exactly the faces whose
 * records the update of rows rlo..rhi reads. Records of a band are packed
 * by the window's faces per slice (fa, fb), so a band holds rb slices
 * within the same shared-memory records as a whole-patch band of RB. For
 * rlo = 1, rhi = M every field is the whole-patch constant. */
template <int M, int RB, int DIR>
struct SweepWin {
    int ts_lo, nsl; /* slices ts_lo .. ts_lo + nsl - 1                  */
    int na_lo, fa;  /* normal-solve faces na_lo .. na_lo + fa - 1        */
    int nb_lo, fb;  /* limited faces nb_lo .. nb_lo + fb - 1             */
    int rb;         /* slices per band                                   */
    __device__ __forceinline__ SweepWin(int rlo, int rhi)
    {
        if (DIR == 0) {
            ts_lo = rlo - 1; nsl = rhi - rlo + 3;
            na_lo = 0; fa = M + 3;
            nb_lo = 1; fb = M + 1;
            rb = RB;
        } else {
            ts_lo = 0; nsl = M + 2;
            na_lo = rlo - 1; fa = rhi - rlo + 4;
            nb_lo = rlo; fb = rhi - rlo + 2;
            rb = min(RB * (M + 3) / fa, RB * (M + 1) / fb);
        }
    }
};

/* Build, for every band of one sweep direction, the normal-solve faces
 * (list A) and the limited faces (list B) ordered by class, so that a warp
 * runs one code path. Classes: 0..2 both cells wet, by the wave structure
 * riemanntype will find (0 two shocks, the costly branch, first so that one
 * class boundary at most splits its warps; 1 two rarefactions; 2 a shock
 * and a rarefaction; list B puts all wet pairs in class 0); 3 one cell wet;
 * 4 both dry. The wave structure is estimated without a square root (F_max <= 0 as
 * delu <= 0 and delu^2 hmin hmax >= (hmax - hmin)^2 g (hmin + hmax) / 2); a
 * borderline face in the neighbouring class only costs divergence, since
 * every face's solve is the same computation wherever it is listed. Two
 * passes (count, then place) over all faces. */
template <int M, int NT, int RB, int DIR, bool EXACT>
__device__ __forceinline__ void build_lists(const double* sm, const unsigned char* wet, int* cnt, uint16_t* la,
                                            uint16_t* lb, double g, const SweepWin<M, RB, DIR>& w)
{
    using G = Geo<M>;
    using L = Smem<M, RB, EXACT>;
    constexpr int N = G::N;
    constexpr int NC = L::NCLS;
    unsigned char* fcls = const_cast<unsigned char*>(reinterpret_cast<const unsigned char*>(sm)) + L::OFF_FCLS_BYTES;
    auto cidx = [](int n, int t) -> int {
        return DIR == 0 ? (t + 1) * N + (n + 1) : (n + 1) * N + (t + 1);
    };
    /* cnt layout: [band][list 0|1][class 0..4][0 = count, 1 = position] */
    auto C = [&](int band, int list, int cls, int w2) -> int& {
        return cnt[((band * 2 + list) * NC + cls) * 2 + w2];
    };
    for (int k = threadIdx.x; k < L::CNT_INTS; k += NT) cnt[k] = 0;
    __syncthreads();
    for (int f = threadIdx.x; f < w.nsl * w.fa; f += NT) {
        const int ts = f / w.fa, n = w.na_lo + f % w.fa;
        const int t = w.ts_lo + ts;
        const int kl = cidx(n - 1, t), kr = cidx(n, t);
        const int nw = wet[kl] + wet[kr];
        int cls = nw == 0 ? 4 : nw == 1 ? 3 : 0;
        if (nw == 2 && EXACT) {
            const double hL = sm[L::OFF_H + kl], hR = sm[L::OFF_H + kr];
            const double uL = sm[(DIR == 0 ? L::OFF_U : L::OFF_V) + kl];
            const double uR = sm[(DIR == 0 ? L::OFF_U : L::OFF_V) + kr];
            const double cL = sm[L::OFF_C + kl], cR = sm[L::OFF_C + kr];
            constexpr bool F = false;
            const double delu = uR - uL;
            const double hmin = d_min<F>(hL, hR), hmax = d_max<F>(hL, hR);
            const double dh = hmax - hmin;
            if (d_gtz<F>(delu + 2.0 * (d_min<F>(cL, cR) - d_max<F>(cL, cR)))) cls = 1;
            else if (d_lez<F>(delu) && d_ge<F>(delu * delu * (hmin * hmax), dh * dh * (0.5 * g) * (hmin + hmax)))
                cls = 0;
            else cls = 2;
        } else if (nw == 2) {
            /* The class only orders the list (a face in the neighbouring
             * class costs divergence, not bits), so the contracted build
             * estimates it in single precision off the FP64 pipe. */
            const float hL = __double2float_rn(sm[L::OFF_H + kl]), hR = __double2float_rn(sm[L::OFF_H + kr]);
            const float uL = __double2float_rn(sm[(DIR == 0 ? L::OFF_U : L::OFF_V) + kl]);
            const float uR = __double2float_rn(sm[(DIR == 0 ? L::OFF_U : L::OFF_V) + kr]);
            const float cL = __double2float_rn(sm[L::OFF_C + kl]), cR = __double2float_rn(sm[L::OFF_C + kr]);
            const float delu = uR - uL;
            const float hmin = fminf(hL, hR), hmax = fmaxf(hL, hR);
            const float dh = hmax - hmin;
            if (delu + 2.0f * (fminf(cL, cR) - fmaxf(cL, cR)) > 0.0f) cls = 1;
            else if (delu <= 0.0f &&
                     delu * delu * (hmin * hmax) >= dh * dh * (0.5f * (float)g) * (hmin + hmax))
                cls = 0;
            else cls = 2;
        }
        fcls[f] = (unsigned char)cls;
        atomicAdd(&C(ts / w.rb, 0, cls, 0), 1);
    }
    for (int f = threadIdx.x; f < w.nsl * w.fb; f += NT) {
        const int ts = f / w.fb, n = w.nb_lo + f % w.fb;
        const int t = w.ts_lo + ts;
        const int nw = wet[cidx(n - 1, t)] + wet[cidx(n, t)];
        atomicAdd(&C(ts / w.rb, 1, nw == 0 ? 4 : nw == 1 ? 3 : 0, 0), 1);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < L::NBAND * 2; e += NT) {
        const int band = e >> 1, list = e & 1;
        int acc = 0;
        for (int cls = 0; cls < NC; ++cls) {
            C(band, list, cls, 1) = acc;
            acc += C(band, list, cls, 0);
        }
    }
    __syncthreads();
    for (int f = threadIdx.x; f < w.nsl * w.fa; f += NT) {
        const int band = (f / w.fa) / w.rb;
        const int pos = atomicAdd(&C(band, 0, fcls[f], 1), 1);
        la[band * w.rb * w.fa + pos] = (uint16_t)(f - band * w.rb * w.fa);
    }
    for (int f = threadIdx.x; f < w.nsl * w.fb; f += NT) {
        const int ts = f / w.fb, n = w.nb_lo + f % w.fb;
        const int t = w.ts_lo + ts;
        const int nw = wet[cidx(n - 1, t)] + wet[cidx(n, t)];
        const int band = ts / w.rb;
        const int pos = atomicAdd(&C(band, 1, nw == 0 ? 4 : nw == 1 ? 3 : 0, 1), 1);
        lb[band * w.rb * w.fb + pos] = (uint16_t)(f - band * w.rb * w.fb);
    }
    __syncthreads();
}

/* One sweep direction over all slices, banded. Accumulates into the flux
 * accumulators; returns this thread's max |s| over normal faces. */
template <int M, int NT, int RB, int DIR, bool EXACT>
__device__ __forceinline__ double sweep(double* sm, const unsigned char* wet, int* cnt,
                                        uint16_t* la, uint16_t* lb, const gf_phys& P, double dtdn,
                                        double c16g, double rsg, double crit, double crit2,
                                        int rlo, int rhi)
{
    using G = Geo<M>;
    using L = Smem<M, RB, EXACT>;
    constexpr int N = G::N;
    constexpr bool FAST = !EXACT;
    double* W = sm + L::OFF_W;
    double* O = sm + L::OFF_O;
    const double g = P.grav, drytol = P.dry_tolerance;
    const double half_dtdn = 0.5 * dtdn;
    /* local component l -> global component (h, hu, hv) */
    constexpr int G1 = (DIR == 0) ? 1 : 2; /* normal momentum     */
    constexpr int G2 = (DIR == 0) ? 2 : 1; /* transverse momentum */
    constexpr int MM = L::PLANE; /* component stride of the accumulators */
    double smax = 0.0;

    auto cidx = [](int n, int t) -> int {
        return DIR == 0 ? (t + 1) * N + (n + 1) : (n + 1) * N + (t + 1);
    };
    auto aidx = [](int n, int t) -> int {
        return DIR == 0 ? (n - 1) + L::MS * (t - 1) : (t - 1) + L::MS * (n - 1);
    };
    auto C = [&](int band, int list, int cls) -> int {
        return cnt[((band * 2 + list) * L::NCLS + cls) * 2 + 0];
    };

    const SweepWin<M, RB, DIR> win(rlo, rhi);
    const int fa = win.fa, fb = win.fb;
    build_lists<M, NT, RB, DIR, EXACT>(sm, wet, cnt, la, lb, g, win);
    /* cells the gather writes: slice-direction t clamped to the window's rows
     * in the x sweep, cell-direction n clamped to them in the y sweep */
    const int gt_lo = DIR == 0 ? rlo : 1, gt_hi = DIR == 0 ? rhi : M;
    const int gn_lo = DIR == 0 ? 1 : rlo, gn_hi = DIR == 0 ? M : rhi;
    /* record of limited face `face` (nb_lo..) of band slice ts */
    auto orec = [&](int ts, int face) -> const double* {
        return O + (ts * fb + (face - win.nb_lo)) * L::O_STRIDE;
    };
    /* per-cell record of cell `cell` of band slice ts (contracted build) */
    double* C2 = sm + L::OFF_C2;
    auto crec = [&](int ts, int cell) -> double* {
        return C2 + (ts * fb + (cell - win.nb_lo)) * L::C_STRIDE;
    };

    /* Contracted build: DX, DY. Exact build: fm(i+1,j), fp(i,j), gm(i,j+1),
     * gp(i,j) of the reference, in sweep coordinates N_M, N_P (normal) and
     * T_M, T_P (transverse), each summed in the reference's order (slices in
     * increasing order, x sweeps before y sweeps). */
    double* ACCN = sm + L::OFF_ACC + (DIR == 0 ? 0 : 3 * MM);
    double* ACCT = sm + L::OFF_ACC + (DIR == 0 ? 3 * MM : 0);
    double* NM = sm + L::OFF_ACC + (DIR == 0 ? 0 : 6 * MM);
    double* NP = NM + 3 * MM;
    double* TM = sm + L::OFF_ACC + (DIR == 0 ? 6 * MM : 0);
    double* TP = TM + 3 * MM;

    auto gather = [&](int t0, int t1) {
        /* slices t0..t1 feed cells n in [1, M], t in [t0-1, t1+1] (interior),
         * within the window */
        const int ta = max(gt_lo, t0 - 1), tb = min(gt_hi, t1 + 1);
        const int nn = gn_hi - gn_lo + 1;
        const int cnt_c = (tb - ta + 1) * nn;
        for (int e = threadIdx.x; e < cnt_c; e += NT) {
            const int t = ta + e / nn;
            const int n = gn_lo + e % nn;
            const int a = aidx(n, t);
            if (EXACT) {
                if (t - 1 >= t0 && t - 1 <= t1) { /* slice below: up-going parts */
                    const double* fr = orec(t - 1 - t0, n + 1);
                    const double* fl = orec(t - 1 - t0, n);
#pragma unroll
                    for (int c = 0; c < 3; ++c) TP[a + c * MM] += (0.0 - fr[9 + c]) - fl[15 + c];
                }
                if (t >= t0 && t <= t1) {
                    const double* fr = orec(t - t0, n + 1);
                    const double* fl = orec(t - t0, n);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        NM[a + c * MM] += fr[c];
                        NP[a + c * MM] += fl[3 + c];
                        TM[a + c * MM] += (0.0 - fr[9 + c]) - fl[15 + c];
                        TP[a + c * MM] += (0.0 - fr[6 + c]) - fl[12 + c];
                    }
                }
                if (t + 1 >= t0 && t + 1 <= t1) { /* slice above: down-going parts */
                    const double* fr = orec(t + 1 - t0, n + 1);
                    const double* fl = orec(t + 1 - t0, n);
#pragma unroll
                    for (int c = 0; c < 3; ++c) TM[a + c * MM] += (0.0 - fr[6 + c]) - fl[12 + c];
                }
            } else {
                /* each slice's part enters the accumulators on its own, slices in
                 * increasing order, so the sums do not depend on where the band
                 * boundaries fall: every tile shape gives the same bits. A
                 * slice's per-cell record holds its flux difference N and the
                 * up-going (U) and down-going (Dn) transverse parts. */
                if (t - 1 >= t0 && t - 1 <= t1) { /* slice below: up-going parts */
                    const double* r = crec(t - 1 - t0, n);
                    ACCT[a] += half_dtdn * r[3];
                    ACCT[a + MM] += half_dtdn * r[4];
                    ACCT[a + 2 * MM] += half_dtdn * r[5];
                }
                if (t >= t0 && t <= t1) {
                    const double* r = crec(t - t0, n);
                    ACCN[a] += r[0];
                    ACCN[a + MM] += r[1];
                    ACCN[a + 2 * MM] += r[2];
                    ACCT[a] += half_dtdn * (r[6] - r[3]);
                    ACCT[a + MM] += half_dtdn * (r[7] - r[4]);
                    ACCT[a + 2 * MM] += half_dtdn * (r[8] - r[5]);
                }
                if (t + 1 >= t0 && t + 1 <= t1) { /* slice above: down-going parts */
                    const double* r = crec(t + 1 - t0, n);
                    ACCT[a] -= half_dtdn * r[6];
                    ACCT[a + MM] -= half_dtdn * r[7];
                    ACCT[a + 2 * MM] -= half_dtdn * r[8];
                }
            }
        }
    };

    /* a2 / b2 both cells wet (list A by wave structure), a1 / b1 one wet,
     * a0 / b0 both dry */
    auto counts_a = [&](int band, int& a2, int& a1, int& a0) {
        a2 = C(band, 0, 0) + C(band, 0, 1) + C(band, 0, 2);
        a1 = C(band, 0, 3);
        a0 = C(band, 0, 4);
    };
    auto counts_b = [&](int band, int& b2, int& b1, int& b0) {
        b2 = C(band, 1, 0);
        b1 = C(band, 1, 3);
        b0 = C(band, 1, 4);
    };

    /* ---- stage A: normal Riemann solves, faces 0..M+2, by class ---- */
    auto stage_a = [&](int t0, int band) {
        const uint16_t* lA = la + band * win.rb * fa;
        int a2, a1, a0;
        counts_a(band, a2, a1, a0);
        for (int idx = threadIdx.x; idx < a2 + a1 + a0; idx += NT) {
            const int f = lA[idx];
            double* w = W + f * L::W_STRIDE;
            if (idx >= a2 + a1) { /* both cells dry: no waves */
#pragma unroll
                for (int q = 0; q < L::W_STRIDE; ++q) w[q] = 0.0;
                continue;
            }
            const int t = t0 + f / fa;
            const int n = win.na_lo + f % fa;
            const gf_cell cl = load_cell<DIR, EXACT, L>(sm, wet, cidx(n - 1, t));
            const gf_cell cr = load_cell<DIR, EXACT, L>(sm, wet, cidx(n, t));
            double s[3], fw[3][3];
            gf_rpn2_face<FAST>(cl, cr, g, drytol, c16g, rsg, crit, crit2, s, fw);
#pragma unroll
            for (int mw = 0; mw < 3; ++mw) {
                w[mw] = s[mw];
                w[3 + 3 * mw + 0] = fw[mw][0];
                w[3 + 3 * mw + 1] = fw[mw][1];
                w[3 + 3 * mw + 2] = fw[mw][2];
                smax = d_max_nn<FAST>(smax, fabs(s[mw]));
            }
        }
    };

    /* Fluctuations from the unlimited f-waves (rpn2_geoclaw.f:359-376) and
     * the limited second-order term cqxx of one face (flux2: limiter.f /
     * philim.f and the correction loop). The middle f-wave is (0, beta2, 0) in
     * local order: the contracted build skips its two zero components (adding
     * +0.0 to a sum that starts at +0.0 changes no bits). */
    auto face_terms = [&](const double* wc, double amdq[3], double apdq[3], double cq[3]) {
        double s[3], fw[3][3];
#pragma unroll
        for (int mw = 0; mw < 3; ++mw) {
            s[mw] = wc[mw];
            fw[mw][0] = wc[3 + 3 * mw]; fw[mw][1] = wc[4 + 3 * mw]; fw[mw][2] = wc[5 + 3 * mw];
        }
        amdq[0] = amdq[1] = amdq[2] = 0.0;
        apdq[0] = apdq[1] = apdq[2] = 0.0;
        cq[0] = cq[1] = cq[2] = 0.0;
#pragma unroll
        for (int mw = 0; mw < 3; ++mw) {
            if (FAST && mw == 1) {
                if (d_ltz<FAST>(s[1])) {
                    amdq[1] += fw[1][1];
                } else if (d_gtz<FAST>(s[1])) {
                    apdq[1] += fw[1][1];
                } else {
                    amdq[1] += 0.5 * fw[1][1];
                    apdq[1] += 0.5 * fw[1][1];
                }
                continue;
            }
            if (FAST && mw == 0) { /* into zero sums: assigned (a zero's sign aside) */
                if (d_ltz<FAST>(s[0])) {
                    amdq[0] = fw[0][0]; amdq[1] = fw[0][1]; amdq[2] = fw[0][2];
                } else if (d_gtz<FAST>(s[0])) {
                    apdq[0] = fw[0][0]; apdq[1] = fw[0][1]; apdq[2] = fw[0][2];
                } else {
                    amdq[0] = 0.5 * fw[0][0]; amdq[1] = 0.5 * fw[0][1]; amdq[2] = 0.5 * fw[0][2];
                    apdq[0] = amdq[0]; apdq[1] = amdq[1]; apdq[2] = amdq[2];
                }
                continue;
            }
            if (d_ltz<FAST>(s[mw])) {
                amdq[0] += fw[mw][0]; amdq[1] += fw[mw][1]; amdq[2] += fw[mw][2];
            } else if (d_gtz<FAST>(s[mw])) {
                apdq[0] += fw[mw][0]; apdq[1] += fw[mw][1]; apdq[2] += fw[mw][2];
            } else {
                amdq[0] += 0.5 * fw[mw][0]; amdq[1] += 0.5 * fw[mw][1]; amdq[2] += 0.5 * fw[mw][2];
                apdq[0] += 0.5 * fw[mw][0]; apdq[1] += 0.5 * fw[mw][1]; apdq[2] += 0.5 * fw[mw][2];
            }
        }
        if (P.order == 1) return;
        const double* wl = wc - L::W_STRIDE; /* face n-1 */
        const double* wr = wc + L::W_STRIDE; /* face n+1 */
#pragma unroll
        for (int mw = 0; mw < 3; ++mw) {
            const double* fa = fw[mw];
            if (FAST && mw == 1) {
                /* the middle wave has one non-zero component: its norm and
                 * projections are single products */
                double lim = 1.0;
                const double a = fa[1];
                if (P.mthlim[1] != 0) {
                    const double wnorm2 = a * a;
                    if (!d_eqz<FAST>(wnorm2)) {
                        /* the upwind neighbour's projection only */
                        const double up = d_gtz<FAST>(s[1]) ? (wl + 3 + 3)[1] : (wr + 3 + 3)[1];
                        lim = gf_philim<FAST>(wnorm2, up * a, P.mthlim[1]);
                    }
                }
                const double fac = with_sign_of(1.0 - fabs(s[1]) * dtdn, s[1]);
                cq[1] += (fac * lim) * a;
                continue;
            }
            double lim = 1.0;
            if (P.mthlim[mw] != 0) {
                /* dot products in the global (h, hu, hv) order */
                const double a0 = fa[0], a1 = (DIR == 0) ? fa[1] : fa[2], a2 = (DIR == 0) ? fa[2] : fa[1];
                const double* ql = wl + 3 + 3 * mw;
                const double* qr = wr + 3 + 3 * mw;
                const double l0 = ql[0], l1 = (DIR == 0) ? ql[1] : ql[2], l2 = (DIR == 0) ? ql[2] : ql[1];
                const double r0 = qr[0], r1 = (DIR == 0) ? qr[1] : qr[2], r2 = (DIR == 0) ? qr[2] : qr[1];
                const double wnorm2 = a0 * a0 + a1 * a1 + a2 * a2;
                if (!d_eqz<FAST>(wnorm2)) {
                    /* the upwind neighbour's projection only (the same
                     * products in the same order) */
                    const bool up = d_gtz<FAST>(s[mw]);
                    const double p0 = up ? l0 : r0, p1 = up ? l1 : r1, p2 = up ? l2 : r2;
                    const double dot = p0 * a0 + p1 * a1 + p2 * a2;
                    lim = gf_philim<FAST>(wnorm2, dot, P.mthlim[mw]);
                }
            }
            const double fac = FAST ? with_sign_of(1.0 - fabs(s[mw]) * dtdn, s[mw])
                                    : copysign(1.0, s[mw]) * (1.0 - fabs(s[mw]) * dtdn);
            if (FAST) {
                const double fl = fac * lim;
                cq[0] += fl * fa[0];
                cq[1] += fl * fa[1];
                cq[2] += fl * fa[2];
            } else {
                cq[0] += fac * (lim * fa[0]);
                cq[1] += fac * (lim * fa[1]);
                cq[2] += fac * (lim * fa[2]);
            }
        }
    };

    /* ---- exact build, stage B: limiter, 2nd-order terms, both transverse
     * splits of every face (flux2's per-face order) ---- */
    auto stage_b_exact = [&](int t0, int band) {
        const uint16_t* lB = lb + band * win.rb * fb;
        int b2, b1, b0;
        counts_b(band, b2, b1, b0);
        for (int idx = threadIdx.x; idx < b2 + b1 + b0; idx += NT) {
            const int f = lB[idx];
            double* o = O + f * L::O_STRIDE;
            if (idx >= b2 + b1) {
#pragma unroll
                for (int q = 0; q < L::O_STRIDE; ++q) o[q] = 0.0;
                continue;
            }
            const int t = t0 + f / fb;
            const int n = win.nb_lo + f % fb;
            const int kl = cidx(n - 1, t), kr = cidx(n, t);
            const double* wc = W + ((t - t0) * fa + (n - win.na_lo)) * L::W_STRIDE;
            double amdq[3], apdq[3], cq[3];
            face_terms(wc, amdq, apdq, cq);
            double faddm[3] = {amdq[0], amdq[1], amdq[2]};
            double faddp[3] = {-apdq[0], -apdq[1], -apdq[2]};
            if (P.order != 1) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    faddm[c] += 0.5 * cq[c];
                    faddp[c] += 0.5 * cq[c];
                }
                if (P.transverse == 2) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        amdq[c] += cq[c];
                        apdq[c] -= cq[c];
                    }
                }
            }
            double A[3] = {0, 0, 0}, B[3] = {0, 0, 0}, Cc[3] = {0, 0, 0}, D[3] = {0, 0, 0};
            if (P.transverse != 0) {
                double bm[3], bp[3];
                if (wet[kl]) { /* rpt2 imp=1: left-going part into cell n-1 */
                    const gf_cell cl = load_cell<DIR, EXACT, L>(sm, wet, kl);
                    gf_rpt2_face<FAST>(cl, sm[L::OFF_B + cidx(n - 1, t - 1)],
                                       sm[L::OFF_B + cidx(n - 1, t + 1)], drytol, amdq, bm, bp);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        A[c] = half_dtdn * bm[c];
                        B[c] = half_dtdn * bp[c];
                    }
                }
                if (wet[kr]) { /* rpt2 imp=2: right-going part into cell n */
                    const gf_cell cr = load_cell<DIR, EXACT, L>(sm, wet, kr);
                    gf_rpt2_face<FAST>(cr, sm[L::OFF_B + cidx(n, t - 1)],
                                       sm[L::OFF_B + cidx(n, t + 1)], drytol, apdq, bm, bp);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        Cc[c] = half_dtdn * bm[c];
                        D[c] = half_dtdn * bp[c];
                    }
                }
            }
            /* write in global component order (h, hu, hv) */
            o[0] = faddm[0]; o[G1] = faddm[1]; o[G2] = faddm[2];
            o[3] = faddp[0]; o[3 + G1] = faddp[1]; o[3 + G2] = faddp[2];
            o[6] = A[0]; o[6 + G1] = A[1]; o[6 + G2] = A[2];
            o[9] = B[0]; o[9 + G1] = B[1]; o[9 + G2] = B[2];
            o[12] = Cc[0]; o[12 + G1] = Cc[1]; o[12 + G2] = Cc[2];
            o[15] = D[0]; o[15 + G1] = D[1]; o[15 + G2] = D[2];
        }
    };

    /* ---- contracted build, stage B1: per limited face, the fluctuations
     * amdq, apdq and the limited second-order term cq (local order) ---- */
    auto stage_b1 = [&](int t0, int band) {
        const uint16_t* lB = lb + band * win.rb * fb;
        int b2, b1, b0;
        counts_b(band, b2, b1, b0);
        for (int idx = threadIdx.x; idx < b2 + b1 + b0; idx += NT) {
            const int f = lB[idx];
            double* o = O + f * L::O_STRIDE;
            if (idx >= b2 + b1) {
#pragma unroll
                for (int q = 0; q < L::O_STRIDE; ++q) o[q] = 0.0;
                continue;
            }
            const int t = t0 + f / fb;
            const int n = win.nb_lo + f % fb;
            const double* wc = W + ((t - t0) * fa + (n - win.na_lo)) * L::W_STRIDE;
            double amdq[3], apdq[3], cq[3];
            face_terms(wc, amdq, apdq, cq);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                o[c] = amdq[c];
                o[3 + c] = apdq[c];
                o[6 + c] = cq[c];
            }
        }
    };

    /* ---- contracted build, stage B2: per cell n of each band slice, from
     * its faces n (apdq, cq) and n+1 (amdq, cq): the flux difference
     * N = faddm(n+1) - faddp(n) = P + Q/2 with P = amdq(n+1) + apdq(n),
     * Q = cq(n+1) - cq(n), and the transverse split of the fluctuations that
     * enter the cell. rpt2 is linear in its input and the cell alone decides
     * its branches, so the splits of amdq(n+1) and apdq(n) (with the
     * second-order terms for transverse = 2) are one split of their sum
     * P + Q (P for transverse = 1): bm is the down-going part Dn, bp the
     * up-going part U, equal to the sum of the reference's two splits up to
     * rounding. ---- */
    auto stage_b2 = [&](int t0, int t1) {
        const int ncell = fb - 1;
        const int cnt_c = (t1 - t0 + 1) * ncell;
        for (int e = threadIdx.x; e < cnt_c; e += NT) {
            const int ts = e / ncell;
            const int n = win.nb_lo + e % ncell;
            const int t = t0 + ts;
            const int k = cidx(n, t);
            double* r = crec(ts, n);
            if (!(wet[cidx(n - 1, t)] | wet[k] | wet[cidx(n + 1, t)])) {
                /* faces n and n+1 both between dry cells: no waves */
#pragma unroll
                for (int q = 0; q < L::C_STRIDE; ++q) r[q] = 0.0;
                continue;
            }
            const double* orr = O + (ts * fb + (n + 1 - win.nb_lo)) * L::O_STRIDE; /* face n+1 */
            const double* orl = O + (ts * fb + (n - win.nb_lo)) * L::O_STRIDE;     /* face n   */
            double Pv[3], Qv[3], Nv[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                Pv[c] = orr[c] + orl[3 + c];
                Qv[c] = orr[6 + c] - orl[6 + c];
                Nv[c] = Pv[c] + 0.5 * Qv[c];
            }
            double bm[3] = {0.0, 0.0, 0.0}, bp[3] = {0.0, 0.0, 0.0};
            if (P.transverse != 0 && wet[k]) {
                double x[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) x[c] = P.transverse == 2 ? Pv[c] + Qv[c] : Pv[c];
                const gf_cell cc = load_cell<DIR, EXACT, L>(sm, wet, k);
                gf_rpt2_face<FAST>(cc, sm[L::OFF_B + cidx(n, t - 1)], sm[L::OFF_B + cidx(n, t + 1)], drytol, x,
                                   bm, bp);
            }
            /* global component order (h, hu, hv) */
            r[0] = Nv[0]; r[G1] = Nv[1]; r[G2] = Nv[2];
            r[3] = bp[0]; r[3 + G1] = bp[1]; r[3 + G2] = bp[2];
            r[6] = bm[0]; r[6 + G1] = bm[1]; r[6 + G2] = bm[2];
        }
    };

    const int ts_end = win.ts_lo + win.nsl;
    int prev_t0 = -1, prev_t1 = -1;
    if (EXACT) {
        for (int t0 = win.ts_lo, band = 0; t0 < ts_end; t0 += win.rb, ++band) {
            const int t1 = min(t0 + win.rb, ts_end) - 1; /* last slice of band */
            stage_a(t0, band);
            if (prev_t0 >= 0) gather(prev_t0, prev_t1);
            __syncthreads();
            stage_b_exact(t0, band);
            __syncthreads();
            prev_t0 = t0;
            prev_t1 = t1;
        }
        gather(prev_t0, prev_t1);
        __syncthreads();
        return smax;
    }
    /* Contracted build, pipelined over bands with two barriers per band:
     * [stage A of band b | B2 of band b-1], [B1 of band b | gather of band
     * b-1]. Each stage reads what the phase before the last barrier wrote. */
    for (int t0 = win.ts_lo, band = 0;; t0 += win.rb, ++band) {
        const bool have = t0 < ts_end;
        const int t1 = have ? min(t0 + win.rb, ts_end) - 1 : -1;
        if (have) stage_a(t0, band);
        if (prev_t0 >= 0) stage_b2(prev_t0, prev_t1);
        __syncthreads();
        if (have) stage_b1(t0, band);
        if (prev_t0 >= 0) gather(prev_t0, prev_t1);
        __syncthreads();
        if (!have) break;
        prev_t0 = t0;
        prev_t1 = t1;
    }
    return smax;
}

/* Manning friction source term on one interior cell (geoclaw_src2_fort.f90:41-71).
 * The contracted build forms h^(-7/3) = y^7 from y = h^(-1/3) and one
 * reciprocal of 1 + dt gamma instead of pow and three divisions: y by
 * Newton's iteration for the inverse cube root, y <- y + y (1 - h y^3) / 3,
 * two steps from the single-precision value (each step doubles the correct
 * bits, 23 -> 46 -> the FP64 rounding), so no FP64 division or cube root
 * is taken. */
template <bool FAST>
__device__ __forceinline__ void src2_cell(const gf_phys& P, double dt, double bathy, double nvar,
                                          double& h, double& hu, double& hv)
{
    if (!P.friction_forcing) return;
    if (h < 1.0e-30) {
        hu = 0.0;
        hv = 0.0;
    } else if (h <= P.friction_depth) {
        double coeff = 0.0;
        if (!P.variable_friction) {
            for (int nman = P.num_manning; nman >= 1; --nman)
                if (bathy < P.manning_break[nman - 1]) coeff = P.manning_coefficient[nman - 1];
        } else {
            coeff = nvar;
        }
        if (FAST) {
            /* 1e-30 <= h here: a normal single-precision number */
            double y = (double)rcbrtf((float)h);
#pragma unroll
            for (int it = 0; it < 2; ++it) {
                const double e = fma(-h, (y * y) * y, 1.0);
                y = fma(y * (1.0 / 3.0), e, y);
            }
            const double y2 = y * y;
            const double hm73 = ((y2 * y2) * y2) * y; /* h^(-7/3) */
            const double gamma = d_sqrt<FAST>(hu * hu + hv * hv) * P.grav * (coeff * coeff) * hm73;
            const double rdg = gf_rcp(1.0 + dt * gamma);
            hu = hu * rdg;
            hv = hv * rdg;
        } else {
            const double gamma =
                sqrt(hu * hu + hv * hv) * P.grav * (coeff * coeff) / pow(h, 7.0 / 3.0);
            const double dgamma = 1.0 + dt * gamma;
            hu = hu / dgamma;
            hv = hv / dgamma;
        }
    }
}

/* One work item of the fused update: stage the patch, b4step2, both face
 * sweeps, flux differencing + src2, CFL. All threads of the CTA take part;
 * returns false (on every thread) when the staging copy's wait timed out,
 * after the error flag is set and the copy has landed or been waited for. */
template <int M, int NT, int RB, bool EXACT>
__device__ __forceinline__ bool patch_item(double* sm, uint64_t* bar, uint32_t& phase, gf_patch_work wk,
                                           int wi, const gf_phys* __restrict__ phys_table,
                                           double dt_uniform, const double* __restrict__ group_dt,
                                           const int* __restrict__ group_par, int maux,
                                           double* __restrict__ cfl_out,
                                           unsigned long long* __restrict__ group_max, int* __restrict__ err,
                                           int rlo = 1, int rhi = M, double* part = nullptr)
{
    using G = Geo<M>;
    using L = Smem<M, RB, EXACT>;
    constexpr int N = G::N;
    constexpr int S = G::S;
    constexpr bool FAST = !EXACT;
    int* cnt = reinterpret_cast<int*>(sm + L::OFF_INT);
    uint16_t* la = reinterpret_cast<uint16_t*>(cnt + L::CNT_INTS);
    uint16_t* lb = la + L::LIST_A;
    unsigned char* wet = reinterpret_cast<unsigned char*>(sm) + L::OFF_WET_BYTES;
    double* red = sm + L::OFF_RED;

    const double dt = group_dt ? group_dt[wk.group] : dt_uniform;
    /* a group with no step this round (dt <= 0) is skipped as a whole */
    if (group_dt && !(dt > 0.0)) return true;
    if (group_par && group_par[wk.group]) {
        /* the group's state lives in the second buffer: read there, write back */
        double* t = wk.q;
        wk.q = wk.qout;
        wk.qout = t;
    }
    /* culled: this update would be an exact identity (the ghost fill decided) */
    if (wk.fl && wk.fl->skip) return true;
    const gf_phys P = phys_table[wk.phys];
    const double g = P.grav, drytol = P.dry_tolerance;

    /* after a wait of this launch (or an earlier one of the same step) gave
     * up, the step has failed: later items leave at once */
    if (__syncthreads_or(threadIdx.x == 0 && err && *reinterpret_cast<volatile int*>(err) != 0)) return false;

    /* ---- stage the patch (h, hu, hv planes and b) with bulk copies ---- */
    if (threadIdx.x == 0) {
        mbar_expect_tx(bar, (uint32_t)(4 * S * sizeof(double)));
        bulk_g2s(sm + L::OFF_H, wk.q, (uint32_t)(3 * S * sizeof(double)), bar);
        bulk_g2s(sm + L::OFF_B, wk.aux, (uint32_t)(S * sizeof(double)), bar);
    }
    const uint32_t ph = phase;
    phase ^= 1u;
    if (!__syncthreads_and(mbar_wait(bar, ph, kWaitPolls))) {
        if (threadIdx.x == 0) atomicExch(err, 1);
        mbar_wait(bar, ph, kWaitPolls); /* let any copy in flight land */
        return false;
    }

    /* ---- b4step2 on all cells + per-cell quotients ---- */
    int any_wet = 0, changed = 0;
    for (int k = threadIdx.x; k < S; k += NT) {
        double h = sm[L::OFF_H + k];
        if (d_lt<FAST>(h, drytol)) {
            /* b4step2 changes this cell's bits unless h >= 0 and both momenta are +0 */
            changed |= (__double_as_longlong(h) < 0) | (__double_as_longlong(sm[L::OFF_HU + k]) != 0) |
                       (__double_as_longlong(sm[L::OFF_HV + k]) != 0);
            h = d_max<FAST>(h, 0.0);
            sm[L::OFF_H + k] = h;
            sm[L::OFF_HU + k] = 0.0;
            sm[L::OFF_HV + k] = 0.0;
        }
        const bool w = d_gt<FAST>(h, drytol);
        wet[k] = w ? 1 : 0;
        any_wet |= w;
        double u = 0.0, v = 0.0, c = 0.0, rh = 0.0, rc = 0.0;
        if (w) {
            if (FAST) {
                /* rc^2 = 1 / (g h), so 1 / h = g rc^2 within a few ulps:
                 * two products instead of a reciprocal */
                const double gh = g * h;
                rc = rsqrt(gh);
                c = gh * rc;
                rh = g * (rc * rc);
                u = sm[L::OFF_HU + k] * rh;
                v = sm[L::OFF_HV + k] * rh;
            } else {
                u = sm[L::OFF_HU + k] / h;
                v = sm[L::OFF_HV + k] / h;
                c = sqrt(g * h);
            }
        }
        sm[L::OFF_U + k] = u;
        sm[L::OFF_V + k] = v;
        sm[L::OFF_C + k] = c;
        if (FAST) {
            sm[L::OFF_RH + k] = rh;
            sm[L::OFF_RC + k] = rc;
        }
    }
    for (int k = threadIdx.x; k < L::NACC * 3 * L::PLANE; k += NT) sm[L::OFF_ACC + k] = 0.0;
    any_wet = __syncthreads_or(any_wet);
    if (wk.fl) changed = __syncthreads_or(changed);

    const double dtdx = dt / wk.dx, dtdy = dt / wk.dy;
    double smax_x = 0.0, smax_y = 0.0;
    if (any_wet) {
        const double c16g = 1.0 / (16.0 * g);
        const double rsg = rsqrt(g);
        const double crit = fmax(drytol * g, 1e-6);
        const double crit2 = sqrt(crit);
        smax_x = sweep<M, NT, RB, 0, EXACT>(sm, wet, cnt, la, lb, P, dtdx, c16g, rsg, crit, crit2, rlo, rhi);
        smax_y = sweep<M, NT, RB, 1, EXACT>(sm, wet, cnt, la, lb, P, dtdy, c16g, rsg, crit, crit2, rlo, rhi);
    }

    /* ---- flux-difference update, src2, write interior ---- */
    double* gq = wk.qout ? wk.qout : wk.q;
    const double* gaux = wk.aux;
    const int fidx = P.friction_index - 1;
    for (int e = threadIdx.x; e < (rhi - rlo + 1) * M; e += NT) {
        const int i = 1 + e % M, j = rlo + e / M;
        const int k = (j + 1) * N + (i + 1);
        double h = sm[L::OFF_H + k], hu = sm[L::OFF_HU + k], hv = sm[L::OFF_HV + k];
        constexpr int PL = L::PLANE;
        const int a = (i - 1) + L::MS * (j - 1); /* accumulator index of the cell */
        if (EXACT) {
            /* q - dtdx*(fm(i+1,j) - fp(i,j)) - dtdy*(gm(i,j+1) - gp(i,j)) */
            const double* FM = sm + L::OFF_ACC;
            const double* FP = FM + 3 * PL;
            const double* GM = FP + 3 * PL;
            const double* GP = GM + 3 * PL;
            h = h - dtdx * (FM[a] - FP[a]) - dtdy * (GM[a] - GP[a]);
            hu = hu - dtdx * (FM[a + PL] - FP[a + PL]) - dtdy * (GM[a + PL] - GP[a + PL]);
            hv = hv - dtdx * (FM[a + 2 * PL] - FP[a + 2 * PL]) - dtdy * (GM[a + 2 * PL] - GP[a + 2 * PL]);
        } else {
            const double* DX = sm + L::OFF_ACC;
            const double* DY = sm + L::OFF_ACC + 3 * PL;
            h = h - dtdx * DX[a] - dtdy * DY[a];
            hu = hu - dtdx * DX[a + PL] - dtdy * DY[a + PL];
            hv = hv - dtdx * DX[a + 2 * PL] - dtdy * DY[a + 2 * PL];
        }
        if (P.src_term > 0) {
            const double nvar = (P.variable_friction && fidx >= 0 && fidx < maux)
                                    ? gaux[(size_t)fidx * S + k]
                                    : 0.0;
            src2_cell<FAST>(P, dt, sm[L::OFF_B + k], nvar, h, hu, hv);
        }
        gq[k] = h;
        gq[S + k] = hu;
        gq[2 * S + k] = hv;
    }

    if (wk.fl && threadIdx.x == 0) {
        wk.fl->ident = (!any_wet && !changed) ? 1 : 0;
        wk.fl->wet = any_wet ? 1 : 0;
    }

    /* ---- CFL: warp-shuffle max, then across warps ---- */
    double cx = smax_x, cy = smax_y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cx = fmax(cx, __shfl_xor_sync(0xffffffffu, cx, o));
        cy = fmax(cy, __shfl_xor_sync(0xffffffffu, cy, o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        red[warp] = cx;
        red[32 + warp] = cy;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double mx = 0.0, my = 0.0;
        for (int w2 = 0; w2 < NT / 32; ++w2) {
            mx = fmax(mx, red[w2]);
            my = fmax(my, red[32 + w2]);
        }
        if (part) { /* a window of a split item: the cluster forms the patch CFL */
            part[0] = mx;
            part[1] = my;
        }
    }
    if (part) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        return true;
    }
    if (threadIdx.x == 0) {
        double mx = 0.0, my = 0.0;
        for (int w2 = 0; w2 < NT / 32; ++w2) {
            mx = fmax(mx, red[w2]);
            my = fmax(my, red[32 + w2]);
        }
        double cfl = fmax(dtdx * mx, dtdy * my);
        if (cfl > P.maxcfl_cap) cfl = 0.0;
        if (cfl_out) cfl_out[wi] = cfl;
        if (group_max) atomicMax(group_max + wk.group, dkey(cfl));
    }
    /* shared memory is restaged by the bulk (async-proxy) copies of the next
     * work item: order this item's generic-proxy accesses before them */
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    return true;
}

/* The fused kernel for one patch size: one CTA per work item, or a
 * persistent grid striding over the work list. */
template <int M, int NT, int RB, int MINB, bool EXACT>
__global__ void __launch_bounds__(NT, MINB)
    patch_update_kernel(const gf_patch_work* __restrict__ work, int nwork,
                        const gf_phys* __restrict__ phys_table, double dt_uniform,
                        const double* __restrict__ group_dt, const int* __restrict__ group_par,
                        int maux, double* __restrict__ cfl_out,
                        unsigned long long* __restrict__ group_max, int* __restrict__ err)
{
    using L = Smem<M, RB, EXACT>;
    extern __shared__ __align__(128) double sm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + L::OFF_BAR);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    uint32_t phase = 0;
    for (int wi = blockIdx.x; wi < nwork; wi += gridDim.x)
        if (!patch_item<M, NT, RB, EXACT>(sm, bar, phase, work[wi], wi, phys_table, dt_uniform, group_dt,
                                          group_par, maux, cfl_out, group_max, err))
            return;
}

/* Latency form: one patch split over a thread-block cluster of K CTAs on
 * K SMs. CTA r of a cluster updates interior rows r*M/K+1 .. (r+1)*M/K of
 * the cluster's work item; each stages the whole patch and computes exactly
 * the faces those rows read (SweepWin), so the interior values are the same
 * bits as the one-CTA kernel's (the same operations, summed per cell in the
 * same slice order). The patch CFL is the maximum of the CTAs' partial wave
 * speed maxima, read by rank 0 through distributed shared memory after a
 * cluster barrier; a second barrier keeps every CTA resident until it has
 * been read. A lone patch then runs on K SMs instead of one. */
template <int M, int NT, int RB, int K, bool EXACT>
__global__ void __cluster_dims__(K, 1, 1) __launch_bounds__(NT, 1)
    patch_update_window_kernel(const gf_patch_work* __restrict__ work, int nwork,
                               const gf_phys* __restrict__ phys_table, double dt_uniform,
                               const double* __restrict__ group_dt, const int* __restrict__ group_par,
                               int maux, double* __restrict__ cfl_out,
                               unsigned long long* __restrict__ group_max, int* __restrict__ err)
{
    static_assert(M % K == 0, "the rows split evenly over the cluster");
    namespace cg = cooperative_groups;
    using L = Smem<M, RB, EXACT>;
    constexpr int R = M / K;
    extern __shared__ __align__(128) double sm[];
    cg::cluster_group cluster = cg::this_cluster();
    const int r = (int)cluster.block_rank();
    const int wi = blockIdx.x / K;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + L::OFF_BAR);
    double* part = sm + L::OFF_RED + 62; /* past the warp slots of the CFL reduction */
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        part[0] = 0.0;
        part[1] = 0.0;
    }
    __syncthreads();
    /* both tests are the same on every CTA of the cluster: it leaves whole */
    if (wi >= nwork) return;
    const gf_patch_work wk = work[wi];
    if (group_dt && !(group_dt[wk.group] > 0.0)) return;
    if (wk.fl && wk.fl->skip) return;
    uint32_t phase = 0;
    patch_item<M, NT, RB, EXACT>(sm, bar, phase, wk, wi, phys_table, dt_uniform, group_dt, group_par,
                                 maux, cfl_out, group_max, err, 1 + r * R, (r + 1) * R, part);
    cluster.sync();
    if (r == 0 && threadIdx.x == 0) {
        double mx = 0.0, my = 0.0;
        for (int q = 0; q < K; ++q) {
            const double* p = cluster.map_shared_rank(part, q);
            mx = fmax(mx, p[0]);
            my = fmax(my, p[1]);
        }
        const gf_phys& P = phys_table[wk.phys];
        const double dt = group_dt ? group_dt[wk.group] : dt_uniform;
        const double dtdx = dt / wk.dx, dtdy = dt / wk.dy;
        double cfl = fmax(dtdx * mx, dtdy * my);
        if (cfl > P.maxcfl_cap) cfl = 0.0;
        if (cfl_out) cfl_out[wi] = cfl;
        if (group_max) atomicMax(group_max + wk.group, dkey(cfl));
    }
    cluster.sync();
}

/* Shared-memory bytes of the mixed kernel: the largest class layout, then
 * the mbarrier and the two work-cursor slots. */
template <int RB8, int RB16, int RB32, bool EXACT>
struct MixedSmem {
    static constexpr size_t B8 = Smem<8, RB8, EXACT>::BYTES, B16 = Smem<16, RB16, EXACT>::BYTES,
                            B32 = Smem<32, RB32, EXACT>::BYTES;
    static constexpr size_t MAXB = B8 > B16 ? (B8 > B32 ? B8 : B32) : (B16 > B32 ? B16 : B32);
    static constexpr size_t OFF_CTL = (MAXB + 15) / 16 * 16;
    static constexpr size_t BYTES = OFF_CTL + 32;
};

/* All patch sizes in one persistent launch. The work list holds the mx = 32
 * items, then the mx = 16 items, then the mx = 8 items; CTAs take items in
 * that order from a device cursor (sched[0]) so that the long items start
 * first and the short ones fill the tail. sched[1] counts CTAs that found
 * the list empty; the last of them resets both counters for the next launch
 * (both start at zero). */
template <int NT, int RB8, int RB16, int RB32, bool EXACT>
__global__ void __launch_bounds__(NT, 1)
    patch_update_mixed_kernel(const gf_patch_work* __restrict__ work, int n32, int n16, int n8,
                              const gf_phys* __restrict__ phys_table, double dt_uniform,
                              const double* __restrict__ group_dt, const int* __restrict__ group_par,
                              int maux, double* __restrict__ cfl_out,
                              unsigned long long* __restrict__ group_max, int* __restrict__ err,
                              unsigned int* __restrict__ sched)
{
    using X = MixedSmem<RB8, RB16, RB32, EXACT>;
    extern __shared__ __align__(128) double sm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(sm) + X::OFF_CTL);
    volatile int* slot = reinterpret_cast<volatile int*>(reinterpret_cast<char*>(sm) + X::OFF_CTL + 8);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    const int nwork = n32 + n16 + n8;
    uint32_t phase = 0;
    /* the cursor value goes through one of two slots by iteration parity: a
     * skipped item has no barrier after its read, and the next write goes to
     * the other slot */
    for (int it = 0;; ++it) {
        if (threadIdx.x == 0) slot[it & 1] = (int)atomicAdd(sched, 1u);
        __syncthreads();
        const int wi = slot[it & 1];
        if (wi >= nwork) break;
        bool ok;
        if (wi < n32)
            ok = patch_item<32, NT, RB32, EXACT>(sm, bar, phase, work[wi], wi, phys_table, dt_uniform, group_dt,
                                                 group_par, maux, cfl_out, group_max, err);
        else if (wi < n32 + n16)
            ok = patch_item<16, NT, RB16, EXACT>(sm, bar, phase, work[wi], wi, phys_table, dt_uniform, group_dt,
                                                 group_par, maux, cfl_out, group_max, err);
        else
            ok = patch_item<8, NT, RB8, EXACT>(sm, bar, phase, work[wi], wi, phys_table, dt_uniform, group_dt,
                                               group_par, maux, cfl_out, group_max, err);
        if (!ok) break;
    }
    if (threadIdx.x == 0) {
        if (atomicAdd(sched + 1, 1u) == gridDim.x - 1) {
            atomicExch(sched, 0u);
            atomicExch(sched + 1, 0u);
        }
    }
}

} // namespace GF_KNS

#endif
