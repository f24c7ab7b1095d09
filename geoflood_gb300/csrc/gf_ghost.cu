/*
 * Ghost-cell fill of a same-level patch batch on the device.
 *
 * Step 1 copies face and corner ghost cells from aligned same-level
 * neighbours (fclaw2d_source/fc2d_geoclaw_copy_fort.f:11-107). Step 2 applies
 * the physical boundary rule of every side with no neighbour, in the
 * reference's order left, right, bottom, top over the full ghost extent
 * (fortran_source/geoflood_bc2_fort.f90:7-409), including the hydrograph
 * inflow state (hydrograph/hydrograh_module.f90:224-331). Step 1 reads only
 * neighbours' interior cells and step 2 only its own patch, so one CTA per
 * patch needs no grid-wide barrier.
 */
#include <cuda_runtime.h>

#include "gf_internal.h"

namespace gf {

namespace {

__device__ __forceinline__ double* plane(double* base, long patch, int field, int S, int nf)
{
    return base + (patch * nf + field) * (long)S;
}

/* Riemann_invariants / two_shock (hydrograh_module.f90:224-331), discharge
 * form; tol is the single-precision literal 1.0e-6 of the Fortran. */
__device__ void inflow_riemann(double g, double q0hu, double h1, double hu1, double& h0, bool two)
{
    const double tol = (double)1.0e-6f;
    const double u1 = hu1 / h1;
    const double Fr = two ? 1.0 : 0.5;
    h0 = pow(q0hu / sqrt(g) * Fr, 2.0 / 3.0);
    for (int i = 1; i <= 100; ++i) {
        double fxn, dfxn;
        if (!two) {
            fxn = q0hu / h0 - 2 * sqrt(g * h0) - u1 + 2 * sqrt(g * h1);
            if (fabs(fxn) < tol) return;
            dfxn = -q0hu / (h0 * h0) - sqrt(g / h0);
        } else {
            fxn = q0hu / h0 - u1 - (h0 - h1) * sqrt((g / 2.0) * (1.0 / h0 + 1.0 / h1));
            if (fabs(fxn) < tol) return;
            const double num = sqrt(g * (1.0 / h0 + 1.0 / h1));
            const double deno = 2 * sqrt(2.0) * (h0 * h0) * num;
            dfxn = -q0hu / (h0 * h0) - num / sqrt(2.0) + g * (h0 - h1) / deno;
        }
        h0 = h0 - fxn / dfxn;
    }
}

/* Inflow ghost state inside the channel window; false = mirror (wall) case. */
__device__ bool inflow_state(const gf_phys& P, double q0hu, double h1, double hu1, double& h,
                             double& hu)
{
    if (h1 < P.dry_tolerance) {
        const double hh = pow(q0hu / sqrt(P.grav), 2.0 / 3.0);
        h = hh > 0.001 ? hh : 0.001;
        hu = q0hu;
        return true;
    }
    if (q0hu != 0.0) {
        double h0;
        inflow_riemann(P.grav, q0hu, h1, hu1, h0, false);
        if (h0 > h1) inflow_riemann(P.grav, q0hu, h1, hu1, h0, true);
        h = h0;
        hu = q0hu;
        return true;
    }
    return false;
}

template <int M>
__global__ void __launch_bounds__(128) ghost_fill_kernel(const gf_ghost_block* __restrict__ blocks,
                                                         const gf_ghost_ref* __restrict__ list,
                                                         int nlist,
                                                         const gf_phys* __restrict__ phys_table)
{
    constexpr int N = M + 4, S = N * N, MBC = 2;
    if ((int)blockIdx.x >= nlist) return;
    /* list == nullptr: one block, patch = blockIdx.x */
    const gf_ghost_ref ref = list ? list[blockIdx.x] : gf_ghost_ref{0, (int)blockIdx.x};
    const gf_ghost_block& blk = blocks[ref.block];
    if (blk.skip) return;
    const long p = ref.local;
    double* __restrict__ q = blk.q;
    const gf_bc_spec bc = blk.bc;
    const int* __restrict__ nbr = blk.nbr;
    int nb[8];
#pragma unroll
    for (int s = 0; s < 8; ++s) nb[s] = nbr[8 * p + s];

    /* dry-patch culling: the patch's last update was an identity, no
     * neighbour holds water and no side takes inflow, so this step's update
     * would be the identity again; mark it skipped and leave its ghosts */
    if (blk.fl) {
        bool skip = blk.fl[p].ident != 0;
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            if (nb[s] >= 0) skip = skip && blk.fl[nb[s]].wet == 0;
            else if (nb[s] != -1) skip = false;               /* filled by another route */
            else if (s < 4 && bc.mthbc[s] == 0) skip = false; /* hydrograph side */
        }
        __syncthreads(); /* every thread has read the flags before thread 0 writes */
        if (threadIdx.x == 0) blk.fl[p].skip = skip ? 1 : 0;
        if (skip) return;
    }

    /* ---- step 1: same-level face and corner copies ---- */
    for (int k = threadIdx.x; k < S; k += blockDim.x) {
        const int i = k % N - 1, j = k / N - 1; /* Fortran indices 1-mbc..M+mbc */
        const bool L = i <= 0, R = i >= M + 1, B = j <= 0, T = j >= M + 1;
        if (!(L || R || B || T)) continue;
        int src;
        if ((L || R) && (B || T)) src = nb[4 + (T ? 2 : 0) + (R ? 1 : 0)];
        else src = nb[L ? 0 : R ? 1 : B ? 2 : 3];
        if (src < 0) continue;
        const int i2 = i + (L ? M : R ? -M : 0), j2 = j + (B ? M : T ? -M : 0);
        const int k2 = (j2 + 1) * N + (i2 + 1);
#pragma unroll
        for (int f = 0; f < 3; ++f) plane(q, p, f, S, 3)[k] = plane(q, src, f, S, 3)[k2];
    }
    const bool phys_side[4] = {nb[0] == -1, nb[1] == -1, nb[2] == -1, nb[3] == -1};
    if (!(phys_side[0] || phys_side[1] || phys_side[2] || phys_side[3])) return;
    __syncthreads();

    const gf_phys P = phys_table[blk.phys_of ? blk.phys_of[p] : blk.phys];
    const gf_patch_geom G = blk.geom[p];
    double* qh = plane(q, p, 0, S, 3);
    double* qu = plane(q, p, 1, S, 3);
    double* qv = plane(q, p, 2, S, 3);
    double* b = plane(blk.aux, p, 0, S, blk.maux);
    auto at = [](int i, int j) { return (j + 1) * N + (i + 1); };

    /* ---- step 2a: x sides (left then right are disjoint), all rows ---- */
    for (int e = threadIdx.x; e < 2 * N * MBC; e += blockDim.x) {
        const int side = e / (N * MBC); /* 0 left, 1 right */
        const int r = e % (N * MBC);
        const int j = r / MBC + 1 - MBC, ibc = r % MBC + 1;
        if (!phys_side[side]) continue;
        const int rule = bc.mthbc[side];
        const int ig = side == 0 ? 1 - ibc : M + ibc;        /* ghost          */
        const int im = side == 0 ? ibc : M + 1 - ibc;        /* mirror source  */
        const int ie = side == 0 ? 1 : M;                    /* boundary cell  */
        const int kg = at(ig, j);
        bool mirror = false;
        if (rule == 0 && bc.hydro_side[side]) {
            const double y = G.ylower + (j - 0.5) * G.dy;
            bool inflow = false;
            if (fabs(y - bc.y0) <= bc.width / 2.0) {
                double h, hu;
                inflow = inflow_state(P, bc.q0hu, qh[at(ie, j)], qu[at(ie, j)], h, hu);
                if (inflow) { qh[kg] = h; qu[kg] = hu; qv[kg] = 0.0; }
            }
            mirror = !inflow;
        } else if (rule == 1) {
            const int ks = at(ie, j);
            b[kg] = b[ks];
            qh[kg] = qh[ks]; qu[kg] = qu[ks]; qv[kg] = qv[ks];
        } else if (rule == 3) {
            mirror = true;
        }
        if (mirror) {
            const int ks = at(im, j);
            b[kg] = b[ks];
            qh[kg] = qh[ks]; qu[kg] = -qu[ks]; qv[kg] = qv[ks];
        }
    }
    __syncthreads();

    /* ---- step 2b: y sides (bottom then top are disjoint), all columns ---- */
    for (int e = threadIdx.x; e < 2 * N * MBC; e += blockDim.x) {
        const int side = 2 + e / (N * MBC); /* 2 bottom, 3 top */
        const int r = e % (N * MBC);
        const int i = r / MBC + 1 - MBC, jbc = r % MBC + 1;
        if (!phys_side[side]) continue;
        const int rule = bc.mthbc[side];
        const int jg = side == 2 ? 1 - jbc : M + jbc;
        const int jm = side == 2 ? jbc : M + 1 - jbc;
        const int je = side == 2 ? 1 : M;
        const int kg = at(i, jg);
        bool mirror = false;
        if (rule == 0 && bc.hydro_side[side]) {
            const double x = G.xlower + (i - 0.5) * G.dx;
            bool inflow = false;
            if (fabs(x - bc.x0) <= bc.width / 2.0) {
                double h, hu;
                /* the reference feeds q(2) (x momentum) on the y sides too */
                inflow = inflow_state(P, bc.q0hu, qh[at(i, je)], qu[at(i, je)], h, hu);
                if (inflow) { qh[kg] = h; qu[kg] = hu; qv[kg] = 0.0; }
            }
            mirror = !inflow;
        } else if (rule == 1) {
            const int ks = at(i, je);
            b[kg] = b[ks];
            qh[kg] = qh[ks]; qu[kg] = qu[ks]; qv[kg] = qv[ks];
        } else if (rule == 3) {
            mirror = true;
        }
        if (mirror) {
            const int ks = at(i, jm);
            b[kg] = b[ks];
            qh[kg] = qh[ks]; qu[kg] = qu[ks]; qv[kg] = -qv[ks];
        }
    }
}

} // namespace

cudaError_t launch_ghost_fill(int m, const gf_ghost_block* blocks, const gf_ghost_ref* list,
                              int nlist, const gf_phys* phys, cudaStream_t st)
{
    if (nlist <= 0) return cudaSuccess;
    switch (m) {
    case 32: ghost_fill_kernel<32><<<nlist, 128, 0, st>>>(blocks, list, nlist, phys); break;
    case 16: ghost_fill_kernel<16><<<nlist, 128, 0, st>>>(blocks, list, nlist, phys); break;
    case 8: ghost_fill_kernel<8><<<nlist, 128, 0, st>>>(blocks, list, nlist, phys); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

} // namespace gf
