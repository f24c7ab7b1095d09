/*
 * qad, the coarse/fine conservation fix-up of GeoClaw's geolib
 * (src/fc2d_geoclaw/geolib_source/qad.f:4-371), on the device.
 *
 * For one side of a fine patch: the Riemann problem between the fine
 * patch's first ghost cell and the coarse cell that ghost cell lies in is
 * solved at each of the side's mx fine faces (rpn2_geoclaw.f with
 * riemann_aug_JCP, the same face solver as the patch update, in its
 * IEEE-exact form), and the fluctuations amdq + apdq, times the fine face
 * length and the time step, are added into svdflx, one entry per coarse cell
 * along the side (two fine faces each, in order). Sides and signs follow
 * qad.f: 1 left (coarse | ghost, +hy), 2 top (ghost | coarse, -hx), 3 right
 * (ghost | coarse, -hy), 4 bottom (coarse | ghost, +hx).
 *
 * The reference tree does not compile qad.f; nothing in GeoFlood calls it.
 * Built without floating-point contraction (like the other coarse/fine
 * kernels) so the result matches the oracle's restatement.
 *
 * One CTA per side task; thread f solves fine face f, then thread c sums
 * coarse cell c's two faces into svdflx.
 */
#include <cuda_runtime.h>

#include "gf_internal.h"
#include "gf_riemann.cuh"

namespace gf {
namespace {

template <int M>
__global__ void __launch_bounds__(M) qad_kernel(const gf_qad_dev_task* __restrict__ tasks,
                                                const gf_phys* __restrict__ phys_tab, double dt)
{
    constexpr int N = M + 4;
    constexpr int S = N * N;
    const gf_qad_dev_task T = tasks[blockIdx.x];
    const gf_phys& P = phys_tab[T.phys];
    const double g = P.grav, drytol = P.dry_tolerance;
    const int side = T.side;
    const bool xdir = (side == 1 || side == 3);
    __shared__ double am[3][M], ap[3][M];

    const int f = threadIdx.x; /* fine face: row (sides 1, 3) or column (2, 4), 0-based */
    {
        /* fine ghost cell (0-based array index incl. halo) */
        int gi, gj;
        if (side == 1) { gi = 1; gj = 2 + f; }
        else if (side == 2) { gi = 2 + f; gj = M + 2; }
        else if (side == 3) { gi = M + 2; gj = 2 + f; }
        else { gi = 2 + f; gj = 1; }
        /* the coarse cell holding it: fine index (1-based) fi maps to coarse
         * (fi - o + 1) / 2 for the task's offset o (gf_xfer_task convention) */
        const int fi = gi - 1, fj = gj - 1;
        const int ci = (fi - T.ox + 1) >> 1, cj = (fj - T.oy + 1) >> 1; /* 1-based, host-checked */
        const int kg = gj * N + gi, kc = (cj + 1) * N + (ci + 1);
        double qg[3], qc[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            qg[m] = T.qf[m * S + kg];
            qc[m] = T.qc[m * S + kc];
        }
        const double bg = T.af[kg], bc = T.ac[kc];
        /* left / right states of the face: coarse | ghost on sides 1 and 4 */
        const bool coarse_left = (side == 1 || side == 4);
        const double* ql = coarse_left ? qc : qg;
        const double* qr = coarse_left ? qg : qc;
        const double bl = coarse_left ? bc : bg, br = coarse_left ? bg : bc;
        /* rpn2_geoclaw.f:110-120: a negative depth is set to a dry state */
        double hl = ql[0], hr = qr[0];
        const int mu = xdir ? 1 : 2, mv = xdir ? 2 : 1;
        double s[3] = {0.0, 0.0, 0.0}, fw[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
        if (hl < 0.0) hl = 0.0;
        if (hr < 0.0) hr = 0.0;
        if (!(hl <= drytol && hr <= drytol)) { /* :131-133 both dry: no waves */
            gf_cell Lc, Rc;
            Lc.b = bl;
            Rc.b = br;
            Lc.wet = hl > drytol;
            Rc.wet = hr > drytol;
            Lc.h = hl; Lc.hun = ql[mu]; Lc.hut = ql[mv];
            Rc.h = hr; Rc.hun = qr[mu]; Rc.hut = qr[mv];
            Lc.un = Lc.wet ? Lc.hun / hl : 0.0;
            Lc.ut = Lc.wet ? Lc.hut / hl : 0.0;
            Lc.c = Lc.wet ? sqrt(g * hl) : 0.0;
            Rc.un = Rc.wet ? Rc.hun / hr : 0.0;
            Rc.ut = Rc.wet ? Rc.hut / hr : 0.0;
            Rc.c = Rc.wet ? sqrt(g * hr) : 0.0;
            Lc.rh = Lc.rc = Rc.rh = Rc.rc = 0.0;
            const double c16g = 1.0 / (16.0 * g);
            const double rsg = rsqrt(g);
            const double crit = fmax(drytol * g, 1e-6);
            const double crit2 = sqrt(crit);
            gf_rpn2_face<false>(Lc, Rc, g, drytol, c16g, rsg, crit, crit2, s, fw);
        }
        /* fluctuations (rpn2_geoclaw.f:359-376), back in (h, hu, hv) order */
        double a[3] = {0.0, 0.0, 0.0}, b[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int mw = 0; mw < 3; ++mw) {
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                if (s[mw] < 0.0) {
                    a[m] = a[m] + fw[mw][m];
                } else if (s[mw] > 0.0) {
                    b[m] = b[m] + fw[mw][m];
                } else {
                    a[m] = a[m] + 0.5 * fw[mw][m];
                    b[m] = b[m] + 0.5 * fw[mw][m];
                }
            }
        }
        am[0][f] = a[0]; am[mu][f] = a[1]; am[mv][f] = a[2];
        ap[0][f] = b[0]; ap[mu][f] = b[1]; ap[mv][f] = b[2];
    }
    __syncthreads();
    const double h = xdir ? T.hy : T.hx;
    const double sgn = (side == 1 || side == 4) ? 1.0 : -1.0;
    for (int e = threadIdx.x; e < 3 * (M / 2); e += M) {
        const int c = e / 3, m = e % 3;
        double v = T.svdflx[m + 3 * c];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const int ff = 2 * c + l;
            v = v + sgn * am[m][ff] * h * dt + sgn * ap[m][ff] * h * dt;
        }
        T.svdflx[m + 3 * c] = v;
    }
}

} // namespace

cudaError_t launch_qad(int m, const gf_qad_dev_task* tasks, int ntask, const gf_phys* phys,
                       double dt, cudaStream_t st)
{
    if (ntask <= 0) return cudaSuccess;
    switch (m) {
    case 32: qad_kernel<32><<<ntask, 32, 0, st>>>(tasks, phys, dt); break;
    case 16: qad_kernel<16><<<ntask, 16, 0, st>>>(tasks, phys, dt); break;
    case 8: qad_kernel<8><<<ntask, 8, 0, st>>>(tasks, phys, dt); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

} // namespace gf
