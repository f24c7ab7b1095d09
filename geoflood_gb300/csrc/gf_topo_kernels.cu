/*
 * Cell-averaged topography on the device: setaux's bathymetry for every
 * cell of a raster (a level of a forest, or any uniform grid).
 *
 * One thread per cell. The cell's integral follows cellgridintegrate
 * (src/fc2d_geoclaw/geolib_source/cellgridintegrate2.f:1-90): the finest
 * grid overlapping the cell alone if it holds the whole cell, else the
 * inclusion-exclusion over the ranked grids of rectintegral
 * (geolib_source/topo_module.f90:1460-1548), I(R, m) = I(R, m+1) -
 * I(R n G_m, m+1) + T(G_m, R n G_m), evaluated here with an explicit stack
 * instead of recursion; T is topointegral (geolib_source/topointegral.f):
 * the exact integral of the bilinear interpolant over each node cell of G
 * the rectangle touches (bilinearintegral.f). Then the cell average is the
 * integral over dx * dy (fortran_source/geoclaw_setaux_fort.f90:107-168),
 * and cells outside the domain copy the nearest cell inside (:178-215).
 * Compiled without FMA contraction, in the Fortran expressions' order.
 */
#include <cuda_runtime.h>

#include "gf_internal.h"

namespace gf {

namespace {

struct Rect {
    double x1, x2, y1, y2;
};

__device__ __forceinline__ bool cut(const Rect& r, const gf_topo_grid& g, Rect* o, double* area)
{
    o->x1 = fmax(r.x1, g.xlow);
    o->x2 = fmin(r.x2, g.xhi);
    o->y1 = fmax(r.y1, g.ylow);
    o->y2 = fmin(r.y2, g.yhi);
    if (o->x2 > o->x1 && o->y2 > o->y1) {
        *area = (o->x2 - o->x1) * (o->y2 - o->y1);
        return true;
    }
    *area = 0.0;
    return false;
}

/* integral of the bilinear interpolant of g over r (r within g's extent up
 * to rounding, which the clamp absorbs) */
__device__ double grid_integral(Rect r, const gf_topo_grid& g)
{
    double s = 0.0;
    const double xxhi = g.xlow + (g.mx - 1) * g.dx, yyhi = g.ylow + (g.my - 1) * g.dy;
    if ((r.x1 - g.xlow) < 0.0 || (r.x2 - xxhi) > 0.0) {
        r.x1 = fmax(g.xlow, r.x1);
        r.x2 = fmin(xxhi, r.x2);
    }
    if ((r.y1 - g.ylow) < 0.0 || (r.y2 - yyhi) > 0.0) {
        r.y1 = fmax(g.ylow, r.y1);
        r.y2 = fmin(yyhi, r.y2);
    }
    const int j0 = max((int)((r.y1 - g.ylow) / g.dy) + 1, 1);
    const int i0 = max((int)((r.x1 - g.xlow) / g.dx) + 1, 1);
    const int i1 = min((int)ceil((r.x2 - g.xlow) / g.dx) + 1, g.mx);
    const int j1 = min((int)ceil((r.y2 - g.ylow) / g.dy) + 1, g.my);
    for (int jj = j0; jj < j1; ++jj) {
        const double y1 = g.ylow + (jj - 1.0) * g.dy, y2 = g.ylow + jj * g.dy;
        /* nodes are stored north to south: row (my - jj) holds y1 */
        const double* row1 = g.z + (long)(g.my - jj) * g.mx;
        const double* row2 = row1 - g.mx;
        const double ylo = fmax(r.y1, y1), yhi = fmin(r.y2, y2);
        const double sumeta = (yhi + ylo - 2.0 * y1) / g.dy;
        for (int ii = i0; ii < i1; ++ii) {
            const double x1 = g.xlow + (ii - 1.0) * g.dx, x2 = g.xlow + ii * g.dx;
            const double z11 = row1[ii - 1], z21 = row1[ii], z12 = row2[ii - 1], z22 = row2[ii];
            const double xlo = fmax(r.x1, x1), xhi = fmin(r.x2, x2);
            const double area = (yhi - ylo) * (xhi - xlo);
            const double sumxi = (xhi + xlo - 2.0 * x1) / g.dx;
            const double a = z21 - z11, b = z12 - z11, c = z22 - z21 - z12 + z11;
            s = s + (0.5 * (a * sumxi + b * sumeta) + 0.25 * c * sumxi * sumeta + z11) * area;
        }
    }
    return s;
}

/* inclusion-exclusion over ranks m..n-1 without recursion: frames hold the
 * rectangle, the rank, the stage and the partial sums */
__device__ double ranked_integral(Rect r0, int m0, const gf_topo_grid* grids, const int* order, int n)
{
    struct Frame {
        Rect r, cut;
        double a;
        int m, stage;
    };
    Frame st[GF_TOPO_MAX_FILES];
    int sp = 0;
    double ret = 0.0;
    st[0].r = r0;
    st[0].m = m0;
    st[0].stage = 0;
    while (sp >= 0) {
        Frame& F = st[sp];
        const gf_topo_grid& G = grids[order[F.m]];
        if (F.m == n - 1) {
            Rect c;
            double area;
            ret = cut(F.r, G, &c, &area) ? grid_integral(c, G) : 0.0;
            --sp;
            continue;
        }
        if (F.stage == 0) {
            F.stage = 1;
            st[sp + 1].r = F.r;
            st[sp + 1].m = F.m + 1;
            st[sp + 1].stage = 0;
            ++sp;
            continue;
        }
        if (F.stage == 1) {
            F.a = ret;
            double area;
            cut(F.r, G, &F.cut, &area);
            if (area > 0) {
                F.stage = 2;
                st[sp + 1].r = F.cut;
                st[sp + 1].m = F.m + 1;
                st[sp + 1].stage = 0;
                ++sp;
                continue;
            }
            ret = F.a;
            --sp;
            continue;
        }
        /* stage 2: ret holds the coarser ranks' integral over the cut */
        ret = F.a - ret + grid_integral(F.cut, G);
        --sp;
    }
    return ret;
}

__device__ bool cell_integral(const Rect& cell, const gf_topo_grid* grids, const int* order, int n,
                              double* out)
{
    for (int m = 0; m < n; ++m) {
        const gf_topo_grid& G = grids[order[m]];
        const double cellarea = (cell.x2 - cell.x1) * (cell.y2 - cell.y1);
        Rect c;
        double area;
        if (cut(cell, G, &c, &area)) {
            if (area == cellarea) *out = 0.0 + grid_integral(c, G);
            else *out = ranked_integral(cell, m, grids, order, n);
            return true;
        }
    }
    *out = 0.0;
    return false;
}

__global__ void topo_raster_kernel(const gf_topo_grid* __restrict__ grids, const int* __restrict__ order,
                                   int n, int nx, int ny, int halo, double xlower, double ylower,
                                   double dx, double dy, double xupper, double yupper,
                                   double* __restrict__ out, int* __restrict__ err)
{
    const long p = nx + 2 * halo;
    const long total = p * (ny + 2 * halo);
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        const int gi = (int)(e % p) - halo, gj = (int)(e / p) - halo;
        Rect cell;
        cell.x1 = xlower + (double)gi * dx;
        cell.x2 = xlower + (double)(gi + 1) * dx;
        cell.y1 = ylower + (double)gj * dy;
        cell.y2 = ylower + (double)(gj + 1) * dy;
        const double x = 0.5 * (cell.x1 + cell.x2), y = 0.5 * (cell.y1 + cell.y2);
        if (y > yupper || y < ylower || x > xupper || x < xlower) continue;
        double v;
        if (!cell_integral(cell, grids, order, n, &v)) *err = 1;
        out[e] = v / (dx * dy);
    }
}

/* cells outside the domain take the cell inside that setaux's index shift
 * names: i + max(0, ceil((xlower - x)/dx)) - max(0, ceil((x - xupper)/dx)) */
__global__ void topo_outside_kernel(double* __restrict__ out, int nx, int ny, int halo, double xlower,
                                    double ylower, double dx, double dy, double xupper, double yupper)
{
    const long p = nx + 2 * halo;
    const long total = p * (ny + 2 * halo);
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        const int i = (int)(e % p), j = (int)(e / p);
        const double x = xlower + ((i - halo) + 0.5) * dx, y = ylower + ((j - halo) + 0.5) * dy;
        if (!(y < ylower || y > yupper || x < xlower || x > xupper)) continue;
        const int ii = i + (int)fmax(0.0, ceil((xlower - x) / dx)) - (int)fmax(0.0, ceil((x - xupper) / dx));
        const int jj = j + (int)fmax(0.0, ceil((ylower - y) / dy)) - (int)fmax(0.0, ceil((y - yupper) / dy));
        out[e] = out[(long)jj * p + ii];
    }
}

int grid_of(long total)
{
    long b = (total + 127) / 128;
    if (b > 152L * 32) b = 152L * 32;
    return (int)(b < 1 ? 1 : b);
}

} // namespace

cudaError_t launch_topo_raster(const gf_topo_grid* grids, const int* order, int n, int nx, int ny, int halo,
                               double xlower, double ylower, double dx, double dy, double xupper,
                               double yupper, double* out, int* err, cudaStream_t st)
{
    if (n < 1 || n > GF_TOPO_MAX_FILES) return cudaErrorInvalidValue;
    const long total = (long)(nx + 2 * halo) * (ny + 2 * halo);
    topo_raster_kernel<<<grid_of(total), 128, 0, st>>>(grids, order, n, nx, ny, halo, xlower, ylower, dx, dy,
                                                       xupper, yupper, out, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || halo == 0) return e;
    topo_outside_kernel<<<grid_of(total), 128, 0, st>>>(out, nx, ny, halo, xlower, ylower, dx, dy, xupper, yupper);
    return cudaGetLastError();
}

} // namespace gf
