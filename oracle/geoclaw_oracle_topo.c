/*
 * CPU oracle, cell-averaged topography from topo grids -- TEST
 * INFRASTRUCTURE ONLY.
 *
 * Restates (paths relative to the GeoFlood source tree):
 *   intersection       src/fc2d_geoclaw/geolib_source/topo_module.f90:1552-1580
 *   rectintegral       topo_module.f90:1460-1548
 *   topoarea           topo_module.f90:1384-1456
 *   file ranking       topo_module.f90:298-318 (finest first; equal cell
 *                      areas: the later file first)
 *   cellgridintegrate  geolib_source/cellgridintegrate2.f:1-90
 *   topointegral       geolib_source/topointegral.f (bilinear, Cartesian)
 *   bilinearintegral   geolib_source/bilinearintegral.f (Cartesian form)
 *   fc2d_geoclaw_setaux, bathymetry part
 *                      fortran_source/geoclaw_setaux_fort.f90:107-215
 * Each grid holds node values z in file order: rows north to south, x
 * fastest (topo(i) of read_topo_file). Arithmetic follows the Fortran
 * expressions' order; built without contraction.
 */
#include <math.h>
#include <string.h>

#include "geoclaw_oracle.h"

static void intersection(int* ind, double* area, double* xlo, double* xhi, double* ylo, double* yhi,
                         double x1lo, double x1hi, double y1lo, double y1hi, double x2lo, double x2hi,
                         double y2lo, double y2hi)
{
    *xlo = fmax(x1lo, x2lo);
    *xhi = fmin(x1hi, x2hi);
    *ylo = fmax(y1lo, y2lo);
    *yhi = fmin(y1hi, y2hi);
    if (*xhi > *xlo && *yhi > *ylo) {
        *area = (*xhi - *xlo) * (*yhi - *ylo);
        *ind = 1;
    } else {
        *area = 0.0;
        *ind = 0;
    }
}

static double bilinearintegral(double xim, double xip, double yjm, double yjp, double x1, double x2,
                               double y1, double y2, double dxx, double dyy, double z11, double z12,
                               double z21, double z22)
{
    const double xlow = fmax(xim, x1), ylow = fmax(yjm, y1);
    const double xhi = fmin(xip, x2), yhi = fmin(yjp, y2);
    const double area = (yhi - ylow) * (xhi - xlow);
    const double sumxi = (xhi + xlow - 2.0 * x1) / dxx;
    const double sumeta = (yhi + ylow - 2.0 * y1) / dyy;
    const double a = z21 - z11, b = z12 - z11, c = z22 - z21 - z12 + z11, d = z11;
    return (0.5 * (a * sumxi + b * sumeta) + 0.25 * c * sumxi * sumeta + d) * area;
}

double orc_topointegral(double xim, double xip, double yjm, double yjp, const orc_topo_grid* g)
{
    double s = 0.0;
    const double xxhi = g->xlow + (g->mx - 1) * g->dx;
    const double yyhi = g->ylow + (g->my - 1) * g->dy;
    if ((xim - g->xlow) < 0.0 || (xip - xxhi) > 0.0) {
        xim = fmax(g->xlow, xim);
        xip = fmin(xxhi, xip);
    }
    if ((yjm - g->ylow) < 0.0 || (yjp - yyhi) > 0.0) {
        yjm = fmax(g->ylow, yjm);
        yjp = fmin(yyhi, yjp);
    }
    int jjstart = (int)((yjm - g->ylow) / g->dy) + 1;
    int iistart = (int)((xim - g->xlow) / g->dx) + 1;
    int iiend = (int)ceil((xip - g->xlow) / g->dx) + 1;
    int jjend = (int)ceil((yjp - g->ylow) / g->dy) + 1;
    if (iistart < 1) iistart = 1;
    if (jjstart < 1) jjstart = 1;
    if (iiend > g->mx) iiend = g->mx;
    if (jjend > g->my) jjend = g->my;
    for (int jj = jjstart; jj <= jjend - 1; ++jj) {
        const double y1 = g->ylow + (jj - 1.0) * g->dy;
        const double y2 = g->ylow + jj * g->dy;
        const int jz1 = g->my - jj + 1, jz2 = jz1 - 1; /* rows stored north to south */
        for (int ii = iistart; ii <= iiend - 1; ++ii) {
            const double x1 = g->xlow + (ii - 1.0) * g->dx;
            const double x2 = g->xlow + ii * g->dx;
            const double z11 = g->z[(size_t)(jz1 - 1) * g->mx + (ii - 1)];
            const double z12 = g->z[(size_t)(jz2 - 1) * g->mx + (ii - 1)];
            const double z21 = g->z[(size_t)(jz1 - 1) * g->mx + ii];
            const double z22 = g->z[(size_t)(jz2 - 1) * g->mx + ii];
            s = s + bilinearintegral(xim, xip, yjm, yjp, x1, x2, y1, y2, g->dx, g->dy, z11, z12, z21, z22);
        }
    }
    return s;
}

void orc_topo_rank(const orc_topo_grid* g, int n, int* order)
{
    for (int i = 0; i < n; ++i) {
        int finer_than = 0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            const double ai = g[i].dx * g[i].dy, aj = g[j].dx * g[j].dy;
            if (ai < aj) ++finer_than;
            if (ai == aj && j < i) ++finer_than;
        }
        order[n - finer_than - 1] = i;
    }
}

/* m: 0-based rank */
static double rectintegral(double x1, double x2, double y1, double y2, int m, const orc_topo_grid* g,
                           const int* order, int n)
{
    const orc_topo_grid* G = &g[order[m]];
    int ind;
    double area, a, b, c, d;
    if (m == n - 1) {
        intersection(&ind, &area, &a, &b, &c, &d, x1, x2, y1, y2, G->xlow, G->xhi, G->ylow, G->yhi);
        return ind ? orc_topointegral(a, b, c, d, G) : 0.0;
    }
    const double int1 = rectintegral(x1, x2, y1, y2, m + 1, g, order, n);
    intersection(&ind, &area, &a, &b, &c, &d, x1, x2, y1, y2, G->xlow, G->xhi, G->ylow, G->yhi);
    if (area > 0) {
        const double int2 = rectintegral(a, b, c, d, m + 1, g, order, n);
        const double int3 = orc_topointegral(a, b, c, d, G);
        return int1 - int2 + int3;
    }
    return int1;
}

static double topoarea(double x1, double x2, double y1, double y2, int m, const orc_topo_grid* g,
                       const int* order, int n)
{
    const orc_topo_grid* G = &g[order[m]];
    int ind;
    double area, a, b, c, d;
    if (m == n - 1) {
        intersection(&ind, &area, &a, &b, &c, &d, x1, x2, y1, y2, G->xlow, G->xhi, G->ylow, G->yhi);
        return area;
    }
    const double area1 = topoarea(x1, x2, y1, y2, m + 1, g, order, n);
    double area_m;
    intersection(&ind, &area_m, &a, &b, &c, &d, x1, x2, y1, y2, G->xlow, G->xhi, G->ylow, G->yhi);
    if (area_m > 0) {
        const double area2 = topoarea(a, b, c, d, m + 1, g, order, n);
        return area1 - area2 + area_m;
    }
    return area1;
}

double orc_topo_area(double x1, double x2, double y1, double y2, const orc_topo_grid* g, const int* order,
                     int n)
{
    return n > 0 ? topoarea(x1, x2, y1, y2, 0, g, order, n) : 0.0;
}

int orc_cellgridintegrate(double* out, double xim, double xip, double yjm, double yjp,
                          const orc_topo_grid* g, const int* order, int n)
{
    double topoint = 0.0;
    for (int m = 0; m < n; ++m) {
        const orc_topo_grid* G = &g[order[m]];
        const double cellarea = (xip - xim) * (yjp - yjm);
        int ind;
        double area, a, b, c, d;
        intersection(&ind, &area, &a, &b, &c, &d, xim, xip, yjm, yjp, G->xlow, G->xhi, G->ylow, G->yhi);
        if (ind == 1) {
            if (area == cellarea) {
                *out = topoint + orc_topointegral(a, b, c, d, G);
                return 0;
            }
            *out = rectintegral(xim, xip, yjm, yjp, m, g, order, n);
            return 0;
        }
    }
    *out = 0.0;
    return -1; /* the cell overlaps no topo grid: the reference stops */
}

int orc_setaux_raster(const orc_topo_grid* g, const int* order, int n, int nx, int ny, int halo,
                      double xlower, double ylower, double dx, double dy, double xupper, double yupper,
                      double* out)
{
    const long p = nx + 2 * halo;
    int rc = 0;
    for (int j = 0; j < ny + 2 * halo; ++j) {
        const int gj = j - halo;
        const double ym = ylower + (double)gj * dy, yp = ylower + (double)(gj + 1) * dy;
        const double y = 0.5 * (ym + yp);
        for (int i = 0; i < nx + 2 * halo; ++i) {
            const int gi = i - halo;
            const double xm = xlower + (double)gi * dx, xp = xlower + (double)(gi + 1) * dx;
            const double x = 0.5 * (xm + xp);
            if (y > yupper || y < ylower || x > xupper || x < xlower) continue;
            double v;
            if (orc_cellgridintegrate(&v, xm, xp, ym, yp, g, order, n)) rc = -1;
            out[(long)j * p + i] = v / (dx * dy);
        }
    }
    /* cells outside the domain take the nearest cell inside (setaux's two
     * copy loops, geoclaw_setaux_fort.f90:178-215) */
    for (int pass = 0; pass < 2; ++pass) {
        for (int j = 0; j < ny + 2 * halo; ++j) {
            const double y = ylower + ((j - halo) + 0.5) * dy;
            for (int i = 0; i < nx + 2 * halo; ++i) {
                const double x = xlower + ((i - halo) + 0.5) * dx;
                const int out_y = (y < ylower) || (y > yupper), out_x = (x < xlower) || (x > xupper);
                if (pass == 0 ? !out_y : !out_x) continue;
                const double cx1 = ceil((xlower - x) / dx), cx2 = ceil((x - xupper) / dx);
                const double cy1 = ceil((ylower - y) / dy), cy2 = ceil((y - yupper) / dy);
                const int ii = i + (int)fmax(0.0, cx1) - (int)fmax(0.0, cx2);
                const int jj = j + (int)fmax(0.0, cy1) - (int)fmax(0.0, cy2);
                out[(long)j * p + i] = out[(long)jj * p + ii];
            }
        }
    }
    return rc;
}
