/*
 * Output in the reference's file formats (host side).
 *
 *  - ASCII frames fort.tXXXX / fort.qXXXX as written by
 *    fc2d_geoclaw_fort_write_header / _write_file
 *    (fclaw2d_source/fc2d_geoclaw_output_ascii_fort.f:1-117): a header of
 *    time, meqn + 1, ngrids, num_aux, num_dim, num_ghost; per patch six
 *    i5 lines (grid number, AMR level, block, MPI rank, mx, my), four e24.16
 *    lines (xlow, ylow, dx, dy), a blank line, then per row of cells one
 *    5E26.16 line per cell with h, hu, hv, eta (values below 1e-99 in
 *    magnitude written as 0) and a blank line after each row.
 *  - Gauges gaugeXXXXX.txt (src/fc2d_geoclaw/fc2d_geoclaw_gauges_default.c:
 *    183-199, 272-302): the header lines and one "%5d %15.7e ..." row per
 *    sample; samples interpolated as fc2d_geoclaw_update_gauge does
 *    (fortran_source/geoclaw_gauges_fort.f90:1-77).
 *
 * Fortran Ew.d fields are formatted here from the correctly rounded
 * decimal digits of the value: 0.d1...dd E+xx, with the E dropped for
 * three-digit exponents as the Fortran standard prescribes.
 */
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gf_internal.h"

namespace {

/* Fortran Ew.d of x into out (right-justified in w characters). */
void fort_e(double x, int w, int d, std::string& out)
{
    char digits[64];
    int e10 = 0;
    bool neg = std::signbit(x);
    double ax = std::fabs(x);
    std::string mant;
    if (ax == 0.0) {
        mant.assign(d, '0');
        e10 = 0;
    } else {
        char buf[64];
        std::snprintf(buf, sizeof buf, "%.*e", d - 1, ax); /* D.DDDe+XX */
        int k = 0;
        for (const char* p = buf; *p && *p != 'e'; ++p)
            if (*p != '.') digits[k++] = *p;
        digits[k] = 0;
        mant.assign(digits, d);
        e10 = std::atoi(std::strchr(buf, 'e') + 1) + 1; /* 0.D... scaling */
    }
    char field[96];
    const int ae = e10 < 0 ? -e10 : e10;
    char expo[16];
    if (ae <= 99) std::snprintf(expo, sizeof expo, "E%c%02d", e10 < 0 ? '-' : '+', ae);
    else std::snprintf(expo, sizeof expo, "%c%03d", e10 < 0 ? '-' : '+', ae);
    std::snprintf(field, sizeof field, "%s0.%s%s", neg ? "-" : "", mant.c_str(), expo);
    const int len = (int)std::strlen(field);
    if (len < w) out.append(w - len, ' ');
    out += field;
}

void fort_i(int v, int w, std::string& out)
{
    char b[32];
    std::snprintf(b, sizeof b, "%*d", w, v);
    out += b;
}

std::string frame_name(const char* dir, char kind, int iframe)
{
    char b[32];
    std::snprintf(b, sizeof b, "fort.%c%04d", kind, iframe % 10000);
    std::string p = dir && *dir ? std::string(dir) + "/" : std::string();
    return p + b;
}

inline double tiny0(double v) { return std::fabs(v) < 1e-99 ? 0.0 : v; }

} // namespace

extern "C" {

int gf_write_ascii_frame(const char* dir, int iframe, double time, int npatch, int mx, int maux,
                         const double* q, const double* aux, const int* grid_number,
                         const int* level, const int* block, const double* xlower,
                         const double* ylower, const double* dx, const double* dy)
{
    const int mbc = GF_MBC, meqn = 3;
    if (iframe < 0 || npatch < 0 || mx < 1 || maux < 1 || (npatch > 0 && (!q || !aux || !level ||
        !xlower || !ylower || !dx || !dy)))
        return GF_ERR_ARG;
    std::string t;
    fort_e(time, 30, 20, t);
    t += "    time\n";
    fort_i(meqn + 1, 5, t);
    t += "                 meqn\n";
    fort_i(npatch, 5, t);
    t += "                 ngrids\n";
    fort_i(maux, 5, t);
    t += "                 num_aux\n";
    fort_i(2, 5, t);
    t += "                 num_dim\n";
    fort_i(mbc, 5, t);
    t += "                 num_ghost\n";
    FILE* ft = std::fopen(frame_name(dir, 't', iframe).c_str(), "w");
    if (!ft) return GF_ERR_ARG;
    std::fputs(t.c_str(), ft);
    std::fclose(ft);
    FILE* fq = std::fopen(frame_name(dir, 'q', iframe).c_str(), "w");
    if (!fq) return GF_ERR_ARG;
    const int n4 = mx + 2 * mbc;
    const size_t S = (size_t)n4 * n4;
    std::string s;
    for (int k = 0; k < npatch; ++k) {
        s.clear();
        fort_i(grid_number ? grid_number[k] : k, 5, s);
        s += "                 grid_number\n";
        fort_i(level[k], 5, s);
        s += "                 AMR_level\n";
        fort_i(block ? block[k] : 0, 5, s);
        s += "                 block_number\n";
        fort_i(0, 5, s);
        s += "                 mpi_rank\n";
        fort_i(mx, 5, s);
        s += "                 mx\n";
        fort_i(mx, 5, s);
        s += "                 my\n";
        fort_e(xlower[k], 24, 16, s);
        s += "    xlow\n";
        fort_e(ylower[k], 24, 16, s);
        s += "    ylow\n";
        fort_e(dx[k], 24, 16, s);
        s += "    dx\n";
        fort_e(dy[k], 24, 16, s);
        s += "    dy\n\n";
        const double* qk = q + (size_t)k * 3 * S;
        const double* ak = aux + (size_t)k * maux * S;
        for (int j = 1; j <= mx; ++j) {
            for (int i = 1; i <= mx; ++i) {
                const size_t c = (size_t)(j + mbc - 1) * n4 + (i + mbc - 1);
                double v[3];
                for (int m = 0; m < 3; ++m) v[m] = tiny0(qk[c * 3 + m]);
                const double eta = tiny0(v[0] + ak[c * maux]);
                fort_e(v[0], 26, 16, s);
                fort_e(v[1], 26, 16, s);
                fort_e(v[2], 26, 16, s);
                fort_e(eta, 26, 16, s);
                s += "\n";
            }
            s += "  \n"; /* list-directed write of ' ' */
        }
        std::fputs(s.c_str(), fq);
    }
    std::fclose(fq);
    return GF_OK;
}

int gf_sample_gauge(int mx, int maux, const double* q, const double* aux, double xlower,
                    double ylower, double dx, double dy, double dry_tolerance, double xc,
                    double yc, double* out /* h, hu, hv, topo */)
{
    if (!q || !aux || !out || mx < 1 || maux < 1 || !(dx > 0) || !(dy > 0)) return GF_ERR_ARG;
    const int mbc = GF_MBC, n4 = mx + 2 * mbc;
    const int ii = (int)((xc - xlower) / dx) + 1;
    const int jj = (int)((yc - ylower) / dy) + 1;
    /* the gauge may sit on the patch's upper edge (ii = mx + 1): the stencil
     * then reaches the second ghost column, still inside the array */
    if (ii < 1 || ii > mx + 1 || jj < 1 || jj > mx + 1) return GF_ERR_ARG;
    const double xcent = xlower + (ii - .5) * dx, ycent = ylower + (jj - .5) * dy;
    const double xoff = (xc - xcent) / dx, yoff = (yc - ycent) / dy;
    const double drytol2 = 0.1 * dry_tolerance;
    auto at = [&](int i, int j) { return (size_t)(j + mbc - 1) * n4 + (i + mbc - 1); };
    const size_t c00 = at(ii, jj), c10 = at(ii + 1, jj), c01 = at(ii, jj + 1), c11 = at(ii + 1, jj + 1);
    const double* h = q;
    if (h[c00 * 3] < drytol2 || h[c10 * 3] < drytol2 || h[c01 * 3] < drytol2 || h[c11 * 3] < drytol2) {
        for (int m = 0; m < 3; ++m) out[m] = q[c00 * 3 + m];
        out[3] = aux[c00 * maux];
    } else {
        for (int m = 0; m < 3; ++m)
            out[m] = (1.0 - xoff) * (1.0 - yoff) * q[c00 * 3 + m] + xoff * (1.0 - yoff) * q[c10 * 3 + m] +
                     (1.0 - xoff) * yoff * q[c01 * 3 + m] + xoff * yoff * q[c11 * 3 + m];
        out[3] = (1.0 - xoff) * (1.0 - yoff) * aux[c00 * maux] + xoff * (1.0 - yoff) * aux[c10 * maux] +
                 (1.0 - xoff) * yoff * aux[c01 * maux] + xoff * yoff * aux[c11 * maux];
    }
    for (int m = 0; m < 3; ++m) out[m] = tiny0(out[m]);
    return GF_OK;
}

int gf_write_gauge_header(const char* dir, int id, double xc, double yc)
{
    char name[32];
    std::snprintf(name, sizeof name, "gauge%05d.txt", id);
    std::string p = dir && *dir ? std::string(dir) + "/" + name : std::string(name);
    FILE* fp = std::fopen(p.c_str(), "w");
    if (!fp) return GF_ERR_ARG;
    std::fprintf(fp, "# gauge_id= %5d location=( %17.10e %17.10e ) num_eqn= %2d\n", id, xc, yc, 4);
    std::fprintf(fp, "# Columns: level time h    hu    hv    eta\n");
    std::fclose(fp);
    return GF_OK;
}

int gf_write_gauge_rows(const char* dir, int id, int nrow, const int* level, const double* t,
                        const double* qv /* nrow x (h, hu, hv, topo) */)
{
    if (nrow < 0 || (nrow > 0 && (!level || !t || !qv))) return GF_ERR_ARG;
    char name[32];
    std::snprintf(name, sizeof name, "gauge%05d.txt", id);
    std::string p = dir && *dir ? std::string(dir) + "/" + name : std::string(name);
    FILE* fp = std::fopen(p.c_str(), "a");
    if (!fp) return GF_ERR_ARG;
    for (int k = 0; k < nrow; ++k) {
        const double* v = qv + 4 * k;
        const double eta = tiny0(v[0] + v[3]);
        std::fprintf(fp, "%5d %15.7e %15.7e %15.7e %15.7e %15.7e\n", level[k], t[k], v[0], v[1], v[2], eta);
    }
    std::fclose(fp);
    return GF_OK;
}

/* The file layout GeoClaw's setrun writes: five '#' header lines, one blank
 * line, the gauge count, one "id x y t1 t2" line per gauge, eight lines
 * skipped, then the min_time_increment of every gauge on one line. Read
 * line by line with strtod like the reference reader; a header line that
 * does not start with '#' is an error (the reference exits there). */
int gf_read_gauges_data(const char* path, int cap, int* n, int* id, double* xc, double* yc,
                        double* t1, double* t2, double* min_time_increment)
{
    if (!path || !n || cap < 0) return GF_ERR_ARG;
    *n = 0;
    FILE* fp = std::fopen(path, "r");
    if (!fp) return GF_ERR_ARG;
    char line[512];
    auto next_line = [&]() -> bool { return std::fgets(line, sizeof line, fp) != nullptr; };
    int rc = GF_OK;
    for (int i = 0; i < 5 && rc == GF_OK; ++i)
        if (!next_line() || line[0] != '#') rc = GF_ERR_ARG;
    if (rc == GF_OK && !next_line()) rc = GF_ERR_ARG; /* blank line */
    if (rc == GF_OK && !next_line()) rc = GF_ERR_ARG;
    int count = 0;
    if (rc == GF_OK) {
        const double v = std::strtod(line, nullptr);
        if (!(v >= 0) || v > 1e7) rc = GF_ERR_ARG;
        else count = (int)v;
    }
    if (rc == GF_OK) *n = count;
    if (rc == GF_OK && count > 0 && count <= cap) {
        if (!id || !xc || !yc || !t1 || !t2 || !min_time_increment) rc = GF_ERR_ARG;
        for (int i = 0; i < count && rc == GF_OK; ++i) {
            if (!next_line()) {
                rc = GF_ERR_ARG;
                break;
            }
            char* p = line;
            id[i] = (int)std::strtod(p, &p);
            xc[i] = std::strtod(p, &p);
            yc[i] = std::strtod(p, &p);
            t1[i] = std::strtod(p, &p);
            t2[i] = std::strtod(p, nullptr);
        }
        for (int i = 0; i < 8 && rc == GF_OK; ++i)
            if (!next_line()) rc = GF_ERR_ARG;
        if (rc == GF_OK && !next_line()) rc = GF_ERR_ARG;
        if (rc == GF_OK) {
            char* p = line;
            for (int i = 0; i < count; ++i) min_time_increment[i] = std::strtod(p, &p);
        }
    }
    std::fclose(fp);
    return rc;
}

} // extern "C"
