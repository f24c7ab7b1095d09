/*
 * Topography sets: GeoClaw topo file readers, file ranking, coverage, and
 * the host side of the cell-average launches (gf_topo_kernels.cu).
 *
 * Readers follow read_topo_header / read_topo_file
 * (src/fc2d_geoclaw/geolib_source/topo_module.f90:491-769, 785-1059):
 *   type 1   records "x y z", rows north to south; the first row's length
 *            is found by reading until y changes, the extent from the first
 *            and last records;
 *   type 2/3 a six-line header whose numbers parse_values extracts
 *            (utility_module.f90:53-108): ncols, nrows, xll, yll, cellsize
 *            (one or two values), nodata; "xllcorner" / "yllcorner" move the
 *            corner half a cell to the first node; then one value per record
 *            (type 2) or one row per record (type 3, a row may continue on
 *            the next records);
 *   a negative type negates z; nodata nodes take topo_missing, and the
 *   default 99999 is refused when a file has any (the reference stops).
 * Ranking (topo_module.f90:298-318): finest cell area first; of two files
 * with equal cell areas, the later one first.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gf_internal.h"

namespace {

struct TopoGrid {
    int mx = 0, my = 0;
    double xlow = 0, ylow = 0, xhi = 0, yhi = 0, dx = 0, dy = 0;
    std::vector<double> z; /* file order */
};

/* a Fortran real constant (list-directed input): [+-]digits[.digits][e|d[+-]digits] */
bool fort_real(std::string w, double* v)
{
    while (!w.empty() && w.back() == ',') w.pop_back();
    size_t i = 0, n = w.size();
    if (n == 0) return false;
    if (w[i] == '+' || w[i] == '-') ++i;
    size_t dig = 0;
    while (i < n && std::isdigit((unsigned char)w[i])) ++i, ++dig;
    if (i < n && w[i] == '.') {
        ++i;
        while (i < n && std::isdigit((unsigned char)w[i])) ++i, ++dig;
    }
    if (dig == 0) return false;
    if (i < n && (w[i] == 'e' || w[i] == 'E' || w[i] == 'd' || w[i] == 'D')) {
        w[i] = 'e';
        ++i;
        if (i < n && (w[i] == '+' || w[i] == '-')) ++i;
        size_t ed = 0;
        while (i < n && std::isdigit((unsigned char)w[i])) ++i, ++ed;
        if (ed == 0) return false;
    }
    if (i != n) return false;
    *v = std::strtod(w.c_str(), nullptr);
    return true;
}

std::vector<std::string> words(const std::string& line)
{
    std::vector<std::string> out;
    size_t i = 0;
    while (i < line.size()) {
        while (i < line.size() && std::isspace((unsigned char)line[i])) ++i;
        size_t j = i;
        while (j < line.size() && !std::isspace((unsigned char)line[j])) ++j;
        if (j > i) out.push_back(line.substr(i, j - i));
        i = j;
    }
    return out;
}

std::vector<double> parse_values(const std::string& line)
{
    std::vector<double> v;
    double x;
    for (const std::string& w : words(line))
        if (fort_real(w, &x)) v.push_back(x);
    return v;
}

bool read_lines(const char* path, std::vector<std::string>* lines)
{
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return false;
    std::string cur;
    char buf[1 << 16];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof buf, fp)) > 0) {
        for (size_t i = 0; i < k; ++i) {
            if (buf[i] == '\n') {
                lines->push_back(cur);
                cur.clear();
            } else {
                cur.push_back(buf[i]);
            }
        }
    }
    if (!cur.empty()) lines->push_back(cur);
    std::fclose(fp);
    return true;
}

inline int fortran_nint(double v) { return (int)(v >= 0 ? std::floor(v + 0.5) : -std::floor(-v + 0.5)); }

std::string lower(std::string s)
{
    for (char& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

/* returns an error text or nullptr */
/* ---- NetCDF classic files (topo type 4) ----
 * The classic format's header, big-endian throughout: "CDF" and a version
 * byte (1: 32-bit offsets, 2: 64-bit offsets, 5: 64-bit sizes), the record
 * count, then the dimension, global attribute and variable lists, each a tag
 * (0x0A / 0x0C / 0x0B, or 0 when absent) and a count. Names and attribute
 * values are padded to 4 bytes. A non-record variable's values lie
 * contiguous at its `begin` offset, last dimension fastest. NetCDF-4 files
 * (HDF5 containers) are not read. */
struct NcVar {
    std::string name;
    std::vector<int> dims;
    int type = 0;
    uint64_t begin = 0;
    std::string positive; /* the text attribute "positive", if any */
};

struct NcFile {
    std::vector<std::pair<std::string, uint64_t>> dims;
    std::vector<NcVar> vars;
    std::vector<unsigned char> buf;
};

int nc_type_size(int t)
{
    switch (t) {
    case 1: case 2: case 7: return 1;  /* byte, char, ubyte */
    case 3: case 8: return 2;          /* short, ushort     */
    case 4: case 5: case 9: return 4;  /* int, float, uint  */
    case 6: case 10: case 11: return 8; /* double, int64, uint64 */
    default: return 0;
    }
}

struct NcReader {
    const std::vector<unsigned char>& b;
    size_t i = 0;
    bool ok = true;
    bool wide = false; /* CDF-5: 64-bit counts */
    explicit NcReader(const std::vector<unsigned char>& buf) : b(buf) {}
    uint64_t be(int n)
    {
        if (i + n > b.size()) {
            ok = false;
            return 0;
        }
        uint64_t v = 0;
        for (int k = 0; k < n; ++k) v = (v << 8) | b[i + k];
        i += n;
        return v;
    }
    uint64_t count() { return be(wide ? 8 : 4); }
    void pad() { i = (i + 3) & ~(size_t)3; }
    std::string name()
    {
        const uint64_t n = count();
        if (!ok || i + n > b.size()) {
            ok = false;
            return {};
        }
        std::string s(reinterpret_cast<const char*>(&b[i]), (size_t)n);
        i += n;
        pad();
        return s;
    }
    /* an attribute list; returns the text attribute `want` (or "") */
    std::string atts(const char* want)
    {
        std::string found;
        const uint64_t tag = be(4), n = count();
        if (tag == 0) return found;
        if (tag != 0x0C) {
            ok = false;
            return found;
        }
        for (uint64_t k = 0; k < n && ok; ++k) {
            const std::string nm = name();
            const int type = (int)be(4);
            const uint64_t nel = count();
            const int sz = nc_type_size(type);
            if (!sz || i + nel * sz > b.size()) {
                ok = false;
                break;
            }
            if (type == 2 && nm == want) found.assign(reinterpret_cast<const char*>(&b[i]), (size_t)nel);
            i += nel * sz;
            pad();
        }
        return found;
    }
};

const char* nc_parse(NcFile* f)
{
    const std::vector<unsigned char>& b = f->buf;
    if (b.size() >= 4 && b[0] == 0x89 && b[1] == 'H' && b[2] == 'D' && b[3] == 'F')
        return "NetCDF-4 (HDF5) topo files are not read: convert to the classic format";
    if (b.size() < 8 || b[0] != 'C' || b[1] != 'D' || b[2] != 'F' || !(b[3] == 1 || b[3] == 2 || b[3] == 5))
        return "not a NetCDF classic file";
    const int version = b[3];
    NcReader r(b);
    r.i = 4;
    r.wide = version == 5;
    r.count(); /* record count */
    uint64_t tag = r.be(4), n = r.count();
    if (tag != 0 && tag != 0x0A) return "NetCDF header: bad dimension list";
    for (uint64_t k = 0; k < n && r.ok; ++k) {
        std::string nm = r.name();
        const uint64_t len = r.count();
        f->dims.emplace_back(nm, len);
    }
    r.atts("");
    tag = r.be(4);
    n = r.count();
    if (tag != 0 && tag != 0x0B) return "NetCDF header: bad variable list";
    for (uint64_t k = 0; k < n && r.ok; ++k) {
        NcVar v;
        v.name = r.name();
        const uint64_t nd = r.count();
        for (uint64_t d = 0; d < nd && r.ok; ++d) {
            const uint64_t id = r.count();
            if (id >= f->dims.size()) return "NetCDF header: bad dimension id";
            v.dims.push_back((int)id);
        }
        v.positive = r.atts("positive");
        v.type = (int)r.be(4);
        r.count(); /* vsize */
        v.begin = r.be(version == 1 ? 4 : 8);
        f->vars.push_back(std::move(v));
    }
    return r.ok ? nullptr : "NetCDF header ends early";
}

/* a non-record variable's values as doubles, last dimension fastest */
const char* nc_values(const NcFile& f, const NcVar& v, std::vector<double>* out)
{
    uint64_t n = 1;
    for (int d : v.dims) {
        if (f.dims[d].second == 0) return "NetCDF record variables are not read";
        n *= f.dims[d].second;
    }
    const int sz = nc_type_size(v.type);
    if (!sz || v.type == 2) return "NetCDF variable of a non-numeric type";
    if (v.begin + n * sz > f.buf.size()) return "NetCDF variable beyond the end of the file";
    out->resize((size_t)n);
    const unsigned char* p = &f.buf[(size_t)v.begin];
    for (uint64_t k = 0; k < n; ++k, p += sz) {
        uint64_t u = 0;
        for (int j = 0; j < sz; ++j) u = (u << 8) | p[j];
        double x;
        switch (v.type) {
        case 1: x = (double)(int8_t)u; break;
        case 3: x = (double)(int16_t)u; break;
        case 4: x = (double)(int32_t)u; break;
        case 5: {
            uint32_t w = (uint32_t)u;
            float fl;
            std::memcpy(&fl, &w, 4);
            x = fl;
            break;
        }
        case 6: std::memcpy(&x, &u, 8); break;
        case 7: x = (double)(uint8_t)u; break;
        case 8: x = (double)(uint16_t)u; break;
        case 9: x = (double)(uint32_t)u; break;
        case 10: x = (double)(int64_t)u; break;
        default: x = (double)u; break;
        }
        (*out)[(size_t)k] = x;
    }
    return nullptr;
}

/* topo type 4 as read_topo_file / read_topo_header read it
 * (geolib_source/topo_module.f90:624-732, :926-1035, get_dim_info :1599-1623):
 * x and y dimensions named lon / longitude / x and lat / latitude / y (any
 * case), their coordinate variables of the same names, and the last 2-D
 * variable as z in either dimension order; rows stored north first; z
 * negated when its attribute positive is "down" and the type is negative.
 * The whole grid is kept (the reference crops it to the domain plus one
 * spacing, which leaves every cell integral inside the domain unchanged). */
const char* read_netcdf(const char* path, int topo_type, TopoGrid* g)
{
    NcFile f;
    {
        std::FILE* fp = std::fopen(path, "rb");
        if (!fp) return "cannot open the topo file";
        unsigned char chunk[65536];
        size_t got;
        while ((got = std::fread(chunk, 1, sizeof chunk, fp)) > 0) f.buf.insert(f.buf.end(), chunk, chunk + got);
        std::fclose(fp);
    }
    if (const char* e = nc_parse(&f)) return e;
    auto upper = [](std::string s) {
        for (char& c : s) c = (char)std::toupper((unsigned char)c);
        return s;
    };
    int xd = -1, yd = -1;
    for (size_t d = 0; d < f.dims.size(); ++d) {
        const std::string u = upper(f.dims[d].first);
        if (u == "LON" || u == "LONGITUDE" || u == "X") xd = (int)d;
        else if (u == "LAT" || u == "LATITUDE" || u == "Y") yd = (int)d;
    }
    if (xd < 0 || yd < 0) return "NetCDF topo: no x / y (lon / lat) dimensions";
    const NcVar *xv = nullptr, *yv = nullptr, *zv = nullptr;
    for (const NcVar& v : f.vars) {
        if (v.name == f.dims[xd].first) xv = &v;
        else if (v.name == f.dims[yd].first) yv = &v;
        else if (v.dims.size() == 2) zv = &v;
    }
    if (!xv || !yv) return "NetCDF topo: no coordinate variables for x and y";
    if (!zv) return "NetCDF topo: no topography variable";
    std::vector<double> xs, ys, zs;
    if (const char* e = nc_values(f, *xv, &xs)) return e;
    if (const char* e = nc_values(f, *yv, &ys)) return e;
    if (const char* e = nc_values(f, *zv, &zs)) return e;
    const int mx = (int)xs.size(), my = (int)ys.size();
    if (mx < 2 || my < 2) return "NetCDF topo: need at least 2 x 2 nodes";
    const bool yx = zv->dims[0] == yd && zv->dims[1] == xd; /* x fastest */
    const bool xy = zv->dims[0] == xd && zv->dims[1] == yd;
    if (!yx && !xy) return "NetCDF z variable has dimensions that don't align with x and y";
    g->mx = mx;
    g->my = my;
    g->xlow = xs[0];
    g->ylow = ys[0];
    g->dx = xs[1] - xs[0];
    g->dy = ys[1] - ys[0];
    g->xhi = xs[mx - 1];
    g->yhi = ys[my - 1];
    g->z.resize((size_t)mx * my);
    for (int j = 0; j < my; ++j)
        for (int i = 0; i < mx; ++i) {
            const int jy = my - 1 - j; /* row 0 is the northernmost */
            g->z[(size_t)j * mx + i] = yx ? zs[(size_t)jy * mx + i] : zs[(size_t)i * my + jy];
        }
    if (topo_type < 0 && lower(zv->positive) == "down")
        for (double& z : g->z) z = -z;
    return nullptr;
}

const char* read_topo(const char* path, int topo_type, double topo_missing, TopoGrid* g)
{
    if (std::abs(topo_type) == 4) {
        if (const char* e = read_netcdf(path, topo_type, g)) return e;
        if (!(g->dx > 0) || !(g->dy > 0)) return "topo grid spacing must be positive";
        if (topo_type < 0)
            for (double& z : g->z) z = -z;
        return nullptr;
    }
    std::vector<std::string> lines;
    if (!read_lines(path, &lines)) return "cannot open the topo file";
    const int t = std::abs(topo_type);
    if (t == 1) {
        std::vector<std::vector<double>> recs;
        for (const std::string& l : lines) {
            std::vector<double> v = parse_values(l);
            if (!v.empty()) recs.push_back(std::move(v));
        }
        if (recs.size() < 4 || recs[0].size() < 3) return "topo type 1: too few records";
        for (const auto& r : recs)
            if (r.size() < 3) return "topo type 1: a record without x y z";
        const double xll = recs[0][0], yhi = recs[0][1];
        size_t k = 1;
        int mx = 1;
        double y = yhi;
        while (y == yhi) {
            if (k >= recs.size()) return "topo type 1: a single row";
            y = recs[k][1];
            ++k;
            ++mx;
        }
        mx -= 1;
        const long size = (long)recs.size();
        const int my = (int)(size / mx);
        if (mx < 2 || my < 2 || (long)mx * my > size) return "topo type 1: bad grid shape";
        g->mx = mx;
        g->my = my;
        g->xlow = xll;
        g->yhi = yhi;
        g->xhi = recs.back()[0];
        g->ylow = recs.back()[1];
        g->dx = (g->xhi - g->xlow) / (mx - 1);
        g->dy = (g->yhi - g->ylow) / (my - 1);
        g->z.resize((size_t)mx * my);
        for (size_t i = 0; i < g->z.size(); ++i) g->z[i] = recs[i][2];
    } else if (t == 2 || t == 3) {
        if (lines.size() < 6) return "topo type 2/3: header too short";
        std::vector<double> v[6];
        for (int k = 0; k < 6; ++k) {
            v[k] = parse_values(lines[k]);
            if (v[k].empty()) return "topo type 2/3: a header line without a number";
        }
        g->mx = fortran_nint(v[0][0]);
        g->my = fortran_nint(v[1][0]);
        if (g->mx < 2 || g->my < 2) return "topo type 2/3: need at least 2 x 2 nodes";
        g->xlow = v[2][0];
        g->ylow = v[3][0];
        g->dx = v[4][0];
        g->dy = v[4].size() == 2 ? v[4][1] : g->dx;
        const double nodata = v[5][0];
        if (lower(lines[2]).find("xllcorner") != std::string::npos) g->xlow = g->xlow + 0.5 * g->dx;
        if (lower(lines[3]).find("yllcorner") != std::string::npos) g->ylow = g->ylow + 0.5 * g->dy;
        g->xhi = g->xlow + (g->mx - 1) * g->dx;
        g->yhi = g->ylow + (g->my - 1) * g->dy;
        const size_t need = (size_t)g->mx * g->my;
        g->z.assign(need, 0.0);
        size_t k = 6;
        if (t == 2) {
            for (size_t i = 0; i < need; ++i) {
                std::vector<double> r;
                while (k < lines.size() && (r = parse_values(lines[k])).empty()) ++k;
                if (k >= lines.size()) return "topo type 2: file ends early";
                g->z[i] = r[0];
                ++k;
            }
        } else {
            for (int j = 0; j < g->my; ++j) {
                std::vector<double> row;
                while ((int)row.size() < g->mx) {
                    if (k >= lines.size()) return "topo type 3: file ends early";
                    std::vector<double> r = parse_values(lines[k++]);
                    row.insert(row.end(), r.begin(), r.end());
                }
                std::copy(row.begin(), row.begin() + g->mx, g->z.begin() + (size_t)j * g->mx);
            }
        }
        long missing = 0;
        for (double& z : g->z)
            if (z == nodata) {
                z = topo_missing;
                ++missing;
            }
        if (missing > 0 && topo_missing == 99999.0)
            return "the topo file has missing data and topo_missing is the default 99999";
    } else {
        return "topo type must be +-1, +-2, +-3 or +-4";
    }
    if (!(g->dx > 0) || !(g->dy > 0)) return "topo grid spacing must be positive";
    if (topo_type < 0)
        for (double& z : g->z) z = -z;
    return nullptr;
}

} // namespace

struct gf_topo {
    double missing = 99999.0;
    std::vector<TopoGrid> grids;
    std::string err;
    /* device copy (one device at a time) */
    int dev = -1;
    bool stale = true;
    double* d_z = nullptr;
    gf_topo_grid* d_grid = nullptr;
    int* d_order = nullptr;
    std::vector<int> order;
};

namespace {

void rank(gf_topo* t)
{
    const int n = (int)t->grids.size();
    t->order.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        int finer_than = 0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            const double ai = t->grids[i].dx * t->grids[i].dy, aj = t->grids[j].dx * t->grids[j].dy;
            if (ai < aj) ++finer_than;
            if (ai == aj && j < i) ++finer_than;
        }
        t->order[n - finer_than - 1] = i;
    }
}

void release_device(gf_topo* t)
{
    if (t->dev >= 0) {
        cudaSetDevice(t->dev);
        if (t->d_z) cudaFree(t->d_z);
        if (t->d_grid) cudaFree(t->d_grid);
        if (t->d_order) cudaFree(t->d_order);
    }
    t->d_z = nullptr;
    t->d_grid = nullptr;
    t->d_order = nullptr;
    t->dev = -1;
    t->stale = true;
}

void overlap(double a1, double a2, double b1, double b2, double c1, double c2, double d1, double d2,
             double* xlo, double* xhi, double* ylo, double* yhi, double* area)
{
    *xlo = std::max(a1, c1);
    *xhi = std::min(a2, c2);
    *ylo = std::max(b1, d1);
    *yhi = std::min(b2, d2);
    *area = (*xhi > *xlo && *yhi > *ylo) ? (*xhi - *xlo) * (*yhi - *ylo) : 0.0;
}

/* topoarea (topo_module.f90:1384-1456), m = 0-based rank */
double topo_area(const gf_topo* t, double x1, double x2, double y1, double y2, int m)
{
    const TopoGrid& G = t->grids[t->order[m]];
    double a, b, c, d, area;
    overlap(x1, x2, y1, y2, G.xlow, G.xhi, G.ylow, G.yhi, &a, &b, &c, &d, &area);
    if (m == (int)t->grids.size() - 1) return area;
    const double area1 = topo_area(t, x1, x2, y1, y2, m + 1);
    if (area > 0) return area1 - topo_area(t, a, b, c, d, m + 1) + area;
    return area1;
}

} // namespace

namespace gf {

/* upload the grids to device `dev` (once per change); *grid, *order set */
int topo_device(gf_topo* t, int dev, cudaStream_t st, const gf_topo_grid** grid, const int** order, int* n)
{
    *n = (int)t->grids.size();
    if (*n == 0) return GF_ERR_STATE;
    if (t->dev != dev || t->stale) {
        release_device(t);
        rank(t);
        size_t total = 0;
        for (const TopoGrid& g : t->grids) total += g.z.size();
        if (cudaMalloc(&t->d_z, total * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&t->d_grid, t->grids.size() * sizeof(gf_topo_grid)) != cudaSuccess ||
            cudaMalloc(&t->d_order, t->grids.size() * sizeof(int)) != cudaSuccess) {
            t->dev = dev;
            release_device(t);
            return GF_ERR_NOMEM;
        }
        t->dev = dev;
        std::vector<gf_topo_grid> hg(t->grids.size());
        size_t off = 0;
        for (size_t k = 0; k < t->grids.size(); ++k) {
            const TopoGrid& g = t->grids[k];
            if (cudaMemcpy(t->d_z + off, g.z.data(), g.z.size() * sizeof(double), cudaMemcpyHostToDevice) !=
                cudaSuccess)
                return GF_ERR_CUDA;
            hg[k] = gf_topo_grid{t->d_z + off, g.mx, g.my, g.xlow, g.ylow, g.xhi, g.yhi, g.dx, g.dy};
            off += g.z.size();
        }
        if (cudaMemcpy(t->d_grid, hg.data(), hg.size() * sizeof(gf_topo_grid), cudaMemcpyHostToDevice) !=
                cudaSuccess ||
            cudaMemcpy(t->d_order, t->order.data(), t->order.size() * sizeof(int), cudaMemcpyHostToDevice) !=
                cudaSuccess)
            return GF_ERR_CUDA;
        t->stale = false;
    }
    (void)st;
    *grid = t->d_grid;
    *order = t->d_order;
    return GF_OK;
}

/* cell averages of a raster into device memory `out` (row pitch nx + 2 halo) */
int topo_raster_device(gf_ctx* c, gf_topo* t, int nx, int ny, int halo, double xlower, double ylower, double dx,
                       double dy, double xupper, double yupper, double* out, cudaStream_t st)
{
    const gf_topo_grid* grid;
    const int* order;
    int n;
    int rc = topo_device(t, ctx_device(c), st, &grid, &order, &n);
    if (rc == GF_ERR_STATE) return ctx_fail(c, rc, "the topo set has no grids");
    if (rc) return ctx_fail(c, rc, "topo upload failed");
    int* d_err = nullptr;
    cudaError_t e = cudaMallocAsync(&d_err, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_err, 0, sizeof(int), st);
    if (e == cudaSuccess)
        e = launch_topo_raster(grid, order, n, nx, ny, halo, xlower, ylower, dx, dy, xupper, yupper, out, d_err,
                               st);
    int h_err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (d_err) cudaFreeAsync(d_err, st);
    if (e != cudaSuccess) return ctx_cuda_fail(c, e, "topo raster");
    if (h_err) return ctx_fail(c, GF_ERR_ARG, "a cell overlaps no topo grid (the reference stops here)");
    return GF_OK;
}

} // namespace gf

extern "C" {

int gf_topo_create(gf_topo** out)
{
    if (!out) return GF_ERR_ARG;
    *out = new gf_topo;
    return GF_OK;
}

void gf_topo_destroy(gf_topo* t)
{
    if (!t) return;
    release_device(t);
    delete t;
}

int gf_topo_set_missing(gf_topo* t, double topo_missing)
{
    if (!t || !std::isfinite(topo_missing)) return GF_ERR_ARG;
    t->missing = topo_missing;
    return GF_OK;
}

int gf_topo_read_file(gf_topo* t, const char* path, int topo_type)
{
    if (!t || !path) return GF_ERR_ARG;
    if ((int)t->grids.size() >= GF_TOPO_MAX_FILES) return GF_ERR_UNSUPPORTED;
    TopoGrid g;
    const char* err = read_topo(path, topo_type, t->missing, &g);
    if (err) {
        t->err = err;
        return GF_ERR_ARG;
    }
    t->grids.push_back(std::move(g));
    t->stale = true;
    return GF_OK;
}

int gf_topo_add_grid(gf_topo* t, int mx, int my, double xll, double yll, double dx, double dy, const double* z)
{
    if (!t || !z || mx < 2 || my < 2 || !(dx > 0) || !(dy > 0)) return GF_ERR_ARG;
    if ((int)t->grids.size() >= GF_TOPO_MAX_FILES) return GF_ERR_UNSUPPORTED;
    TopoGrid g;
    g.mx = mx;
    g.my = my;
    g.xlow = xll;
    g.ylow = yll;
    g.dx = dx;
    g.dy = dy;
    g.xhi = xll + (mx - 1) * dx;
    g.yhi = yll + (my - 1) * dy;
    g.z.assign(z, z + (size_t)mx * my);
    t->grids.push_back(std::move(g));
    t->stale = true;
    return GF_OK;
}

/* topo.data as read_topo_settings reads it (topo_module.f90:183-226) after
 * opendatafile (amrlib_source/opendatafile.f), which consumes the leading
 * '#' lines and the first line after them */
int gf_topo_read_data(gf_topo* t, const char* topo_data_path)
{
    if (!t || !topo_data_path) return GF_ERR_ARG;
    std::vector<std::string> L;
    if (!read_lines(topo_data_path, &L)) return GF_ERR_ARG;
    size_t k = 0;
    while (k < L.size() && !L[k].empty() && L[k][0] == '#') ++k;
    ++k; /* the first line that is not a comment */
    auto next_nonblank = [&]() -> const std::string* {
        while (k < L.size() && words(L[k]).empty()) ++k;
        return k < L.size() ? &L[k++] : nullptr;
    };
    const std::string* r = next_nonblank();
    double v;
    if (!r || !fort_real(words(*r)[0], &v)) return GF_ERR_ARG;
    const double missing = v;
    if (k >= L.size()) return GF_ERR_ARG;
    const std::string& tl = L[k++]; /* read(iunit, "(i1)") */
    const int test_topo = (tl.empty() || tl[0] == ' ') ? 0 : (std::isdigit((unsigned char)tl[0]) ? tl[0] - '0' : -1);
    if (test_topo != 0) {
        t->err = "analytic test topography (test_topography > 0) is not supported";
        return GF_ERR_UNSUPPORTED;
    }
    r = next_nonblank();
    if (!r || !fort_real(words(*r)[0], &v) || v < 0) return GF_ERR_ARG;
    const int nfiles = (int)v;
    std::string dir(topo_data_path);
    const size_t slash = dir.find_last_of('/');
    dir = slash == std::string::npos ? std::string() : dir.substr(0, slash + 1);
    t->missing = missing;
    for (int i = 0; i < nfiles; ++i) {
        r = next_nonblank();
        if (!r) return GF_ERR_ARG;
        std::string name;
        const size_t q1 = r->find_first_of("'\"");
        if (q1 != std::string::npos) {
            const size_t q2 = r->find((*r)[q1], q1 + 1);
            if (q2 == std::string::npos) return GF_ERR_ARG;
            name = r->substr(q1 + 1, q2 - q1 - 1);
        } else {
            name = words(*r)[0];
        }
        r = next_nonblank();
        if (!r || !fort_real(words(*r)[0], &v)) return GF_ERR_ARG;
        const int type = (int)v;
        std::string path = name;
        if (name[0] != '/') {
            FILE* probe = std::fopen(name.c_str(), "rb");
            if (probe) std::fclose(probe);
            else path = dir + name;
        }
        int rc = gf_topo_read_file(t, path.c_str(), type);
        if (rc) return rc;
    }
    return GF_OK;
}

int gf_topo_count(const gf_topo* t) { return t ? (int)t->grids.size() : -1; }

int gf_topo_grid_info(const gf_topo* t, int k, int* mx, int* my, double* xlow, double* ylow, double* xhi,
                      double* yhi, double* dx, double* dy, double* z)
{
    if (!t || k < 0 || k >= (int)t->grids.size()) return GF_ERR_ARG;
    const TopoGrid& g = t->grids[k];
    if (mx) *mx = g.mx;
    if (my) *my = g.my;
    if (xlow) *xlow = g.xlow;
    if (ylow) *ylow = g.ylow;
    if (xhi) *xhi = g.xhi;
    if (yhi) *yhi = g.yhi;
    if (dx) *dx = g.dx;
    if (dy) *dy = g.dy;
    if (z) std::copy(g.z.begin(), g.z.end(), z);
    return GF_OK;
}

int gf_topo_covered_area(const gf_topo* t, double x1, double x2, double y1, double y2, double* area)
{
    if (!t || !area) return GF_ERR_ARG;
    if (t->grids.empty()) {
        *area = 0.0;
        return GF_OK;
    }
    gf_topo* tt = const_cast<gf_topo*>(t);
    if (tt->order.size() != tt->grids.size() || tt->stale) rank(tt);
    *area = topo_area(t, x1, x2, y1, y2, 0);
    return GF_OK;
}

int gf_topo_raster(gf_ctx* c, gf_topo* t, int nx, int ny, int halo, double xlower, double ylower, double dx,
                   double dy, double xupper, double yupper, double* out)
{
    if (!c || !t || !out || nx < 1 || ny < 1 || halo < 0 || halo > 8 || !(dx > 0) || !(dy > 0)) return GF_ERR_ARG;
    /* the domain holds at least one cell, so every cell outside it has a
     * nearest cell inside within the raster */
    if (!(xupper - xlower >= dx) || !(yupper - ylower >= dy)) return GF_ERR_ARG;
    cudaError_t e = cudaSetDevice(gf::ctx_device(c));
    if (e != cudaSuccess) return gf::ctx_cuda_fail(c, e, "cudaSetDevice");
    cudaStream_t st = gf::ctx_stream(c);
    const size_t cells = (size_t)(nx + 2 * halo) * (ny + 2 * halo);
    double* d = nullptr;
    e = cudaMallocAsync(&d, cells * sizeof(double), st);
    if (e != cudaSuccess) return gf::ctx_cuda_fail(c, e, "topo raster buffer");
    int rc = gf::topo_raster_device(c, t, nx, ny, halo, xlower, ylower, dx, dy, xupper, yupper, d, st);
    if (!rc) {
        e = cudaMemcpyAsync(out, d, cells * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = gf::ctx_cuda_fail(c, e, "topo raster download");
    }
    cudaFreeAsync(d, st);
    cudaStreamSynchronize(st);
    return rc;
}

} // extern "C"
