/*
 * CPU oracle for the GeoClaw patch update (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of the reference's Fortran hot path, used as the
 * parity checker for the CUDA path and as the timed CPU baseline. Nothing in
 * the shipped library links or calls this code.
 *
 * Arrays use the reference's Fortran layout:
 *   q(meqn, 1-mbc:mx+mbc, 1-mbc:my+mbc), aux(maux, 1-mbc:mx+mbc, 1-mbc:my+mbc)
 * i.e. the equation index is fastest, then i, then j, all contiguous.
 *
 * Parity status: the reference's Fortran cannot be compiled here (no Fortran
 * compiler, ForestClaw, p4est or MPI), and its own tests carry no golden
 * vectors for this path. The Riemann-solver core is cross-checked against
 * the reference's CUDA device functions compiled for the host by
 * oracle/build_ref.sh (see oracle/ref_riemann_shim.cpp); everything else is
 * checked against known-answer tests derived from the mathematics.
 */
#ifndef GEOCLAW_ORACLE_H
#define GEOCLAW_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Physics and method parameters (geoclaw_module / fc2d_geoclaw_options). */
typedef struct orc_params {
    double grav;              /* geoclaw_module.f90: grav                       */
    double dry_tolerance;     /* geoclaw_module.f90: dry_tolerance              */
    double sea_level;         /* geoclaw_module.f90: sea_level                  */
    double friction_depth;    /* geoclaw_module.f90: friction_depth             */
    int    friction_forcing;  /* geoclaw_module.f90: friction_forcing           */
    int    num_manning;       /* geoclaw_module.f90: num_manning (<= 4)         */
    double manning_coefficient[4];
    double manning_break[4];
    int    variable_friction; /* friction_module.f90: variable_friction         */
    int    friction_index;    /* friction_module.f90: friction_index (1-based)  */
    int    order;             /* method(2): 1 or 2                              */
    int    transverse;        /* method(3): 0, 1 or 2                           */
    int    mthlim[3];         /* limiter per wave family (philim.f)             */
    int    src_term;          /* fc2d_geoclaw_options: src_term                 */
    double maxcfl_cap;        /* fc2d_geoclaw.h MAXCFL_CAP (100)                */
} orc_params;

void orc_default_params(orc_params* p);

/* fc2d_geoclaw_b4step2 (geoclaw_b4step2_fort.f90:183-186). */
void orc_b4step2(const orc_params* p, int mbc, int mx, int my, double* q);

/* fc2d_geoclaw_step2 + the flux-difference update of fc2d_geoclaw_step2_wrap
 * (geoclaw_step2_fort.f90:80-250, geoclaw_step2_wrap_fort.f:94-115).
 * Returns cflgrid. */
double orc_step2(const orc_params* p, int mbc, int mx, int my, double* q,
                 const double* aux, int maux, double dx, double dy, double dt);

/* fc2d_geoclaw_src2 friction part (geoclaw_src2_fort.f90:41-71). */
void orc_src2(const orc_params* p, int mbc, int mx, int my, double* q,
              const double* aux, int maux, double dt);

/* geoclaw_update (fc2d_geoclaw.cpp:352-387): b4step2, step2, CFL cap, src2.
 * Returns the patch CFL number. */
double orc_patch_update(const orc_params* p, int mbc, int mx, int my,
                        double* q, const double* aux, int maux,
                        double dx, double dy, double t, double dt);

/* One level step over npatch patches of identical shape (the loop ForestClaw
 * runs over single_step_update). Patch k's arrays start at q + k*qstride and
 * aux + k*astride. dx[k], dy[k] per patch. Threads over patches (OpenMP)
 * when nthreads > 1. Returns the max CFL over patches. */
double orc_level_update(const orc_params* p, int npatch, int mbc, int mx,
                        int my, double* q, long qstride, const double* aux,
                        int maux, long astride, const double* dx,
                        const double* dy, double t, double dt, int nthreads);

/* Single-face entry points, exposed for the Riemann-solver pin against the
 * reference's own solver. */
void orc_riemanntype(double hL, double hR, double uL, double uR, double* hm,
                     double* s1m, double* s2m, int* rare1, int* rare2,
                     int maxiter, double drytol, double g);
void orc_riemann_aug_JCP(int maxiter, double hL, double hR, double huL,
                         double huR, double hvL, double hvR, double bL,
                         double bR, double uL, double uR, double vL,
                         double vR, double phiL, double phiR, double sE1,
                         double sE2, double drytol, double g, double* sw,
                         double* fw /* fw(3,3), column-major */);

/* rpn2 over a 1-D slice (rpn2_geoclaw.f:84-376). q1d(3, 1-mbc:mx+mbc),
 * aux1d(maux, ...). fwave(3,3,1-mbc:mx+mbc), s(3,...), amdq/apdq(3,...). */
void orc_rpn2(const orc_params* p, int ixy, int mbc, int mx, double* q1d,
              const double* aux1d, int maux, double* fwave, double* s,
              double* amdq, double* apdq);

/* rpt2 over a 1-D slice (rpt2_geoclaw.f:61-187). */
void orc_rpt2(const orc_params* p, int ixy, int imp, int mbc, int mx,
              const double* q1d, const double* aux1, const double* aux2,
              const double* aux3, int maux, const double* asdq,
              double* bmasdq, double* bpasdq);

/* Single-face views of rpn2 / rpt2 (see geoclaw_oracle.c). */
void orc_rpn2_face(const orc_params* p, int ixy, const double* ql, const double* qr, double bl,
                   double br, double* fwave, double* s, double* amdq, double* apdq);
/* qad (geolib_source/qad.f:4-371), one side of a fine patch (see
 * geoclaw_oracle_qad.c). */
void orc_qad_side(const orc_params* p, int side, int mbc, int mx, int my, int maux,
                  const double* qf, const double* af, const double* qc1d, const double* auxc1d,
                  double hx, double hy, double delt, double* svdflx);
void orc_rpt2_face(const orc_params* p, int ixy, int imp, const double* ql, const double* qr,
                   const double* aux1, const double* aux2, const double* aux3, const double* asdq,
                   double* bmasdq, double* bpasdq);

#ifdef __cplusplus
}
#endif
#endif

#ifdef __cplusplus
extern "C" {
#endif
/* Hydrograph inflow (hydrograph/hydrograh_module.f90), discharge type. */
typedef struct orc_hydro {
    int use;           /* use_hydrograph == 'True'                      */
    int side[4];       /* boundary_location(k) matches side k (1..4)     */
    double width;      /* b: channel width                               */
    double x0, y0;     /* channel centre                                 */
    int n;             /* rows of the table                              */
    const double* time;
    const double* hu;  /* discharge per unit width                       */
} orc_hydro;

/* fc2d_geoclaw_bc2 (fortran_source/geoflood_bc2_fort.f90:7-409); mthbc[k]
 * is the rule of side k (left, right, bottom, top), -1 = not physical. */
void orc_bc2(const orc_params* p, const orc_hydro* hy, int mbc, int mx, int my,
             double xlower, double ylower, double dx, double dy, double* q,
             double* aux, int maux, double t, const int* mthbc);

/* fc2d_geoclaw_fort_copy_face / _copy_corner (fclaw2d_source/
 * fc2d_geoclaw_copy_fort.f:11-107) for aligned same-level neighbours. */
void orc_copy_face(int mx, int my, int mbc, int meqn, double* qthis,
                   const double* qneighbor, int iface);
void orc_copy_corner(int mx, int my, int mbc, int meqn, double* qthis,
                     const double* qneighbor, int icorner);

/* Ghost fill of a same-level batch: face and corner copies from the
 * neighbour table nbr[8*k + s] (s = 0..3 faces left,right,bottom,top;
 * 4..7 corners ll,lr,ul,ur; -1 = physical boundary), then bc2 on the
 * physical sides of every patch. */
void orc_level_ghost_fill(const orc_params* p, const orc_hydro* hy, int npatch,
                          int mbc, int mx, int my, double* q, double* aux,
                          int maux, const int* nbr, const double* xlower,
                          const double* ylower, double dx, double dy,
                          double t, const int* mthbc);
#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
extern "C" {
#endif
/* Refinement regions (geolib_source/regions_module.f90 region_type). */
typedef struct orc_region {
    double x_low, x_hi, y_low, y_hi, t_low, t_hi;
    int min_level, max_level;
} orc_region;

/* refinement_data_module (geolib_source/refinement_data_module.f90:11-40). */
typedef struct orc_refine {
    double wave_tolerance;
    double speed_tolerance[8];
    int num_speed_tolerance;
    double deep_depth;
    int max_level_deep;
    double max_velocity_depth_product;
    int num_flowgrades;
    double flowgradevalue[4];
    int flowgradevariable[4];
    int flowgradetype[4];
    int flowgrademinlevel[4];
    int num_regions;
    orc_region regions[16];
} orc_refine;

/* Coarse ghost cells from a fine neighbour (kind 0 face, code = iface of the
 * coarse patch; kind 1 corner, code = icorner). (ox, oy): fine index of the
 * coarse patch's cell (1,1) lower-left corner, minus one. */
void orc_average_ghost(const orc_params* p, int mbc, int mx, int my, int maux, double* qc,
                       const double* ac, const double* qf, const double* af, int kind, int code,
                       int ox, int oy);
/* Fine ghost cells from a coarse neighbour (same conventions). */
void orc_interpolate_ghost(const orc_params* p, int mbc, int mx, int my, int maux,
                           const double* qc, const double* ac, double* qf, const double* af,
                           int kind, int code, int ox, int oy);
void orc_interpolate2fine(const orc_params* p, int mbc, int mx, int my, int maux,
                          const double* qc, const double* ac, double* qf, const double* af,
                          int igrid);
void orc_average2coarse(const orc_params* p, int mbc, int mx, int my, int maux, double* qc,
                        const double* ac, const double* qf, const double* af, int igrid);
int orc_timeinterp(int mbc, int mx, int my, int psize, const double* qcurr, const double* qlast,
                   double* qinterp, double alpha);
int orc_test_regions(const orc_refine* rf, int level, double xl, double yl, double xu, double yu,
                     double t, int refine);
int orc_flag2refine(const orc_params* p, const orc_refine* rf, int mbc, int mx, int my, int maux,
                    const double* q, const double* aux, int i, int j, int level, int maxlevel,
                    int init_flag, int is_coarsening);
int orc_tag4refinement(const orc_params* p, const orc_refine* rf, int mbc, int mx, int my,
                       int maux, const double* q, const double* aux, double xlower,
                       double ylower, double dx, double dy, double t, int level, int maxlevel,
                       int init_flag);
int orc_tag4coarsening(const orc_params* p, const orc_refine* rf, int mbc, int mx, int my,
                       int maux, const double* const* q, const double* const* aux,
                       const double* xlower, const double* ylower, double dx, double dy, double t,
                       int level, int maxlevel, int init_flag);

/* Topo grids (geoclaw_oracle_topo.c): node values z in file order (rows
 * north to south, x fastest), node extent [xlow, xhi] x [ylow, yhi]. */
typedef struct orc_topo_grid {
    const double* z;
    int mx, my;
    double xlow, ylow, xhi, yhi, dx, dy;
} orc_topo_grid;
void orc_topo_rank(const orc_topo_grid* g, int n, int* order);
double orc_topointegral(double xim, double xip, double yjm, double yjp, const orc_topo_grid* g);
int orc_cellgridintegrate(double* out, double xim, double xip, double yjm, double yjp,
                          const orc_topo_grid* g, const int* order, int n);
double orc_topo_area(double x1, double x2, double y1, double y2, const orc_topo_grid* g,
                     const int* order, int n);
/* Cell averages of a uniform raster of nx x ny cells plus a halo (row
 * pitch nx + 2 halo), as setaux sets aux(1) on the cells of a patch. */
int orc_setaux_raster(const orc_topo_grid* g, const int* order, int n, int nx, int ny, int halo,
                      double xlower, double ylower, double dx, double dy, double xupper,
                      double yupper, double* out);
#ifdef __cplusplus
}
#endif
