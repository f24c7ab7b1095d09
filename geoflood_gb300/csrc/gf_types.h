/*
 * Shared host/device types for the GB300 patch-update path.
 *
 * Device layout of a level batch (structure of arrays, per patch contiguous):
 *   q   : [patch][field h|hu|hv][j = 0..my+3][i = 0..mx+3]   (mbc = 2 halo)
 *   aux : [patch][field][j][i], field 0 = bathymetry b
 * Each patch block starts on a 16-byte boundary so it can be staged into
 * shared memory with one bulk-async (TMA) copy per field group.
 */
#ifndef GF_TYPES_H
#define GF_TYPES_H

#include <stdint.h>

#include "geoflood_gb300.h"

#define GF_MBC 2
#define GF_MEQN 3

/* Activity of one patch (dry-patch culling of the served form). The update
 * kernel records, for the state it read (the patch and its two-cell halo):
 * `wet` = some cell deeper than the dry tolerance, and `ident` = no cell
 * wet and b4step2 changed nothing, so that update was an exact identity
 * and left the same interior in both state buffers. Before the next
 * update the ghost fill sets `skip` for a patch whose update would again be
 * the identity: ident set, no neighbour (faces and corners) wet, no
 * hydrograph side. Ghost fill and update then leave the patch alone. */
typedef struct gf_patch_flags {
    unsigned char skip;
    unsigned char ident;
    unsigned char wet;
    unsigned char pad;
} gf_patch_flags;

/* One unit of work for the patch-update kernel: a patch of any forest. */
typedef struct gf_patch_work {
    double* q;          /* device: 3 planes of (mx+4)*(my+4) doubles   */
    double* qout;       /* interior cells of the result; null = q      */
    const double* aux;  /* device: maux planes of (mx+4)*(my+4) doubles */
    gf_patch_flags* fl; /* activity flags, or null: always updated     */
    double dx, dy;
    int phys;           /* index into the gf_phys table                */
    int group;          /* time-step group: dt slot and CFL max slot   */
} gf_patch_work;

/* Position and spacing of one patch (lower-left corner of cell (1,1)). */
typedef struct gf_patch_geom {
    double xlower, ylower, dx, dy;
} gf_patch_geom;

/* Physical boundary rules of a level and the hydrograph inflow state for
 * the current time (q0hu = interpolated discharge per unit width). */
typedef struct gf_bc_spec {
    int mthbc[4];      /* left, right, bottom, top: 0 inflow, 1 extrap, 2 periodic, 3 wall */
    int hydro_side[4]; /* side uses the hydrograph (rule 0)                                */
    double width, x0, y0;
    double q0hu;
} gf_bc_spec;

/* Ghost fill of one block of same-level patches sharing a layout (a level
 * of one forest, or one served scenario). nbr holds 8 entries per patch
 * (left, right, bottom, top, ll, lr, ul, ur) as block-local indices, -1 for
 * a physical side and -2 for a side filled by another route (coarse/fine). */
typedef struct gf_ghost_block {
    double* q;                  /* block's q, patch p at q + 3*S*p             */
    double* aux;                /* block's aux, patch p at aux + maux*S*p      */
    const int* nbr;
    const gf_patch_geom* geom;
    const int* phys_of;         /* per-patch physics slot, or null = phys      */
    gf_patch_flags* fl;         /* per-patch activity (culling), or null       */
    gf_bc_spec bc;
    int phys, maux;
    int skip;                   /* non-zero: leave this block alone this round */
    int pad;
} gf_ghost_block;

/* Per-group q-pointer offset of a group with no step this round: its
 * coarse/fine transfer tasks are skipped. */
#define GF_QDELTA_SKIP (-0x7fffffffffffffffLL - 1)

/* A patch of a ghost-fill list: (block, block-local patch index). */
typedef struct gf_ghost_ref {
    int block, local;
} gf_ghost_ref;

/* Time-step controller of one served scenario, kept on the device
 * (ForestClaw outstyle 1, src/fc2d_geoclaw/fc2d_geoclaw_run.c:190-395). */
typedef struct gf_group_state {
    double* qb[2];             /* the scenario's two state buffers            */
    double t_curr, tend, dt_outer, dt_minlevel, dt_step;
    double desired_cfl, max_cfl, max_cfl_seen;
    double level_factor;       /* step = dt_minlevel / level_factor           */
    long long steps, rejects;
    int nint, nout;            /* output interval in progress / count         */
    int took_small;
    int active;                /* 0: the run is over (or never started)       */
    int cur;                   /* state buffer holding the current solution   */
    int hydro_off, nhydro;     /* samples in the lane's hydrograph table      */
    int regrid_interval;       /* accepted steps between regrids (0: never)   */
    int since_regrid;          /* accepted steps since the last regrid        */
    int paused;                /* 1: waiting for the host to regrid           */
} gf_group_state;

/* Fill of one patch's planes from pyramid windows (gf_forest_kernels.cu):
 * field f of the patch (slot planes dst[f]) is the (mx+4)^2 window of the
 * padded level raster src[f] (row length nx + 4) starting at patch
 * (I, J) of that level. */
#define GF_FILL_MAX_FIELDS 8
typedef struct gf_fill_task {
    const double* src[GF_FILL_MAX_FIELDS];
    double* dst[GF_FILL_MAX_FIELDS];
    int nfield;
    int nx;          /* interior cells per row of the level */
    int I, J;        /* patch index at that level */
} gf_fill_task;

/* One coarse/fine transfer (gf_amr.cu): kind GF_XFER_*, code = coarse
 * face / corner or child index, (ox, oy) = fine index of the coarse patch's
 * lower-left corner minus one. */
typedef struct gf_xfer_task {
    double* qc;
    const double* ac;
    double* qf;
    const double* af;
    int kind, code, ox, oy, phys;
    int group; /* with a per-group offset table: q pointers are shifted by it */
} gf_xfer_task;

/* One side of one fine patch for qad (gf_amr.cu): the fine patch's q and
 * aux, the coarse patch holding the coarse cells along that side, qad.f's
 * side number (1 left, 2 top, 3 right, 4 bottom), (ox, oy) as in
 * gf_xfer_task, the fine spacings, and the side's svdflx entries
 * (3 x mx/2 doubles, accumulated). */
typedef struct gf_qad_dev_task {
    const double* qf;
    const double* af;
    const double* qc;
    const double* ac;
    double* svdflx;
    double hx, hy;
    int side, ox, oy, phys;
} gf_qad_dev_task;

typedef struct gf_tinterp_task {
    const double* qcurr;
    const double* qlast;
    double* qinterp;
} gf_tinterp_task;

/* A refinement tag task: one patch (nsib = 1) or four siblings (nsib = 4,
 * order ll, lr, ul, ur). */
typedef struct gf_tag_task {
    const double* q[4];
    const double* aux[4];
    double xlower[4], ylower[4];
    double dx, dy;
    int level, nsib, phys;
    /* rf != null: this task's criteria, time, maxlevel and init_flag replace
     * the launch's (one launch then tags many forests) */
    const gf_refine* rf;
    double t;
    int maxlevel, init_flag;
} gf_tag_task;

/* Subcycling (gf_forest_kernels.cu): one patch's time interpolation
 * (qi = qold + alpha (qnew - qold) on the two cell layers along each face,
 * qold's ghost ring copied) or one patch copy (src -> dst, all planes). */
typedef struct gf_slot_task {
    const double* a;  /* qold / src */
    const double* b;  /* qnew       */
    double* c;        /* qi / dst   */
} gf_slot_task;

/* One topo grid on the device (gf_topo_kernels.cu): node values in file order
 * (rows north to south, x fastest), node extent and spacing. */
typedef struct gf_topo_grid {
    const double* z;
    int mx, my;
    double xlow, ylow, xhi, yhi, dx, dy;
} gf_topo_grid;

/* One gauge of a forest (gf_forest_kernels.cu): the slot of the leaf
 * holding it (-1: outside the domain), the Fortran index (ii, jj) of the
 * cell containing it, its offsets from that cell's centre in cells, and its
 * recording window. */
typedef struct gf_gauge_task {
    int slot, level, ii, jj;
    double xoff, yoff;
    double t1, t2, incr;
} gf_gauge_task;

#endif
