/*
 * geoflood_gb300 -- C ABI of the GB300 (sm_103a) GeoClaw patch update.
 *
 * This is the drop-in boundary for the reference's patch-update hot path.
 * Each entry point names the reference interface it replaces (paths are
 * relative to the GeoFlood source tree). All functions return GF_OK (0) or a
 * negative gf_status; none throws or exits. A context is single-threaded;
 * contexts are independent. Host arrays use the reference's Fortran layout
 *   q(meqn, 1-mbc:mx+mbc, 1-mbc:my+mbc), aux(maux, 1-mbc:mx+mbc, 1-mbc:my+mbc)
 * (equation index fastest), with meqn = 3 (h, hu, hv), mbc = 2 and aux(1)
 * the bathymetry. Patch sizes mx = my in {8, 16, 32}. Arithmetic is FP64.
 */
#ifndef GEOFLOOD_GB300_H
#define GEOFLOOD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum gf_status {
    GF_OK = 0,
    GF_ERR_ARG = -1,      /* invalid argument (size, layout, null pointer) */
    GF_ERR_CUDA = -2,     /* a CUDA runtime call failed                    */
    GF_ERR_NOMEM = -3,    /* device or pinned allocation failed            */
    GF_ERR_DEVICE = -4,   /* a kernel reported a bounded wait that expired */
    GF_ERR_STATE = -5,    /* call out of order (e.g. no physics set)       */
    GF_ERR_UNSUPPORTED = -6
};

#define GF_MAX_MANNING 4
#define GF_MAX_PHYS 1024

/* Physics and method parameters of one scenario.
 * Replaces geoclaw_module (geolib_source/geoclaw_module.f90:30-48, set_geo
 * :57-161), friction_module (geolib_source/friction_module.f90:62-190) and the
 * [geoclaw] options order/mthlim/src_term (fc2d_geoclaw_options.c:44-91). */
typedef struct gf_phys {
    double grav;
    double dry_tolerance;
    double sea_level;
    double friction_depth;
    double manning_coefficient[GF_MAX_MANNING];
    double manning_break[GF_MAX_MANNING];
    int num_manning;
    int friction_forcing;
    int variable_friction; /* 1: Manning n per cell from aux(friction_index) */
    int friction_index;    /* 1-based aux field                              */
    int order;             /* method(2): 1 or 2                              */
    int transverse;        /* method(3): 0, 1 or 2                           */
    int mthlim[3];         /* philim.f limiter per wave family (1..5, 0 off)  */
    int src_term;          /* call src2 after step2                          */
    double maxcfl_cap;     /* fc2d_geoclaw.h:40 MAXCFL_CAP (100): a larger
                              patch CFL is returned as 0                     */
} gf_phys;

/* Defaults of the reference examples: g = 9.81, dry tolerance 1e-3,
 * Manning 0.035 below a break of 1e10, MC limiter, order 2, transverse 2. */
void gf_phys_default(gf_phys* p);

/* --------------------------------------------------------------- context */
typedef struct gf_ctx gf_ctx;

/* Create a context on CUDA device `device` (the reference's
 * fc2d_cudaclaw_initialize_GPUs, src/fc2d_cpu_cuda/cuda_source/
 * cudaclaw_initialize.cu:37-74, without the MPI rank mapping). */
int gf_ctx_create(int device, gf_ctx** out);
void gf_ctx_destroy(gf_ctx* ctx);
/* Text of the last error on this context ("" if none). */
const char* gf_ctx_last_error(const gf_ctx* ctx);

/* The context's CUDA stream (a cudaStream_t), for event timing and
 * ordering with other work. */
int gf_ctx_stream(gf_ctx* ctx, void** stream);

/* Floating-point contraction of the patch kernel. allow = 1 (default) runs
 * the production build, which fuses multiply-adds; allow = 0 runs a build
 * compiled without contraction that also sums the fluxes in the reference's
 * order, so each FP64 operation rounds as the Fortran expression is written
 * (fortran_source/geoclaw_step2_wrap_fort.f:97-115 for the final sum). */
int gf_ctx_set_fp_contract(gf_ctx* ctx, int allow);
/* Batched forest rounds (gf_forest_batch_run, the forest server) update
 * the patches of every size in one persistent launch over one work list
 * (on = 1, the default) or launch once per patch size (on = 0). Results
 * are the same either way. */
int gf_ctx_set_mixed_update(gf_ctx* ctx, int on);

/* Store physics set `slot` (0 <= slot < GF_MAX_PHYS). Replaces the
 * module set-up fc2d_geoclaw_module_setup (fc2d_geoclaw.cpp, calling
 * fortran_source/geoclaw_set_modules_fort.f90:1-63) and, for the GPU build,
 * setprob_cuda (src/fc2d_cpu_cuda/riemann_source/variables.cu:72-113). */
int gf_ctx_set_phys(gf_ctx* ctx, int slot, const gf_phys* phys);

/* ---------------------------------------------- plain per-patch drop-in */
/* One patch, host arrays in the Fortran layout: b4step2, step2, CFL cap and
 * src2 with physics slot 0, exactly the work of the single_step_update hook
 * geoclaw_update (src/fc2d_geoclaw/fc2d_geoclaw.cpp:352-387). Interior cells
 * of q are updated in place; ghost cells are left as they were on entry
 * (ghost filling rewrites them before the next step). *cfl receives the
 * patch CFL number (0 if above maxcfl_cap). */
int gf_patch_update(gf_ctx* ctx, int mx, int my, int mbc, int meqn, int maux,
                    double dx, double dy, double t, double dt, double* q,
                    const double* aux, double* cfl);

/* A buffer of patches with host arrays, one launch: the batched GPU hook
 * cudaclaw_update + cudaclaw_step2_batch (src/fc2d_cpu_cuda/fc2d_cpucuda.cpp:
 * 410-495, src/fc2d_cpu_cuda/cuda_source/cudaclaw_step2.cu:57-324).
 * q[k], aux[k] point at patch k's arrays; dx[k], dy[k] its spacing.
 * cfl (nullable) receives per-patch CFL; *maxcfl the maximum. */
int gf_patch_update_batch(gf_ctx* ctx, int npatch, int mx, int my, int mbc,
                          int meqn, int maux, const double* dx,
                          const double* dy, double t, double dt,
                          double* const* q, const double* const* aux,
                          double* cfl, double* maxcfl);

/* The buffered per-patch hook of the reference's GPU build, cudaclaw_update
 * (src/fc2d_cpu_cuda/fc2d_cpucuda.cpp:410-495, buffer_len from the
 * [cudaclaw] buffer-len option, 1024 in the reference's examples):
 * ForestClaw's level step hands the patches one at a time with iter =
 * 0..total-1. Each call records the patch (q and aux stay in the caller's
 * storage); when (iter+1) % buffer_len == 0 or iter+1 == total, every
 * recorded patch is updated as gf_patch_update_batch updates it and
 * *maxcfl receives the largest patch CFL of that flush. Other calls set
 * *maxcfl = 0 and leave q as it is until the flush (ForestClaw takes the
 * maximum over all returns). A patch's CFL is capped as gf_patch_update
 * caps it (above maxcfl_cap: 0); the reference's GPU build caps the
 * flush's maximum instead (:488). Patches of one buffer share mx, my,
 * maux; iter must count up from 0 without gaps (GF_ERR_STATE otherwise). */
typedef struct gf_step_buffer gf_step_buffer;
int gf_step_buffer_create(gf_ctx* ctx, int buffer_len, gf_step_buffer** out);
void gf_step_buffer_destroy(gf_step_buffer* buf);
int gf_step_buffer_update(gf_step_buffer* buf, int iter, int total, int mx,
                          int my, int mbc, int meqn, int maux, double dx,
                          double dy, double t, double dt, double* q,
                          const double* aux, double* maxcfl);

/* ------------------------------------------- device-resident level batch */
typedef struct gf_level gf_level;

/* A batch of npatch patches of size mx x my kept in HBM as planes
 * [patch][h|hu|hv][j][i] and [patch][aux field][j][i]. Replaces the per-patch
 * device buffers of cudaclaw_allocate_fluxes / fc2d_cudaclaw_allocate_buffers
 * (src/fc2d_cpu_cuda/cuda_source/cudaclaw_allocate.cu:21-138). */
int gf_level_create(gf_ctx* ctx, int npatch, int mx, int my, int maux,
                    gf_level** out);
void gf_level_destroy(gf_level* lev);

/* Per-patch cell sizes and physics slots (phys may be NULL: slot 0). */
int gf_level_set_geometry(gf_level* lev, const double* dx, const double* dy,
                          const int* phys);

/* Ghost-fill layout: nbr[8*k + s] is the same-level neighbour of patch k
 * across face s (0 left, 1 right, 2 bottom, 3 top) or corner 4 + c
 * (c = 0 lower-left, 1 lower-right, 2 upper-left, 3 upper-right), or -1 on
 * a physical boundary; xlower/ylower (nullable) position each patch.
 * Periodic sides are expressed by wrapping the neighbour table. */
int gf_level_set_layout(gf_level* lev, const int* nbr, const double* xlower,
                        const double* ylower);

/* Physical boundary rule per side (left, right, bottom, top): 0 hydrograph
 * inflow, 1 zero-order extrapolation, 2 periodic, 3 solid wall -- the
 * [geoclaw] mthbc option (fc2d_geoclaw_options.c:44-91). Default 1 1 1 1. */
int gf_level_set_bc(gf_level* lev, const int* mthbc);

/* Discharge hydrograph (time, hu per unit width; n rows) applied by rule 0
 * on the flagged sides (side[4]: left, right, bottom, top) inside the
 * channel |y - y0| <= width/2 (x for bottom/top): the data read by
 * read_hydrograph_data (hydrograph/hydrograh_module.f90:36-152). */
int gf_level_set_hydrograph(gf_level* lev, int n, const double* time,
                            const double* hu, const int* side, double width,
                            double x0, double y0);

/* Fill every ghost cell of the level at time t: same-level face and corner
 * copies (fc2d_geoclaw_fort_copy_face/_corner, fclaw2d_source/
 * fc2d_geoclaw_copy_fort.f:11-107) then physical boundaries
 * (fc2d_geoclaw_bc2, fortran_source/geoflood_bc2_fort.f90:7-409). */
int gf_level_ghost_fill(gf_level* lev, double t);
int gf_level_ghost_fill_async(gf_level* lev, double t);

/* Copy npatch Fortran-layout blocks (contiguous, patch k at
 * q + k*meqn*(mx+4)*(my+4)) to the device; aux may be NULL to keep the
 * resident bathymetry. */
int gf_level_upload(gf_level* lev, const double* q, const double* aux);
int gf_level_download(gf_level* lev, double* q);
int gf_level_download_aux(gf_level* lev, double* aux);

/* One level step on device-resident state (no host copies of q): the work
 * ForestClaw's level step does through single_step_update for every patch,
 * plus the CFL reduction (fc2d_geoclaw_run.c:305-312 within one process).
 * *maxcfl receives the maximum patch CFL. */
int gf_level_step(gf_level* lev, double t, double dt, double* maxcfl);

/* The same step end to end from host buffers: upload q (Fortran layout),
 * step, fill ghost cells at t + dt if a layout is set, download q. aux stays
 * resident. The patches go in chunks: one chunk's copies (on a second
 * stream) run beside other chunks' transposes, updates and ghost fills, so
 * with pinned q most of the traffic hides behind the update. */
int gf_level_step_host(gf_level* lev, double* q, double t, double dt,
                       double* maxcfl);
/* Chunks of gf_level_step_host: 0 (default) picks whole waves of the update
 * kernel, at most 8 chunks; 1 runs one chunk (no overlap); n > 1 n equal
 * chunks. The result does not depend on it. */
int gf_level_set_pipeline(gf_level* lev, int nchunks);

/* Asynchronous form of gf_level_step: enqueue the step on the context
 * stream and return; gf_level_sync waits and reports the max CFL of the
 * last enqueued step. */
int gf_level_step_async(gf_level* lev, double t, double dt);
int gf_level_sync(gf_level* lev, double* maxcfl);

/* Per-patch CFL numbers of the last step (npatch doubles). */
int gf_level_patch_cfl(gf_level* lev, double* cfl);

/* Device pointers of the resident planes (for graph capture / tooling). */
int gf_level_device_planes(gf_level* lev, double** q, double** aux);

/* ------------------------------------------ coarse/fine and regrid */
/* Transfer kinds between a coarse and a fine level (refinement ratio 2,
 * aligned patches):
 *   GF_XFER_AVG_FACE / _AVG_CORNER: coarse ghost cells from a fine neighbour
 *     (fc2d_geoclaw_fort_average_face/_corner, fclaw2d_source/
 *     fc2d_geoclaw_average_fort.f:33, 323; patch_vt->average_face/_corner);
 *   GF_XFER_INTERP_FACE / _INTERP_CORNER: fine ghost cells from a coarse
 *     neighbour (fc2d_geoclaw_interpolate_fort.f:24, 261);
 *   GF_XFER_INTERP2FINE: child from parent on refinement
 *     (fc2d_geoclaw_fort_interpolate2fine, interpolate_fort.f:405-579);
 *   GF_XFER_AVG2COARSE: parent from child on coarsening
 *     (fc2d_geoclaw_fort_average2coarse, average_fort.f:482-602).
 * code: the coarse patch's face (0..3) or corner (0..3) toward the fine
 * patch, or the child index igrid (0..3). (ox, oy): fine-cell index of the
 * coarse patch's lower-left corner relative to the fine patch's, i.e. the
 * coarse cell (ic, jc) covers fine cells 2ic-1+ox .. 2ic+ox (unused for the
 * parent/child kinds). */
enum gf_xfer_kind {
    GF_XFER_AVG_FACE = 0,
    GF_XFER_AVG_CORNER = 1,
    GF_XFER_INTERP_FACE = 2,
    GF_XFER_INTERP_CORNER = 3,
    GF_XFER_INTERP2FINE = 4,
    GF_XFER_AVG2COARSE = 5
};
typedef struct gf_transfer {
    int kind;
    int coarse; /* patch index in the coarse level */
    int fine;   /* patch index in the fine level   */
    int code;
    int ox, oy;
} gf_transfer;

/* Run ntask transfers; tasks of one call must not write a patch another
 * task of the same call reads (the caller orders averaging before
 * interpolation, as ForestClaw's ghost fill does). */
int gf_level_transfer(gf_level* coarse, gf_level* fine, int ntask,
                      const gf_transfer* tasks);

/* Time interpolation of the 2-cell interior boundary strip of every patch,
 * dst = last + alpha (curr - last) (fc2d_geoclaw_fort_timeinterp,
 * fclaw2d_source/fc2d_geoclaw_timeinterp_fort.f:1-69). The three levels
 * must hold the same patches. */
int gf_level_timeinterp(gf_level* dst, gf_level* curr, gf_level* last, double alpha);

/* Refinement regions and criteria: regions_module region_type and
 * refinement_data_module (geolib_source/refinement_data_module.f90:11-40). */
typedef struct gf_region {
    double x_low, x_hi, y_low, y_hi, t_low, t_hi;
    int min_level, max_level;
} gf_region;
#define GF_MAX_SPEEDS 8
#define GF_MAX_FLOWGRADES 4
#define GF_MAX_REGIONS 16
typedef struct gf_refine {
    double wave_tolerance;
    double speed_tolerance[GF_MAX_SPEEDS];
    int num_speed_tolerance;
    double deep_depth;
    int max_level_deep;
    double max_velocity_depth_product;
    int num_flowgrades;
    double flowgradevalue[GF_MAX_FLOWGRADES];
    int flowgradevariable[GF_MAX_FLOWGRADES]; /* 1 depth, 2 momentum, 3 surface */
    int flowgradetype[GF_MAX_FLOWGRADES];
    int flowgrademinlevel[GF_MAX_FLOWGRADES];
    int num_regions;
    gf_region regions[GF_MAX_REGIONS];
} gf_refine;

/* Refinement tag of every patch of the level (1 refine, 0 not):
 * geoclaw_patch_tag4refinement (src/fc2d_geoclaw/fc2d_geoclaw.cpp:405-457 ->
 * fc2d_geoclaw_test_regions, fc2d_geoclaw_fort_tag4refinement,
 * fc2d_geoflood_flag2refine). The level's xlower/ylower come from
 * gf_level_set_layout. */
int gf_level_tag4refinement(gf_level* lev, const gf_refine* rf, int level,
                            int maxlevel, int init_flag, double t, int* tags);

/* Coarsening tag of nfam sibling families (fam[4k..4k+3] = patches ll, lr,
 * ul, ur; 1 = may coarsen): geoclaw_patch_tag4coarsening
 * (fc2d_geoclaw.cpp:461-506 -> fc2d_geoclaw_fort_tag4coarsening). */
int gf_level_tag4coarsening(gf_level* lev, const gf_refine* rf, int nfam,
                            const int* fam, int level, int maxlevel,
                            int init_flag, double t, int* tags);

/* Coarse/fine conservation fix-up qad (src/fc2d_geoclaw/geolib_source/
 * qad.f:4-371, AMRClaw's routine as GeoClaw carries it; the reference tree
 * does not compile it and no GeoFlood path calls it). For each task, one
 * side of fine patch `fine` (side 1 left, 2 top, 3 right, 4 bottom, qad.f's
 * numbering) whose first ghost layer lies in coarse patch `coarse` ((ox,
 * oy) as in gf_transfer): the Riemann problem between each fine ghost cell
 * and the coarse cell holding it is solved, and the fluctuations times the
 * fine face length and dt are added into svdflx[task][c][m] (host array of
 * ntask x mx/2 x 3 doubles, accumulated in place), one entry per coarse cell
 * c along the side (bottom to top on sides 1 and 3, left to right on 2 and
 * 4), signed as qad.f signs each side. The fine patch's ghost cells must be
 * filled. Physics from the fine patch's slot. */
typedef struct gf_qad_task {
    int fine, coarse, side, ox, oy;
} gf_qad_task;
int gf_level_qad(gf_level* coarse, gf_level* fine, int ntask,
                 const gf_qad_task* tasks, double dt, double* svdflx);

/* ------------------------------------------- allocation-free drop-in */
/* For callers that cannot allocate device memory at step time: memory owned
 * by another allocator (a framework's caching pool or a fixed budget a raw
 * cudaMalloc would bypass), a service at its memory limit where allocation
 * can fail mid-step, or a latency-critical stream that cudaFree would stall
 * by synchronising the device. No counterpart in the reference: its GPU
 * path allocates per call (cuda_source/cudaclaw_step2.cu:179, 279-287).
 *
 * Same work as gf_patch_update_batch, but q and aux are DEVICE buffers the
 * caller owns: npatch contiguous Fortran-layout blocks (q updated in place,
 * interior cells only), dx/dy/cfl/maxcfl host arrays, `phys` a host struct,
 * `stream` a cudaStream_t (NULL = legacy default stream). Nothing is
 * allocated: staging lives in one static device array of
 * GF_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * exit. Limits: npatch <= GF_NOALLOC_MAX_PATCHES (16), maux <=
 * GF_NOALLOC_MAX_MAUX (4), mx = my in {8, 16, 32}; larger sizes return
 * GF_ERR_ARG, other shapes GF_ERR_UNSUPPORTED, and `phys` is held to the
 * rules of gf_ctx_set_phys (with variable friction, friction_index must
 * lie in 1..maux), GF_ERR_ARG otherwise; all of these are checked before
 * any device memory is touched. The first call on a device looks up the
 * array's device address, so make that first call before any stream
 * capture. The call is synchronous: it waits for `stream` to finish its
 * work before it returns. It makes `device` current while it runs and
 * puts the caller's current device back before returning. All calls share
 * the array: calls whose GPU work overlaps race, so issue them one after
 * another. */
#define GF_NOALLOC_MAX_PATCHES 16
#define GF_NOALLOC_MAX_MAUX 4
#define GF_NOALLOC_SCRATCH_BYTES 1163008
int gf_patch_update_noalloc(int device, const gf_phys* phys, int npatch,
                            int mx, int my, int mbc, int meqn, int maux,
                            const double* dx, const double* dy, double dt,
                            double* q, const double* aux, double* cfl,
                            double* maxcfl, void* stream);

/* ------------------------------------------------ multi-level forests */
/* A forest of nbx x nby root blocks refined as quadtrees between minlevel
 * and maxlevel, patches of mx x mx cells, resident on the device. This is
 * the ForestClaw level machinery the patch-update path sits in, restated
 * for one GPU (ForestClaw itself is an external library, absent from the
 * reference tree): leaves with full (face and corner) 2:1 balance; ghost
 * fill = fine->coarse averages (fc2d_geoclaw_average_fort.f:33,323), same-
 * level copies and physical boundaries (fc2d_geoclaw_copy_fort.f,
 * geoflood_bc2_fort.f90), then coarse->fine interpolation level by level
 * (fc2d_geoclaw_interpolate_fort.f:24,261) with the boundaries re-applied
 * to interpolated patches; regrid from the reference's tags
 * (fc2d_geoclaw_tag4refinement_fort.f90, _tag4coarsening_fort.f90) with
 * interpolate2fine / average2coarse for the new patches; time stepping by
 * outstyle 1 (fc2d_geoclaw_run.c:190-395) with all levels advanced by the
 * same step (subcycle = F, advance-one-step = T, as the reference's
 * examples set them) or, with opts.subcycle = 1, level by level with
 * time-interpolated coarse ghost cells (ForestClaw's subcycle = T,
 * fclaw2d_advance_all_levels; fclaw2d_source/fc2d_geoclaw_timeinterp_fort.f
 * for the interpolation), and a regrid every regrid_interval accepted steps.
 *
 * Static fields and the initial state come as rasters at the finest level
 * (maxlevel): maux aux fields then h, hu, hv, each ny x nx doubles with x
 * fastest, nx = nbx*mx*2^maxlevel, ny = nby*mx*2^maxlevel. A patch at a
 * coarser level takes the cell averages of the raster (a pyramid of 2 x 2
 * averages), like setaux's cell-averaged topography. */
typedef struct gf_forest gf_forest;

typedef struct gf_forest_opts {
    int mx;                /* 8, 16 or 32 (my = mx)                          */
    int maux;              /* aux fields, bathymetry first (1..3)            */
    int nbx, nby;          /* root blocks                                    */
    int minlevel, maxlevel; /* 0 <= minlevel <= maxlevel <= 10               */
    double x0, y0;         /* lower-left corner of the domain                */
    double dx0, dy0;       /* cell size at level 0                           */
    int phys_slot;         /* physics set in the context's table             */
    int mthbc[4];          /* left, right, bottom, top: 0 inflow, 1 extrap, 3 wall */
    int regrid_interval;   /* accepted steps between regrids (0: never)      */
    int max_patches;       /* slot capacity (0: 5/4 of nbx*nby*4^maxlevel, the
                              most a regrid can hold at once)                */
    gf_refine refine;      /* refinement criteria                            */
    int subcycle;          /* 1: level l takes 2^(l - lmin) steps of dt / 2^(l - lmin)
                              per coarse step (ForestClaw subcycle = T); 0: every
                              level takes the finest level's step             */
} gf_forest_opts;

typedef struct gf_forest_stats {
    long long steps, rejects, regrids;
    long long cell_updates;  /* interior cells x accepted steps, all leaves */
    double t;                /* simulated time reached                      */
    double dt;               /* controller's dt at minlevel                 */
    double max_cfl_seen;
    int npatch, npatch_max;  /* leaves now / at most                        */
    int levels_used;         /* finest level present                        */
} gf_forest_stats;

void gf_forest_opts_default(gf_forest_opts* o);
/* fields: (maux + 3) rasters at maxlevel, see above (host memory). */
int gf_forest_create(gf_ctx* c, const gf_forest_opts* o, const double* fields, gf_forest** out);
void gf_forest_destroy(gf_forest* f);
/* Inflow hydrograph (as gf_level_set_hydrograph); call before gf_forest_init. */
int gf_forest_set_hydrograph(gf_forest* f, int n, const double* time, const double* hu,
                             const int* side, double width, double x0, double y0);
/* Leaves at minlevel, then initial refinement (init_flag = 1) until no tag
 * fires or maxlevel is reached; every new patch takes the rasters. */
int gf_forest_init(gf_forest* f);
int gf_forest_ghost_fill(gf_forest* f, double t);
/* One step of every leaf with dt from its state at t (ghost fill included);
 * the result is held until gf_forest_accept. *cfl = max over leaves. */
int gf_forest_step(gf_forest* f, double t, double dt, double* cfl);
int gf_forest_accept(gf_forest* f, int accept);
/* Tag, refine/coarsen, balance, transfer; *changed = 1 if the leaves changed. */
int gf_forest_regrid(gf_forest* f, double t, int* changed);
/* outstyle-1 run from t = 0 to t_final with nout output intervals. */
int gf_forest_run(gf_forest* f, double t_final, int nout, double initial_dt, double desired_cfl,
                  double max_cfl, int max_steps, gf_forest_stats* st);
int gf_forest_get_stats(gf_forest* f, gf_forest_stats* st);
/* Leaves in canonical order (level, then J, then I). */
int gf_forest_npatch(const gf_forest* f);
int gf_forest_patches(const gf_forest* f, int* level, int* I, int* J);
/* State / aux of the leaves in canonical order, Fortran layout per patch. */
int gf_forest_download(gf_forest* f, double* q);
int gf_forest_download_aux(gf_forest* f, double* aux);
int gf_forest_upload(gf_forest* f, const double* q);

/* Batched form: n forests of one context run the same outstyle-1 loop
 * (each with its own dt, CFL, output times and regrid cadence) in shared
 * launches. The time-step control runs on the device; one round (step
 * control, coarse/fine exchange, ghost fill, patch update of every leaf of
 * every forest, CFL reduction) is captured as a CUDA graph per epoch and
 * replayed; a forest whose regrid is due waits on the device until the
 * host regrids it, after which the epoch is rebuilt and captured again.
 * Subcycled forests (subcycle = 1) share launches in groups instead: the
 * forests whose leaves span the same levels take their coarse steps
 * together, each launch of the subcycled schedule carrying every member's
 * tasks (each member its own level dts, boundary times and CFL), one CUDA
 * graph per group step, each member under its own outstyle-1 control
 * (fclaw2d_advance_all_levels' schedule, fc2d_geoclaw_run.c:229-395). Each
 * forest's result equals its own gf_forest_run. */
typedef struct gf_forest_batch_stats {
    long long rounds;        /* graph replays                               */
    long long epochs;        /* captures (membership or tables changed)     */
    long long regrids;       /* forest regrids                              */
    long long launches;      /* kernel launches inside the replayed rounds  */
    long long cell_updates;  /* all forests                                 */
    double s_rounds;         /* host seconds waiting on replayed rounds      */
    double s_regrid;         /* host seconds in regrids                      */
    double s_epoch;          /* host seconds building and capturing epochs   */
} gf_forest_batch_stats;
int gf_forest_batch_run(gf_forest** forests, int n, double t_final, int nout, double initial_dt,
                        double desired_cfl, double max_cfl, gf_forest_batch_stats* st);

/* ----------------------------------------------------------- topography */
/* A set of topo grids (DEMs) and the cell-averaged bathymetry setaux makes
 * of them. Replaces topo_module's readers and ranking
 * (geolib_source/topo_module.f90:160-402, 491-1059) and setaux's
 * bathymetry (fortran_source/geoclaw_setaux_fort.f90:107-215 with
 * cellgridintegrate2.f, topointegral.f, bilinearintegral.f): the bathymetry
 * of a cell is the integral over the cell of the piecewise-bilinear surface
 * through the nodes of the finest grid covering each part of it, divided by
 * the cell area; cells outside the domain copy the nearest cell inside.
 * Reading is host-only (no device needed); the integrals run on the device
 * of the context or forest that uses the set. */
typedef struct gf_topo gf_topo;
#define GF_TOPO_MAX_FILES 16

int gf_topo_create(gf_topo** out);
void gf_topo_destroy(gf_topo* t);
/* Value stored for no-data nodes of later files (default 99999, which the
 * reference refuses when a file has missing data: so do these readers). */
int gf_topo_set_missing(gf_topo* t, double topo_missing);
/* Append a topo file of type +-1, +-2, +-3 or +-4 (negative: z is negated).
 * Type 4 is a classic NetCDF file (CDF-1, -2 or -5) read as the reference
 * reads it: x / y dimensions named lon / longitude / x and lat / latitude /
 * y, coordinate variables of the same names, the last 2-D variable as z;
 * NetCDF-4 (HDF5) files are refused. The whole grid is kept. */
int gf_topo_read_file(gf_topo* t, const char* path, int topo_type);
/* Append every file that a topo.data (test_topography = 0) lists; relative
 * names are taken relative to the directory of topo.data. */
int gf_topo_read_data(gf_topo* t, const char* topo_data_path);
/* Append a grid from memory: mx x my nodes, lower-left node (xll, yll),
 * spacing dx, dy, z in file order (rows north to south, x fastest). */
int gf_topo_add_grid(gf_topo* t, int mx, int my, double xll, double yll, double dx, double dy,
                     const double* z);
int gf_topo_count(const gf_topo* t);
/* Header of grid k (any pointer may be NULL) and its nodes (z may be NULL). */
int gf_topo_grid_info(const gf_topo* t, int k, int* mx, int* my, double* xlow, double* ylow,
                      double* xhi, double* yhi, double* dx, double* dy, double* z);
/* Area of the rectangle covered by the grids (topoarea): the reference
 * stops when it is below 99 % of the domain. */
int gf_topo_covered_area(const gf_topo* t, double x1, double x2, double y1, double y2, double* area);
/* Cell averages of a uniform raster: nx x ny cells of dx x dy from
 * (xlower, ylower) plus `halo` cells each side, out (ny + 2 halo) x
 * (nx + 2 halo) host doubles, row pitch nx + 2 halo; (xupper, yupper) is
 * the domain's upper corner (cells beyond it copy the nearest cell inside).
 * Computed on the context's device. */
int gf_topo_raster(gf_ctx* c, gf_topo* t, int nx, int ny, int halo, double xlower, double ylower,
                   double dx, double dy, double xupper, double yupper, double* out);
/* Replace a forest's bathymetry (aux field 1) at every level by the cell
 * averages of t -- setaux at each level -- before gf_forest_init; with
 * qinit != 0 also set its initial state as fc2d_geoclaw_qinit does without
 * qinit files (fortran_source/geoclaw_qinit_fort.f90:24-27):
 * h = max(0, sea_level - b), hu = hv = 0, sea_level of the forest's
 * physics. gf_forest_create accepts fields = NULL for this use. */
int gf_forest_set_topo(gf_forest* f, gf_topo* t, int qinit);

/* ------------------------------------------------------------- output */
/* ASCII frame fort.tXXXX + fort.qXXXX in directory dir (NULL or "": the
 * working directory), as fc2d_geoclaw_output_ascii
 * (src/fc2d_geoclaw/fc2d_geoclaw_output_ascii.c:38-109) and the Fortran
 * writers fc2d_geoclaw_fort_write_header / _write_file
 * (fclaw2d_source/fc2d_geoclaw_output_ascii_fort.f:1-117) write it: time
 * as e30.20, the patch headers as i5 / e24.16, one 5E26.16 line of h, hu,
 * hv, eta = h + aux(1) per interior cell (values below 1e-99 in magnitude
 * written as 0), a blank record after each row. The npatch patches (Fortran
 * layout, ghosts included) are written in the order given; grid_number and
 * block may be NULL (0..npatch-1 and 0). iframe is taken modulo 10000. */
int gf_write_ascii_frame(const char* dir, int iframe, double time, int npatch, int mx, int maux,
                         const double* q, const double* aux, const int* grid_number,
                         const int* level, const int* block, const double* xlower,
                         const double* ylower, const double* dx, const double* dy);
/* Gauge value at (xc, yc) in one patch (Fortran layout, ghosts included):
 * out = h, hu, hv, bathymetry, bilinear between the cell holding the gauge
 * and its +x / +y neighbours unless one of the four is drier than
 * 0.1 * dry_tolerance (fc2d_geoclaw_update_gauge,
 * fortran_source/geoclaw_gauges_fort.f90:1-77). */
int gf_sample_gauge(int mx, int maux, const double* q, const double* aux, double xlower,
                    double ylower, double dx, double dy, double dry_tolerance, double xc,
                    double yc, double* out);
/* gaugeXXXXX.txt: the header (geoclaw_create_gauge_files_default,
 * src/fc2d_geoclaw/fc2d_geoclaw_gauges_default.c:172-200) and appended rows
 * "level t h hu hv eta" (geoclaw_print_gauges_default, :275-305); qv holds
 * nrow x (h, hu, hv, bathymetry). */
int gf_write_gauge_header(const char* dir, int id, double xc, double yc);
int gf_write_gauge_rows(const char* dir, int id, int nrow, const int* level, const double* t,
                        const double* qv);
/* gauges.data as geoclaw_read_gauges_data_default reads it
 * (fc2d_geoclaw_gauges_default.c:56-167): *n = number of gauges; the arrays
 * are filled when cap >= *n. */
int gf_read_gauges_data(const char* path, int cap, int* n, int* id, double* xc, double* yc,
                        double* t1, double* t2, double* min_time_increment);

/* Forest output. Frames list the leaves in p4est order: blocks (trees of
 * the nbx x nby brick) along the brick's Morton curve, leaves of a block
 * along the Morton curve of their lower-left corners; grid_number is the
 * position in that order, block the tree number. */
int gf_forest_write_ascii(gf_forest* f, const char* dir, int iframe);
/* With dir set, gf_forest_run writes frame 0 before its first step (once
 * per forest) and the next frame after each output interval (frames != 0),
 * and appends gauge rows there. */
int gf_forest_set_output(gf_forest* f, const char* dir, int frames);
/* Gauges sampled by gf_forest_run at the start of the first run and after
 * every accepted step, before any regrid: gauge k records at time t when
 * t1[k] <= t <= t2[k] and t >= (its last record) + min_time_increment[k],
 * from the leaf holding (xc, yc), with ghost cells exchanged at t. Writes
 * the gauge file headers in the output directory. n = 0 removes them. */
int gf_forest_set_gauges(gf_forest* f, int n, const int* id, const double* xc, const double* yc,
                         const double* t1, const double* t2, const double* min_time_increment);
/* Record the gauges at time t from the current state (for host-driven
 * loops over gf_forest_step / gf_forest_accept); rows are buffered on the
 * device until gf_forest_flush_gauges appends them to the files. */
int gf_forest_sample_gauges(gf_forest* f, double t);
int gf_forest_flush_gauges(gf_forest* f);

/* ------------------------------------------------- served scenarios */
/* A request loop over flood scenarios (continuous batching). Each admitted
 * scenario keeps its state resident on the device; every batching round
 * steps all active scenarios of one size lane and one patch size with
 * shared launches (one ghost fill and one patch update), each scenario with
 * its own dt and CFL slot; the queues of different patch sizes step
 * independently, on streams of their lane's priority. Time stepping per scenario follows ForestClaw's outstyle 1
 * loop (src/fc2d_geoclaw/fc2d_geoclaw_run.c:190-395): dt clipped to hit each
 * output time with the 1% tolerance, a step whose CFL exceeds max_cfl is
 * retaken with dt * desired_cfl / cfl, otherwise the next dt is
 * dt * desired_cfl / cfl. A rejected step costs no copy: the update writes
 * into the second of two state buffers and the scenario's current buffer
 * only flips on acceptance. Replaces the per-rank driver loop for many
 * independent runs; the single level per scenario is a one-level forest.
 *
 * The caller keeps q, aux and q_out alive until the scenario is DONE,
 * FAILED or CANCELLED (pinned memory keeps the copies asynchronous). */
typedef struct gf_server gf_server;

enum gf_scenario_state {
    GF_SCEN_QUEUED = 0,
    GF_SCEN_ACTIVE = 1,
    GF_SCEN_DONE = 2,
    GF_SCEN_FAILED = 3,
    GF_SCEN_CANCELLED = 4
};

#define GF_SERVER_MAX_LANES 4

typedef struct gf_scenario {
    int mx;                /* 8, 16 or 32 (my = mx)                              */
    int npx, npy;          /* patch grid of the level, patch index = py*npx + px */
    int maux;              /* aux fields, bathymetry first (1..3)                */
    double dx, dy;         /* cell size                                          */
    double xlower, ylower; /* lower-left corner of the domain                    */
    const double* q;       /* host, Fortran layout per patch: q(3, mx+4, mx+4)   */
    const double* aux;     /* host, aux(maux, mx+4, mx+4) per patch, ghosts set  */
    double* q_out;         /* host, final state in the layout of q (nullable)    */
    gf_phys phys;
    int mthbc[4];          /* left, right, bottom, top: 0 inflow, 1 extrap, 3 wall */
    int hydro_side[4];     /* sides fed by the hydrograph (rule 0)               */
    int nhydro;            /* hydrograph samples (0 = none)                      */
    const double* hydro_time;
    const double* hydro_hu; /* discharge per unit width at hydro_time            */
    double hydro_width, hydro_x0, hydro_y0;
    double t_final;        /* simulated horizon                                  */
    int nout;              /* output intervals (dt lands on each output time)    */
    double initial_dt, desired_cfl, max_cfl;
} gf_scenario;

typedef struct gf_server_opts {
    size_t hbm_budget;      /* device bytes all admitted scenarios may hold      */
    int max_active;         /* scenarios admitted at once (<= 1024)              */
    int nlanes;             /* size lanes, each with its own stream (1..4)       */
    long long lane_cells[GF_SERVER_MAX_LANES]; /* lane k: cells < lane_cells[k]; last lane takes the rest */
    int priority;           /* 1: smaller lanes on higher-priority streams       */
    int backfill;           /* 1: admit later arrivals that fit while the head waits */
    int reserve_sms;        /* > 0: lanes after the first run persistent grids that
                               leave this many SMs free for it; 0 (default): one CTA
                               per patch, stream priority shares the SMs */
    int mixed_update;       /* 1: lanes after the first update every patch size in one
                               persistent launch (same results); 0 (default): one launch
                               per size, which keeps the small sizes' occupancy */
    int cull_dry;           /* 1 (default): skip the ghost fill and update of a patch
                               whose update would be an exact identity (it and its
                               halo dry and unchanged by b4step2 at its last update,
                               no neighbour wet, no hydrograph side); interior results
                               are the same bits; a skipped patch's ghost cells keep
                               their last values. 0: every patch every step */
    int split_sizes;        /* 1 (default): each lane keeps one round queue per patch
                               size, stepping independently; 0: one queue per lane,
                               its sizes as parallel branches of every round (same
                               results either way) */
} gf_server_opts;

typedef struct gf_scenario_info {
    int state;              /* gf_scenario_state                                 */
    int lane;
    long long steps, rejects, cell_updates; /* accepted steps; interior cells x steps */
    double t;               /* simulated time reached                            */
    double dt;              /* current dt of the controller                      */
    double t_submit, t_admit, t_done; /* seconds on the server clock (-1: not yet) */
    double max_cfl_seen;
    size_t device_bytes;
} gf_scenario_info;

typedef struct gf_server_stats {
    long long submitted, admitted, done, rounds, launches;
    long long cell_updates;  /* accepted steps over all scenarios               */
    size_t bytes_in_use, bytes_peak;
    int active, queued;
} gf_server_stats;

void gf_server_opts_default(gf_server_opts* o);
int gf_server_create(int device, const gf_server_opts* opts, gf_server** out);
void gf_server_destroy(gf_server* s);
const char* gf_server_last_error(const gf_server* s);
/* Device bytes a scenario holds while admitted (0 for an invalid one). */
size_t gf_scenario_footprint(const gf_scenario* sc);
/* Queue a scenario (validated here; GF_ERR_NOMEM if it can never fit). */
int gf_server_submit(gf_server* s, const gf_scenario* sc, long long* id);
/* One non-blocking pass of the request loop: finish completed rounds, admit,
 * launch the next rounds. *busy = 1 while any work is queued or in flight. */
int gf_server_pump(gf_server* s, int* busy);
/* Run the request loop on a background thread / stop it. */
int gf_server_start(gf_server* s);
int gf_server_stop(gf_server* s);
/* Pump (or, with the loop thread running, sleep) until the scenario ends or
 * timeout_s passes (GF_ERR_STATE on timeout). */
int gf_server_wait(gf_server* s, long long id, double timeout_s);
int gf_server_poll(gf_server* s, long long id, gf_scenario_info* info);
int gf_server_cancel(gf_server* s, long long id);
int gf_server_stats_get(gf_server* s, gf_server_stats* st);
double gf_server_clock(const gf_server* s);

/* ---------------------------------------------------- served AMR forests */
/* A request loop over adaptive flood scenarios: each request is a forest
 * (gf_forest_create / set_hydrograph / set_topo / init on admission) that
 * then runs its outstyle-1 loop (src/fc2d_geoclaw/fc2d_geoclaw_run.c:190-395,
 * regrids every regrid_interval steps) inside the batched engine of
 * gf_forest_batch_run, with every other admitted forest of any mx in the
 * same replayed rounds. Members join between iterations (about half a
 * millisecond of rounds each) and leave when their run ends; each
 * membership change re-captures the round's graph. A request's result
 * equals its own gf_forest_run bit for bit.
 *
 * Admission is by device footprint (gf_forest_footprint) against the
 * budget, first come first served (backfill: later requests that fit pass
 * a head that does not). Forests batch in up to three lanes by size, each
 * on its own stream: a lane's rounds last as long as its largest member's
 * update, so smaller forests run in their own lanes, at higher priority and
 * on SMs the larger lanes' updates leave free. A finished forest stays resident, counted against
 * the budget, until gf_fserver_release; read it meanwhile through
 * gf_fserver_forest (or gf_fserver_download while the loop thread runs).
 * The caller keeps fields and topo alive until the request leaves QUEUED.
 * Subcycled forests (opts.subcycle = 1) run in lane 3, side by side: each
 * coarse step the forest's own graph on a stream of a pool, so the loop
 * never waits on the device. */
typedef struct gf_fserver gf_fserver;

typedef struct gf_forest_request {
    gf_forest_opts opts;   /* phys_slot is ignored: the server assigns one      */
    gf_phys phys;
    const double* fields;  /* rasters as gf_forest_create (NULL: zero rasters)  */
    gf_topo* topo;         /* nullable: bathymetry from DEMs (gf_forest_set_topo) */
    int qinit;             /* with topo: still water at phys.sea_level          */
    int nhydro;            /* hydrograph samples (0 = none), copied on submit    */
    const double* hydro_time;
    const double* hydro_hu;
    int hydro_side[4];
    double hydro_width, hydro_x0, hydro_y0;
    double t_final;
    int nout;
    double initial_dt, desired_cfl, max_cfl;
} gf_forest_request;

#define GF_FSERVER_LANES 3 /* lanes of shared rounds at most                    */
typedef struct gf_fserver_opts {
    size_t hbm_budget;     /* device bytes admitted and unreleased forests may hold */
    int max_active;        /* forests running at once (1..GF_MAX_PHYS)          */
    int backfill;
    long long lane_cells[GF_FSERVER_LANES - 1]; /* ascending, 0 ends the list: lane k
                              takes forests with fewer cells after initial refinement
                              than lane_cells[k], the last lane the rest; each lane
                              its own stream, smaller lanes at higher priority     */
    int reserve_sms;       /* a lane's update leaves this many SMs free per smaller
                              lane that has forests running                      */
} gf_fserver_opts;

typedef struct gf_forest_request_info {
    int state;             /* gf_scenario_state                                 */
    long long steps, rejects, regrids, cell_updates;
    double t, dt, max_cfl_seen;
    double t_submit, t_admit, t_done; /* seconds on the server clock (-1: not yet) */
    int npatch, npatch_max;
    size_t footprint;      /* bytes reserved at admission                       */
    size_t device_bytes;   /* bytes the forest holds (0 before admission)       */
    int lane;              /* 0..2 shared-round lanes by size, 3 subcycled (-1 before admission) */
} gf_forest_request_info;

typedef struct gf_fserver_stats {
    long long submitted, admitted, done, failed;
    long long lane_admitted[4];  /* per lane (shared-round lanes 0..2, subcycled 3) */
    long long iterations, epochs, rounds, launches, regrids, cell_updates;
    long long sub_steps;     /* subcycled coarse steps launched               */
    double s_admit, s_epoch, s_rounds, s_regrid; /* host seconds per phase      */
    size_t bytes_in_use, bytes_peak;
    int active, queued, held;
} gf_fserver_stats;

/* Device bytes a forest with these options may hold at most (0: invalid). */
size_t gf_forest_footprint(const gf_forest_opts* o);
void gf_fserver_opts_default(gf_fserver_opts* o);
int gf_fserver_create(int device, const gf_fserver_opts* opts, gf_fserver** out);
void gf_fserver_destroy(gf_fserver* s);
const char* gf_fserver_last_error(const gf_fserver* s);
/* The server's context (fp-contract mode, topo rasters); owned by the server. */
gf_ctx* gf_fserver_ctx(gf_fserver* s);
/* Queue a request (validated here; GF_ERR_NOMEM if it can never fit). */
int gf_fserver_submit(gf_fserver* s, const gf_forest_request* r, long long* id);
/* One pass of the loop: admit, run one iteration of the batch, retire the
 * finished. *busy = 1 while requests are queued or running. */
int gf_fserver_pump(gf_fserver* s, int* busy);
int gf_fserver_start(gf_fserver* s);
int gf_fserver_stop(gf_fserver* s);
int gf_fserver_wait(gf_fserver* s, long long id, double timeout_s);
int gf_fserver_poll(gf_fserver* s, long long id, gf_forest_request_info* info);
int gf_fserver_cancel(gf_fserver* s, long long id);
/* A DONE request's forest (borrowed; valid until gf_fserver_release). */
int gf_fserver_forest(gf_fserver* s, long long id, gf_forest** f);
/* npatch and the leaves' state / aux of a DONE request, canonical order
 * (as gf_forest_patches / gf_forest_download); any argument may be NULL. */
int gf_fserver_download(gf_fserver* s, long long id, int* npatch, int* level, int* I, int* J,
                        double* q, double* aux);
/* Destroy a finished request's forest and return its bytes to the budget. */
int gf_fserver_release(gf_fserver* s, long long id);
int gf_fserver_stats_get(gf_fserver* s, gf_fserver_stats* st);
double gf_fserver_clock(const gf_fserver* s);

/* ------------------------------------------------------------ tiling */
/* Tile shapes of the production patch kernel (threads per patch x slices
 * per band) per patch size, measured on this device: the fastest for whole
 * levels (throughput) and the fastest lone small batch (latency) become
 * the process-wide choice; the served form's smallest lane uses the
 * latency choice, everything else the throughput choice. Synthetic
 * all-wet patches, physics slot 0 of the context, `reps` timed launches
 * per variant. No reference counterpart (tuning support). */
#define GF_MAX_TILES 12
typedef struct gf_tile_result {
    int mx;
    int nvariant;
    int threads[GF_MAX_TILES], band[GF_MAX_TILES];
    int cluster[GF_MAX_TILES];       /* > 1: one patch split over a cluster of
                                        that many CTAs (the latency form)   */
    double throughput[GF_MAX_TILES]; /* cell-updates/s, ~4M-cell level     */
    double latency_us[GF_MAX_TILES]; /* one launch over 8 patches           */
    int best_throughput, best_latency;
} gf_tile_result;
int gf_autotune(gf_ctx* ctx, int reps, gf_tile_result* out /* [3]: mx 8, 16, 32 */);
/* Number of tile variants of patch size mx. */
int gf_tile_count(int mx);
/* Current choice (goal 0 throughput, 1 latency) or a manual one. Levels,
 * forests and batched rounds take the throughput choice; a batch through
 * gf_patch_update / gf_patch_update_batch / gf_step_buffer_update, and a
 * step of the served form's smallest lane, take the latency choice when
 * all their patches run in one wave of it (no more patches than the
 * clusters of that tile the GPU holds resident at once). */
int gf_tile_get(int mx, int goal);
int gf_tile_set(int mx, int goal, int variant);

/* ----------------------------------------------------------- probes */
/* Measured FP64 pipe rates of `device` in operations per second:
 * rates[0] double fma, [1] double division, [2] double sqrt, [3] float fma.
 * The patch update is FP64-issue bound; this is its roofline denominator.
 * No reference counterpart (measurement support). */
int gf_measure_fp64_rates(int device, double* rates);
/* Failure detection of the device waits: every wait in this library's
 * kernels (the patch staging copies' mbarrier) polls at most a fixed number
 * of times, then records an error the host turns into GF_ERR_DEVICE, and
 * the kernel returns. This runs that bounded wait in one CTA on a barrier
 * phase that nothing completes (arrive = 0: *timed_out = 1) or that the CTA
 * completes itself (arrive = 1: *timed_out = 0), for at most max_iter polls;
 * *ms (nullable) is the kernel's duration. The context stays usable. */
int gf_probe_bounded_wait(int device, int arrive, unsigned int max_iter, int* timed_out, double* ms);

#ifdef __cplusplus
}
#endif
#endif
