/*
 * Stand-ins for the ForestClaw / GeoFlood declarations that the C++ units in
 * INTEGRATION.md use, with the argument lists the reference's own calls give
 * them (src/fc2d_geoclaw/fc2d_geoclaw.cpp:275-387, src/fc2d_cpu_cuda/
 * fc2d_cpucuda.cpp:410-495). Test infrastructure: only the declarations a
 * maintainer's translation unit would get from ForestClaw's headers, so the
 * snippets compile against include/geoflood_gb300.h without ForestClaw.
 */
#ifndef GF_FORESTCLAW_STUB_H
#define GF_FORESTCLAW_STUB_H
#include <assert.h>
#include <stdio.h>

typedef struct fclaw2d_global fclaw2d_global_t;
typedef struct fclaw2d_patch fclaw2d_patch_t;

/* fclaw2d_update_single_step.h: the buffer a buffered update hook receives */
typedef struct fclaw2d_single_step_buffer_data {
    int total_count;
    int iter;
    void* user;
} fclaw2d_single_step_buffer_data_t;

/* fc2d_geoclaw_options.h: the [geoclaw] method settings the hooks read */
typedef struct fc2d_geoclaw_options {
    int method[7];
    int mthlim[4];
    int src_term;
} fc2d_geoclaw_options_t;

#ifdef __cplusplus
extern "C" {
#endif
void fclaw2d_clawpatch_grid_data(fclaw2d_global_t* glob, fclaw2d_patch_t* patch, int* mx,
                                 int* my, int* mbc, double* xlower, double* ylower, double* dx,
                                 double* dy);
void fclaw2d_clawpatch_soln_data(fclaw2d_global_t* glob, fclaw2d_patch_t* patch, double** q,
                                 int* meqn);
void fclaw2d_clawpatch_aux_data(fclaw2d_global_t* glob, fclaw2d_patch_t* patch, double** aux,
                                int* maux);
void fclaw2d_clawpatch_save_current_step(fclaw2d_global_t* glob, fclaw2d_patch_t* patch);
const fc2d_geoclaw_options_t* fc2d_geoclaw_get_options(fclaw2d_global_t* glob);
#ifdef __cplusplus
}
#endif

#define fclaw_global_essentialf(...) fprintf(stderr, __VA_ARGS__)
#define FCLAW_ASSERT(c) assert(c)

#endif
