/* Empty definitions of the stand-ins in forestclaw_stub.h, so the linked
 * snippets leave no symbol but the library's unresolved. Never called. */
#include "forestclaw_stub.h"

extern "C" {
void fclaw2d_clawpatch_grid_data(fclaw2d_global_t*, fclaw2d_patch_t*, int*, int*, int*, double*,
                                 double*, double*, double*) {}
void fclaw2d_clawpatch_soln_data(fclaw2d_global_t*, fclaw2d_patch_t*, double**, int*) {}
void fclaw2d_clawpatch_aux_data(fclaw2d_global_t*, fclaw2d_patch_t*, double**, int*) {}
void fclaw2d_clawpatch_save_current_step(fclaw2d_global_t*, fclaw2d_patch_t*) {}
const fc2d_geoclaw_options_t* fc2d_geoclaw_get_options(fclaw2d_global_t*) { return nullptr; }
}
