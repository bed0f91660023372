/* solve_mex(h): build_subspace + lin_sys_solves + apply_V as one persistent
 * launch (gm_solve); X is overwritten, not accumulated, and get_xsol_mex
 * reads it as after the three separate calls. */
#include "gm_mex_common.h"
GM_MEX_VOID("solve", gm_solve)
