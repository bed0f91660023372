/* solve_mex(h): build_subspace + lin_sys_solves + apply_V as one persistent
 * launch (gm_solve).  X is overwritten, while the reference's apply_V
 * accumulates into X (apply_V.cu:45,91): get_xsol_mex reads the same X as
 * after the three separate calls only when X was zero before them, as it is
 * after lanczos_create, update_U and update_U_monodomain. */
#include "gm_mex_common.h"
GM_MEX_VOID("solve", gm_solve)
