/* update_U_mex: replaces the reference gateway update_U.cpp (handle -> gm_update_U). */
#include "gm_mex_common.h"
GM_MEX_VOID("update_U", gm_update_U)
