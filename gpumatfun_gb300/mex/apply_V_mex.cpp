/* apply_V_mex: replaces the reference gateway apply_V.cpp (handle -> gm_apply_V). */
#include "gm_mex_common.h"
GM_MEX_VOID("apply_V", gm_apply_V)
