/* lin_sys_solves_mex: replaces the reference gateway lin_sys_solves.cpp (handle -> gm_lin_sys_solves). */
#include "gm_mex_common.h"
GM_MEX_VOID("lin_sys_solves", gm_lin_sys_solves)
