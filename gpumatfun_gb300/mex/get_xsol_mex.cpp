/* get_xsol_mex: replaces the reference gateway get_xsol.cpp (handle -> n x 2 matrix via gm_get_xsol). */
#include "gm_mex_common.h"
GM_MEX_GET("get_xsol", gm_get_xsol)
