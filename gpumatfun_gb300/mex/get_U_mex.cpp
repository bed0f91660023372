/* get_U_mex: replaces the reference gateway get_U.cpp (handle -> n x 2 matrix via gm_get_U). */
#include "gm_mex_common.h"
GM_MEX_GET("get_U", gm_get_U)
