/* update_U_monodomain_mex: replaces the reference gateway update_U_monodomain.cpp (handle -> gm_update_U_monodomain). */
#include "gm_mex_common.h"
GM_MEX_VOID("update_U_monodomain", gm_update_U_monodomain)
