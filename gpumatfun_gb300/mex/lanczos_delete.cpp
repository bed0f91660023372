/* lanczos_delete: replaces the reference gateway lanczos_delete.cpp. */
#include "gm_mex_common.h"
GM_MEX_VOID("lanczos_delete", gm_lanczos_delete)
