/* build_subspace_mex: replaces the reference gateway build_subspace.cpp (handle -> gm_build_subspace). */
#include "gm_mex_common.h"
GM_MEX_VOID("build_subspace", gm_build_subspace)
