/* Shared helpers of the MEX gateways over the C ABI (include/gpumatfun.h).
 * The gateways keep the reference's MATLAB-visible names and argument order
 * (lanczosEngine.m:8-55) and its error identifiers (MATLAB:<fn>:<id>); they are
 * built only where MATLAB's mex.h is available (see build_mex.m). */
#ifndef GM_MEX_COMMON_H
#define GM_MEX_COMMON_H
#include <mex.h>
#include <stdint.h>
#include <string.h>
#include "../../include/gpumatfun.h"

static gm_handle gm_mex_handle(const mxArray* a, const char* fn) {
  if (!mxIsUint64(a)) {
    char id[128];
    snprintf(id, sizeof(id), "MATLAB:%s:inputNotHandle", fn);
    mexErrMsgIdAndTxt(id, "First input argument must be a handle.");
  }
  return (gm_handle)(uintptr_t)(*(uint64_t*)mxGetData(a));
}

static void gm_mex_check(int rc, gm_handle h, const char* fn) {
  if (rc == GM_OK) return;
  char id[128];
  snprintf(id, sizeof(id), "MATLAB:%s:status%d", fn, rc);
  mexErrMsgIdAndTxt(id, "%s", gm_last_error(h));
}

/* gateway for calls of the form fn(handle) with no outputs */
#define GM_MEX_VOID(FN, CALL)                                                         \
  void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {     \
    if (nrhs != 1) mexErrMsgIdAndTxt("MATLAB:" FN ":invalidNumInputs", "Handle input argument required."); \
    if (nlhs != 0) mexErrMsgIdAndTxt("MATLAB:" FN ":maxlhs", "No output arguments are required."); \
    gm_handle h = gm_mex_handle(prhs[0], FN);                                          \
    gm_mex_check(CALL(h), h, FN);                                                      \
  }

/* gateway for fn(handle) -> n x nrhs double matrix */
#define GM_MEX_GET(FN, CALL)                                                          \
  void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {     \
    if (nrhs != 1) mexErrMsgIdAndTxt("MATLAB:" FN ":invalidNumInputs", "Handle input argument required."); \
    if (nlhs != 1) mexErrMsgIdAndTxt("MATLAB:" FN ":maxlhs", "One output arguments is required."); \
    gm_handle h = gm_mex_handle(prhs[0], FN);                                          \
    int64_t info[16];  /* gm_info writes 16 entries */                                                                  \
    gm_mex_check(gm_info(h, info), h, FN);                                             \
    plhs[0] = mxCreateDoubleMatrix((mwSize)info[0], (mwSize)info[1], mxREAL);         \
    gm_mex_check(CALL(h, mxGetPr(plhs[0])), h, FN);                                    \
  }
#endif
