/* get_aabb_mex: the MEX file lanczosEngine.get_aabb calls (lanczosEngine.m:25-27),
 * absent from the reference; returns aabb ((m+1) x 4). */
#include "gm_mex_common.h"
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 1 || nlhs != 1) mexErrMsgIdAndTxt("MATLAB:get_aabb:invalidNumInputs", "Handle input argument required.");
  gm_handle h = gm_mex_handle(prhs[0], "get_aabb");
  int64_t info[16];  /* gm_info writes 16 entries */
  gm_mex_check(gm_info(h, info), h, "get_aabb");
  plhs[0] = mxCreateDoubleMatrix((mwSize)(info[2] + 1), (mwSize)(2 * info[1]), mxREAL);
  gm_mex_check(gm_get_aabb(h, mxGetPr(plhs[0])), h, "get_aabb");
}
