/* fe_forward_mex: x = f(A(kappa)) b on an engine made by fe_create_mex
 * (gm_fe_forward).   x = fe_forward_mex(h, kappa, b) */
#include "gm_mex_common.h"
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 3) mexErrMsgIdAndTxt("MATLAB:fe_forward:invalidNumInputs", "Three input arguments are required.");
  if (nlhs != 1) mexErrMsgIdAndTxt("MATLAB:fe_forward:maxlhs", "One output argument is required.");
  gm_handle h = gm_mex_handle(prhs[0], "fe_forward");
  int64_t info[16];  /* gm_info writes 16 entries */
  gm_mex_check(gm_info(h, info), h, "fe_forward");
  if (!mxIsDouble(prhs[1]) || !mxIsDouble(prhs[2]) || mxGetNumberOfElements(prhs[2]) != (size_t)info[0])
    mexErrMsgIdAndTxt("MATLAB:fe_forward:badInput", "kappa and b must be real doubles, b with n entries.");
  plhs[0] = mxCreateDoubleMatrix((mwSize)info[0], 1, mxREAL);
  gm_mex_check(gm_fe_forward(h, mxGetPr(prhs[1]), mxGetPr(prhs[2]), mxGetPr(plhs[0])), h, "fe_forward");
}
