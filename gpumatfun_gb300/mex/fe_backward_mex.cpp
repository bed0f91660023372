/* fe_backward_mex: the backward entry of the adjoint (gm_fe_backward).
 *   [dkappa, db] = fe_backward_mex(h, kappa, b, g)
 * for dL/dx = g at x = f(A(kappa)) b: dkappa = dL/dkappa (one per triangle),
 * db = dL/db = f(A) g. */
#include "gm_mex_common.h"
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 4) mexErrMsgIdAndTxt("MATLAB:fe_backward:invalidNumInputs", "Four input arguments are required.");
  if (nlhs < 1 || nlhs > 2) mexErrMsgIdAndTxt("MATLAB:fe_backward:maxlhs", "One or two output arguments are required.");
  gm_handle h = gm_mex_handle(prhs[0], "fe_backward");
  int64_t info[16];  /* gm_info writes 16 entries */
  gm_mex_check(gm_info(h, info), h, "fe_backward");
  const size_t n = (size_t)info[0];
  for (int i = 1; i < 4; ++i)
    if (!mxIsDouble(prhs[i]) || mxIsComplex(prhs[i])) mexErrMsgIdAndTxt("MATLAB:fe_backward:badInput", "Inputs must be real doubles.");
  if (mxGetNumberOfElements(prhs[2]) != n || mxGetNumberOfElements(prhs[3]) != n)
    mexErrMsgIdAndTxt("MATLAB:fe_backward:badInput", "b and g must have n entries.");
  plhs[0] = mxCreateDoubleMatrix(mxGetNumberOfElements(prhs[1]), 1, mxREAL);
  double* db = nullptr;
  if (nlhs == 2) {
    plhs[1] = mxCreateDoubleMatrix((mwSize)n, 1, mxREAL);
    db = mxGetPr(plhs[1]);
  }
  gm_mex_check(gm_fe_backward(h, mxGetPr(prhs[1]), mxGetPr(prhs[2]), mxGetPr(prhs[3]), mxGetPr(plhs[0]), db), h,
               "fe_backward");
}
