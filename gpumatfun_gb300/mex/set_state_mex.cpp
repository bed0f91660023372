/* set_state_mex(h, U, ode): resumes a time loop from a checkpoint taken with
 * get_U_mex and get_ode_mex (U exactly as get_U returned it, n x 2; ode n x 1
 * or [] to keep the device copy). */
#include "gm_mex_common.h"
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 3 || nlhs != 0) mexErrMsgIdAndTxt("MATLAB:set_state:invalidNumInputs", "Handle, U and ode input arguments required.");
  gm_handle h = gm_mex_handle(prhs[0], "set_state");
  int64_t info[16];  /* gm_info writes 16 entries */
  gm_mex_check(gm_info(h, info), h, "set_state");
  if (!mxIsDouble(prhs[1]) || mxGetM(prhs[1]) != (mwSize)info[0] || mxGetN(prhs[1]) != (mwSize)info[1])
    mexErrMsgIdAndTxt("MATLAB:set_state:badU", "Invalid U input argument.");
  const double* ode = nullptr;
  if (mxGetNumberOfElements(prhs[2]) != 0) {
    if (!mxIsDouble(prhs[2]) || mxGetNumberOfElements(prhs[2]) != (size_t)info[0])
      mexErrMsgIdAndTxt("MATLAB:set_state:bad_ode", "Invalid ode input argument.");
    ode = mxGetPr(prhs[2]);
  }
  gm_mex_check(gm_set_state(h, mxGetPr(prhs[1]), ode), h, "set_state");
}
