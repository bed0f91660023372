/* get_ode_mex: the FitzHugh-Nagumo recovery variable (n x 1), which the
 * reference keeps on the device between update_U_monodomain steps; with
 * get_U_mex it is the checkpoint of a time loop (see set_state_mex). */
#include "gm_mex_common.h"
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 1 || nlhs != 1) mexErrMsgIdAndTxt("MATLAB:get_ode:invalidNumInputs", "Handle input argument required.");
  gm_handle h = gm_mex_handle(prhs[0], "get_ode");
  int64_t info[16];  /* gm_info writes 16 entries */
  gm_mex_check(gm_info(h, info), h, "get_ode");
  plhs[0] = mxCreateDoubleMatrix((mwSize)info[0], 1, mxREAL);
  gm_mex_check(gm_get_ode(h, mxGetPr(plhs[0])), h, "get_ode");
}
