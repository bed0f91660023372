/* set_y_mex: the MEX file lanczosEngine.set_y calls (lanczosEngine.m:29-31),
 * absent from the reference; sets Yreal/Yimag (m x 2C) before apply_V. */
#include "gm_mex_common.h"
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 3 || nlhs != 0) mexErrMsgIdAndTxt("MATLAB:set_y:invalidNumInputs", "Handle, yreal and yimag required.");
  gm_handle h = gm_mex_handle(prhs[0], "set_y");
  int64_t info[16];  /* gm_info writes 16 entries */
  gm_mex_check(gm_info(h, info), h, "set_y");
  const size_t want = (size_t)info[2] * info[1] * info[4];
  if (!mxIsDouble(prhs[1]) || !mxIsDouble(prhs[2]) || mxGetNumberOfElements(prhs[1]) != want ||
      mxGetNumberOfElements(prhs[2]) != want)
    mexErrMsgIdAndTxt("MATLAB:set_y:badY", "yreal and yimag must be m x 2C real matrices.");
  gm_mex_check(gm_set_y(h, mxGetPr(prhs[1]), mxGetPr(prhs[2])), h, "set_y");
}
