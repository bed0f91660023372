/* get_basis_mex: the Krylov basis V of the last build_subspace, which the
 * reference keeps on the device only (lanczos.h, V); returns n x (m*nrhs),
 * the m basis vectors of right-hand side r in columns r*m .. r*m+m-1. */
#include "gm_mex_common.h"
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 1 || nlhs != 1) mexErrMsgIdAndTxt("MATLAB:get_basis:invalidNumInputs", "Handle input argument required.");
  gm_handle h = gm_mex_handle(prhs[0], "get_basis");
  int64_t info[16];  /* gm_info writes 16 entries */
  gm_mex_check(gm_info(h, info), h, "get_basis");
  plhs[0] = mxCreateDoubleMatrix((mwSize)info[0], (mwSize)(info[2] * info[1]), mxREAL);
  gm_mex_check(gm_get_basis(h, mxGetPr(plhs[0])), h, "get_basis");
}
