/* time_loop_mex(h, nsteps, monodomain, use_graph): nsteps of solve +
 * update_U (monodomain = 0) or + update_U_monodomain (monodomain = 1), the
 * steps captured once into a CUDA graph and replayed when use_graph is
 * nonzero (gm_time_loop).  The loop the reference's scripts drive from
 * MATLAB one MEX call at a time. */
#include <math.h>
#include "gm_mex_common.h"
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 4 || nlhs != 0)
    mexErrMsgIdAndTxt("MATLAB:time_loop:invalidNumInputs", "Handle, nsteps, monodomain and use_graph input arguments required.");
  gm_handle h = gm_mex_handle(prhs[0], "time_loop");
  for (int i = 1; i < 4; ++i)
    if (!mxIsDouble(prhs[i]) || mxGetNumberOfElements(prhs[i]) != 1)
      mexErrMsgIdAndTxt("MATLAB:time_loop:badScalar", "nsteps, monodomain and use_graph must be numeric scalars.");
  const double ns = mxGetScalar(prhs[1]);
  if (!(ns >= 0) || ns > 2147483647.0 || ns != floor(ns))
    mexErrMsgIdAndTxt("MATLAB:time_loop:bad_nsteps", "Invalid nsteps input argument (a whole number >= 0).");
  const double mono = mxGetScalar(prhs[2]), graph = mxGetScalar(prhs[3]);
  if (mono != mono) mexErrMsgIdAndTxt("MATLAB:time_loop:bad_monodomain", "Invalid monodomain input argument (NaN).");
  if (graph != graph) mexErrMsgIdAndTxt("MATLAB:time_loop:bad_use_graph", "Invalid use_graph input argument (NaN).");
  gm_mex_check(gm_time_loop(h, (int)ns, mono != 0 ? 1 : 0, graph != 0 ? 1 : 0), h, "time_loop");
}
