/* deflation_pairs_mex: the k smallest eigenpairs of a symmetric sparse A on
 * the GPU (gm_deflation_pairs), in place of the host eigensolve of the
 * reference's set-up, [Q, L] = eigs(K, M, k, 'sm') (process_nonuniform.m:
 * 38-40, 106-110); with the lumped mass M pass A = M^{-1/2} K M^{-1/2}.
 *   [lambda, Q] = deflation_pairs_mex(A, k)
 *   [lambda, Q, stats] = deflation_pairs_mex(A, k, tol, max_degree, max_iter, seed)
 * lambda is k x 1 ascending, Q is n x k with orthonormal columns; stats is the
 * 9-vector of gm_deflation_pairs. */
#include <math.h>
#include <vector>
#include "gm_mex_common.h"
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 2 && nrhs != 6)
    mexErrMsgIdAndTxt("MATLAB:deflation_pairs:invalidNumInputs", "Two or six input arguments are required.");
  if (nlhs < 1 || nlhs > 3)
    mexErrMsgIdAndTxt("MATLAB:deflation_pairs:maxlhs", "One to three output arguments are required.");
  const mxArray* A = prhs[0];
  if (!mxIsSparse(A) || !mxIsDouble(A) || mxIsComplex(A) || mxGetM(A) != mxGetN(A))
    mexErrMsgIdAndTxt("MATLAB:deflation_pairs:inputNotSparse", "A must be a real square sparse matrix.");
  for (int i = 1; i < nrhs; ++i)
    if (!mxIsDouble(prhs[i]) || mxGetNumberOfElements(prhs[i]) != 1)
      mexErrMsgIdAndTxt("MATLAB:deflation_pairs:badScalar", "k and the options must be numeric scalars.");
  const double kd = mxGetScalar(prhs[1]);
  if (!(kd >= 1) || kd != floor(kd) || kd > 1e6) mexErrMsgIdAndTxt("MATLAB:deflation_pairs:bad_k", "Invalid k input argument.");
  double tol = 1e-8, deg = 1000, iters = 200, seed = 0;
  if (nrhs == 6) {
    tol = mxGetScalar(prhs[2]);
    deg = mxGetScalar(prhs[3]);
    iters = mxGetScalar(prhs[4]);
    seed = mxGetScalar(prhs[5]);
    if (deg != floor(deg) || iters != floor(iters) || seed != floor(seed) || !(seed >= 0) || fabs(deg) > 1e9 || iters > 1e9)
      mexErrMsgIdAndTxt("MATLAB:deflation_pairs:badOption", "max_degree, max_iter and seed must be whole numbers.");
  }
  const size_t n = mxGetN(A);
  const mwIndex* jc = mxGetJc(A);
  const mwIndex* ir = mxGetIr(A);
  // A is symmetric, so its CSC arrays are the CSR arrays of A itself
  std::vector<int64_t> ptr(n + 1);
  for (size_t i = 0; i <= n; ++i) ptr[i] = (int64_t)jc[i];
  std::vector<int32_t> col(ptr[n]);
  for (int64_t t = 0; t < ptr[n]; ++t) col[t] = (int32_t)ir[t];
  const int k = (int)kd;
  plhs[0] = mxCreateDoubleMatrix((mwSize)k, 1, mxREAL);
  mxArray* Q = mxCreateDoubleMatrix((mwSize)n, (mwSize)k, mxREAL);
  mxArray* st = mxCreateDoubleMatrix(9, 1, mxREAL);
  const int rc = gm_deflation_pairs((int64_t)n, ptr.data(), col.data(), mxGetPr(A), k, tol, (int)deg, (int)iters,
                                    (uint64_t)seed, mxGetPr(plhs[0]), mxGetPr(Q), mxGetPr(st));
  gm_mex_check(rc, nullptr, "deflation_pairs");
  if (nlhs >= 2) plhs[1] = Q;
  if (nlhs >= 3) plhs[2] = st;
}
