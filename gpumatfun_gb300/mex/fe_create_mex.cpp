/* fe_create_mex: creates an engine for the adjoint of the finite-element
 * fractional operator A(kappa) = M^{-1/2} K(kappa) M^{-1/2} and attaches its
 * element structure (gm_lanczos_create with keep_entry_map, then
 * gm_fe_attach).  No counterpart in the reference, whose matrices are fixed.
 *
 *   h = fe_create_mex(A, N, gamma, gamma_s_real, gamma_s_imag, wts, shifts,
 *                     ent_ptr, ent_tri, ent_coef, tri_nodes, tri_kc [, mixed])
 *
 * A: the sparse operator at some kappa (its pattern and initial values);
 * wts (C x 2) the weights of f for both columns; shifts (4 N C) as for
 * lanczos_create; the entry lists and triangle arrays as documented at
 * gm_fe_attach (ent_ptr, ent_tri, tri_nodes zero-based, given as doubles
 * in CSC order of A); mixed = 1 selects the mixed-precision engine. */
#include <vector>
#include "gm_mex_common.h"

static const double* dbl(const mxArray* a, const char* what) {
  if (!mxIsDouble(a) || mxIsComplex(a)) mexErrMsgIdAndTxt("MATLAB:fe_create:badInput", "Invalid %s input argument.", what);
  return mxGetPr(a);
}

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 12 && nrhs != 13) mexErrMsgIdAndTxt("MATLAB:fe_create:invalidNumInputs", "Twelve or thirteen input arguments are required.");
  if (nlhs != 1) mexErrMsgIdAndTxt("MATLAB:fe_create:maxlhs", "One output argument is required.");
  const mxArray* A = prhs[0];
  if (!mxIsSparse(A) || mxIsComplex(A) || mxGetM(A) != mxGetN(A))
    mexErrMsgIdAndTxt("MATLAB:fe_create:inputNotSparse", "Invalid sparse matrix input argument.");
  const mwSize n = mxGetM(A);
  const mwIndex* jc = mxGetJc(A);
  const mwIndex* ir = mxGetIr(A);
  const size_t nnz = jc[n];
  /* A is symmetric, so its CSC arrays are the CSR arrays of A (row j = column j) */
  std::vector<int64_t> ptr(jc, jc + n + 1), ind(ir, ir + nnz);
  gm_create_args a;
  gm_default_args(&a);
  a.n = (int64_t)n;
  a.nnz = (int64_t)nnz;
  a.format = GM_CSR;
  a.ptr = ptr.data();
  a.ind = ind.data();
  a.values = mxGetPr(A);
  a.nrhs = 2;
  std::vector<double> U(2 * n, 0.0);
  a.U = U.data();
  a.subspace_size = (int)mxGetScalar(prhs[1]);
  a.gamma_size = (int)mxGetNumberOfElements(prhs[2]);
  a.gamma = dbl(prhs[2], "gamma");
  a.contour_size = (int)mxGetN(prhs[3]);
  a.gamma_s_real = dbl(prhs[3], "gamma_s_real");
  a.gamma_s_imag = dbl(prhs[4], "gamma_s_imag");
  const int C = a.contour_size;
  if ((int)mxGetM(prhs[5]) != C || mxGetN(prhs[5]) != 2) mexErrMsgIdAndTxt("MATLAB:fe_create:bad_wts", "Invalid wts input argument.");
  std::vector<double> wts(4 * (size_t)C);
  for (int r = 0; r < 2; ++r) memcpy(wts.data() + 2 * C * r, mxGetPr(prhs[5]), sizeof(double) * 2 * C);
  a.wts = wts.data();
  a.shifts = dbl(prhs[6], "shifts");
  double cs[2] = {1.0, 1.0};
  a.col_scale = cs;
  a.keep_entry_map = 1;
  a.sync_mode = 0;
  if (nrhs == 13 && mxGetScalar(prhs[12]) != 0.0) a.precision = GM_MIXED;
  const size_t ntri = mxGetM(prhs[10]);
  if (mxGetNumberOfElements(prhs[7]) != nnz + 1 || mxGetN(prhs[10]) != 3 || mxGetM(prhs[11]) != ntri || mxGetN(prhs[11]) != 9)
    mexErrMsgIdAndTxt("MATLAB:fe_create:badStructure", "Inconsistent element structure arguments.");
  const double* ep = dbl(prhs[7], "ent_ptr");
  const double* et = dbl(prhs[8], "ent_tri");
  const double* tn = dbl(prhs[10], "tri_nodes");
  const double* kc = dbl(prhs[11], "tri_kc");
  std::vector<int64_t> ent_ptr(ep, ep + nnz + 1);
  const size_t ncon = (size_t)ent_ptr[nnz];
  if (mxGetNumberOfElements(prhs[8]) != ncon || mxGetNumberOfElements(prhs[9]) != ncon)
    mexErrMsgIdAndTxt("MATLAB:fe_create:badStructure", "Inconsistent entry lists.");
  std::vector<int32_t> ent_tri(et, et + ncon);
  /* column-major ntri x 3 / ntri x 9 -> row-major */
  std::vector<int64_t> nodes(3 * ntri);
  std::vector<double> kcr(9 * ntri);
  for (size_t t = 0; t < ntri; ++t) {
    for (int c = 0; c < 3; ++c) nodes[3 * t + c] = (int64_t)tn[t + ntri * c];
    for (int c = 0; c < 9; ++c) kcr[9 * t + c] = kc[t + ntri * c];
  }
  gm_handle h = nullptr;
  int rc = gm_lanczos_create(&a, &h);
  if (rc != GM_OK) mexErrMsgIdAndTxt("MATLAB:fe_create:create", "%s", gm_last_error(nullptr));
  rc = gm_fe_attach(h, (int64_t)ntri, ent_ptr.data(), ent_tri.data(), dbl(prhs[9], "ent_coef"), nodes.data(), kcr.data());
  if (rc != GM_OK) {
    const char* msg = gm_last_error(h);
    char buf[512];
    snprintf(buf, sizeof(buf), "%s", msg);
    gm_lanczos_delete(h);
    mexErrMsgIdAndTxt("MATLAB:fe_create:attach", "%s", buf);
  }
  plhs[0] = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
  *(uint64_t*)mxGetData(plhs[0]) = (uint64_t)(uintptr_t)h;
}
