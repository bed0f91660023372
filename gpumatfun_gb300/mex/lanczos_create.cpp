/* lanczos_create: replaces the reference gateway lanczos_create.cpp:35-766.
 * Same 26 positional arguments (U, A, Q, lambda, N, gamma, gamma_s_real,
 * gamma_s_imag, exp_lambda, phi_lambda, dt, ode, aode, bode, code, vrest,
 * vamp, vth, vpeak, c1ion, c2ion, mass, wts1, wts2, shifts, valvec) and the
 * same error identifiers; returns the engine handle as a 1x1 uint64.
 * An optional 27th argument, a struct, sets engine options by field name:
 * precision ('fp64' | 'mixed'), reorth, val_prefetch, matrix_powers,
 * sync_policy, threads_per_block, blocks_per_sm, sell_sigma (numbers as
 * gm_create_args documents them); absent fields keep their defaults. */
#include <vector>
#include "gm_mex_common.h"

static const double* real_arg(const mxArray* a, const char* id, const char* msg) {
  if (!mxIsDouble(a) || mxIsComplex(a)) mexErrMsgIdAndTxt(id, msg);
  return mxGetPr(a);
}
static double scalar_arg(const mxArray* a, const char* id) {
  if (!mxIsDouble(a) || mxGetM(a) != 1 || mxGetN(a) != 1) mexErrMsgIdAndTxt(id, "Invalid scalar input argument.");
  return mxGetScalar(a);
}

static void read_options(const mxArray* o, gm_create_args* a) {
  if (!mxIsStruct(o)) mexErrMsgIdAndTxt("MATLAB:lanczos_create:badOptions", "Options must be a struct.");
  const mxArray* p = mxGetField(o, 0, "precision");
  if (p) {
    if (!mxIsChar(p)) mexErrMsgIdAndTxt("MATLAB:lanczos_create:badOptions", "precision must be 'fp64' or 'mixed'.");
    char* s = mxArrayToString(p);
    const bool mixed = s && strcmp(s, "mixed") == 0, fp64 = s && strcmp(s, "fp64") == 0;
    mxFree(s);
    if (!mixed && !fp64) mexErrMsgIdAndTxt("MATLAB:lanczos_create:badOptions", "precision must be 'fp64' or 'mixed'.");
    a->precision = mixed ? GM_MIXED : GM_FP64;
  }
  struct { const char* name; int* dst; } ints[] = {
      {"reorth", &a->reorth}, {"val_prefetch", &a->val_prefetch}, {"matrix_powers", &a->matrix_powers},
      {"sync_policy", &a->sync_policy}, {"threads_per_block", &a->threads_per_block},
      {"blocks_per_sm", &a->blocks_per_sm}, {"sell_sigma", &a->sell_sigma}};
  for (auto& f : ints) {
    const mxArray* v = mxGetField(o, 0, f.name);
    if (!v) continue;
    if (!mxIsDouble(v) || mxGetNumberOfElements(v) != 1)
      mexErrMsgIdAndTxt("MATLAB:lanczos_create:badOptions", "Option %s must be a numeric scalar.", f.name);
    *f.dst = (int)mxGetScalar(v);
  }
}

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 26 && nrhs != 27)
    mexErrMsgIdAndTxt("MATLAB:lanczos_create:invalidNumInputs", "Twenty-five input arguments are required.");
  if (nlhs != 1) mexErrMsgIdAndTxt("MATLAB:lanczos_create:maxlhs", "One output argument is required.");
  const mxArray *U = prhs[0], *A = prhs[1], *Q = prhs[2];
  if (!mxIsDouble(U) || mxIsComplex(U)) mexErrMsgIdAndTxt("MATLAB:lanczos_create:badU", "Invalid U input argument.");
  if (!mxIsSparse(A)) mexErrMsgIdAndTxt("MATLAB:lanczos_create:inputNotSparse", "Invalid sparse matrix input argument.");
  if (mxGetM(A) != mxGetN(A)) mexErrMsgIdAndTxt("MATLAB:lanczos_create:inputNotSquare", "Sparse matrix must be square.");
  if (mxIsComplex(A)) mexErrMsgIdAndTxt("MATLAB:lanczos_create:inputNotReal", "First input argument must be a real matrix.");
  const mwSize n = mxGetM(A);
  if (mxGetM(U) != n || mxGetN(U) != 2) mexErrMsgIdAndTxt("MATLAB:lanczos_create:badU", "Invalid U input argument.");
  const mwIndex* jc = mxGetJc(A);
  const mwIndex* ir = mxGetIr(A);
  std::vector<int64_t> ptr(jc, jc + n + 1), ind(ir, ir + jc[n]);
  gm_create_args a;
  gm_default_args(&a);
  a.n = (int64_t)n;
  a.nnz = (int64_t)jc[n];  /* the stored entries, not mxGetNzmax (lanczos_create.cpp:101) */
  a.format = GM_CSC;
  a.ptr = ptr.data();
  a.ind = ind.data();
  a.values = mxGetPr(A);
  a.nrhs = 2;
  a.U = mxGetPr(U);
  a.num_eigs = (int)mxGetN(Q);
  a.Q = real_arg(Q, "MATLAB:lanczos_create:badQ", "Invalid Q input argument.");
  a.lambda = real_arg(prhs[3], "MATLAB:lanczos_create:bad_lambda", "Invalid lambda input argument.");
  a.subspace_size = (int)scalar_arg(prhs[4], "MATLAB:lanczos_create:bad_N");
  a.gamma_size = (int)mxGetNumberOfElements(prhs[5]);
  a.gamma = real_arg(prhs[5], "MATLAB:lanczos_create:bad_gamma", "Invalid gamma input argument.");
  a.contour_size = (int)mxGetN(prhs[6]);
  if ((int)mxGetM(prhs[6]) != a.gamma_size) mexErrMsgIdAndTxt("MATLAB:lanczos_create:bad_gamma_s_real", "Invalid gamma_s_real input argument.");
  if ((int)mxGetM(prhs[7]) != a.gamma_size || (int)mxGetN(prhs[7]) != a.contour_size)
    mexErrMsgIdAndTxt("MATLAB:lanczos_create:bad_gamma_s_imag", "Invalid gamma_s_imag input argument.");
  a.gamma_s_real = mxGetPr(prhs[6]);
  a.gamma_s_imag = mxGetPr(prhs[7]);
  const int k = a.num_eigs;
  if ((int)mxGetNumberOfElements(prhs[8]) != k) mexErrMsgIdAndTxt("MATLAB:lanczos_create:bad_exp_lambda", "Invalid exp_lambda input argument.");
  if ((int)mxGetNumberOfElements(prhs[9]) != k) mexErrMsgIdAndTxt("MATLAB:lanczos_create:bad_phi_lambda", "Invalid phi_lambda input argument.");
  std::vector<double> flam(2 * (size_t)k);
  memcpy(flam.data(), mxGetPr(prhs[8]), sizeof(double) * k);
  memcpy(flam.data() + k, mxGetPr(prhs[9]), sizeof(double) * k);
  a.flam = flam.data();
  a.dt = scalar_arg(prhs[10], "MATLAB:lanczos_create:bad_dt");
  if (mxGetNumberOfElements(prhs[11]) != n) mexErrMsgIdAndTxt("MATLAB:lanczos_create:bad_ode", "Invalid ode input argument.");
  a.ode = mxGetPr(prhs[11]);
  a.aode = scalar_arg(prhs[12], "MATLAB:lanczos_create:bad_aode");
  a.bode = scalar_arg(prhs[13], "MATLAB:lanczos_create:bad_bode");
  a.code = scalar_arg(prhs[14], "MATLAB:lanczos_create:bad_code");
  a.vrest = scalar_arg(prhs[15], "MATLAB:lanczos_create:bad_vrest");
  a.vamp = scalar_arg(prhs[16], "MATLAB:lanczos_create:bad_vamp");
  a.vth = scalar_arg(prhs[17], "MATLAB:lanczos_create:bad_vth");
  a.vpeak = scalar_arg(prhs[18], "MATLAB:lanczos_create:bad_vpeak");
  a.c1ion = scalar_arg(prhs[19], "MATLAB:lanczos_create:bad_c1ion");
  a.c2ion = scalar_arg(prhs[20], "MATLAB:lanczos_create:bad_c2ion");
  if (mxGetNumberOfElements(prhs[21]) != n) mexErrMsgIdAndTxt("MATLAB:lanczos_create:bad_mass", "Invalid mass input argument.");
  a.mass = mxGetPr(prhs[21]);
  if ((int)mxGetM(prhs[22]) != a.contour_size || mxGetN(prhs[22]) != 2) mexErrMsgIdAndTxt("MATLAB:lanczos_create:bad_wts1", "Invalid wts1 input argument.");
  if ((int)mxGetM(prhs[23]) != a.contour_size || mxGetN(prhs[23]) != 2) mexErrMsgIdAndTxt("MATLAB:lanczos_create:bad_wts2", "Invalid wts2 input argument.");
  std::vector<double> wts(4 * (size_t)a.contour_size);
  memcpy(wts.data(), mxGetPr(prhs[22]), sizeof(double) * 2 * a.contour_size);
  memcpy(wts.data() + 2 * a.contour_size, mxGetPr(prhs[23]), sizeof(double) * 2 * a.contour_size);
  a.wts = wts.data();
  if (mxGetNumberOfElements(prhs[24]) != (size_t)4 * a.subspace_size * a.contour_size)
    mexErrMsgIdAndTxt("MATLAB:lanczos_create:bad_shifts", "Invalid shifts input argument c.");
  a.shifts = mxGetPr(prhs[24]);
  /* prhs[25] is valvec = [-1 0 1]: the reference keeps BLAS scalars on the
   * device; the engine needs none. */
  if (nrhs == 27) read_options(prhs[26], &a);
  gm_handle h = nullptr;
  int rc = gm_lanczos_create(&a, &h);
  if (rc != GM_OK) mexErrMsgIdAndTxt("MATLAB:lanczos_create:engine", "%s", gm_last_error(nullptr));
  plhs[0] = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
  *(uint64_t*)mxGetData(plhs[0]) = (uint64_t)(uintptr_t)h;
}
