/*
 * gpumatfun.h -- C ABI of the GB300-native f(A)b engine.
 *
 * The engine computes f(A) b for a sparse symmetric A by polynomial-
 * preconditioned Lanczos, deflation by k known eigenvectors and the
 * Hale-Higham-Trefethen contour integral evaluated through batched shifted
 * complex tridiagonal solves.  Each entry point below replaces one MEX
 * gateway of the reference (GPUMatfun, MATLAB -> MEX -> CUDA) and keeps its
 * meaning; the MEX shim in gpumatfun_gb300/mex/ maps the MATLAB arguments
 * onto these calls.
 *
 * Conventions
 *  - Host arrays are column-major, as MATLAB stores them.
 *  - Every function returns a gm_status; GM_OK is 0.  On failure the
 *    message is available from gm_last_error(h) (or gm_last_error(NULL)
 *    for failures before a handle exists).
 *  - A handle owns all its device memory and one CUDA stream.  A handle is
 *    not thread-safe; different handles may be used from different threads.
 *  - With sync_mode = 1 (default) each call waits for its kernels and
 *    checks the device status word; with sync_mode = 0 calls are
 *    asynchronous on the handle's stream until gm_sync or a gm_get_* call.
 */
#ifndef GPUMATFUN_H
#define GPUMATFUN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GM_CREATE_ARGS_VERSION 1

typedef struct gm_engine* gm_handle;

typedef enum gm_status {
  GM_OK = 0,
  GM_ERR_ARG = 1,          /* invalid argument (shape, size, pointer)           */
  GM_ERR_OOM = 2,          /* device allocation failed                          */
  GM_ERR_CUDA = 3,         /* CUDA runtime error                                */
  GM_ERR_BREAKDOWN = 4,    /* Lanczos breakdown in every right-hand side        */
  GM_ERR_TIMEOUT = 5,      /* a bounded grid-barrier wait expired               */
  GM_ERR_STATE = 6,        /* call out of order (e.g. apply before solves)      */
  GM_ERR_NONFINITE = 7,    /* NaN/Inf met in the recurrence                     */
  GM_ERR_UNSUPPORTED = 8,  /* option not available on this device/build         */
  GM_ERR_NOCONV = 9        /* iteration limit reached before the tolerance      */
} gm_status;

typedef enum gm_precision {
  GM_FP64 = 0,   /* FP64 values, basis and arithmetic (the reference's precision) */
  GM_MIXED = 1   /* FP32 values and Krylov basis; exact products and compensated
                    sums on the FP32 pipe; FP64 alpha/beta recurrence, tridiagonal
                    solves and quadrature */
} gm_precision;

typedef enum gm_matrix_format {
  GM_CSC = 0,    /* MATLAB sparse storage: colptr (jc), rowind (ir), values (pr) */
  GM_CSR = 1
} gm_matrix_format;

/* Arguments of gm_lanczos_create.  The first block carries exactly the 26
 * positional arguments of lanczos_create (lanczos_create.cpp:7-32,
 * lanczosEngine.m:9); nrhs generalises the reference's fixed pair of
 * right-hand sides (column 0 = exp part with wts1/exp_lambda, column 1 = phi
 * part with wts2/phi_lambda). */
typedef struct gm_create_args {
  int struct_version;          /* GM_CREATE_ARGS_VERSION                         */
  /* A: n x n sparse (lanczos_create.cpp:69-118) */
  int64_t n;
  int64_t nnz;                 /* stored entries; taken as colptr[n] when 0      */
  int format;                  /* gm_matrix_format                               */
  const int64_t* ptr;          /* n+1 column (CSC) or row (CSR) pointers          */
  const int64_t* ind;          /* nnz row (CSC) or column (CSR) indices           */
  const double* values;        /* nnz                                             */
  /* U: n x nrhs right-hand sides (ARG_U) */
  int nrhs;
  const double* U;
  /* deflation: Q n x k, lambda k (unused on device, as in the reference),
   * flam k x nrhs = f_r(lambda) (exp_lambda / phi_lambda for the reference) */
  int num_eigs;
  const double* Q;
  const double* lambda;
  const double* flam;
  /* Krylov dimension (ARG_N) and polynomial preconditioner (ARG_gamma) */
  int subspace_size;
  int gamma_size;              /* d + 1 */
  const double* gamma;
  /* contour: gamma_s_{real,imag} (d+1) x C; wts: nrhs blocks of C x 2
   * [re, im] (wts1, wts2); shifts: 2*m*C*nrhs (the reference's 4mC) */
  int contour_size;
  const double* gamma_s_real;
  const double* gamma_s_imag;
  const double* wts;
  const double* shifts;
  /* time stepping (ARG_dt, ARG_ode .. ARG_c2ion, ARG_mass) */
  double dt;
  const double* col_scale;     /* nrhs; NULL = reference convention [1, dt]     */
  const double* mass;          /* n; NULL = ones                                  */
  const double* ode;           /* n; NULL = zeros                                 */
  double aode, bode, code, vrest, vamp, vth, vpeak, c1ion, c2ion;
  /* engine options (no counterpart in the reference) */
  int precision;               /* gm_precision                                    */
  int sync_mode;               /* 1 = synchronous checked calls (default)        */
  int threads_per_block;       /* 0 = 512                                         */
  int blocks_per_sm;           /* 0 = occupancy-limited, at most 2                */
  int sell_sigma;              /* SELL-32 sorting window in rows; 0/1 = unsorted  */
  double barrier_timeout_s;    /* 0 = 5 s                                         */
  double breakdown_tol;        /* 0 = 64 eps, relative to |alpha_j| + beta_j      */
  int sync_policy;             /* ordering of consecutive SpMV passes: 0 = waits on
                                  the blocks owning referenced rows (default),
                                  1 = grid barriers                               */
  int col_staging;             /* SELL column indices staged in shared memory by TMA
                                  bulk copies (with the value prefetch): 0 = when
                                  the matrix is not held in the L2 window or
                                  val_prefetch = 1 (default), 1 = never (read
                                  directly), 2 = always                            */
  int keep_entry_map;          /* 1 = keep the map from stored entries (CSR order)
                                  to device slots, needed by gm_fe_attach          */
  int l2_window;               /* 0 = launches keep the SELL matrix resident in L2
                                  (persisting access-policy window) when it fits
                                  the device's persisting limit and the matrix plus
                                  one SpMV pass's vectors fit in L2 (default),
                                  1 = off, 2 = on whenever the matrix fits the
                                  persisting limit                                 */
  const double* row_weight;    /* mixed engine, n entries: the FP32-stored matrix
                                  gets a per-row diagonal correction so that
                                  A' w = A w exactly for this w (the operator's
                                  near-null vector: ones for a graph Laplacian,
                                  M^{1/2} 1 for M^{-1/2} K M^{-1/2}); NULL = ones  */
  int diag_compensation;       /* mixed engine: 0 = on (default), 1 = off          */
  int max_blocks;              /* > 0: at most this many blocks in the grid
                                  (a tuning knob); 0 = engine default            */
  int matrix_powers;           /* 1 = two Horner levels of the polynomial per SpMV
                                  pass (halo rows recomputed per block, the level
                                  in between in shared memory), where it applies:
                                  one problem, no sigma sorting, the vector fits
                                  shared memory; 0 = one level per pass            */
  int reorth;                  /* Gram-Schmidt reorthogonalisation of every new
                                  Lanczos vector against the stored basis, with
                                  FP64 dot products: 0 = none (the reference's
                                  three-term recurrence, default), 1 = classical
                                  Gram-Schmidt once, 2 = twice (CGS2).  Adds
                                  2 (resp. 4) reads of V_0..V_j per step.        */
  int val_prefetch;            /* L2 bulk prefetch (TMA) of each slice's values
                                  with its column copy: 0 = when the matrix is not
                                  held in the L2 persisting window (default),
                                  1 = always, 2 = never.  More bytes in flight per
                                  warp for a matrix streamed from HBM.           */
} gm_create_args;

/* Fill *args with defaults (zeros, struct_version, sync_mode = 1, nrhs = 2). */
void gm_default_args(gm_create_args* args);

/* Replaces lanczos_create (lanczos_create.cpp:35-766 and the engine
 * constructor lanczos_impl.cu:5-91): uploads A, Q, U and the method
 * parameters, scales U's columns by col_scale, keeps Usol = U and deflates:
 * Z = Q^T U, U <- U - Q Z, update = Q (f(lambda) o Z). */
int gm_lanczos_create(const gm_create_args* args, gm_handle* out);

/* One problem of a batch: its matrix, right-hand sides and method arrays
 * (same meaning and layout as the fields of gm_create_args). */
typedef struct gm_batch_problem {
  int64_t n;
  int format;
  const int64_t* ptr;
  const int64_t* ind;
  const double* values;
  const double* U;              /* n x nrhs */
  const double* gamma;          /* gamma_size */
  const double* gamma_s_real;   /* gamma_size x C */
  const double* gamma_s_imag;
  const double* wts;            /* nrhs blocks of C x 2 */
  const double* shifts;         /* 2 m C nrhs */
} gm_batch_problem;

/* Several independent problems (uneven sizes allowed) in one engine: every
 * launch runs all of them at once, each on its own group of blocks with its
 * own barriers and reductions.  common supplies nrhs, subspace_size,
 * gamma_size, contour_size, precision and the engine options; num_eigs must
 * be 0.  Vectors (U, X, solution) are the problems' rows stacked in order
 * (n = sum of n_p); aabb, Y and m_eff are per problem, in problem order.
 * No counterpart in the reference (it runs one problem per engine). */
int gm_batch_create(int nprob, const gm_batch_problem* probs, const gm_create_args* common, gm_handle* out);

/* Replaces lanczos_delete (lanczos_delete.cpp:6-35). */
int gm_lanczos_delete(gm_handle h);

/* Replaces build_subspace_mex (build_subspace.cpp:6-35, build_subspace.cu:5-91):
 * m steps of Lanczos on A p(A) for every right-hand side; fills V and aabb. */
int gm_build_subspace(gm_handle h);

/* Replaces lin_sys_solves_mex (lin_sys_solves.cpp:6-35, lin_sys_solves.cu:5-21):
 * y_{r,j} = w_{r,j} beta0_r (sigma_j I - T_r)^{-1} e1 for every node and RHS. */
int gm_lin_sys_solves(gm_handle h);

/* Replaces apply_V_mex (apply_V.cpp:6-35, apply_V.cu:5-95):
 * X_r += sum_j Im(q_j(A) V_r y_{r,j}). */
int gm_apply_V(gm_handle h);

/* Replaces update_U_mex (update_U.cpp:6-35, update_U.cu:5-32): Fisher-KPP
 * exponential-Euler step, re-deflation, X = 0.  Needs nrhs = 2. */
int gm_update_U(gm_handle h);

/* Replaces update_U_monodomain_mex (update_U_monodomain.cpp:6-35,
 * update_U_monodomain.cu:5-43): FitzHugh-Nagumo step. Needs nrhs = 2. */
int gm_update_U_monodomain(gm_handle h);

/* Replaces get_U_mex (get_U.cpp:6-38, lanczos_impl.cu:502-506): copies Usol
 * (n x nrhs, column-major) to dst. */
int gm_get_U(gm_handle h, double* dst);

/* Replaces get_xsol_mex (get_xsol.cpp:6-38, lanczos_impl.cu:508-512): copies
 * X (n x nrhs, column-major) to dst. */
int gm_get_xsol(gm_handle h, double* dst);

/* Implements lanczosEngine.get_aabb (lanczosEngine.m:25-27), whose MEX file
 * the reference never shipped: copies aabb ((m+1) x 2*nrhs, alpha columns then
 * beta columns) to dst. */
int gm_get_aabb(gm_handle h, double* dst);

/* Implements lanczosEngine.set_y (lanczosEngine.m:29-31), whose MEX file the
 * reference never shipped: sets Yreal/Yimag (m x nrhs*C) for apply_V. */
int gm_set_y(gm_handle h, const double* yreal, const double* yimag);

/* Copies Yreal and Yimag (m x nrhs*C each) to the host (either may be NULL). */
int gm_get_y(gm_handle h, double* yreal, double* yimag);

/* Copies the Krylov basis V to the host as FP64: for each right-hand side r an
 * n x m column-major block (dst[(r*m + j)*n + i] = v_j(i)); rows in the
 * caller's order (stacked problems for a batch).  In the mixed engine these
 * are the FP32-stored vectors.  The basis of build_subspace (lanczos.h:47,
 * V), which the reference keeps on the device only. */
int gm_get_basis(gm_handle h, double* dst);

/* ---- additions with no reference counterpart ------------------------------ */

/* Time-loop checkpoint and resume.  The state of a time loop after any step is
 * Usol (gm_get_U: n x nrhs, column-major, with the column scaling applied)
 * and the FitzHugh-Nagumo recovery variable ode (n; update_U_monodomain.cu
 * keeps it on the device between steps).  gm_get_ode copies ode to the host;
 * gm_set_state restores Usol exactly as gm_get_U returned it (no column
 * scaling, unlike gm_set_U) and ode (NULL keeps the device copy),
 * re-deflates and clears X, so the next steps continue the trajectory bit
 * for bit. */
int gm_get_ode(gm_handle h, double* ode_host);
int gm_set_state(gm_handle h, const double* Usol_host, const double* ode_host);

/* New right-hand sides (n x nrhs, column-major, host): U <- U_host o col_scale,
 * Usol = U, re-deflate, X = 0. */
int gm_set_U(gm_handle h, const double* U_host);

/* As gm_set_U with U a device pointer (column-major n x nrhs) on the
 * handle's device; asynchronous on the handle's stream. */
int gm_set_U_device(gm_handle h, const double* U_dev);

/* Copies the deflation update Q (f(lambda) o Q^T U) (n x nrhs) to dst. */
int gm_get_update(gm_handle h, double* dst);

/* f(A) b for every column: X + update (n x nrhs, column-major) to dst. */
int gm_get_solution(gm_handle h, double* dst);

/* The same solution, column-major n x nrhs, into device memory on the
 * handle's stream (no host synchronisation unless sync_mode is set). */
int gm_get_solution_device(gm_handle h, double* dst_dev);

/* One f(A)b evaluation in a single persistent launch: build_subspace,
 * lin_sys_solves and apply_V fused; then X + update is available. */
int gm_solve(gm_handle h);

/* End to end with host buffers: set_U(b_host), gm_solve, solution -> x_host. */
int gm_solve_host(gm_handle h, const double* b_host, double* x_host);

/* Finite-element operator A(kappa) = M^{-1/2} K(kappa) M^{-1/2}, K(kappa) =
 * sum_e kappa_e K_e (unit-coefficient P1 element stiffness K_e), for the
 * adjoint of fractional diffusion.  No counterpart in the reference (its
 * matrices are fixed inputs).  The engine must be created from a CSR matrix
 * with keep_entry_map = 1.
 *   ent_ptr  (nnz+1) : for stored entry t (CSR order) of A, its contributions
 *   ent_tri, ent_coef: are kappa[ent_tri[p]] * ent_coef[p], p in ent_ptr[t]..
 *   tri_nodes (ntri x 3): row of each vertex, -1 for a boundary vertex
 *   tri_kc   (ntri x 9): msi_a K_e[a][c] msi_c (row-major), msi = M^{-1/2}  */
int gm_fe_attach(gm_handle h, int64_t ntri, const int64_t* ent_ptr, const int32_t* ent_tri, const double* ent_coef,
                 const int64_t* tri_nodes, const double* tri_kc);

/* Recomputes A's stored values from kappa (device pointer, ntri doubles) on
 * the handle's stream; Krylov state is invalidated. */
int gm_fe_assemble(gm_handle h, const double* kappa_dev);

/* dL/dkappa (device pointer, ntri doubles) for L = 1/2 ||f(A) b - d||^2, after
 * a solve (gm_solve, or build_subspace + lin_sys_solves) with U = [b, g],
 * g = f(A) b - d (nrhs = 2, both columns with the weights of f, no deflation):
 *   dL/dkappa_e = Im sum_j w_j s_j^T (M^{-1/2} K_e M^{-1/2}) r_j,
 *   r_j = (xi_j - A)^{-1} b,  s_j = (xi_j - A)^{-1} g,
 * with (xi_j - A)^{-1} = q_j(A) (sigma_j - A p(A))^{-1} from the engine's
 * shifted solves (q_j the shifted polynomial, gamma_s(:, j)).
 * dL/db = f(A) g is column 1 of the solution. */
int gm_fe_gradient(gm_handle h, double* dkappa_dev);

/* One forward evaluation x = f(A(kappa)) b: assemble A(kappa), solve, copy
 * the solution.  kappa (ntri), b and x (n) may be host or device memory (UVA);
 * results in host memory are complete on return, device results follow the
 * handle's stream order.  An nrhs = 1 engine keeps this solve's Krylov state
 * (basis and shifted solutions) for gm_fe_backward_stored; an nrhs = 2 engine
 * solves [b, 0]. */
int gm_fe_forward(gm_handle h, const double* kappa, const double* b, double* x);

/* The backward entry: dkappa = dL/dkappa (ntri) and, when db is not NULL,
 * db = dL/db = f(A) g (n), for dL/dx = g at x = f(A(kappa)) b.  The Krylov
 * state of b is recomputed (nrhs = 1: b, then g, in two stored states;
 * nrhs = 2: [b, g] in one solve).  Pointers as in gm_fe_forward. */
int gm_fe_backward(gm_handle h, const double* kappa, const double* b, const double* g, double* dkappa, double* db);

/* The same for the kappa and b of the last gm_fe_forward on this nrhs = 1
 * handle, reusing its stored Krylov state: one solve (for g) instead of two.
 * GM_ERR_STATE when no forward state is stored (after gm_fe_assemble, gm_set_U
 * or a forward on another input). */
int gm_fe_backward_stored(gm_handle h, const double* g, double* dkappa, double* db);

/* nsteps steps of the reference's time loop (nicksmethodgpu_problem.m:7-16,
 * nicksmethodgpu_problem_monodomain.m:7-16): build_subspace + lin_sys_solves
 * + apply_V fused, then update_U (mode 0, Fisher-KPP) or update_U_monodomain
 * (mode 1, FitzHugh-Nagumo).  With use_graph = 1 the nsteps steps are
 * captured once into a CUDA graph (cached per nsteps and mode) and replayed
 * by a single graph launch.  Needs nrhs = 2; the last step's timing is
 * phase slot [4] of gm_phase_times.  use_graph = 1 on the legacy or the
 * per-thread default stream (which cannot be captured) returns GM_ERR_ARG
 * before any work.  On every return the handle's synchronous mode is as
 * before the call, and after a failed call the basis, solves and lift count
 * as not computed (GM_ERR_STATE from apply_V until the next build). */
int gm_time_loop(gm_handle h, int nsteps, int mode, int use_graph);

/* Waits for the handle's stream and returns the device status. */
int gm_sync(gm_handle h);

/* Uses an external CUDA stream (cudaStream_t passed as void*); NULL restores
 * the handle's own stream.  The legacy default stream (the stream PyTorch's
 * default stream is) is selected by its CUDA handle value, cudaStreamLegacy
 * ((void*)1); cudaStreamPerThread ((void*)2) likewise. */
int gm_set_stream(gm_handle h, void* stream);

/* Device milliseconds of the last launch of each phase group, measured with
 * CUDA events on the handle's stream: [0] deflate/update, [1] build_subspace,
 * [2] lin_sys_solves, [3] apply_V, [4] fused solve. */
int gm_phase_times(gm_handle h, float* ms5);

/* Engine facts: [0] n, [1] nrhs, [2] m, [3] d, [4] C, [5] k, [6] precision,
 * [7] grid blocks, [8] threads per block, [9] SELL padded entries,
 * [10] device bytes held, [11] kernel launches so far, [12] problems,
 * [13] 1 when matrix-powers passes are active, [14] bytes per SELL value
 * when the values are prefetched into L2 (0: no prefetch), [15] Gram-Schmidt passes per
 * Lanczos step.  info has 16 entries. */
int gm_info(gm_handle h, int64_t* info16);

/* gm_info's entries followed by: [16] bytes of the matrix under the L2
 * persisting access-policy window (0: no window, the matrix streams from
 * HBM on every pass), [17] column-index staging depth in 32-column groups
 * per stage (0: staging off), [18] 1 when passes wait on their neighbour
 * blocks only, 0 when every pass ends at a grid barrier.  Fills the first
 * min(count, GM_INFO_EX_COUNT) entries. */
#define GM_INFO_EX_COUNT 19
int gm_info_ex(gm_handle h, int64_t* info, int count);

/* Effective Krylov dimension per (problem, RHS) after the last build (< m
 * after a breakdown). */
int gm_get_meff(gm_handle h, int* meff);

/* Largest m * nrhs * C accepted by gm_lin_sys_solves_noalloc. */
#define GM_NOALLOC_MAX_ENTRIES 32768

/* The shifted tridiagonal solves of gm_lin_sys_solves for callers that
 * cannot allocate device memory -- applications whose device memory is all
 * owned by their own allocator (MATLAB's gpuArray manager, a framework's
 * caching pool, a fixed-budget embedded solver) and latency-critical loops
 * where cudaMalloc's implicit device synchronisation is not acceptable.  No
 * counterpart in the reference.
 *
 * All pointers are device pointers on the current device, supplied by the
 * caller: aabb ((m+1) x 2*nrhs, column-major, alpha columns then beta
 * columns, as gm_get_aabb returns), meff (nrhs ints, clamped to [0, m];
 * NULL = m), wts
 * (nrhs blocks of C x 2 [re, im]), shifts (2*m*C*nrhs) and the outputs
 * yreal, yimag (m x nrhs*C, as gm_get_y).  stream is a cudaStream_t (NULL =
 * legacy default stream); the call is asynchronous on it.
 *
 * The only other memory used is a fixed table of 1 MiB + 32 bytes in a
 * file-scope __device__ array, so m * nrhs * C must not exceed
 * GM_NOALLOC_MAX_ENTRIES (GM_ERR_ARG otherwise, message in
 * gm_last_error(NULL)).  Every call looks up the table's device address
 * with the current device (a lookup, no allocation), so the entry point
 * stays valid across a cudaDeviceReset; the first call on a device also
 * loads the library's device code there, so make it before any stream
 * capture.  All calls share the table and it keeps the last call's contents
 * (no entry needs to start at zero): calls whose kernels overlap on the GPU
 * race and must be ordered on one stream. */
int gm_lin_sys_solves_noalloc(int m, int nrhs, int contour_size, const double* aabb, const int* meff,
                              const double* wts, const double* shifts, double* yreal, double* yimag,
                              void* stream);

/* The k smallest eigenpairs of the symmetric matrix A (n x n, CSR: int64
 * row pointer, int32 column indices, FP64 values; host or device memory),
 * for the engine's deflation vectors Q and lambda.  Replaces the host
 * eigensolve of the reference's set-up, eigs(K, M, k, 'sm') on the
 * generalised problem (process_nonuniform.m:38-40, 106-110; with the lumped
 * mass M this is the symmetric A = M^{-1/2} K M^{-1/2} the engine takes).
 *
 * Method: Chebyshev-filtered subspace iteration over a block of 32 vectors on
 * the GPU: scaled Chebyshev filter on [largest Ritz value, Gershgorin bound],
 * CholQR2, Rayleigh-Ritz with a Jacobi eigensolver of the 32 x 32
 * projection, all in FP64 except the filter while the wanted residuals are
 * above 1e-7, which runs in float-float arithmetic (about 48 bits) on the
 * FP32 pipe; a negative max_degree keeps the filter in FP64 throughout.
 * 1 <= k <= 24, n >= 64.  Iterates until every wanted relative residual
 * ||A q_j - lambda_j q_j|| / |lambda_j| <= tol, or for at most max_iter
 * filter applications of degree <= |max_degree|; seed fixes the start block.
 * Outputs (host or device): lambda (k, ascending) and Q (n x k, column-major,
 * orthonormal columns).  stats (9 doubles, may be NULL): [0] iterations,
 * [1] block SpMVs, [2] device seconds, [3] largest wanted relative residual,
 * [4] Gershgorin bound, [5] last filter cut, [6] largest Ritz value of the
 * block, [7] nnz, [8] block SpMVs in float-float.  Returns GM_ERR_NOCONV
 * (outputs and stats still written) when the tolerance was not reached;
 * messages in gm_last_error(NULL).  Allocates about 6 n 256 + 20 nnz bytes of
 * device memory for the duration of the call and synchronises the device. */
int gm_deflation_pairs(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, int k,
                       double tol, int max_degree, int max_iter, uint64_t seed, double* lambda, double* Q,
                       double* stats);

/* Last error message of h (or of the last failed create when h is NULL). */
const char* gm_last_error(gm_handle h);

/* Library version string. */
const char* gm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GPUMATFUN_H */
