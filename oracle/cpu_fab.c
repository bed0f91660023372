/*
 * cpu_fab.c -- C/OpenMP restatement of GPUMatfun's CPU f(A)b path
 * (test infrastructure and timed CPU baseline; never part of the product).
 *
 * Follows, statement by statement:
 *   nicksmethodcpu.m:7-43   Lanczos, C shifted tridiagonal solves per RHS,
 *                           per-node V*y and shifted-polynomial Horner,
 *                           summing imaginary parts;
 *   lanczos.m:21-53         three-term recurrence on A p(A) without
 *                           reorthogonalisation, both RHS columns together;
 *   jacobi_poly_eval.m:12-18  Horner with (complex) coefficients, which
 *                           multiplies A by the stacked [real, imag] block
 *                           even when the imaginary part is zero (as the
 *                           reference does inside lanczos.m:24).
 * The tridiagonal systems (sigma_j I - H) y = beta_0 e1 are solved with
 * Gaussian elimination with partial pivoting specialised to tridiagonal
 * matrices (what MATLAB's sparse backslash does for this structure).
 *
 * Layouts: CSR (rowptr int64, col int32, val double); dense matrices
 * column-major; complex arrays interleaved (re, im).
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;

int cpu_fab_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Y(:, 0..nc-1) = A X(:, 0..nc-1), X and Y n x nc column-major */
static void spmm(long n, const long* rp, const int* ci, const double* va, int nc, const double* X, double* Y) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    for (int c = 0; c < nc; ++c) {
      double s = 0.0;
      for (long t = rp[i]; t < rp[i + 1]; ++t) s += va[t] * X[(long)c * n + ci[t]];
      Y[(long)c * n + i] = s;
    }
  }
}

/* jacobi_poly_eval.m with coefficients (gr, gi) of length d1, input B = [br, bi]
 * (n x nb each), output x = [xr, xi]; work holds 4 n nb doubles. */
static void jacobi_poly_eval(long n, const long* rp, const int* ci, const double* va, int d1, const double* gr,
                             const double* gi, int nb, const double* br, const double* bi, double* xr, double* xi,
                             double* work) {
  double* X2 = work;               /* [xr, xi] stacked, n x 2nb */
  double* AX = work + 2L * n * nb; /* A [xr, xi] */
#pragma omp parallel for schedule(static)
  for (long t = 0; t < n * nb; ++t) {
    xr[t] = br[t] * gr[0] - bi[t] * gi[0];
    xi[t] = br[t] * gi[0] + bi[t] * gr[0];
  }
  for (int i = 1; i < d1; ++i) {
    memcpy(X2, xr, sizeof(double) * n * nb);
    memcpy(X2 + n * nb, xi, sizeof(double) * n * nb);
    spmm(n, rp, ci, va, 2 * nb, X2, AX);
#pragma omp parallel for schedule(static)
    for (long t = 0; t < n * nb; ++t) {
      xr[t] = AX[t] + br[t] * gr[i] - bi[t] * gi[i];
      xi[t] = AX[n * nb + t] + br[t] * gi[i] + bi[t] * gr[i];
    }
  }
}

static double dot(long n, const double* a, const double* b) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (long i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* tridiagonal solve with partial pivoting: sub/super = beta[1..m-1] (real),
 * diagonal = sigma - alpha (the matrix is sigma I - H), rhs = b0 e1. */
static void tri_solve_pivot(int m, const double* alpha, const double* beta, cplx sigma, double b0, cplx* y,
                            cplx* wk) {
  cplx* dl = wk;          /* sub-diagonal */
  cplx* dd = wk + m;      /* diagonal */
  cplx* du = wk + 2 * m;  /* super-diagonal */
  cplx* du2 = wk + 3 * m; /* second super-diagonal after pivoting */
  for (int q = 0; q < m; ++q) {
    dd[q] = sigma - alpha[q];
    dl[q] = q + 1 < m ? -beta[q + 1] : 0.0;
    du[q] = q + 1 < m ? -beta[q + 1] : 0.0;
    du2[q] = 0.0;
    y[q] = 0.0;
  }
  y[0] = b0;
  for (int q = 0; q < m - 1; ++q) {
    if (cabs(dd[q]) >= cabs(dl[q])) {
      cplx f = dl[q] / dd[q];
      dd[q + 1] -= f * du[q];
      y[q + 1] -= f * y[q];
      dl[q] = 0.0;
    } else {
      cplx f = dd[q] / dl[q];
      dd[q] = dl[q];
      cplx t = dd[q + 1];
      dd[q + 1] = du[q] - f * t;
      du[q] = t;
      if (q + 2 < m) {
        du2[q] = du[q + 1];
        du[q + 1] = -f * du2[q];
      }
      cplx ty = y[q];
      y[q] = y[q + 1];
      y[q + 1] = ty - f * y[q + 1];
    }
  }
  y[m - 1] /= dd[m - 1];
  if (m > 1) y[m - 2] = (y[m - 2] - du[m - 2] * y[m - 1]) / dd[m - 2];
  for (int q = m - 3; q >= 0; --q) y[q] = (y[q] - du[q] * y[q + 1] - du2[q] * y[q + 2]) / dd[q];
}

/*
 * f(A) applied to the (already deflated) columns of U (n x R) by the
 * reference CPU algorithm; out (n x R) receives sum_j Im(q_j(A) V y_j).
 * wts: R blocks of C x 2 [re, im]; sigma: C complex (re, im interleaved).
 * Returns 0 on success, -1 on allocation failure.
 */
int cpu_fab(long n, const long* rp, const int* ci, const double* va, int R, const double* U, int m, int d1,
            const double* gamma, int C, const double* gs_re, const double* gs_im, const double* wts,
            const double* sigma, double* out, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  double* V = (double*)malloc(sizeof(double) * (size_t)n * m * R);  /* V_r: n x m */
  double* w = (double*)malloc(sizeof(double) * (size_t)n * R);
  double* vj = (double*)malloc(sizeof(double) * (size_t)n * R);
  double* zi = (double*)calloc((size_t)n * R, sizeof(double));
  double* xr = (double*)malloc(sizeof(double) * (size_t)n * (R > 1 ? R : 1));
  double* xi = (double*)malloc(sizeof(double) * (size_t)n * (R > 1 ? R : 1));
  double* work = (double*)malloc(sizeof(double) * (size_t)n * 8 * (R > 1 ? R : 1));
  double* alpha = (double*)calloc((size_t)(m + 1) * R, sizeof(double));
  double* beta = (double*)calloc((size_t)(m + 1) * R, sizeof(double));
  double* gz = (double*)calloc((size_t)d1, sizeof(double));
  cplx* y = (cplx*)malloc(sizeof(cplx) * (size_t)m * C);
  cplx* wk = (cplx*)malloc(sizeof(cplx) * 4 * (size_t)m);
  double* yre = (double*)malloc(sizeof(double) * (size_t)m);
  double* yim = (double*)malloc(sizeof(double) * (size_t)m);
  double* Br = (double*)malloc(sizeof(double) * (size_t)n);
  double* Bi = (double*)malloc(sizeof(double) * (size_t)n);
  if (!V || !w || !vj || !zi || !xr || !xi || !work || !alpha || !beta || !gz || !y || !wk || !yre || !yim || !Br ||
      !Bi)
    return -1;

  /* lanczos.m:7-19 */
  for (int r = 0; r < R; ++r) {
    const double* a = U + (long)r * n;
    beta[(long)r * (m + 1)] = sqrt(dot(n, a, a));
    const double ib = beta[(long)r * (m + 1)];
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) V[(long)r * n * m + i] = a[i] / ib;
  }
  /* lanczos.m:21-49, all RHS columns together as w = [V1(:,m) V2(:,m)] */
  for (int j = 0; j < m; ++j) {
    for (int r = 0; r < R; ++r) memcpy(vj + (long)r * n, V + (long)r * n * m + (long)j * n, sizeof(double) * n);
    jacobi_poly_eval(n, rp, ci, va, d1, gamma, gz, R, vj, zi, xr, xi, work);
    spmm(n, rp, ci, va, R, xr, w);
    for (int r = 0; r < R; ++r) {
      double* wr = w + (long)r * n;
      const double* vr = vj + (long)r * n;
      if (j != 0) {
        const double b = beta[(long)r * (m + 1) + j];
        const double* vp = V + (long)r * n * m + (long)(j - 1) * n;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) wr[i] -= b * vp[i];
      }
      const double al = dot(n, wr, vr);
      alpha[(long)r * (m + 1) + j] = al;
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) wr[i] -= al * vr[i];
      const double bn = sqrt(dot(n, wr, wr));
      beta[(long)r * (m + 1) + j + 1] = bn;
      if (j < m - 1) {
        double* vn = V + (long)r * n * m + (long)(j + 1) * n;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) vn[i] = wr[i] / bn;
      }
    }
  }
  /* nicksmethodcpu.m:18-43 per RHS */
  for (int r = 0; r < R; ++r) {
    const double* al = alpha + (long)r * (m + 1);
    const double* be = beta + (long)r * (m + 1);
    const double* wr = wts + (long)r * 2 * C;
    for (int j = 0; j < C; ++j) {
      cplx sg = sigma[2 * j] + I * sigma[2 * j + 1];
      tri_solve_pivot(m, al, be, sg, be[0], y + (long)j * m, wk);
      cplx wj = wr[j] + I * wr[C + j];
      for (int q = 0; q < m; ++q) y[(long)j * m + q] *= wj;
    }
    double* o = out + (long)r * n;
    memset(o, 0, sizeof(double) * n);
    const double* Vr = V + (long)r * n * m;
    for (int j = 0; j < C; ++j) {
      for (int q = 0; q < m; ++q) {
        yre[q] = creal(y[(long)j * m + q]);
        yim[q] = cimag(y[(long)j * m + q]);
      }
      /* Y1real = V1*y1real(:,i); Y1imag = V1*y1imag(:,i) */
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) {
        double sr = 0.0, si = 0.0;
        for (int q = 0; q < m; ++q) {
          const double v = Vr[(long)q * n + i];
          sr += v * yre[q];
          si += v * yim[q];
        }
        Br[i] = sr;
        Bi[i] = si;
      }
      jacobi_poly_eval(n, rp, ci, va, d1, gs_re + (long)j * d1, gs_im + (long)j * d1, 1, Br, Bi, xr, xi, work);
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) o[i] += xi[i];
    }
  }
  free(V); free(w); free(vj); free(zi); free(xr); free(xi); free(work); free(alpha); free(beta);
  free(gz); free(y); free(wk); free(yre); free(yim); free(Br); free(Bi);
  return 0;
}
