// gm_deflation_pairs: the k smallest eigenpairs of a symmetric matrix on the
// GPU, for the deflation vectors of the f(A)b engine.
//
// The reference computes them on the host with MATLAB's eigs(K, M, k, 'sm')
// (process_nonuniform.m:38-40, 106-110): shift-invert Arnoldi, which needs a
// sparse factorisation.  On the GPU the method is Chebyshev-filtered subspace
// iteration (Y. Zhou, Y. Saad, M. L. Tiago, J. R. Chelikowsky, "Self-consistent-
// field calculations using Chebyshev-filtered subspace iteration", J. Comput.
// Phys. 219 (2006), with the scaled three-term filter of their Algorithm 4.1)
// over a block of 32 vectors, all in FP64:
//
//   X <- C_deg(A) X        Chebyshev polynomial of degree deg on the unwanted
//                          interval [a, b] (a = the block's largest Ritz value,
//                          b = Gershgorin bound of A), scaled so that the
//                          block's lowest Ritz value a0 stays O(1)
//   X <- X R^{-1}          CholQR, twice (G = X^T X = R^T R)
//   H = X^T A X, H = W diag(theta) W^T  (Rayleigh-Ritz; cyclic Jacobi in one warp)
//   X <- X W, residuals ||A x_j - theta_j x_j|| / |theta_j| for the k wanted
//
// until every wanted relative residual is below tol.  The degree is chosen
// per iteration so that the filter amplifies a0 over a by at most 1e4 (a
// bounded condition number for CholQR) and is capped by max_degree.
//
// Layout: block vectors [n][32] row-major (one row of the block is 256
// contiguous bytes), so lane j of a warp owns column j: the SpMM gathers
// X[c][0..31] as one coalesced 256-byte row per stored entry, and every
// 32 x 32 product (Gram matrices, X W) is a per-row multiply with the small
// matrix in shared memory.  The matrix is CSR (int64 row pointer, int32
// column indices, FP64 values), one warp per row.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/gpumatfun.h"
#include "fab_common.cuh"

namespace gm {
void set_global_error(const char* msg);  // engine.cu: the text gm_last_error(NULL) returns
}  // namespace gm

namespace {

constexpr int P = 32;            // block width: one column per lane
constexpr double kCondCap = 1e4;  // largest amplification of a0 over a per filter
constexpr double kFFUntil = 1e-7; // float-float filter while the wanted residuals are above this

int eig_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  gm::set_global_error(buf);
  return code;
}

// Y_out = c1 (A X) + c2 X + c3 Y_prev, lane = column, one warp per row.
// A row has few stored entries, so the kernel waits on the dependent chain
// of memory accesses (row pointer, then column indices and values, then the
// gathered rows of X).  The chain is shortened: the next row's pointers are
// loaded while the current row is processed, and the epilogue's X and Y_prev
// rows are loaded before the gathers.  Entries are taken 8 at a time, their
// gathers all in flight before the products.
__global__ void k_cheb(long long n, const long long* __restrict__ rp, const int* __restrict__ ci,
                       const double* __restrict__ va, const double* __restrict__ X,
                       const double* __restrict__ Yp, double* __restrict__ Yo, double c1, double c2, double c3) {
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  long long b = r < n ? rp[r] : 0, e = r < n ? rp[r + 1] : 0;
  for (; r < n; r += nw) {
    const long long rn = r + nw;
    const long long bn = rn < n ? rp[rn] : 0, en = rn < n ? rp[rn + 1] : 0;
    const double xo = c2 != 0.0 ? X[r * P + lane] : 0.0;
    const double yo = c3 != 0.0 ? Yp[r * P + lane] : 0.0;
    double acc = 0.0;
    for (long long t = b; t < e; t += 8) {
      double av[8], xv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        av[q] = 0.0;
        xv[q] = 0.0;
        if (t + q < e) {
          av[q] = __ldg(va + t + q);
          xv[q] = __ldg(X + (long long)__ldg(ci + t + q) * P + lane);
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) acc = fma(av[q], xv[q], acc);
    }
    Yo[r * P + lane] = fma(c3, yo, fma(c2, xo, c1 * acc));
    b = bn;
    e = en;
  }
}

// The same three-term step in float-float arithmetic on the FP32 pipe
// (about 48 significant bits): values split as hi + lo floats, block vectors
// as (hi, lo) pairs.  Each product is hi*hi exactly (two_prod) plus the two
// cross terms; the row sum keeps its hi part by two_sum and collects every
// rounding error in lo, renormalised once per row.  About 12 FP32
// instructions per product instead of one FP64 FMA on GB300's narrow FP64
// pipe.  Memory access order as in k_cheb.
__global__ void k_cheb_ff(long long n, const long long* __restrict__ rp, const int* __restrict__ ci,
                          const float* __restrict__ vhi, const float* __restrict__ vlo,
                          const float2* __restrict__ X, const float2* __restrict__ Yp, float2* __restrict__ Yo,
                          float2 c1, float2 c2, float2 c3) {
  using gm::ff;
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const float2 z = make_float2(0.f, 0.f);
  long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  long long b = r < n ? rp[r] : 0, e = r < n ? rp[r + 1] : 0;
  for (; r < n; r += nw) {
    const long long rn = r + nw;
    const long long bn = rn < n ? rp[rn] : 0, en = rn < n ? rp[rn + 1] : 0;
    const float2 xo = c2.x != 0.f ? X[r * P + lane] : z;
    const float2 yo = c3.x != 0.f ? Yp[r * P + lane] : z;
    float ahi = 0.f, alo = 0.f;
    for (long long t = b; t < e; t += 8) {
      float2 av[8], xv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        av[q] = z;
        xv[q] = z;
        if (t + q < e) {
          av[q] = make_float2(__ldg(vhi + t + q), __ldg(vlo + t + q));
          xv[q] = __ldg(X + (long long)__ldg(ci + t + q) * P + lane);
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const ff p = gm::two_prod(av[q].x, xv[q].x);
        const float cross = fmaf(av[q].x, xv[q].y, av[q].y * xv[q].x);
        const ff s2 = gm::two_sum(ahi, p.hi);
        ahi = s2.hi;
        alo += s2.lo + (p.lo + cross);
      }
    }
    ff y = gm::ff_mul(gm::fast_two_sum(ahi, alo), ff{c1.x, c1.y});
    if (c2.x != 0.f) y = gm::ff_add(y, gm::ff_mul(ff{xo.x, xo.y}, ff{c2.x, c2.y}));
    if (c3.x != 0.f) y = gm::ff_add(y, gm::ff_mul(ff{yo.x, yo.y}, ff{c3.x, c3.y}));
    Yo[r * P + lane] = make_float2(y.hi, y.lo);
    b = bn;
    e = en;
  }
}

// FP64 block <-> float-float block (hi = fl32(x), lo = fl32(x - hi))
__global__ void k_d2ff(long long count, const double* __restrict__ x, float2* __restrict__ y) {
  const long long nt = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += nt) {
    const float h = (float)x[t];
    y[t] = make_float2(h, (float)(x[t] - (double)h));
  }
}
__global__ void k_ff2d(long long count, const float2* __restrict__ x, double* __restrict__ y) {
  const long long nt = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += nt)
    y[t] = (double)x[t].x + (double)x[t].y;
}

// partial[blk][i * 32 + j] = sum over the block's rows of Y[r][i] Z[r][j]
// (1024 threads: thread (i, j); tiles of 32 rows staged in shared memory).
__global__ void __launch_bounds__(1024) k_gram(long long n, long long rows_per_block, const double* __restrict__ Y,
                                               const double* __restrict__ Z, double* __restrict__ partial) {
  __shared__ double sy[32][P + 1];
  __shared__ double sz[32][P + 1];
  const int t = threadIdx.x, i = t >> 5, j = t & 31;
  const long long r0 = (long long)blockIdx.x * rows_per_block;
  const long long r1 = r0 + rows_per_block < n ? r0 + rows_per_block : n;
  double acc = 0.0;
  for (long long rt = r0; rt < r1; rt += 32) {
    const long long r = rt + i;
    sy[i][j] = r < r1 ? Y[r * P + j] : 0.0;
    sz[i][j] = r < r1 ? Z[r * P + j] : 0.0;
    __syncthreads();
#pragma unroll 8
    for (int q = 0; q < 32; ++q) acc = fma(sy[q][i], sz[q][j], acc);
    __syncthreads();
  }
  partial[(long long)blockIdx.x * (P * P) + t] = acc;
}

// out[t] = sum over the G blocks of partial[b][t], in block order (deterministic).
__global__ void k_gram_sum(const double* __restrict__ partial, int G, double* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P * P) return;
  double s = 0.0;
  for (int b = 0; b < G; ++b) s += partial[(long long)b * (P * P) + t];
  out[t] = s;
}

// Out[r][j] = sum_i Y[r][i] M[i][j] (M 32 x 32 row-major; Out may not alias Y).
__global__ void k_rowmul(long long n, const double* __restrict__ Y, const double* __restrict__ M,
                         double* __restrict__ Out) {
  __shared__ double sm[P * P];
  for (int t = threadIdx.x; t < P * P; t += blockDim.x) sm[t] = M[t];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += nw) {
    const double y = Y[r * P + lane];
    double acc = 0.0;
#pragma unroll
    for (int i = 0; i < P; ++i) acc = fma(__shfl_sync(0xffffffffu, y, i), sm[i * P + lane], acc);
    Out[r * P + lane] = acc;
  }
}

// R[r][j] = AX[r][j] - theta[j] X[r][j]
__global__ void k_resid(long long n, const double* __restrict__ AX, const double* __restrict__ X,
                        const double* __restrict__ theta, double* __restrict__ Rr) {
  const long long nt = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n * P; t += nt)
    Rr[t] = AX[t] - theta[t & (P - 1)] * X[t];
}

// Seeded start block: splitmix64 of (seed, index) mapped to [-1, 1).
__global__ void k_random(long long n, unsigned long long seed, double* __restrict__ X) {
  const long long nt = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n * P; t += nt) {
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(t + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    X[t] = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  }
}

// Q[j][r] (column-major n x k) = X[r][j]
__global__ void k_take_cols(long long n, int k, const double* __restrict__ X, double* __restrict__ Q) {
  const long long nt = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n * k; t += nt) {
    const long long j = t / n, r = t - j * n;
    Q[t] = X[r * P + j];
  }
}

// One warp: G = L L^T (Cholesky, L lower), then M = L^{-T} (so that X M has
// orthonormal columns).  status[0] = 1 when G is not numerically positive
// definite (a pivot at or below 1e-14 of the largest diagonal entry).
__global__ void k_chol_inv(const double* __restrict__ Gin, double* __restrict__ M, int* __restrict__ status) {
  __shared__ double L[P][P + 1];
  __shared__ double Li[P][P + 1];
  __shared__ int bad;
  const int lane = threadIdx.x;
  for (int i = 0; i < P; ++i) L[i][lane] = Gin[i * P + lane];
  if (lane == 0) bad = 0;
  __syncwarp();
  double dmax = 0.0;
  for (int i = 0; i < P; ++i) dmax = fmax(dmax, L[i][i]);
  for (int k = 0; k < P; ++k) {
    if (lane == 0) {
      const double d = L[k][k];
      if (!(d > 1e-14 * dmax)) bad = 1;
      L[k][k] = sqrt(fmax(d, 1e-300));
    }
    __syncwarp();
    if (lane > k) L[lane][k] /= L[k][k];
    __syncwarp();
    for (int j = k + 1; j < P; ++j)
      if (lane >= j) L[lane][j] -= L[lane][k] * L[j][k];
    __syncwarp();
  }
  // column `lane` of L^{-1} by forward substitution
  for (int i = 0; i < P; ++i) {
    double s = i == lane ? 1.0 : 0.0;
    for (int t = 0; t < i; ++t) s -= L[i][t] * Li[t][lane];
    Li[i][lane] = i >= lane ? s / L[i][i] : 0.0;
    __syncwarp();
  }
  // M[i][j] = (L^{-1})[j][i]
  for (int i = 0; i < P; ++i) M[i * P + lane] = Li[lane][i];
  if (lane == 0) status[0] = bad;
}

// One warp: eigendecomposition of the symmetric 32 x 32 H by cyclic Jacobi
// rotations (G. H. Golub, C. F. Van Loan, Matrix Computations, 4th ed.,
// Algorithm 8.5.2 and 8.5.3), FP64.  theta ascending, W[i][j] = component i
// of eigenvector j.
__global__ void k_jacobi(const double* __restrict__ Hin, double* __restrict__ theta, double* __restrict__ W) {
  __shared__ double H[P][P + 1];
  __shared__ double V[P][P + 1];
  __shared__ double cs[2];
  __shared__ int order[P];
  const int lane = threadIdx.x;
  for (int i = 0; i < P; ++i) {
    H[i][lane] = 0.5 * (Hin[i * P + lane] + Hin[lane * P + i]);
    V[i][lane] = i == lane ? 1.0 : 0.0;
  }
  __syncwarp();
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < P; ++i) {
      const double h = H[i][lane];
      tot += h * h;
      if (i != lane) off += h * h;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if (off <= 1e-30 * tot) break;
    for (int p = 0; p < P - 1; ++p)
      for (int q = p + 1; q < P; ++q) {
        if (lane == 0) {
          const double apq = H[p][q];
          double c = 1.0, s = 0.0;
          if (apq != 0.0) {
            const double tau = (H[q][q] - H[p][p]) / (2.0 * apq);
            const double t = tau >= 0.0 ? 1.0 / (tau + sqrt(1.0 + tau * tau)) : -1.0 / (-tau + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
          cs[0] = c;
          cs[1] = s;
        }
        __syncwarp();
        const double c = cs[0], s = cs[1];
        if (s != 0.0) {
          // H <- J^T H J and V <- V J, J the rotation in the (p, q) plane
          double a = H[lane][p], b = H[lane][q];
          H[lane][p] = c * a - s * b;
          H[lane][q] = s * a + c * b;
          __syncwarp();
          a = H[p][lane];
          b = H[q][lane];
          H[p][lane] = c * a - s * b;
          H[q][lane] = s * a + c * b;
          a = V[lane][p];
          b = V[lane][q];
          V[lane][p] = c * a - s * b;
          V[lane][q] = s * a + c * b;
          __syncwarp();
          if (lane == 0) H[p][q] = H[q][p] = 0.0;
        }
        __syncwarp();
      }
  }
  if (lane == 0) {
    for (int i = 0; i < P; ++i) order[i] = i;
    for (int i = 0; i < P; ++i)
      for (int j = i + 1; j < P; ++j)
        if (H[order[j]][order[j]] < H[order[i]][order[i]]) {
          const int t = order[i];
          order[i] = order[j];
          order[j] = t;
        }
  }
  __syncwarp();
  theta[lane] = H[order[lane]][order[lane]];
  for (int i = 0; i < P; ++i) W[i * P + lane] = V[i][order[lane]];
}

struct Solver {
  long long n = 0, nnz = 0;
  int nsm = 0, G = 0;
  long long rows_per_block = 0;
  long long* rp = nullptr;
  int* ci = nullptr;
  double* va = nullptr;
  float* vhi = nullptr;     // float-float split of the values (float-float filter)
  float* vlo = nullptr;
  unsigned grid64 = 0, grid_ff = 0;   // resident 256-thread blocks of k_cheb / k_cheb_ff
  double* buf[6] = {};      // block vectors [n][32]
  double* part = nullptr;   // Gram partials [G][1024]
  double* small = nullptr;  // [0] G/H 1024, [1024] M/W 1024, [2048] theta 32
  int* status = nullptr;
  long long spmm = 0, spmm_ff = 0;
  std::string err;

  ~Solver() {
    cudaFree(rp);
    cudaFree(ci);
    cudaFree(va);
    cudaFree(vhi);
    cudaFree(vlo);
    for (double* b : buf) cudaFree(b);
    cudaFree(part);
    cudaFree(small);
    cudaFree(status);
  }

  unsigned grid_rows() const { return (unsigned)std::max(1, nsm * 8); }   // 256-thread blocks, a warp per row

  cudaError_t spmm_axpby(const double* X, const double* Yp, double* Yo, double c1, double c2, double c3) {
    k_cheb<<<grid64, 256>>>(n, rp, ci, va, X, Yp, Yo, c1, c2, c3);
    ++spmm;
    return cudaGetLastError();
  }

  static float2 to_ff(double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
  }

  cudaError_t spmm_axpby_ff(const float2* X, const float2* Yp, float2* Yo, double c1, double c2, double c3) {
    k_cheb_ff<<<grid_ff, 256>>>(n, rp, ci, vhi, vlo, X, Yp, Yo, to_ff(c1), to_ff(c2), to_ff(c3));
    ++spmm;
    ++spmm_ff;
    return cudaGetLastError();
  }

  // small[0..1024) = Y^T Z
  cudaError_t gram(const double* Y, const double* Z) {
    k_gram<<<G, 1024>>>(n, rows_per_block, Y, Z, part);
    k_gram_sum<<<(P * P + 255) / 256, 256>>>(part, G, small);
    return cudaGetLastError();
  }

  // X <- X R^{-1} twice (CholQR2) through tmp; returns 1 when G was not
  // positive definite, negative on a CUDA error
  int cholqr2(double* X, double* tmp) {
    for (int pass = 0; pass < 2; ++pass) {
      if (gram(X, X) != cudaSuccess) return -1;
      k_chol_inv<<<1, 32>>>(small, small + P * P, status);
      int bad = 0;
      if (cudaMemcpy(&bad, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
      if (bad) return 1;
      k_rowmul<<<grid_rows(), 256>>>(n, X, small + P * P, tmp);
      if (cudaMemcpy(X, tmp, (size_t)n * P * sizeof(double), cudaMemcpyDeviceToDevice) != cudaSuccess) return -1;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
  }
};

}  // namespace

extern "C" int gm_deflation_pairs(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, int k,
                                  double tol, int max_degree, int max_iter, uint64_t seed, double* lambda, double* Q,
                                  double* stats) {
  // a negative max_degree selects the FP64 filter throughout (|max_degree| is the cap)
  const bool use_ff_arg = max_degree >= 0;
  max_degree = max_degree < 0 ? -max_degree : max_degree;
  gm::set_global_error("");
  if (n < 2 * P) return eig_fail(GM_ERR_ARG, "deflation_pairs: n must be at least %d", 2 * P);
  if (k < 1 || k > P - 8) return eig_fail(GM_ERR_ARG, "deflation_pairs: k must be in [1, %d]", P - 8);
  if (!rowptr || !col || !val || !lambda || !Q) return eig_fail(GM_ERR_ARG, "deflation_pairs: null pointer");
  if (!(tol > 0.0) || max_degree < 4 || max_iter < 1)
    return eig_fail(GM_ERR_ARG, "deflation_pairs: need tol > 0, max_degree >= 4, max_iter >= 1");
  // Host copy of the row pointer (host or device memory): nnz and the
  // Gershgorin bound need it.
  std::vector<int64_t> hrp(n + 1);
  cudaError_t st = cudaMemcpy(hrp.data(), rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyDefault);
  if (st != cudaSuccess) return eig_fail(GM_ERR_CUDA, "deflation_pairs: row pointer copy: %s", cudaGetErrorString(st));
  if (hrp[0] != 0) return eig_fail(GM_ERR_ARG, "deflation_pairs: rowptr[0] must be 0");
  for (long long i = 0; i < n; ++i)
    if (hrp[i + 1] < hrp[i]) return eig_fail(GM_ERR_ARG, "deflation_pairs: rowptr must be non-decreasing");
  const long long nnz = hrp[n];
  std::vector<int32_t> hci(nnz);
  std::vector<double> hva(nnz);
  if ((st = cudaMemcpy(hci.data(), col, sizeof(int32_t) * nnz, cudaMemcpyDefault)) != cudaSuccess ||
      (st = cudaMemcpy(hva.data(), val, sizeof(double) * nnz, cudaMemcpyDefault)) != cudaSuccess)
    return eig_fail(GM_ERR_CUDA, "deflation_pairs: matrix copy: %s", cudaGetErrorString(st));
  double b = 0.0, vmin = HUGE_VAL;
  for (long long i = 0; i < n; ++i) {
    double s = 0.0;
    for (long long t = hrp[i]; t < hrp[i + 1]; ++t) {
      if (hci[t] < 0 || hci[t] >= n) return eig_fail(GM_ERR_ARG, "deflation_pairs: column index out of range");
      if (!std::isfinite(hva[t])) return eig_fail(GM_ERR_ARG, "deflation_pairs: non-finite matrix value");
      s += std::fabs(hva[t]);
      if (hva[t] != 0.0) vmin = std::min(vmin, std::fabs(hva[t]));
    }
    b = std::max(b, s);
  }
  if (!(b > 0.0)) return eig_fail(GM_ERR_ARG, "deflation_pairs: zero matrix");

  Solver S;
  S.n = n;
  S.nnz = nnz;
  int dev = 0;
  if ((st = cudaGetDevice(&dev)) != cudaSuccess ||
      (st = cudaDeviceGetAttribute(&S.nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return eig_fail(GM_ERR_CUDA, "deflation_pairs: %s", cudaGetErrorString(st));
  S.G = std::max(1, std::min<int>(2 * S.nsm, (int)((n + 31) / 32)));
  S.rows_per_block = (n + S.G - 1) / S.G;
  auto alloc = [&](void** p, size_t bytes) { return cudaMalloc(p, std::max<size_t>(bytes, 8)); };
  const size_t vbytes = (size_t)n * P * sizeof(double);
  bool ok = alloc((void**)&S.rp, sizeof(long long) * (n + 1)) == cudaSuccess &&
            alloc((void**)&S.ci, sizeof(int) * nnz) == cudaSuccess &&
            alloc((void**)&S.va, sizeof(double) * nnz) == cudaSuccess &&
            alloc((void**)&S.part, sizeof(double) * (size_t)S.G * P * P) == cudaSuccess &&
            alloc((void**)&S.small, sizeof(double) * (2 * P * P + P)) == cudaSuccess &&
            alloc((void**)&S.status, sizeof(int)) == cudaSuccess;
  for (int i = 0; i < 6 && ok; ++i) ok = alloc((void**)&S.buf[i], vbytes) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    return eig_fail(GM_ERR_OOM, "deflation_pairs: device allocation of %.1f GB failed", (6.0 * vbytes + 12.0 * nnz) / 1e9);
  }
  {
    std::vector<float> hi(nnz), lo(nnz);
    for (long long t = 0; t < nnz; ++t) {
      hi[t] = (float)hva[t];
      lo[t] = (float)(hva[t] - (double)hi[t]);
    }
    if (alloc((void**)&S.vhi, sizeof(float) * nnz) != cudaSuccess || alloc((void**)&S.vlo, sizeof(float) * nnz) != cudaSuccess) {
      cudaGetLastError();
      return eig_fail(GM_ERR_OOM, "deflation_pairs: device allocation failed");
    }
    if ((st = cudaMemcpy(S.vhi, hi.data(), sizeof(float) * nnz, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (st = cudaMemcpy(S.vlo, lo.data(), sizeof(float) * nnz, cudaMemcpyHostToDevice)) != cudaSuccess)
      return eig_fail(GM_ERR_CUDA, "deflation_pairs: upload: %s", cudaGetErrorString(st));
  }
  {
    // grids of resident blocks only (grid-stride loops over the rows)
    int nb64 = 0, nbff = 0;
    if ((st = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb64, k_cheb, 256, 0)) != cudaSuccess ||
        (st = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbff, k_cheb_ff, 256, 0)) != cudaSuccess)
      return eig_fail(GM_ERR_CUDA, "deflation_pairs: occupancy: %s", cudaGetErrorString(st));
    S.grid64 = (unsigned)std::max(1, nb64 * S.nsm);
    S.grid_ff = (unsigned)std::max(1, nbff * S.nsm);
  }
  if ((st = cudaMemcpy(S.rp, hrp.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (st = cudaMemcpy(S.ci, hci.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (st = cudaMemcpy(S.va, hva.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice)) != cudaSuccess)
    return eig_fail(GM_ERR_CUDA, "deflation_pairs: upload: %s", cudaGetErrorString(st));

  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0);
  double* X = S.buf[0];   // current block (orthonormal after each iteration)
  double* AX = S.buf[1];
  double* Y = S.buf[2];   // filter ping-pong
  double* Yp = S.buf[3];
  double* Yn = S.buf[4];
  double* T = S.buf[5];   // scratch
  const unsigned ge = (unsigned)std::max(1, S.nsm * 8);
  // float-float filter only where the values and the filter's intermediates
  // stay well inside FP32's exponent range
  bool use_ff = use_ff_arg && b < 1e30 && vmin > 1e-30;
  double theta[P] = {};
  double res[P] = {};
  int iters = 0, rc = GM_OK;
  double a = 0.0, maxres = 0.0;

  // Rayleigh-Ritz of the orthonormal block Y: X = Y W, AX = (A Y) W, theta,
  // and the wanted relative residuals
  auto rayleigh_ritz = [&](double* Yb) -> int {
    if (S.spmm_axpby(Yb, nullptr, T, 1.0, 0.0, 0.0) != cudaSuccess) return -1;
    if (S.gram(Yb, T) != cudaSuccess) return -1;
    k_jacobi<<<1, 32>>>(S.small, S.small + 2 * P * P, S.small + P * P);
    k_rowmul<<<S.grid_rows(), 256>>>(n, Yb, S.small + P * P, X);
    k_rowmul<<<S.grid_rows(), 256>>>(n, T, S.small + P * P, AX);
    k_resid<<<ge, 256>>>(n, AX, X, S.small + 2 * P * P, T);
    if (cudaMemcpy(theta, S.small + 2 * P * P, sizeof(theta), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    if (S.gram(T, T) != cudaSuccess) return -1;
    std::vector<double> g(P * P);
    if (cudaMemcpy(g.data(), S.small, sizeof(double) * P * P, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    maxres = 0.0;
    for (int j = 0; j < P; ++j) {
      res[j] = std::sqrt(std::max(g[j * P + j], 0.0)) / std::max(std::fabs(theta[j]), 1e-300);
      if (j < k) maxres = std::max(maxres, res[j]);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
  };

  k_random<<<ge, 256>>>(n, seed, Y);
  int q = S.cholqr2(Y, T);
  if (q == 0) q = rayleigh_ritz(Y);
  if (q != 0) rc = q < 0 ? eig_fail(GM_ERR_CUDA, "deflation_pairs: %s", cudaGetErrorString(cudaGetLastError()))
                         : eig_fail(GM_ERR_BREAKDOWN, "deflation_pairs: the start block is rank deficient");
  for (; rc == GM_OK && iters < max_iter && !(maxres <= tol); ++iters) {
    a = theta[P - 1];
    const double a0 = theta[0];
    if (!(a < b) || !(a0 < a)) {
      rc = eig_fail(GM_ERR_BREAKDOWN, "deflation_pairs: Ritz values [%g, %g] outside the filter bound %g", a0, a, b);
      break;
    }
    const double e = 0.5 * (b - a), c = 0.5 * (b + a);
    const double rate = std::acosh((c - a0) / e);
    const int deg = (int)std::min<double>(max_degree, std::max(4.0, std::ceil(std::log(kCondCap) / rate)));
    // scaled Chebyshev filter (Zhou, Saad, Tiago, Chelikowsky, Algorithm 4.1).
    // While the wanted residuals are far above kFFUntil it runs in float-float
    // (about 48 bits, on the FP32 pipe); its rounding floors the reachable
    // residual near 1e-7 on an operator with kappa ~ 1e7, so the last
    // iterations, and every Rayleigh-Ritz step, are FP64.
    double sig = e / (a0 - c);
    const double tau = 2.0 / sig;
    const bool ff_now = use_ff && maxres > kFFUntil;
    double* Yf = nullptr;   // the filtered block, FP64
    if (ff_now) {
      float2* pf = reinterpret_cast<float2*>(S.buf[3]);
      float2* yf = reinterpret_cast<float2*>(S.buf[2]);
      float2* nf = reinterpret_cast<float2*>(S.buf[4]);
      k_d2ff<<<ge, 256>>>(n * P, X, pf);
      if (S.spmm_axpby_ff(pf, nullptr, yf, sig / e, -c * sig / e, 0.0) != cudaSuccess) rc = GM_ERR_CUDA;
      for (int i = 2; i <= deg && rc == GM_OK; ++i) {
        const double sig2 = 1.0 / (tau - sig);
        if (S.spmm_axpby_ff(yf, pf, nf, 2.0 * sig2 / e, -2.0 * c * sig2 / e, -sig * sig2) != cudaSuccess)
          rc = GM_ERR_CUDA;
        float2* old = pf;
        pf = yf;
        yf = nf;
        nf = old;
        sig = sig2;
      }
      Yf = yf == reinterpret_cast<float2*>(S.buf[2]) ? S.buf[3] : S.buf[2];
      k_ff2d<<<ge, 256>>>(n * P, yf, Yf);
    } else {
      if (S.spmm_axpby(X, nullptr, Y, sig / e, -c * sig / e, 0.0) != cudaSuccess) rc = GM_ERR_CUDA;
      double* prev = X;
      for (int i = 2; i <= deg && rc == GM_OK; ++i) {
        const double sig2 = 1.0 / (tau - sig);
        if (S.spmm_axpby(Y, prev, Yn, 2.0 * sig2 / e, -2.0 * c * sig2 / e, -sig * sig2) != cudaSuccess)
          rc = GM_ERR_CUDA;
        // rotate: prev <- Y, Y <- Yn (X is kept untouched after the first step)
        double* old = prev == X ? Yp : prev;
        prev = Y;
        Y = Yn;
        Yn = old;
        sig = sig2;
      }
      Yf = Y;
    }
    if (rc != GM_OK) {
      rc = eig_fail(GM_ERR_CUDA, "deflation_pairs: filter launch: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    const double res_before = maxres;
    q = S.cholqr2(Yf, T);
    if (q == 0) q = rayleigh_ritz(Yf);
    // a float-float iteration that no longer halves the residual has met its floor
    if (q == 0 && ff_now && maxres < 1e-3 && maxres > 0.5 * res_before) use_ff = false;
    if (q != 0) {
      rc = q < 0 ? eig_fail(GM_ERR_CUDA, "deflation_pairs: %s", cudaGetErrorString(cudaGetLastError()))
                 : eig_fail(GM_ERR_BREAKDOWN, "deflation_pairs: filtered block rank deficient (degree %d)", deg);
      break;
    }
    // buffers: X and AX hold the new block; Y, Yp, Yn are free again
    Yp = S.buf[3];
    Y = S.buf[2];
    Yn = S.buf[4];
  }
  cudaEventRecord(t1);
  cudaEventSynchronize(t1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (rc == GM_OK) {
    k_take_cols<<<ge, 256>>>(n, k, X, T);
    if ((st = cudaMemcpy(Q, T, sizeof(double) * (size_t)n * k, cudaMemcpyDefault)) != cudaSuccess)
      return eig_fail(GM_ERR_CUDA, "deflation_pairs: output copy: %s", cudaGetErrorString(st));
    if ((st = cudaMemcpy(lambda, theta, sizeof(double) * k, cudaMemcpyDefault)) != cudaSuccess)
      return eig_fail(GM_ERR_CUDA, "deflation_pairs: output copy: %s", cudaGetErrorString(st));
    if (!(maxres <= tol))
      rc = eig_fail(GM_ERR_NOCONV, "deflation_pairs: %d iterations reached relative residual %.3e > tol %.3e", iters,
                    maxres, tol);
  }
  if (stats) {
    stats[0] = iters;
    stats[1] = (double)S.spmm;
    stats[2] = ms * 1e-3;
    stats[3] = maxres;
    stats[4] = b;
    stats[5] = a;
    stats[6] = theta[P - 1];
    stats[7] = (double)nnz;
    stats[8] = (double)S.spmm_ff;
  }
  return rc;
}
