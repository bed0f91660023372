// Finite-element operator assembly and the adjoint (gradient) kernels.
//
// Operator: A(kappa) = M^{-1/2} K(kappa) M^{-1/2} on the interior nodes of a
// P1 mesh, K(kappa) = sum_e kappa_e K_e with K_e the unit-coefficient element
// stiffness (process_nonuniform.m:90-91 forms the same symmetric scaling).
//
// Adjoint of L = 1/2 ||f(A) b - d||^2 (g = f(A) b - d), from the contour form
// f(A) = Im sum_j w_j (xi_j - A)^{-1} (Frechet derivative of the resolvent):
//   dL/db       = f(A) g
//   dL/dkappa_e = Im sum_j w_j s_j^T (dA/dkappa_e) r_j,
//   r_j = (xi_j - A)^{-1} b,  s_j = (xi_j - A)^{-1} g.
// With the polynomial preconditioner p, B = A p(A), sigma_j = xi_j p(xi_j) and
// q_j(x) = (sigma_j - x p(x)) / (xi_j - x) = sum_i gs(i, j) x^(d-i):
//   (xi_j - A)^{-1} = q_j(A) (sigma_j - B)^{-1},
// and the engine's shifted solves give V y_j = w_j (sigma_j - B)^{-1} u for
// right-hand side u.  Hence
//   dL/dkappa_e = Im sum_j S_j^T dA_e R_j,
//   R_j = q_j(A) V_b (y_b,j / w_j),  S_j = q_j(A) V_g y_g,j,
// evaluated as one lift Z = V y per side (n x C complex) and d Horner steps
// X <- A X + gs(i, j) Z.  dA_e is local to the triangle's three nodes:
// (dA_e)_{ac} = msi_a K_e[a][c] msi_c.
#pragma once
#include "fab_kernel.cuh"

namespace gm {

// value of every stored entry of A from kappa, in a fixed order (no atomics):
// val[slot[t]] = 2^-se sum_{p in ent_ptr[t]..} kappa[ent_tri[p]] * ent_coef[p]
template <class VT>
__global__ void k_fe_assemble(long long nnz, const long long* __restrict__ ent_ptr, const int* __restrict__ ent_tri,
                              const double* __restrict__ ent_coef, const double* __restrict__ kappa,
                              const int* __restrict__ slot, VT* __restrict__ val, int se) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nnz) return;
  double acc = 0.0;
  for (long long p = ent_ptr[t]; p < ent_ptr[t + 1]; ++p) acc = fma(kappa[ent_tri[p]], ent_coef[p], acc);
  val[slot[t]] = (VT)ldexp(acc, -se);
}

// Mixed engine: values of one row of A(kappa) in FP32 (stored as A 2^-se) and
// the row's diagonal compensation c_r = sum_t (a_t - fl32(a_t)) w_col / w_r,
// the same correction the engine computes at create (one thread per row,
// fixed order).
__global__ void k_fe_assemble_rows(long long n, const long long* __restrict__ ptr, const int* __restrict__ col,
                                   const long long* __restrict__ ent_ptr, const int* __restrict__ ent_tri,
                                   const double* __restrict__ ent_coef, const double* __restrict__ kappa,
                                   const int* __restrict__ slot, float* __restrict__ val, int se,
                                   const double* __restrict__ w, const int* __restrict__ row2slot,
                                   float* __restrict__ dlo) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double corr = 0.0;
  for (long long t = ptr[r]; t < ptr[r + 1]; ++t) {
    double acc = 0.0;
    for (long long p = ent_ptr[t]; p < ent_ptr[t + 1]; ++p) acc = fma(kappa[ent_tri[p]], ent_coef[p], acc);
    const double exact = ldexp(acc, -se);
    const int st = slot[t];
    const float v = (float)exact;
    val[st] = v;
    corr += (exact - (double)v) * w[col[st]];
  }
  dlo[row2slot[r]] = (float)(corr / w[r]);
}

// The same lift in float-float arithmetic on the FP32 pipe (GB300's FP64
// pipe issues about 1/64 of its FP32 rate).  Each V element is split into
// hi + lo floats once and each coefficient is kept split in shared memory;
// products are exact (two_prod) with the cross terms added, sums compensated:
// about 48 significant bits, against m-term sums of order 1e3 terms.
__device__ __forceinline__ ff ff_madd(ff acc, float ah, float al, float bh, float bl) {
  ff p = two_prod(ah, bh);
  p.lo = fmaf(ah, bl, fmaf(al, bh, p.lo));
  ff s = two_sum(acc.hi, p.hi);
  const float e = s.lo + (acc.lo + p.lo);
  return fast_two_sum(s.hi, e);
}

template <class BT>
__global__ void __launch_bounds__(256) k_fe_lift_ff(long long n, int m, int C, const BT* __restrict__ Vb,
                                                    const BT* __restrict__ Vg, int vstride,
                                                    const double2* __restrict__ yb, const double2* __restrict__ yg,
                                                    double2* __restrict__ Rout, double2* __restrict__ Sout,
                                                    const int* __restrict__ meff_b, const int* __restrict__ meff_g) {
  // Zb[i][j] = sum_q Vb(q, i) yb'[j][q], Zg[i][j] = sum_q Vg(q, i) yg[j][q];
  // V element (q, i) of a side at V[(q n + i) vstride] (the b and g bases are
  // columns of one interleaved basis, or two separate bases).  One row per
  // thread; shifts in chunks of JC, coefficients in tiles of QT Krylov
  // vectors held split in shared memory.
  constexpr int JC = 8, QT = 128;
  __shared__ float4 sy4[2 * JC * QT];  // [side][jj][q]: (re hi, re lo, im hi, im lo)
  const int mb = min(*meff_b, m), mg = min(*meff_g, m);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = (long long)blockIdx.x * blockDim.x; i0 < n; i0 += stride) {   // block-uniform
    const long long i = i0 + threadIdx.x;
    const bool act = i < n;
    for (int j0 = 0; j0 < C; j0 += JC) {
      ff rr[JC], ri[JC], sr[JC], si[JC];
#pragma unroll
      for (int jj = 0; jj < JC; ++jj) rr[jj] = ri[jj] = sr[jj] = si[jj] = ff{0.f, 0.f};
      for (int q0 = 0; q0 < m; q0 += QT) {
        const int qn = min(QT, m - q0);
        __syncthreads();
        for (int t = threadIdx.x; t < 2 * JC * QT; t += blockDim.x) {
          const int side = t / (JC * QT), rest = t % (JC * QT), jj = rest / QT, q = rest % QT;
          const int j = j0 + jj;
          const double2* src = side ? yg : yb;
          const double2 y = (j < C && q < qn) ? src[(long long)j * m + q0 + q] : make_double2(0.0, 0.0);
          const float rh = (float)y.x, ih = (float)y.y;
          sy4[t] = make_float4(rh, (float)(y.x - (double)rh), ih, (float)(y.y - (double)ih));
        }
        __syncthreads();
        if (!act) continue;
        for (int q = 0; q < qn; ++q) {
          const int qq = q0 + q;
          float bh = 0.f, bl = 0.f, gh = 0.f, gl = 0.f;
          if (qq < mb) {
            const BT v = Vb[((long long)qq * n + i) * vstride];
            bh = (float)v;
            bl = (float)(v - (BT)bh);
          }
          if (qq < mg) {
            const BT v = Vg[((long long)qq * n + i) * vstride];
            gh = (float)v;
            gl = (float)(v - (BT)gh);
          }
#pragma unroll
          for (int jj = 0; jj < JC; ++jj) {
            const float4 b = sy4[jj * QT + q];
            const float4 g = sy4[JC * QT + jj * QT + q];
            rr[jj] = ff_madd(rr[jj], bh, bl, b.x, b.y);
            ri[jj] = ff_madd(ri[jj], bh, bl, b.z, b.w);
            sr[jj] = ff_madd(sr[jj], gh, gl, g.x, g.y);
            si[jj] = ff_madd(si[jj], gh, gl, g.z, g.w);
          }
        }
      }
      if (act) {
#pragma unroll
        for (int jj = 0; jj < JC; ++jj) {
          if (j0 + jj < C) {
            Rout[i * C + j0 + jj] = make_double2(ff_to_double(rr[jj]), ff_to_double(ri[jj]));
            Sout[i * C + j0 + jj] = make_double2(ff_to_double(sr[jj]), ff_to_double(si[jj]));
          }
        }
      }
    }
  }
}

// Xout[r][j] = sum_k A[r][k] Xin[k][j] + gs(i, j) Z[r][j] for both sides
// (first step: gs(0, j) Z[r][j] only).  One warp per row, lanes over the
// shifts j, so every stored entry of the row reads one contiguous
// C-vector of X.  A's entries are read through the CSR-entry -> slot map.
template <class VT>
__global__ void k_fe_horner(long long n, int C, int d1, int i, const long long* __restrict__ ptr,
                            const int* __restrict__ c2s, const int* __restrict__ col, const VT* __restrict__ val,
                            const double* __restrict__ gs_re, const double* __restrict__ gs_im,
                            const double2* __restrict__ Zb, const double2* __restrict__ Zg,
                            const double2* __restrict__ Xb, const double2* __restrict__ Xg,
                            double2* __restrict__ Yb, double2* __restrict__ Yg, int first) {
  const int lane = threadIdx.x & 31;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long r = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += nwarps) {
    for (int j = lane; j < C; j += 32) {
      double2 ab = make_double2(0.0, 0.0), ag = make_double2(0.0, 0.0);
      if (!first) {
        for (long long t = ptr[r]; t < ptr[r + 1]; ++t) {
          const int s = c2s[t];
          const long long k = col[s];
          const double v = (double)val[s];
          const double2 xb = Xb[k * C + j], xg = Xg[k * C + j];
          ab.x = fma(v, xb.x, ab.x);
          ab.y = fma(v, xb.y, ab.y);
          ag.x = fma(v, xg.x, ag.x);
          ag.y = fma(v, xg.y, ag.y);
        }
      }
      const double gr = gs_re[i + (long long)d1 * j], gi = gs_im[i + (long long)d1 * j];
      const double2 zb = Zb[r * C + j], zg = Zg[r * C + j];
      ab.x += gr * zb.x - gi * zb.y;
      ab.y += gr * zb.y + gi * zb.x;
      ag.x += gr * zg.x - gi * zg.y;
      ag.y += gr * zg.y + gi * zg.x;
      Yb[r * C + j] = ab;
      Yg[r * C + j] = ag;
    }
  }
}

// dkappa[e] = Im sum_j sum_{a,c} S[n_a][j] Kc_e[a][c] R[n_c][j]  (one thread
// per triangle; boundary nodes (index -1) contribute nothing)
__global__ void k_fe_grad(long long ntri, int C, const long long* __restrict__ nodes, const double* __restrict__ kc,
                          const double2* __restrict__ R, const double2* __restrict__ S, double* __restrict__ dk) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ntri) return;
  long long nd[3];
  double K[9];
#pragma unroll
  for (int a = 0; a < 3; ++a) nd[a] = nodes[e * 3 + a];
#pragma unroll
  for (int t = 0; t < 9; ++t) K[t] = kc[e * 9 + t];
  double acc = 0.0;
  for (int j = 0; j < C; ++j) {
    double2 r[3], s[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      r[a] = nd[a] >= 0 ? R[nd[a] * C + j] : make_double2(0.0, 0.0);
      s[a] = nd[a] >= 0 ? S[nd[a] * C + j] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      double tr = 0.0, ti = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        tr = fma(K[a * 3 + c], r[c].x, tr);
        ti = fma(K[a * 3 + c], r[c].y, ti);
      }
      acc = fma(s[a].x, ti, fma(s[a].y, tr, acc));  // Im(s_a * t_a)
    }
  }
  dk[e] = acc;
}

}  // namespace gm
