// The f(A)b engine's persistent kernel.
//
// One cooperative launch runs any contiguous subset of the phases
//   LANCZOS -> TRISOLVE -> COEF -> APPLY -> UPDATE_* -> DEFLATE
// with bounded grid barriers (GridBar) between passes.  The grid is sized so
// that every block is co-resident (cudaLaunchCooperativeKernel checks it).
//
// HBM layout (n rows, R right-hand sides, interleaved so that one gather of
// x[c] fetches all R values of a column with one vector load):
//   A            SELL-32: slice_off[nslices+1] (int64), col/val per slot,
//                slot = slice*32 + lane, slice-column-major (coalesced);
//                optional perm[slot] -> row (sigma-sorted slices)
//   U, Usol, X,
//   update, S    [n][R] FP64
//   V            [m][n][R] BT (FP64, or FP32 in the mixed engine)
//   W0/W1        [n][R] BT   Lanczos work vector (ping-pong between steps)
//   H0/H1        [n][R] HT   Horner / lift ping-pong (FP64 or float-float)
//   P            [d+1][n][R] HT   lifted polynomial terms V c_i
//   aabb         (m+1) x 2R column-major: alpha_r in column r, beta_r in R+r
//   Yr, Yi       m x (R C) column-major (column r*C + j), as the reference
//   coef         [R][d+1][m] FP64, coef_ff the float-float copy
#pragma once
#include "fab_common.cuh"

namespace gm {

enum Phase : int {
  PH_LANCZOS = 1, PH_TRISOLVE = 2, PH_COEF = 4, PH_APPLY = 8,
  PH_UPDATE_FKPP = 16, PH_UPDATE_FHN = 32, PH_DEFLATE = 64,
  PH_APPLY_SET = 128   // apply writes X = lift (fused solve) instead of X += lift
};

struct KParams {
  long long n, nslices;
  int m, d, C, k;
  int phases;
  int G;
  const long long* slice_off;
  const int* col;
  const void* val;
  const int* perm;
  const double* gamma;
  const double* gs_re;
  const double* gs_im;
  const double* wts;
  const double* shifts;
  const double* flam;
  const double* Q;
  const double* mass;
  double dt, aode, bode, code, vrest, vamp, vpeak, c1ion;
  double bd_tol;
  double* U;
  double* Usol;
  double* upd;
  double* X;
  double* S;
  double* ode;
  void* V;
  void* W0;
  void* W1;
  void* H0;
  void* H1;
  void* P;
  double* aabb;
  double* Yr;
  double* Yi;
  double* coef;
  float2* coef_ff;
  double* tri;
  double* Z;
  double* part;     // [2R + k R][G]
  unsigned* bar;    // [0] count, [1] generation
  int* status;
  int* meff;        // [R]
  unsigned long long timeout_ns;
};

// ------------------------------------------------------------------ helpers
struct Ctx {
  int G, b, tid, nt, lane, warp, nw;
  long long gw, tw, gt, tt;
  __device__ Ctx(int G_) {
    G = G_; b = blockIdx.x; tid = threadIdx.x; nt = blockDim.x;
    lane = tid & 31; warp = tid >> 5; nw = nt >> 5;
    gw = (long long)b * nw + warp; tw = (long long)G * nw;
    gt = (long long)b * nt + tid; tt = (long long)G * nt;
  }
};

// Row of SELL slot (slice s, lane); -1 for padding.
__device__ __forceinline__ long long slot_row(const KParams& kp, long long s, int lane) {
  long long slot = s * 32 + lane;
  if (kp.perm) return kp.perm[slot];
  return slot < kp.n ? slot : -1;
}

// acc[r] = sum_j A(row, col_j) x[col_j][r] over the slice row of this lane.
// The slice's columns are walked in chunks of CH: all CH column indices and
// values are loaded first (coalesced, read-only path), then all CH gathers of
// x are issued, then the CH products are accumulated, so each chunk costs two
// memory latencies instead of 2*CH.
template <class Pol, int R, class XT>
__device__ __forceinline__ void spmv_slot(const KParams& kp, long long s, int lane, const XT* __restrict__ x,
                                          typename Pol::AT (&acc)[R]) {
  using VT = typename Pol::VT;
  constexpr int CH = (R == 1) ? 8 : 4;
  const long long base = kp.slice_off[s];
  const int len = (int)((kp.slice_off[s + 1] - base) >> 5);
  const int* cp = kp.col + base + lane;
  const VT* vp = reinterpret_cast<const VT*>(kp.val) + base + lane;
#pragma unroll
  for (int r = 0; r < R; ++r) acc[r] = Pol::zero();
  for (int jj = 0; jj < len; jj += CH) {
    int cc[CH];
    VT aa[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      if (jj + u < len) {
        cc[u] = __ldg(cp + (long long)(jj + u) * 32);
        aa[u] = __ldg(vp + (long long)(jj + u) * 32);
      } else {
        cc[u] = 0;
        aa[u] = (VT)0;
      }
    }
    XT xv[CH][R];
#pragma unroll
    for (int u = 0; u < CH; ++u)
      if (jj + u < len) VecIO<R>::ld(x + (long long)cc[u] * R, xv[u]);
#pragma unroll
    for (int u = 0; u < CH; ++u)
      if (jj + u < len) {
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] = Pol::acc(acc[r], aa[u], xv[u][r]);
      }
  }
}

template <class Pol> __device__ __forceinline__ typename Pol::AT h_load_at(const typename Pol::HT& h);
template <> __device__ __forceinline__ double h_load_at<PolFP64>(const double& h) { return h; }
template <> __device__ __forceinline__ ff h_load_at<PolMixed>(const float2& h) { return {h.x, h.y}; }

// ------------------------------------------------------------------ LANCZOS
// build_subspace.cu:5-89 with the three-term recurrence as two grid passes
// per step (A: SpMV + beta_j v_{j-1} + alpha partials; B: w -= alpha v_j +
// beta partials), plus d Horner passes for the polynomial preconditioner.
// v_{j+1} = w (1/beta_{j+1}) is formed on the fly in the next step's first
// pass, which also stores it in V.
template <class Pol, int R>
__device__ bool phase_lanczos(const KParams& kp, const Ctx& c) {
  using BT = typename Pol::BT;
  using HT = typename Pol::HT;
  using AT = typename Pol::AT;
  using ST = typename Pol::ST;
  const long long n = kp.n;
  const int m = kp.m, d = kp.d, G = kp.G;
  GridBar bar{kp.bar, kp.bar + 1, kp.status, (unsigned)G, kp.timeout_ns};
  BT* V = reinterpret_cast<BT*>(kp.V);
  BT* const W0 = reinterpret_cast<BT*>(kp.W0);
  BT* const W1 = reinterpret_cast<BT*>(kp.W1);
  HT* const H0 = reinterpret_cast<HT*>(kp.H0);
  HT* const H1 = reinterpret_cast<HT*>(kp.H1);
  double* part_a = kp.part;
  double* part_b = kp.part + (long long)R * G;

  // prologue: W1 = U (storage precision), beta_0 = ||U_r||
  {
    double bp[R];
#pragma unroll
    for (int r = 0; r < R; ++r) bp[r] = 0.0;
    for (long long i = c.gt; i < n; i += c.tt) {
      double u[R];
      VecIO<R>::ld(kp.U + i * R, u);
      BT wb[R];
#pragma unroll
      for (int r = 0; r < R; ++r) { bp[r] = fma(u[r], u[r], bp[r]); wb[r] = (BT)u[r]; }
      VecIO<R>::st(W1 + i * R, wb);
    }
    block_sum_store<R>(bp, part_b + c.b, G);
  }
  if (!bar.sync()) return false;
  double beta[R], rbeta[R];
  bool broken[R];
  {
    double tot[R];
    grid_total<R>(part_b, G, tot);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      beta[r] = sqrt(tot[r]);
      broken[r] = !(beta[r] > 0.0);
      rbeta[r] = broken[r] ? 0.0 : 1.0 / beta[r];
    }
    if (c.b == 0 && c.tid == 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        kp.aabb[(long long)(m + 1) * (R + r)] = beta[r];
        kp.meff[r] = broken[r] ? 0 : m;
        if (!(tot[r] == tot[r]) || isinf(tot[r])) atomicCAS(kp.status, 0, (int)ST_NONFINITE);
      }
    }
  }
  const BT* src = W1;
  for (int j = 0; j < m; ++j) {
    BT* Vj = V + (long long)j * n * R;
    const BT* Vjm1 = j > 0 ? V + (long long)(j - 1) * n * R : V;
    BT* Wout = (j & 1) ? W1 : W0;
    ST sc[R], rb[R], bj[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      sc[r] = Pol::scalar(rbeta[r] * kp.gamma[0]);
      rb[r] = Pol::scalar(rbeta[r]);
      bj[r] = Pol::scalar(beta[r]);
    }
    AT apa[R];
#pragma unroll
    for (int r = 0; r < R; ++r) apa[r] = Pol::zero();
    if (d == 0) {
      for (long long s = c.gw; s < kp.nslices; s += c.tw) {
        AT z[R];
        spmv_slot<Pol, R, BT>(kp, s, c.lane, src, z);
        const long long row = slot_row(kp, s, c.lane);
        if (row >= 0) {
          BT sv[R], v[R];
          VecIO<R>::ld(src + row * R, sv);
#pragma unroll
          for (int r = 0; r < R; ++r) v[r] = Pol::scale_to_b(sv[r], rb[r]);
          VecIO<R>::st(Vj + row * R, v);
          AT w[R];
#pragma unroll
          for (int r = 0; r < R; ++r) w[r] = Pol::mul(z[r], sc[r]);
          if (j > 0) {
            BT vp[R];
            VecIO<R>::ld(Vjm1 + row * R, vp);
#pragma unroll
            for (int r = 0; r < R; ++r) w[r] = Pol::sub_mul(w[r], bj[r], vp[r]);
          }
          BT wb[R];
#pragma unroll
          for (int r = 0; r < R; ++r) { wb[r] = Pol::to_b(w[r]); apa[r] = Pol::dot(apa[r], w[r], v[r]); }
          VecIO<R>::st(Wout + row * R, wb);
        }
      }
    } else {
      // Horner pass 1: u = gamma_1 v_j + A (gamma_0 v_j); stores v_j
      {
        ST g1[R];
#pragma unroll
        for (int r = 0; r < R; ++r) g1[r] = Pol::scalar(kp.gamma[1]);
        for (long long s = c.gw; s < kp.nslices; s += c.tw) {
          AT z[R];
          spmv_slot<Pol, R, BT>(kp, s, c.lane, src, z);
          const long long row = slot_row(kp, s, c.lane);
          if (row >= 0) {
            BT sv[R], v[R];
            VecIO<R>::ld(src + row * R, sv);
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = Pol::scale_to_b(sv[r], rb[r]);
            VecIO<R>::st(Vj + row * R, v);
            HT u[R];
#pragma unroll
            for (int r = 0; r < R; ++r) u[r] = Pol::to_h(Pol::add_mul(Pol::mul(z[r], sc[r]), g1[r], v[r]));
            VecIO<R>::st(H1 + row * R, u);
          }
        }
      }
      if (!bar.sync()) return false;
      for (int h = 2; h <= d; ++h) {
        const ST gh = Pol::scalar(kp.gamma[h]);
        const HT* hin = (h & 1) ? H0 : H1;
        HT* hout = (h & 1) ? H1 : H0;
        for (long long s = c.gw; s < kp.nslices; s += c.tw) {
          AT z[R];
          spmv_slot<Pol, R, HT>(kp, s, c.lane, hin, z);
          const long long row = slot_row(kp, s, c.lane);
          if (row >= 0) {
            BT v[R];
            VecIO<R>::ld(Vj + row * R, v);
            HT u[R];
#pragma unroll
            for (int r = 0; r < R; ++r) u[r] = Pol::to_h(Pol::add_mul(z[r], gh, v[r]));
            VecIO<R>::st(hout + row * R, u);
          }
        }
        if (!bar.sync()) return false;
      }
      // final pass: w = A u - beta_j v_{j-1}
      const HT* hin = (d & 1) ? H1 : H0;
      for (long long s = c.gw; s < kp.nslices; s += c.tw) {
        AT z[R];
        spmv_slot<Pol, R, HT>(kp, s, c.lane, hin, z);
        const long long row = slot_row(kp, s, c.lane);
        if (row >= 0) {
          BT v[R];
          VecIO<R>::ld(Vj + row * R, v);
          AT w[R];
#pragma unroll
          for (int r = 0; r < R; ++r) w[r] = z[r];
          if (j > 0) {
            BT vp[R];
            VecIO<R>::ld(Vjm1 + row * R, vp);
#pragma unroll
            for (int r = 0; r < R; ++r) w[r] = Pol::sub_mul(w[r], bj[r], vp[r]);
          }
          BT wb[R];
#pragma unroll
          for (int r = 0; r < R; ++r) { wb[r] = Pol::to_b(w[r]); apa[r] = Pol::dot(apa[r], w[r], v[r]); }
          VecIO<R>::st(Wout + row * R, wb);
        }
      }
    }
    double ap[R];
#pragma unroll
    for (int r = 0; r < R; ++r) ap[r] = Pol::to_d(apa[r]);
    block_sum_store<R>(ap, part_a + c.b, G);
    if (!bar.sync()) return false;
    double alpha[R];
    grid_total<R>(part_a, G, alpha);
    // pass B: w -= alpha_j v_j; beta_{j+1} = ||w||
    double bp[R];
    {
      ST al[R];
      AT bpa[R];
#pragma unroll
      for (int r = 0; r < R; ++r) { al[r] = Pol::scalar(alpha[r]); bpa[r] = Pol::zero(); }
      for (long long i = c.gt; i < n; i += c.tt) {
        BT wb[R], v[R];
        VecIO<R>::ld(Wout + i * R, wb);
        VecIO<R>::ld(Vj + i * R, v);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          AT w = Pol::sub_mul(Pol::from_b(wb[r]), al[r], v[r]);
          wb[r] = Pol::to_b(w);
          bpa[r] = Pol::dot_self(bpa[r], w);
        }
        VecIO<R>::st(Wout + i * R, wb);
      }
#pragma unroll
      for (int r = 0; r < R; ++r) bp[r] = Pol::to_d(bpa[r]);
    }
    block_sum_store<R>(bp, part_b + c.b, G);
    if (!bar.sync()) return false;
    double tot[R];
    grid_total<R>(part_b, G, tot);
    bool all_broken = true;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const double bn = sqrt(tot[r]);
      if (c.b == 0 && c.tid == 0) {
        kp.aabb[j + (long long)(m + 1) * r] = broken[r] ? 0.0 : alpha[r];
        kp.aabb[(j + 1) + (long long)(m + 1) * (R + r)] = broken[r] ? 0.0 : bn;
        if (!(bn == bn) || isinf(bn) || !(alpha[r] == alpha[r])) atomicCAS(kp.status, 0, (int)ST_NONFINITE);
      }
      const double scale = fabs(alpha[r]) + (j > 0 ? beta[r] : 0.0);
      if (!broken[r] && j + 1 < m && !(bn > kp.bd_tol * scale)) {
        broken[r] = true;
        if (c.b == 0 && c.tid == 0) kp.meff[r] = j + 1;
      }
      beta[r] = broken[r] ? 0.0 : bn;
      rbeta[r] = broken[r] ? 0.0 : 1.0 / bn;
      all_broken = all_broken && broken[r];
    }
    src = Wout;
    if (all_broken) break;
  }
  return true;
}

// ------------------------------------------------------------------ solves
// copyforsolve + linsyssolve + copyafter (lanczos_impl.cu:292-406,
// lin_sys_solves.cu:8-19): system (r, j) has diagonal alpha_r - shift,
// off-diagonals beta_r[1..meff-1] and right-hand side -beta0_r w_{r,j} e1.
// Because the right-hand side is a multiple of e1, the solution needs no
// back substitution of a general right-hand side: with the bottom-up Schur
// complements g_q = (alpha_q - s_q) - beta_{q+1}^2 / g_{q+1}, the solution is
// y_0 = rhs / g_0 and y_q = -beta_q y_{q-1} / g_q.  One warp per system (lane
// 0; the recurrence is serial), complex FP64, one real division per step; the
// reciprocals 1/g_q are kept in the tri scratch for the top-down sweep.
template <int R>
__device__ void phase_trisolve(const KParams& kp, const Ctx& c) {
  const int m = kp.m, C = kp.C;
  if (c.lane != 0) return;
  for (long long sys = c.gw; sys < (long long)R * C; sys += c.tw) {
    const int r = (int)(sys / C), j = (int)(sys % C);
    const int me = kp.meff[r];
    const double* __restrict__ al = kp.aabb + (long long)(m + 1) * r;
    const double* __restrict__ be = kp.aabb + (long long)(m + 1) * (R + r);
    const double* __restrict__ sh = kp.shifts + 2LL * m * sys;
    double* __restrict__ ig = kp.tri + 4LL * m * sys;  // 1/g_q (re, im)
    double* __restrict__ yr = kp.Yr + (long long)m * sys;
    double* __restrict__ yi = kp.Yi + (long long)m * sys;
    const double b0 = be[0];
    const double wr = kp.wts[2LL * C * r + j], wi = kp.wts[2LL * C * r + C + j];
    double igr = 0.0, igi = 0.0;   // 1/g_{q+1}
    for (int q = me - 1; q >= 0; --q) {
      const double b2 = q + 1 < me ? be[q + 1] * be[q + 1] : 0.0;
      const double gr = (al[q] - sh[2 * q]) - b2 * igr;
      const double gi = -sh[2 * q + 1] - b2 * igi;
      const double inv = 1.0 / (gr * gr + gi * gi);
      igr = gr * inv;
      igi = -gi * inv;
      ig[2 * q] = igr;
      ig[2 * q + 1] = igi;
    }
    // y_0 = rhs * (1/g_0), rhs = -(beta0 w)
    double y_r = 0.0, y_i = 0.0;
    if (me > 0) {
      const double xr = -(b0 * wr), xi = -(b0 * wi);
      y_r = xr * ig[0] - xi * ig[1];
      y_i = xr * ig[1] + xi * ig[0];
      yr[0] = y_r;
      yi[0] = y_i;
    }
    for (int q = 1; q < me; ++q) {
      const double tr = -be[q] * y_r, ti = -be[q] * y_i;
      const double gr = ig[2 * q], gi = ig[2 * q + 1];
      y_r = tr * gr - ti * gi;
      y_i = tr * gi + ti * gr;
      yr[q] = y_r;
      yi[q] = y_i;
    }
    for (int q = me; q < m; ++q) { yr[q] = 0.0; yi[q] = 0.0; }
  }
}

// coef[r][i][q] = sum_j Im(gs(i, j) y_{r, j}[q]) = sum_j gs_re y_im + gs_im y_re:
// the m-vectors that collapse apply_V.cu's 2C per-node passes into one lift.
template <int R>
__device__ void phase_coef(const KParams& kp, const Ctx& c) {
  const int m = kp.m, C = kp.C, d1 = kp.d + 1;
  const long long total = (long long)R * d1 * m;
  for (long long t = c.gt; t < total; t += c.tt) {
    const int q = (int)(t % m);
    const int i = (int)((t / m) % d1);
    const int r = (int)(t / ((long long)m * d1));
    double acc = 0.0;
    for (int j = 0; j < C; ++j) {
      const long long col = (long long)r * C + j;
      acc = fma(kp.gs_re[i + (long long)d1 * j], kp.Yi[col * m + q], acc);
      acc = fma(kp.gs_im[i + (long long)d1 * j], kp.Yr[col * m + q], acc);
    }
    kp.coef[t] = acc;
    const float h = (float)acc;
    kp.coef_ff[t] = make_float2(h, (float)(acc - (double)h));
  }
}

// ------------------------------------------------------------------ APPLY
// X_r += sum_i A^(d-i) V_r c_{r,i}: one lift pass P_i = V c_i (V read once),
// then d Horner passes X = A X + P_i.
template <class Pol, int R>
__device__ bool phase_apply(const KParams& kp, const Ctx& c, bool overwrite) {
  using BT = typename Pol::BT;
  using HT = typename Pol::HT;
  using AT = typename Pol::AT;
  const long long n = kp.n;
  const int m = kp.m, d = kp.d, d1 = d + 1;
  GridBar bar{kp.bar, kp.bar + 1, kp.status, (unsigned)kp.G, kp.timeout_ns};
  const BT* V = reinterpret_cast<const BT*>(kp.V);
  HT* P = reinterpret_cast<HT*>(kp.P);
  HT* const H0 = reinterpret_cast<HT*>(kp.H0);
  HT* const H1 = reinterpret_cast<HT*>(kp.H1);
  constexpr int IC = 3;
  for (long long i = c.gt; i < n; i += c.tt) {
    for (int i0 = 0; i0 < d1; i0 += IC) {
      AT acc[IC][R];
#pragma unroll
      for (int ii = 0; ii < IC; ++ii)
#pragma unroll
        for (int r = 0; r < R; ++r) acc[ii][r] = Pol::zero();
      for (int q = 0; q < m; ++q) {
        BT v[R];
        VecIO<R>::ld(V + ((long long)q * n + i) * R, v);
#pragma unroll
        for (int ii = 0; ii < IC; ++ii) {
          if (i0 + ii < d1) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
              const long long ci = ((long long)r * d1 + i0 + ii) * m + q;
              if constexpr (Pol::kMixed) {
                const float2 cf = kp.coef_ff[ci];
                acc[ii][r] = Pol::add(acc[ii][r], ff_mulf(ff{cf.x, cf.y}, v[r]));
              } else {
                acc[ii][r] = fma((double)v[r], kp.coef[ci], acc[ii][r]);
              }
            }
          }
        }
      }
      if (d == 0) {
        double x[R], u[R], s[R];
        if (overwrite) {
#pragma unroll
          for (int r = 0; r < R; ++r) x[r] = 0.0;
        } else {
          VecIO<R>::ld(kp.X + i * R, x);
        }
        VecIO<R>::ld(kp.upd + i * R, u);
#pragma unroll
        for (int r = 0; r < R; ++r) { x[r] += Pol::to_d(acc[0][r]); s[r] = x[r] + u[r]; }
        VecIO<R>::st(kp.X + i * R, x);
        VecIO<R>::st(kp.S + i * R, s);
      } else {
#pragma unroll
        for (int ii = 0; ii < IC; ++ii) {
          if (i0 + ii < d1) {
            HT hv[R];
#pragma unroll
            for (int r = 0; r < R; ++r) hv[r] = Pol::to_h(acc[ii][r]);
            VecIO<R>::st(P + ((long long)(i0 + ii) * n + i) * R, hv);
          }
        }
      }
    }
  }
  if (d == 0) return true;
  if (!bar.sync()) return false;
  for (int h = 1; h <= d; ++h) {
    const HT* hin = h == 1 ? P : ((h & 1) ? H0 : H1);
    HT* hout = (h & 1) ? H1 : H0;
    const HT* Ph = P + (long long)h * n * R;
    for (long long s = c.gw; s < kp.nslices; s += c.tw) {
      AT z[R];
      spmv_slot<Pol, R, HT>(kp, s, c.lane, hin, z);
      const long long row = slot_row(kp, s, c.lane);
      if (row >= 0) {
        HT p[R];
        VecIO<R>::ld(Ph + row * R, p);
        AT x[R];
#pragma unroll
        for (int r = 0; r < R; ++r) x[r] = Pol::add(z[r], h_load_at<Pol>(p[r]));
        if (h < d) {
          HT hv[R];
#pragma unroll
          for (int r = 0; r < R; ++r) hv[r] = Pol::to_h(x[r]);
          VecIO<R>::st(hout + row * R, hv);
        } else {
          double xo[R], u[R], so[R];
          if (overwrite) {
#pragma unroll
            for (int r = 0; r < R; ++r) xo[r] = 0.0;
          } else {
            VecIO<R>::ld(kp.X + row * R, xo);
          }
          VecIO<R>::ld(kp.upd + row * R, u);
#pragma unroll
          for (int r = 0; r < R; ++r) { xo[r] += Pol::to_d(x[r]); so[r] = xo[r] + u[r]; }
          VecIO<R>::st(kp.X + row * R, xo);
          VecIO<R>::st(kp.S + row * R, so);
        }
      }
    }
    if (h < d && !bar.sync()) return false;
  }
  return true;
}

// ------------------------------------------------------------------ UPDATE + DEFLATE
// Pass 1 (optional time step, update_U.cu:8-16 / update_U_monodomain.cu:8-22)
// then Z = Q^T Usol; pass 2: U = Usol - Q Z, update = Q (flam o Z), X = 0
// (lanczos_impl.cu:84-89, update_U.cu:26-38).
template <int R>
__device__ bool phase_deflate(const KParams& kp, const Ctx& c, int mode) {
  const long long n = kp.n;
  const int k = kp.k, G = kp.G;
  GridBar bar{kp.bar, kp.bar + 1, kp.status, (unsigned)G, kp.timeout_ns};
  double* part_z = kp.part + 2LL * R * G;
  constexpr int KC = 4;
  if (mode != 0 && R == 2) {
    for (long long i = c.gt; i < n; i += c.tt) {
      const double* x = kp.X + i * 2;
      const double* up = kp.upd + i * 2;
      double u = ((x[0] + x[1]) + up[0]) + up[1];
      double g;
      if (mode == 1) {
        u = u * (double)(u >= 0.0);
        const double uo = u / kp.mass[i];
        g = kp.mass[i] * uo * (1.0 - uo);
        g = g * kp.dt;
      } else {
        const double p1 = u * (kp.dt * kp.aode);
        const double p2 = kp.ode[i] * (kp.dt * kp.bode);
        const double o = kp.ode[i] + ((p1 + p2) + kp.code);
        kp.ode[i] = o;
        double srcv = ((u - kp.vrest) * u) * (u - kp.vpeak);
        srcv = srcv * ((kp.c1ion / kp.vamp) / kp.vamp);
        g = (srcv - o) * kp.dt;
      }
      kp.Usol[i * 2] = u;
      kp.Usol[i * 2 + 1] = g;
    }
  }
  if (k > 0) {
    for (int e0 = 0; e0 < k; e0 += KC) {
      double zp[KC * R];
#pragma unroll
      for (int t = 0; t < KC * R; ++t) zp[t] = 0.0;
      for (long long i = c.gt; i < n; i += c.tt) {
        double u[R];
        VecIO<R>::ld(kp.Usol + i * R, u);
#pragma unroll
        for (int ee = 0; ee < KC; ++ee) {
          if (e0 + ee < k) {
            const double q = kp.Q[(long long)(e0 + ee) * n + i];
#pragma unroll
            for (int r = 0; r < R; ++r) zp[ee * R + r] = fma(q, u[r], zp[ee * R + r]);
          }
        }
      }
      block_sum_store<KC * R>(zp, part_z + (long long)e0 * R * G + c.b, G);
    }
    if (!bar.sync()) return false;
    // every block totals the k*R entries in the same fixed order
    __shared__ double s_z[256];
    const int kr = k * R;
    for (int t0 = 0; t0 < kr; t0 += 256) {
      for (int t = t0 + c.tid; t < kr && t < t0 + 256; t += c.nt) {
        double acc = 0.0;
        const double* p = part_z + (long long)t * G;
        for (int b = 0; b < G; ++b) acc += p[b];
        s_z[t - t0] = acc;
        if (c.b == 0) kp.Z[t] = acc;
      }
      __syncthreads();
      // pass 2 over this chunk of Z entries (rows by thread stride)
      const int e_lo = t0 / R, e_hi = min(k, (t0 + 256) / R);
      for (long long i = c.gt; i < n; i += c.tt) {
        double u[R], up[R];
        if (t0 == 0) {
          VecIO<R>::ld(kp.Usol + i * R, u);
#pragma unroll
          for (int r = 0; r < R; ++r) up[r] = 0.0;
        } else {
          VecIO<R>::ld(kp.U + i * R, u);
          VecIO<R>::ld(kp.upd + i * R, up);
        }
        double qz[R];
#pragma unroll
        for (int r = 0; r < R; ++r) qz[r] = 0.0;
        for (int e = e_lo; e < e_hi; ++e) {
          const double q = kp.Q[(long long)e * n + i];
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const double z = s_z[e * R + r - t0];
            qz[r] = fma(q, z, qz[r]);
            up[r] = fma(q, kp.flam[e + (long long)k * r] * z, up[r]);
          }
        }
        double x0[R];
#pragma unroll
        for (int r = 0; r < R; ++r) { u[r] = u[r] - qz[r]; x0[r] = 0.0; }
        VecIO<R>::st(kp.U + i * R, u);
        VecIO<R>::st(kp.upd + i * R, up);
        VecIO<R>::st(kp.X + i * R, x0);
      }
      __syncthreads();
    }
  } else {
    for (long long i = c.gt; i < n; i += c.tt) {
      double u[R], z0[R];
      VecIO<R>::ld(kp.Usol + i * R, u);
#pragma unroll
      for (int r = 0; r < R; ++r) z0[r] = 0.0;
      VecIO<R>::st(kp.U + i * R, u);
      VecIO<R>::st(kp.upd + i * R, z0);
      VecIO<R>::st(kp.X + i * R, z0);
    }
  }
  return true;
}

// ------------------------------------------------------------------ kernel
// PH is the compile-time set of phases this entry point can run (the runtime
// mask kp.phases selects among them); specialising on it lets the compiler
// size registers per phase group.
template <class Pol, int R, int PH>
__global__ void __launch_bounds__(512, (R >= 4 ? 1 : 2)) fab_kernel(KParams kp) {
  const Ctx c(kp.G);
  GridBar bar{kp.bar, kp.bar + 1, kp.status, (unsigned)kp.G, kp.timeout_ns};
  if (*(volatile int*)kp.status != 0) return;
  const int ph = kp.phases & PH;
  bool first = true;
  auto sep = [&]() -> bool {
    if (first) { first = false; return true; }
    return bar.sync();
  };
  if ((PH & PH_LANCZOS) && (ph & PH_LANCZOS)) {
    if (!sep()) return;
    if (!phase_lanczos<Pol, R>(kp, c)) return;
  }
  if ((PH & PH_TRISOLVE) && (ph & PH_TRISOLVE)) {
    if (!sep()) return;
    phase_trisolve<R>(kp, c);
  }
  if ((PH & PH_COEF) && (ph & PH_COEF)) {
    if (!sep()) return;
    phase_coef<R>(kp, c);
  }
  if ((PH & PH_APPLY) && (ph & PH_APPLY)) {
    if (!sep()) return;
    if (!phase_apply<Pol, R>(kp, c, (ph & PH_APPLY_SET) != 0)) return;
  }
  if (PH & (PH_DEFLATE | PH_UPDATE_FKPP | PH_UPDATE_FHN)) {
    const int upd_mode = (ph & PH_UPDATE_FKPP) ? 1 : ((ph & PH_UPDATE_FHN) ? 2 : 0);
    if ((ph & PH_DEFLATE) || upd_mode) {
      if (!sep()) return;
      if (!phase_deflate<R>(kp, c, upd_mode)) return;
    }
  }
}

// Phase groups compiled as separate entry points.
constexpr int KG_LANCZOS = PH_LANCZOS;
constexpr int KG_SOLVE = PH_TRISOLVE | PH_COEF;
constexpr int KG_APPLY = PH_APPLY | PH_APPLY_SET;
constexpr int KG_DEFLATE = PH_DEFLATE | PH_UPDATE_FKPP | PH_UPDATE_FHN;

}  // namespace gm
