// Host side of the f(A)b engine: argument checks, CSC/CSR -> SELL-32
// conversion, device allocation, cooperative launches and the C ABI declared
// in include/gpumatfun.h.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/gpumatfun.h"
#include "fab_kernel.cuh"
#include "fe_kernels.cuh"

using gm::KParams;

namespace gm {
void* kernel_fp64(int R, int group);
void* kernel_mixed(int R, int group);
void* kernel_mixed_l2(int group);
}  // namespace gm

namespace {

thread_local std::string g_create_error;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct gm_engine {
  int dev = 0, nsm = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  long long n = 0, nnz = 0, nslices = 0, padded = 0;
  int R = 0, m = 0, d = 0, C = 0, k = 0, prec = 0, sync_mode = 1, nprob = 1;
  int threads = 512, G = 0;
  int scale_exp = 0;             // mixed engine: A stored as A * 2^-scale_exp
  unsigned long long epoch = 0;  // launch counter (progress-flag epochs)
  double dep_avg = 0.0;          // mean neighbour-list length per block
  int Gk[9] = {};                // grid size per phase group (co-residency bound)
  void* kfn[9] = {};
  size_t smem[9] = {};           // dynamic shared memory per phase group
  std::vector<DevBuf> bufs;
  size_t bytes = 0;
  KParams kp{};
  double* stage = nullptr;       // n*R column-major staging for host transfers
  double* col_scale = nullptr;   // device, R
  int* h_status = nullptr;       // pinned: [0] status, [1..R] meff
  cudaEvent_t ev[5][2] = {};
  bool ev_used[5] = {};
  bool have_y = false, have_coef = false, have_V = false;
  bool capturing = false;        // launches are being recorded into a CUDA graph
  int* csr2sell = nullptr;       // device: SELL slot of every stored entry (kept on request)
  void* mat_base = nullptr;      // SELL values + column indices (one allocation)
  size_t mat_bytes = 0;
  bool l2_window = false;        // launches carry an L2 persisting window over the matrix
  cudaAccessPolicyWindow window = {};
  bool keep_map = false;
  bool mpk_req = false;          // matrix-powers passes requested
  long long mpk_nmax = 0;        // largest own + halo rows of a block
  std::vector<int> sell_col_host;  // SELL column indices kept for the halo build
  std::vector<double> roww;      // mixed engine: weights of the diagonal compensation (empty = ones)
  bool comp = false;             // mixed engine: diagonal compensation on
  int* row2slot = nullptr;       // device, kept with the entry map: row -> 32 * slice + lane
  double* d_roww = nullptr;      // device weights (kept with the entry map, mixed)
  // finite-element structure for gm_fe_assemble / gm_fe_gradient
  long long fe_ntri = 0;
  long long* fe_ent_ptr = nullptr;
  int* fe_ent_tri = nullptr;
  double* fe_ent_coef = nullptr;
  long long* fe_nodes = nullptr;
  double* fe_kc = nullptr;
  double2* fe_buf[6] = {};
  double* fe_kappa = nullptr;    // kappa copied in by gm_fe_forward / gm_fe_backward
  // nrhs = 1 adjoint engines keep two Krylov states: slot 0 for b (the
  // forward solve, kept for the backward call), slot 1 for g
  struct FeSlot { void* V; double* Yr; double* Yi; double* aabb; int* meff; };
  FeSlot fe_slot[2] = {};
  int fe_cur = 0;
  bool fe_fwd_ok = false;        // slot 0 holds the basis of the last gm_fe_forward
  double* fe_dk = nullptr;       // dL/dkappa before it is copied out
  long long* csr_ptr = nullptr;  // device CSR row pointer (kept with csr2sell)
  double2* fe_yb = nullptr;
  double2* fe_yg = nullptr;
  cudaGraphExec_t loop_exec = nullptr;
  int loop_steps = -1, loop_mode = -1;
  long long launches = 0;
  std::string err;
};

namespace {

int fail(gm_engine* e, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (e) e->err = buf; else g_create_error = buf;
  return code;
}

int cuda_fail(gm_engine* e, cudaError_t st, const char* what) {
  return fail(e, GM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(st));
}

#define GM_CUDA(e, call)                                   \
  do {                                                     \
    cudaError_t _st = (call);                              \
    if (_st != cudaSuccess) return cuda_fail((e), _st, #call); \
  } while (0)

template <class T>
int dalloc(gm_engine* e, T** p, size_t count) {
  size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  void* q = nullptr;
  cudaError_t st = cudaMalloc(&q, bytes);
  if (st != cudaSuccess) {
    cudaGetLastError();
    return fail(e, GM_ERR_OOM, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(st));
  }
  e->bufs.push_back({q, bytes});
  e->bytes += bytes;
  *p = reinterpret_cast<T*>(q);
  return GM_OK;
}

template <class T>
int dupload(gm_engine* e, T** p, const T* host, size_t count) {
  int rc = dalloc(e, p, count);
  if (rc) return rc;
  if (count) GM_CUDA(e, cudaMemcpy(*p, host, count * sizeof(T), cudaMemcpyHostToDevice));
  return GM_OK;
}

// ------------------------------------------------------------------ helper kernels
__global__ void k_pack_in(const double* __restrict__ cm, double* __restrict__ il, long long n, int R,
                          const double* __restrict__ scale) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * R) return;
  const long long i = t / R;
  const int r = (int)(t % R);
  il[t] = scale ? cm[(long long)r * n + i] * scale[r] : cm[(long long)r * n + i];
}

__global__ void k_pack_out(const double* __restrict__ il, double* __restrict__ cm, long long n, int R) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * R) return;
  const long long i = t / R;
  const int r = (int)(t % R);
  cm[(long long)r * n + i] = il[t];
}

// ------------------------------------------------------------------ sparse conversion
struct Csr {
  std::vector<long long> ptr;
  std::vector<int> col;
  std::vector<double> val;
};

// One problem's matrix as given (CSC as MATLAB stores it, or CSR) -> CSR.
struct ProbIn {
  long long n, nnz_hint;
  int format;
  const long long* ptr;
  const long long* ind;
  const double* values;
  const double* U;
  const double* gamma;
  const double* gs_re;
  const double* gs_im;
  const double* wts;
  const double* shifts;
};

int make_csr(gm_engine* e, const ProbIn& a, Csr& out) {
  const long long n = a.n;
  const long long* ptr = a.ptr;
  const long long* ind = a.ind;
  if (ptr[0] != 0) return fail(e, GM_ERR_ARG, "lanczos_create:inputNotSparse: pointer array must start at 0");
  for (long long i = 0; i < n; ++i)
    if (ptr[i + 1] < ptr[i]) return fail(e, GM_ERR_ARG, "lanczos_create:inputNotSparse: pointer array not monotone at %lld", i);
  const long long nnz = ptr[n];
  if (a.nnz_hint && a.nnz_hint < nnz) return fail(e, GM_ERR_ARG, "lanczos_create:inputNotSparse: nnz %lld < ptr[n] %lld", a.nnz_hint, nnz);
  if (nnz > 2147483647LL) return fail(e, GM_ERR_UNSUPPORTED, "more than 2^31-1 stored entries");
  for (long long t = 0; t < nnz; ++t)
    if (ind[t] < 0 || ind[t] >= n) return fail(e, GM_ERR_ARG, "lanczos_create:inputNotSparse: index %lld out of range at %lld", (long long)ind[t], t);
  out.ptr.assign(n + 1, 0);
  out.col.resize(nnz);
  out.val.resize(nnz);
  if (a.format == GM_CSR) {
    for (long long i = 0; i <= n; ++i) out.ptr[i] = ptr[i];
    for (long long t = 0; t < nnz; ++t) { out.col[t] = (int)ind[t]; out.val[t] = a.values[t]; }
  } else {
    // CSC of A -> CSR of A (counting sort by row).  The reference uploads the
    // CSC arrays as the CSR of A^T and multiplies with the transpose flag
    // (cusparse_wrapper.cpp:33-46,60-62); the product is the same A x.
    std::vector<long long> cnt(n + 1, 0);
    for (long long t = 0; t < nnz; ++t) cnt[ind[t] + 1]++;
    for (long long i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    out.ptr = cnt;
    std::vector<long long> pos(cnt.begin(), cnt.end() - 1);
    for (long long j = 0; j < n; ++j)
      for (long long t = ptr[j]; t < ptr[j + 1]; ++t) {
        const long long p = pos[ind[t]]++;
        out.col[p] = (int)j;
        out.val[p] = a.values[t];
      }
  }
  return GM_OK;
}

// Appends B (rows and columns shifted by row0) to the block-diagonal A.
void append_block(Csr& A, const Csr& B, long long row0) {
  const long long base = A.ptr.empty() ? 0 : A.ptr.back();
  if (A.ptr.empty()) A.ptr.push_back(0);
  for (size_t i = 1; i < B.ptr.size(); ++i) A.ptr.push_back(base + B.ptr[i]);
  for (int c : B.col) A.col.push_back((int)(c + row0));
  A.val.insert(A.val.end(), B.val.begin(), B.val.end());
}

// SELL-32 over the block-diagonal matrix: every problem starts on a new
// slice, so a slice never mixes problems (pad slots map to row -1).
template <class VT>
int upload_sell(gm_engine* e, const Csr& A, int sigma, int scale_exp, const std::vector<long long>& prow0,
                std::vector<long long>& rows, std::vector<long long>& off, std::vector<long long>& pslice0) {
  const int np = (int)prow0.size() - 1;
  // The mixed engine's diagonal compensation reads x_r from the first gather
  // of a row, so with compensation every row stores its diagonal entry first
  // (an explicit zero one where the matrix has none).
  const bool diag_first = sizeof(VT) == 4 && e->comp;
  const long long nrows_all = (long long)A.ptr.size() - 1;
  std::vector<long long> dpos;
  if (diag_first) {
    dpos.assign(nrows_all, -1);
    for (long long r = 0; r < nrows_all; ++r)
      for (long long t = A.ptr[r]; t < A.ptr[r + 1]; ++t)
        if (A.col[t] == r) { dpos[r] = t - A.ptr[r]; break; }
  }
  auto row_len = [&](long long r) -> long long {
    const long long len = A.ptr[r + 1] - A.ptr[r];
    return (diag_first && dpos[r] < 0) ? len + 1 : len;
  };
  pslice0.assign(np + 1, 0);
  for (int p = 0; p < np; ++p) pslice0[p + 1] = pslice0[p] + (prow0[p + 1] - prow0[p] + 31) / 32;
  const long long nsl = pslice0[np];
  const bool sorted = sigma > 1;
  rows.assign(nsl * 32, -1);
  for (int p = 0; p < np; ++p) {
    const long long n_p = prow0[p + 1] - prow0[p];
    long long* rp = rows.data() + pslice0[p] * 32;
    for (long long i = 0; i < n_p; ++i) rp[i] = prow0[p] + i;
    if (sorted) {
      for (long long w0 = 0; w0 < n_p; w0 += sigma) {
        const long long w1 = std::min<long long>(n_p, w0 + sigma);
        std::stable_sort(rp + w0, rp + w1, [&](long long x, long long y) {
          return row_len(x) > row_len(y);
        });
      }
    }
  }
  off.assign(nsl + 1, 0);
  for (long long s = 0; s < nsl; ++s) {
    long long L = 0;
    for (int l = 0; l < 32; ++l) {
      const long long r = rows[s * 32 + l];
      if (r >= 0) L = std::max(L, row_len(r));
    }
    off[s + 1] = off[s] + 32 * L;
  }
  const long long padded = off[nsl];
  if (padded > 2147483647LL * 2) return fail(e, GM_ERR_UNSUPPORTED, "padded SELL size too large");
  std::vector<int> col(padded);
  std::vector<VT> val(padded);
  std::vector<int> c2s;
  if (e->keep_map) c2s.assign(A.ptr.back(), 0);
  for (long long s = 0; s < nsl; ++s) {
    const long long L = (off[s + 1] - off[s]) / 32;
    for (int l = 0; l < 32; ++l) {
      const long long r = rows[s * 32 + l];
      const long long len = r >= 0 ? row_len(r) : 0;
      for (long long jj = 0; jj < L; ++jj) {
        const long long dst = off[s] + jj * 32 + l;
        if (jj < len) {
          // entry index within the row: diagonal first when diag_first
          long long t = jj;
          bool zero_diag = false;
          if (diag_first) {
            const long long dp = dpos[r];
            if (dp < 0) { zero_diag = jj == 0; t = jj - 1; }
            else t = jj == 0 ? dp : (jj <= dp ? jj - 1 : jj);
          }
          if (zero_diag) {
            col[dst] = (int)r;
            val[dst] = (VT)0;
            continue;
          }
          if (e->keep_map) c2s[A.ptr[r] + t] = (int)dst;
          col[dst] = A.col[A.ptr[r] + t];
          val[dst] = (VT)std::ldexp(A.val[A.ptr[r] + t], -scale_exp);
        } else {
          col[dst] = r >= 0 ? (int)r : 0;
          val[dst] = (VT)0;
        }
      }
    }
  }
  long long* d_off;
  int rc;
  if ((rc = dupload(e, &d_off, off.data(), off.size()))) return rc;
  if (e->mpk_req && np == 1 && !(sorted || np > 1)) e->sell_col_host = col;
  // Diagonal compensation of the FP32-stored matrix: row r gets the extra
  // diagonal term c_r = sum_t (a_t 2^-e - fl32(a_t 2^-e)) w_col(t) / w_r, so
  // that the stored operator maps w exactly as A does.  The small eigenvalues
  // of a Laplacian-like operator come from cancellation in A w-like products;
  // rounding every entry independently breaks it (an error of order
  // eps_32 * a_ii per row, relative to lambda_min), the compensation keeps it.
  e->kp.dlo = nullptr;
  if (sizeof(VT) == 4 && e->comp) {
    std::vector<float> dlo(nsl * 32, 0.f);
    const bool ones = e->roww.empty();
    std::vector<int> r2s;
    if (e->keep_map) r2s.assign(A.ptr.size() - 1, 0);
    for (long long s = 0; s < nsl; ++s)
      for (int l = 0; l < 32; ++l) {
        const long long r = rows[s * 32 + l];
        if (r < 0) continue;
        if (e->keep_map) r2s[r] = (int)(s * 32 + l);
        double corr = 0.0;
        for (long long t = A.ptr[r]; t < A.ptr[r + 1]; ++t) {
          const double exact = std::ldexp(A.val[t], -scale_exp);
          const double err = exact - (double)(float)exact;
          corr += ones ? err : err * e->roww[A.col[t]];
        }
        dlo[s * 32 + l] = (float)(ones ? corr : corr / e->roww[r]);
      }
    float* d_dlo;
    if ((rc = dupload(e, &d_dlo, dlo.data(), dlo.size()))) return rc;
    e->kp.dlo = d_dlo;
    if (e->keep_map) {
      if ((rc = dupload(e, &e->row2slot, r2s.data(), r2s.size()))) return rc;
      std::vector<double> w = e->roww;
      if (w.empty()) w.assign(A.ptr.size() - 1, 1.0);
      if ((rc = dupload(e, &e->d_roww, w.data(), w.size()))) return rc;
    }
  }
  // values and column indices in one allocation, so that one L2 access-policy
  // window can cover the whole matrix
  const size_t vbytes = ((size_t)padded * sizeof(VT) + 255) & ~(size_t)255;
  const size_t mbytes = vbytes + (size_t)padded * sizeof(int);
  unsigned char* d_mat;
  if ((rc = dalloc(e, &d_mat, mbytes))) return rc;
  VT* d_val = reinterpret_cast<VT*>(d_mat);
  int* d_col = reinterpret_cast<int*>(d_mat + vbytes);
  if (padded) {
    GM_CUDA(e, cudaMemcpy(d_val, val.data(), (size_t)padded * sizeof(VT), cudaMemcpyHostToDevice));
    GM_CUDA(e, cudaMemcpy(d_col, col.data(), (size_t)padded * sizeof(int), cudaMemcpyHostToDevice));
  }
  e->mat_base = d_mat;
  e->mat_bytes = mbytes;
  if (e->keep_map && (rc = dupload(e, &e->csr2sell, c2s.data(), c2s.size()))) return rc;
  if (e->keep_map && (rc = dupload(e, &e->csr_ptr, A.ptr.data(), A.ptr.size()))) return rc;
  e->kp.slice_off = d_off;
  e->kp.col = d_col;
  e->kp.val = d_val;
  e->kp.perm = nullptr;
  if (sorted || np > 1) {
    std::vector<int> p32(rows.size());
    for (size_t s = 0; s < rows.size(); ++s) p32[s] = (int)rows[s];
    int* d_perm;
    if ((rc = dupload(e, &d_perm, p32.data(), p32.size()))) return rc;
    e->kp.perm = d_perm;
  }
  e->nslices = nsl;
  e->padded = padded;
  e->kp.nslices = nsl;
  return GM_OK;
}

// Static partition of the SELL slices over the G blocks (contiguous ranges
// balanced by padded entries plus a per-row cost) and, per block, the sorted
// list of other blocks owning a row that one of its rows references, closed
// under symmetry (see DepSync in fab_common.cuh).
int build_partition(gm_engine* e, const Csr& A, const std::vector<long long>& rows,
                    const std::vector<long long>& off, const std::vector<long long>& pslice0,
                    const std::vector<long long>& prow0) {
  const int np = (int)pslice0.size() - 1;
  // blocks per problem in proportion to its work, at least one, at most one
  // per slice; e->G becomes the total
  std::vector<double> work(np, 0.0);
  std::vector<int> gp(np, 1);
  for (int p = 0; p < np; ++p)
    for (long long s = pslice0[p]; s < pslice0[p + 1]; ++s) work[p] += (double)(off[s + 1] - off[s]) + 32.0 * 4.0;
  if (e->G < np) return fail(e, GM_ERR_UNSUPPORTED, "%d problems need at least as many resident blocks (have %d)", np, e->G);
  for (int extra = e->G - np; extra > 0; --extra) {
    int best = -1;
    double bw = -1.0;
    for (int p = 0; p < np; ++p)
      if (gp[p] < pslice0[p + 1] - pslice0[p] && work[p] / gp[p] > bw) { bw = work[p] / gp[p]; best = p; }
    if (best < 0) break;
    gp[best]++;
  }
  std::vector<int> pb0(np + 1, 0);
  for (int p = 0; p < np; ++p) pb0[p + 1] = pb0[p] + gp[p];
  const int G = pb0[np];
  e->G = G;
  for (int g = 0; g < 9; ++g) e->Gk[g] = G;   // every phase group
  e->kp.G = G;
  std::vector<int> bs(G + 1, 0), bprob(G, 0);
  for (int p = 0; p < np; ++p) {
    double total = 0.0;
    for (long long s = pslice0[p]; s < pslice0[p + 1]; ++s) total += (double)(off[s + 1] - off[s]) + 32.0 * 4.0;
    double acc = 0.0;
    int b = 0;
    const int Gp = gp[p];
    bs[pb0[p]] = (int)pslice0[p];
    for (long long s = pslice0[p]; s < pslice0[p + 1]; ++s) {
      const double w = (double)(off[s + 1] - off[s]) + 32.0 * 4.0;
      while (b < Gp - 1 && acc + 0.5 * w > total * (b + 1) / Gp) bs[pb0[p] + (++b)] = (int)s;
      acc += w;
    }
    while (b < Gp - 1) bs[pb0[p] + (++b)] = (int)pslice0[p + 1];
    bs[pb0[p + 1]] = (int)pslice0[p + 1];
    for (int q = pb0[p]; q < pb0[p + 1]; ++q) bprob[q] = p;
  }
  std::vector<int> owner(e->n, 0);
  for (int q = 0; q < G; ++q)
    for (long long s = bs[q]; s < bs[q + 1]; ++s)
      for (int l = 0; l < 32; ++l) {
        const long long r = rows[s * 32 + l];
        if (r >= 0) owner[r] = q;
      }
  std::vector<unsigned char> adj((size_t)G * G, 0);
  for (int q = 0; q < G; ++q)
    for (long long s = bs[q]; s < bs[q + 1]; ++s)
      for (int l = 0; l < 32; ++l) {
        const long long r = rows[s * 32 + l];
        if (r < 0) continue;
        for (long long t = A.ptr[r]; t < A.ptr[r + 1]; ++t) {
          const int o = owner[A.col[t]];
          if (o != q) {
            adj[(size_t)q * G + o] = 1;
            adj[(size_t)o * G + q] = 1;
          }
        }
      }
  // Matrix-powers passes: per block the halo rows (referenced by its rows,
  // owned elsewhere), local column indices, and waits over two hops.
  const bool mpk = e->mpk_req && !e->sell_col_host.empty();
  std::vector<long long> hptr;
  std::vector<int> hrows, lcol;
  if (mpk) {
    hptr.assign(G + 1, 0);
    lcol.assign(e->sell_col_host.size(), 0);
    std::vector<unsigned char> adj2 = adj;
    long long nmax = 0;
    for (int q = 0; q < G; ++q) {
      const long long rb0 = (long long)bs[q] * 32;
      const long long rb1 = std::min<long long>((long long)bs[q + 1] * 32, e->n);
      std::vector<int> halo;
      for (long long r = rb0; r < rb1; ++r)
        for (long long t = A.ptr[r]; t < A.ptr[r + 1]; ++t) {
          const int col = A.col[t];
          if (col < rb0 || col >= rb1) halo.push_back(col);
        }
      std::sort(halo.begin(), halo.end());
      halo.erase(std::unique(halo.begin(), halo.end()), halo.end());
      const long long nown = rb1 - rb0;
      nmax = std::max<long long>(nmax, nown + (long long)halo.size());
      // two hops: the owners of the halo rows' columns
      for (int hr : halo)
        for (long long t = A.ptr[hr]; t < A.ptr[hr + 1]; ++t) {
          const int o = owner[A.col[t]];
          if (o != q) {
            adj2[(size_t)q * G + o] = 1;
            adj2[(size_t)o * G + q] = 1;
          }
        }
      // local column index of every slot of the block's slices
      for (long long sl = bs[q]; sl < bs[q + 1]; ++sl)
        for (long long slot = off[sl]; slot < off[sl + 1]; ++slot) {
          const int col = e->sell_col_host[slot];
          int li = 0;
          if (col >= rb0 && col < rb1) {
            li = (int)(col - rb0);
          } else {
            const auto it = std::lower_bound(halo.begin(), halo.end(), col);
            if (it != halo.end() && *it == col) li = (int)(nown + (it - halo.begin()));
          }
          lcol[slot] = li;
        }
      hrows.insert(hrows.end(), halo.begin(), halo.end());
      hptr[q + 1] = (long long)hrows.size();
    }
    adj.swap(adj2);
    e->mpk_nmax = nmax;
  }
  e->sell_col_host.clear();
  e->sell_col_host.shrink_to_fit();
  std::vector<int> dp(G + 1, 0), di;
  for (int q = 0; q < G; ++q) {
    for (int o = 0; o < G; ++o)
      if (adj[(size_t)q * G + o]) di.push_back(o);
    dp[q + 1] = (int)di.size();
  }
  e->dep_avg = G ? (double)di.size() / G : 0.0;
  int* d_bs;
  int* d_dp;
  int* d_di;
  int* d_bprob;
  int* d_pb0;
  long long* d_prow0;
  unsigned long long* d_prog;
  int rc;
  if ((rc = dupload(e, &d_bprob, bprob.data(), bprob.size()))) return rc;
  if ((rc = dupload(e, &d_pb0, pb0.data(), pb0.size()))) return rc;
  if ((rc = dupload(e, &d_prow0, prow0.data(), prow0.size()))) return rc;
  e->kp.nprob = np;
  e->kp.blk_prob = d_bprob;
  e->kp.prob_blk0 = d_pb0;
  e->kp.prob_row0 = d_prow0;
  if ((rc = dupload(e, &d_bs, bs.data(), bs.size()))) return rc;
  if ((rc = dupload(e, &d_dp, dp.data(), dp.size()))) return rc;
  if ((rc = dupload(e, &d_di, di.data(), di.size()))) return rc;
  if ((rc = dalloc(e, &d_prog, (size_t)G))) return rc;
  GM_CUDA(e, cudaMemset(d_prog, 0, sizeof(unsigned long long) * G));
  e->kp.blk_slice = d_bs;
  e->kp.dep_ptr = d_dp;
  e->kp.dep_idx = d_di;
  e->kp.prog = d_prog;
  e->kp.mpk = 0;
  if (mpk) {
    long long* d_hptr;
    int* d_hrows;
    int* d_lcol;
    if ((rc = dupload(e, &d_hptr, hptr.data(), hptr.size()))) return rc;
    if (hrows.empty()) hrows.push_back(0);
    if ((rc = dupload(e, &d_hrows, hrows.data(), hrows.size()))) return rc;
    if ((rc = dupload(e, &d_lcol, lcol.data(), lcol.size()))) return rc;
    e->kp.halo_ptr = d_hptr;
    e->kp.halo_rows = d_hrows;
    e->kp.lcol = d_lcol;
    e->kp.mpk = 1;   // confirmed (or withdrawn) once the shared memory is sized
  }
  return GM_OK;
}

// Phase-group kernels (kern_fp64.cu / kern_mixed.cu): 0 lanczos, 1 solves,
// 2 apply, 3 deflate/update, 4 fused lanczos + solves + apply.
enum { KGRP_LANCZOS = 0, KGRP_SOLVE = 1, KGRP_APPLY = 2, KGRP_DEFLATE = 3, KGRP_FUSED = 4,
       KGRP_LANCZOS_MPK = 5, KGRP_FUSED_MPK = 6, KGRP_LANCZOS_RO = 7, KGRP_FUSED_RO = 8, KGRP_N = 9 };

// The dynamic shared memory limit is an attribute of the kernel function,
// shared by every handle of the process (per device): only ever raise it, so
// that a handle created later with less shared memory cannot lower the limit
// under an earlier one.
cudaError_t raise_smem_limit(int dev, void* kfn, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, void*>, size_t> set;
  if (bytes <= 48 * 1024) return cudaSuccess;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = set[{dev, kfn}];
  if (bytes <= cur) return cudaSuccess;
  const cudaError_t st = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (st == cudaSuccess) cur = bytes;
  return st;
}

// The persisting L2 set-aside (cudaLimitPersistingL2CacheSize) belongs to
// the context, not to a handle: left set after its handle is gone, it keeps
// a share of L2 out of reach of ordinary accesses of every later kernel
// (measured: a 3D 256^3 FP64 solve created after a deleted handle with a
// window ran 13% slower).  Handles with a window count themselves per
// device; the set-aside is raised to the largest live window and returned
// to zero with the last one.
std::mutex g_window_mu;
std::map<int, std::pair<int, size_t>> g_window_users;   // device -> (handles, set-aside bytes)

cudaError_t window_acquire(int dev, size_t bytes) {
  std::lock_guard<std::mutex> lock(g_window_mu);
  auto& u = g_window_users[dev];
  if (bytes > u.second) {
    const cudaError_t st = cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, bytes);
    if (st != cudaSuccess) return st;
    u.second = bytes;
  }
  u.first++;
  return cudaSuccess;
}

void window_release(int dev) {
  std::lock_guard<std::mutex> lock(g_window_mu);
  auto it = g_window_users.find(dev);
  if (it == g_window_users.end() || it->second.first <= 0) return;
  if (--it->second.first == 0) {
    cudaCtxResetPersistingL2Cache();
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
    it->second.second = 0;
  }
}

// l2: a mixed engine's matrix is held in the L2 persisting window; one
// right-hand side then runs the SpMV groups compiled for two resident blocks
// per SM (gm::PolMixedL2, no register spills).
void* pick_kernel(int prec, int R, int group, bool l2) {
  if (l2 && R == 1 && prec != GM_FP64) {
    void* k = gm::kernel_mixed_l2(group);
    if (k) return k;
  }
  return prec == GM_FP64 ? gm::kernel_fp64(R, group) : gm::kernel_mixed(R, group);
}

// Tuning builds: -DGM_L2K_MIXED=0 keeps the three-block kernels for an
// L2-held matrix.
#ifndef GM_L2K_MIXED
#define GM_L2K_MIXED 1
#endif

int group_of(int phases) {
  const int solve = gm::PH_TRISOLVE | gm::PH_COEF;
  const int defl = gm::PH_DEFLATE | gm::PH_UPDATE_FKPP | gm::PH_UPDATE_FHN;
  if ((phases & gm::PH_LANCZOS) && (phases & (solve | gm::PH_APPLY))) return KGRP_FUSED;
  if (phases & gm::PH_LANCZOS) return KGRP_LANCZOS;
  if ((phases & solve) && (phases & gm::PH_APPLY)) return KGRP_FUSED;
  if (phases & solve) return KGRP_SOLVE;
  if (phases & gm::PH_APPLY) return KGRP_APPLY;
  return KGRP_DEFLATE;
}

int map_status(gm_engine* e, int st) {
  switch (st) {
    case gm::ST_OK: return GM_OK;
    case gm::ST_TIMEOUT: return fail(e, GM_ERR_TIMEOUT, "a grid-barrier wait exceeded its time limit; the handle is unusable");
    case gm::ST_NONFINITE: return fail(e, GM_ERR_NONFINITE, "non-finite value in the Lanczos recurrence");
    default: return fail(e, GM_ERR_CUDA, "device status %d", st);
  }
}

int check_sync(gm_engine* e) {
  GM_CUDA(e, cudaMemcpyAsync(e->h_status, e->kp.status, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  GM_CUDA(e, cudaMemcpyAsync(e->h_status + 1, e->kp.meff, sizeof(int) * e->R * e->nprob, cudaMemcpyDeviceToHost, e->stream));
  GM_CUDA(e, cudaStreamSynchronize(e->stream));
  return map_status(e, e->h_status[0]);
}

// Launch the persistent kernel with the given phases; slot selects the event
// pair used for gm_phase_times.
// NVTX range per engine phase (build_subspace, lin_sys_solves, apply_V,
// deflate/update, fused solve), visible to Nsight tools and ncu --nvtx; a
// no-op without a tool attached.
struct PhaseRange {
  explicit PhaseRange(int slot) {
    static const char* const names[5] = {"gm:deflate_update", "gm:build_subspace", "gm:lin_sys_solves",
                                         "gm:apply_V", "gm:solve"};
    nvtxRangePushA(names[slot >= 0 && slot < 5 ? slot : 4]);
  }
  ~PhaseRange() { nvtxRangePop(); }
  PhaseRange(const PhaseRange&) = delete;
  PhaseRange& operator=(const PhaseRange&) = delete;
};

int launch(gm_engine* e, int phases, int slot) {
  PhaseRange nvtx_range(slot);
  // The barrier counter returns to 0 after every completed barrier; it is
  // reset explicitly only after an aborted launch (gm_set_U clears errors).
  KParams kp = e->kp;
  kp.phases = phases;
  void* args[] = {&kp};
  int grp = group_of(phases);
  if (e->kp.reorth > 0 && (grp == KGRP_LANCZOS || grp == KGRP_FUSED))
    grp = grp == KGRP_LANCZOS ? KGRP_LANCZOS_RO : KGRP_FUSED_RO;
  else if (e->kp.mpk && (grp == KGRP_LANCZOS || grp == KGRP_FUSED))
    grp = grp == KGRP_LANCZOS ? KGRP_LANCZOS_MPK : KGRP_FUSED_MPK;
  kp.G = e->Gk[grp];
  if (e->capturing) {
    // A captured launch replays with the same parameters, so the progress
    // flags are cleared by a memset node before it and a fixed epoch is used.
    GM_CUDA(e, cudaMemsetAsync(e->kp.prog, 0, sizeof(unsigned long long) * e->G, e->stream));
    kp.epoch = 1;
  } else {
    GM_CUDA(e, cudaEventRecord(e->ev[slot][0], e->stream));
    kp.epoch = ++e->epoch;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kp.G);
  cfg.blockDim = dim3(e->threads);
  cfg.dynamicSmemBytes = e->smem[grp];
  cfg.stream = e->stream;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (e->l2_window) {
    attr[1].id = cudaLaunchAttributeAccessPolicyWindow;
    attr[1].val.accessPolicyWindow = e->window;
    cfg.numAttrs = 2;
  }
  cudaError_t st = cudaLaunchKernelExC(&cfg, e->kfn[grp], args);
  if (st != cudaSuccess) return cuda_fail(e, st, "cooperative launch");
  e->launches++;
  if (e->capturing) return GM_OK;
  GM_CUDA(e, cudaEventRecord(e->ev[slot][1], e->stream));
  e->ev_used[slot] = true;
  if (e->sync_mode) return check_sync(e);
  return GM_OK;
}

int copy_out(gm_engine* e, const double* src_il, double* dst) {
  if (!dst) return fail(e, GM_ERR_ARG, "null output pointer");
  const long long total = e->n * e->R;
  if (e->R == 1) {
    GM_CUDA(e, cudaMemcpyAsync(dst, src_il, total * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  } else {
    k_pack_out<<<(unsigned)((total + 255) / 256), 256, 0, e->stream>>>(src_il, e->stage, e->n, e->R);
    GM_CUDA(e, cudaGetLastError());
    e->launches++;
    GM_CUDA(e, cudaMemcpyAsync(dst, e->stage, total * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  }
  GM_CUDA(e, cudaStreamSynchronize(e->stream));
  return GM_OK;
}

// Usol <- U (column-major n x R, host or device) scaled by col_scale.
int set_usol(gm_engine* e, const double* U, bool on_device, bool scaled = true) {
  if (!U) return fail(e, GM_ERR_ARG, "lanczos_create:badU: null U");
  const long long total = e->n * e->R;
  const double* src = U;
  if (!on_device) {
    GM_CUDA(e, cudaMemcpyAsync(e->stage, U, total * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    src = e->stage;
  }
  k_pack_in<<<(unsigned)((total + 255) / 256), 256, 0, e->stream>>>(src, e->kp.Usol, e->n, e->R,
                                                                   scaled ? e->col_scale : nullptr);
  GM_CUDA(e, cudaGetLastError());
  e->launches++;
  return GM_OK;
}

void destroy(gm_engine* e) {
  if (!e) return;
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->l2_window) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(e->dev);
    window_release(e->dev);
    cudaSetDevice(cur);
  }
  if (e->loop_exec) cudaGraphExecDestroy(e->loop_exec);
  for (auto& b : e->bufs) cudaFree(b.p);
  e->bufs.clear();
  for (int s = 0; s < 5; ++s)
    for (int t = 0; t < 2; ++t)
      if (e->ev[s][t]) cudaEventDestroy(e->ev[s][t]);
  if (e->h_status) cudaFreeHost(e->h_status);
  if (e->own_stream) cudaStreamDestroy(e->own_stream);
  delete e;
}

// Creates the engine for one problem (gm_lanczos_create) or several
// independent problems sharing m, C, d and nrhs (gm_batch_create).
int create_impl(const gm_create_args* a, const std::vector<ProbIn>& probs, gm_engine* e) {
  if (a->struct_version != GM_CREATE_ARGS_VERSION)
    return fail(e, GM_ERR_ARG, "lanczos_create:invalidNumInputs: struct_version %d != %d", a->struct_version, GM_CREATE_ARGS_VERSION);
  const int np = (int)probs.size();
  if (np < 1) return fail(e, GM_ERR_ARG, "batch_create: no problems");
  if (a->gamma_size < 1 || a->gamma_size > GM_MAX_DEG + 1)
    return fail(e, GM_ERR_ARG, "lanczos_create:bad_gamma: polynomial degree must be 0..%d (gamma_size %d)", GM_MAX_DEG, a->gamma_size);
  if (a->nrhs != 1 && a->nrhs != 2 && a->nrhs != 4) return fail(e, GM_ERR_ARG, "lanczos_create:badU: nrhs must be 1, 2 or 4 (got %d)", a->nrhs);
  if (a->num_eigs < 0 || (a->num_eigs > 0 && (!a->Q || !a->flam)))
    return fail(e, GM_ERR_ARG, "lanczos_create:badQ: num_eigs %d needs Q and f(lambda)", a->num_eigs);
  if (np > 1 && a->num_eigs > 0) return fail(e, GM_ERR_UNSUPPORTED, "batch_create: deflation needs a single problem");
  if (a->subspace_size < 1) return fail(e, GM_ERR_ARG, "lanczos_create:bad_N: subspace size must be >= 1");
  if (a->gamma_size < 1) return fail(e, GM_ERR_ARG, "lanczos_create:bad_gamma: gamma_size must be >= 1");
  if (a->contour_size < 1) return fail(e, GM_ERR_ARG, "lanczos_create:bad_gamma_s_real: contour size must be >= 1");
  if (a->precision != GM_FP64 && a->precision != GM_MIXED) return fail(e, GM_ERR_ARG, "unknown precision %d", a->precision);
  if (a->reorth < 0 || a->reorth > 2) return fail(e, GM_ERR_ARG, "reorth must be 0 (none), 1 (CGS) or 2 (CGS2), got %d", a->reorth);
  long long ntot = 0;
  for (int p = 0; p < np; ++p) {
    const ProbIn& q = probs[p];
    if (q.n <= 0) return fail(e, GM_ERR_ARG, "lanczos_create:inputNotSquare: n must be positive (problem %d)", p);
    if (!q.ptr || !q.ind || !q.values) return fail(e, GM_ERR_ARG, "lanczos_create:inputNotSparse: null sparse array (problem %d)", p);
    if (q.format != GM_CSC && q.format != GM_CSR) return fail(e, GM_ERR_ARG, "unknown matrix format %d", q.format);
    if (!q.U) return fail(e, GM_ERR_ARG, "lanczos_create:badU: null U (problem %d)", p);
    if (!q.gamma) return fail(e, GM_ERR_ARG, "lanczos_create:bad_gamma: null gamma (problem %d)", p);
    if (!q.gs_re || !q.gs_im) return fail(e, GM_ERR_ARG, "lanczos_create:bad_gamma_s_real: null shifted coefficients (problem %d)", p);
    if (!q.wts) return fail(e, GM_ERR_ARG, "lanczos_create:bad_wts1: null weights (problem %d)", p);
    if (!q.shifts) return fail(e, GM_ERR_ARG, "lanczos_create:bad_shifts: null shifts (problem %d)", p);
    ntot += q.n;
  }
  if (ntot > 2147483647LL) return fail(e, GM_ERR_UNSUPPORTED, "n above 2^31-1");

  e->keep_map = a->keep_entry_map != 0 && np == 1;
  e->comp = a->precision == GM_MIXED && a->diag_compensation == 0;
  // matrix-powers passes and reorthogonalisation are separate entry points;
  // reorthogonalisation takes precedence
  e->mpk_req = a->matrix_powers != 0 && np == 1 && a->sell_sigma <= 1 && a->gamma_size >= 3 && a->reorth == 0;
  if (e->comp && a->row_weight) {
    if (np != 1) return fail(e, GM_ERR_ARG, "row_weight applies to a single problem");
    e->roww.assign(a->row_weight, a->row_weight + probs[0].n);
    for (double w : e->roww)
      if (!(w > 0.0) || !std::isfinite(w)) return fail(e, GM_ERR_ARG, "row_weight entries must be positive and finite");
  }
  if (a->keep_entry_map && probs[0].format != GM_CSR) return fail(e, GM_ERR_ARG, "keep_entry_map needs a CSR matrix");
  e->n = ntot; e->nprob = np; e->R = a->nrhs; e->m = a->subspace_size; e->d = a->gamma_size - 1;
  e->C = a->contour_size; e->k = a->num_eigs; e->prec = a->precision; e->sync_mode = a->sync_mode;
  e->threads = a->threads_per_block ? a->threads_per_block : GM_MAXT;
  if (e->threads % 32 || e->threads < 64 || e->threads > GM_MAXT)
    return fail(e, GM_ERR_ARG, "threads_per_block must be a multiple of 32 in [64, %d]", GM_MAXT);
  GM_CUDA(e, cudaGetDevice(&e->dev));
  GM_CUDA(e, cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, e->dev));
  int coop = 0;
  GM_CUDA(e, cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, e->dev));
  if (!coop) return fail(e, GM_ERR_UNSUPPORTED, "device does not support cooperative launch");
  GM_CUDA(e, cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking));
  e->stream = e->own_stream;
  for (int s = 0; s < 5; ++s)
    for (int t = 0; t < 2; ++t) GM_CUDA(e, cudaEventCreate(&e->ev[s][t]));
  GM_CUDA(e, cudaHostAlloc((void**)&e->h_status, sizeof(int) * (1 + (size_t)np * e->R), cudaHostAllocDefault));

  int rc;
  Csr csr;
  std::vector<long long> prow0(np + 1, 0);
  for (int p = 0; p < np; ++p) {
    Csr one;
    if ((rc = make_csr(e, probs[p], one))) return rc;
    prow0[p + 1] = prow0[p] + probs[p].n;
    if (np == 1) csr = std::move(one);
    else append_block(csr, one, prow0[p]);
  }
  e->nnz = csr.ptr.back();
  // The mixed engine stores A / 2^e (e = floor(log2 of the largest absolute
  // row sum)) so that A's spectrum, the polynomial coefficients and the
  // Horner intermediates stay inside FP32's exponent range.  The scaling is a
  // power of two, hence exact, and is undone exactly: gamma_i, the shifted
  // coefficients, the shifts and the weights are rescaled so that y and X
  // are unchanged (sigma/s - T/s = (sigma - T)/s, A_s^(d-i) s^(d-i) = A^(d-i)).
  if (e->prec == GM_MIXED) {
    double mx = 0.0;
    for (long long i = 0; i < e->n; ++i) {
      double rs = 0.0;
      for (long long t = csr.ptr[i]; t < csr.ptr[i + 1]; ++t) rs += std::fabs(csr.val[t]);
      mx = std::max(mx, rs);
    }
    e->scale_exp = mx > 0.0 ? (int)std::floor(std::log2(mx)) : 0;
  }
  std::vector<long long> slot_rows, slice_off, pslice0;
  rc = e->prec == GM_FP64 ? upload_sell<double>(e, csr, a->sell_sigma, 0, prow0, slot_rows, slice_off, pslice0)
                          : upload_sell<float>(e, csr, a->sell_sigma, e->scale_exp, prow0, slot_rows, slice_off, pslice0);
  if (rc) return rc;
  // Value prefetch: with each staged slice's column copy, lane 0 also starts
  // an L2 bulk prefetch of the slice's values, so they are on their way from
  // HBM while the warp computes the current slice.  A matrix held in the L2
  // persisting window (see below) gains nothing, so by default the prefetch
  // is on only when the matrix does not fit that window.
  if (a->val_prefetch < 0 || a->val_prefetch > 2) return fail(e, GM_ERR_ARG, "val_prefetch must be 0, 1 or 2");
  if (a->l2_window < 0 || a->l2_window > 2) return fail(e, GM_ERR_ARG, "l2_window must be 0 (auto), 1 (off) or 2 (on)");
  // The persisting L2 window pays when the whole matrix fits the persisting
  // limit and the rest of L2 still holds one SpMV pass's vectors: the
  // gathered input and the output (n R Horner elements each, 8 bytes: FP64
  // or float-float) and the basis row read (n R storage elements).  When
  // they do not fit, a pinned matrix makes the vectors, whose gathers are
  // latency-critical, stream from DRAM on every pass; streaming the matrix
  // with the value prefetch instead keeps the vectors in L2 (measured on the
  // 1M-node FE disk with 4 right-hand sides, mixed precision: with the
  // window the launch moved its whole algorithmic traffic through DRAM at
  // an L2 hit rate of 13%).
  bool use_window = false;
  if (a->l2_window != 1 && e->mat_bytes > 0) {
    int mp = 0, mw = 0, l2 = 0;
    GM_CUDA(e, cudaDeviceGetAttribute(&mp, cudaDevAttrMaxPersistingL2CacheSize, e->dev));
    GM_CUDA(e, cudaDeviceGetAttribute(&mw, cudaDevAttrMaxAccessPolicyWindowSize, e->dev));
    GM_CUDA(e, cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, e->dev));
    const bool fits_limit = mp > 0 && mw > 0 && e->mat_bytes <= (size_t)std::min(mp, mw);
    const double vec_bytes = (double)ntot * e->R * (2.0 * 8.0 + (e->prec == GM_FP64 ? 8.0 : 4.0));
    const bool fits_l2 = (double)e->mat_bytes + vec_bytes <= 0.9 * (double)l2;
    use_window = fits_limit && (a->l2_window == 2 || fits_l2);
  }
  // Column staging: per warp two stages of stage_cap * 32 column indices
  // (slices with more columns are read from global memory directly), with
  // the value prefetch riding on each stage's copy.  It pays for a matrix
  // streamed from HBM (3D 256^3: mixed 56.7 vs 51.8 ms per solve without vs
  // with staging; the 1M-node FE disk with four right-hand sides, whose
  // vectors push the matrix out of L2: 58.4 vs 49.7 ms); for a matrix held in
  // the L2 window it only adds work (the same disk with one right-hand side:
  // mixed 18.2 vs 16.8 ms with vs without, FP64 equal within 0.5%; the 250k
  // adjoint 317 vs 310 ms per gradient), so by default it is on only when the
  // window is not used.
  if (a->col_staging < 0 || a->col_staging > 2) return fail(e, GM_ERR_ARG, "col_staging must be 0 (auto), 1 (off) or 2 (on)");
  long long max_len = 0;
  for (size_t q = 0; q + 1 < slice_off.size(); ++q) max_len = std::max(max_len, (slice_off[q + 1] - slice_off[q]) / 32);
  // (val_prefetch = 1 forces the prefetch, which rides on the stages).
  // Since the SpMV walks one entry per step with the column source fixed per
  // row, the FP64 engine gains from staging an L2-held matrix too (1M-node
  // FE disk FP64 19.68 vs 21.18 ms per solve), where the mixed engine still
  // loses (16.19 vs 14.94 ms): FP64 engines without matrix-powers passes
  // (whose level-between vector shares the dynamic shared memory) stage
  // whenever the slices fit a stage.
  const bool stage_l2 = e->prec == GM_FP64 && !e->mpk_req;
  const bool staging = a->col_staging == 2 ||
                       (a->col_staging == 0 && (!use_window || a->val_prefetch == 1 || stage_l2));
  const int stage_cap = staging ? (int)std::min<long long>(max_len, 24) : 0;
  const size_t stage_smem = stage_cap > 0 ? (size_t)16 * (e->threads / 32) + (size_t)2 * (e->threads / 32) * stage_cap * 128 : 0;
  e->kp.stage_cap = stage_cap;
  e->kp.pf_vals = 0;
  if (stage_cap > 0 && a->val_prefetch != 2) {
    if (a->val_prefetch == 1 || !use_window) e->kp.pf_vals = e->prec == GM_FP64 ? 8 : 4;
  }
  // Grid: blocks_per_sm x SMs, capped by co-residency of each phase-group
  // kernel this engine can launch and by the work (about one SELL slice per
  // warp: small problems get fewer blocks, which makes every grid barrier
  // cheaper).  The matrix-powers and Gram-Schmidt groups, compiled for fewer
  // resident blocks, bound the grid only of engines that launch them.
  const bool l2k = use_window && e->prec != GM_FP64 && GM_L2K_MIXED != 0;
  const long long nsl = (long long)slice_off.size() - 1;
  const int nw = e->threads / 32;
  const long long want = std::max<long long>(np, (nsl + nw - 1) / nw);
  long long Gmax = 0;
  for (int g = 0; g < KGRP_N; ++g) {
    e->kfn[g] = pick_kernel(e->prec, e->R, g, l2k);
    if (!e->kfn[g]) return fail(e, GM_ERR_UNSUPPORTED, "no kernel for nrhs %d", e->R);
    e->smem[g] = (g == KGRP_LANCZOS || g == KGRP_APPLY || g == KGRP_FUSED || g == KGRP_LANCZOS_MPK ||
                  g == KGRP_FUSED_MPK || g == KGRP_LANCZOS_RO || g == KGRP_FUSED_RO) ? stage_smem : 0;
    if (e->smem[g] > 48 * 1024)
      GM_CUDA(e, raise_smem_limit(e->dev, e->kfn[g], e->smem[g]));
    const bool ro_grp = g == KGRP_LANCZOS_RO || g == KGRP_FUSED_RO;
    const bool mpk_grp = g == KGRP_LANCZOS_MPK || g == KGRP_FUSED_MPK;
    if ((ro_grp && a->reorth == 0) || (mpk_grp && !e->mpk_req)) {
      e->Gk[g] = 0;   // never launched
      continue;
    }
    int nb = 0;
    GM_CUDA(e, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, e->kfn[g], e->threads, e->smem[g]));
    if (nb < 1) return fail(e, GM_ERR_UNSUPPORTED, "kernel group %d cannot be resident with %d threads", g, e->threads);
    const int bps = a->blocks_per_sm > 0 ? std::min(a->blocks_per_sm, nb) : nb;
    long long G = (long long)bps * e->nsm;
    if (a->blocks_per_sm <= 0) G = std::min(G, want);
    if (a->max_blocks > 0) G = std::min<long long>(G, std::max<long long>(np, a->max_blocks));
    e->Gk[g] = (int)std::max<long long>(1, G);
    Gmax = Gmax == 0 ? e->Gk[g] : std::min(Gmax, (long long)e->Gk[g]);
  }
  e->G = (int)Gmax;
  // blocks per problem and the slice partition (sets e->G to the blocks used)
  if ((rc = build_partition(e, csr, slot_rows, slice_off, pslice0, prow0))) return rc;
  e->kp.dep_mode = a->sync_policy == 0 ? 1 : 0;
  if (e->kp.mpk) {
    // the level in between lives in dynamic shared memory after the stages;
    // keep it only if the Lanczos kernels stay as resident as the grid needs
    const size_t su_off = (e->smem[KGRP_LANCZOS] + 15) & ~(size_t)15;
    const size_t su_bytes = (size_t)e->mpk_nmax * e->R * 8;
    const int need = (e->G + e->nsm - 1) / e->nsm;
    bool fits = true;
    for (int g : {KGRP_LANCZOS_MPK, KGRP_FUSED_MPK}) {
      const size_t sm = su_off + su_bytes;
      if (raise_smem_limit(e->dev, e->kfn[g], sm) != cudaSuccess) {
        cudaGetLastError();
        fits = false;
        break;
      }
      int nb = 0;
      GM_CUDA(e, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, e->kfn[g], e->threads, sm));
      if (nb < need) { fits = false; break; }
    }
    if (fits) {
      e->smem[KGRP_LANCZOS_MPK] = e->smem[KGRP_FUSED_MPK] = su_off + su_bytes;
      e->kp.su_off = (long long)su_off;
    } else {
      e->kp.mpk = 0;   // the two-hop waits stay: correct, slightly more waiting
    }
  }
  csr = Csr();
  if (use_window) {
    // Persisting L2 lines for the matrix, which every SpMV pass re-reads
    // (only when the whole matrix fits the persisting limit: a partial
    // window pins a sliver of a large matrix and takes L2 from the vectors).
    // The set-aside is a setting of the context, shared by all handles: it
    // is raised to the largest live window and released when the last
    // handle with a window is deleted (window_acquire / window_release).
    int max_window = 0;
    GM_CUDA(e, cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, e->dev));
    const size_t win = std::min<size_t>(e->mat_bytes, (size_t)max_window);
    GM_CUDA(e, window_acquire(e->dev, win));
    e->window.base_ptr = e->mat_base;
    e->window.num_bytes = win;
    e->window.hitRatio = 1.0f;
    e->window.hitProp = cudaAccessPropertyPersisting;
    e->window.missProp = cudaAccessPropertyStreaming;
    e->l2_window = true;
  }

  KParams& kp = e->kp;
  const long long n = e->n;
  const int R = e->R, m = e->m, d = e->d, C = e->C, k = e->k;
  kp.n = n; kp.m = m; kp.d = d; kp.C = C; kp.k = k; kp.G = e->G;
  kp.dt = a->dt; kp.aode = a->aode; kp.bode = a->bode; kp.code = a->code; kp.vrest = a->vrest;
  kp.vamp = a->vamp; kp.vpeak = a->vpeak; kp.c1ion = a->c1ion;
  kp.bd_tol = a->breakdown_tol > 0 ? a->breakdown_tol : 64.0 * 2.220446049250313e-16;
  const double tmo = a->barrier_timeout_s > 0 ? a->barrier_timeout_s : 5.0;
  kp.timeout_ns = (unsigned long long)(tmo * 1e9);

  double *gam, *gsr, *gsi, *wts, *shf, *flam = nullptr, *Q = nullptr, *mass, *ode;
  {
    // per-problem method arrays, concatenated in problem order
    const int se = e->scale_exp;
    std::vector<double> g, gr, gi, w, sh;
    for (int p = 0; p < np; ++p) {
      const ProbIn& q = probs[p];
      const size_t g0 = g.size(), gr0 = gr.size(), w0 = w.size(), sh0 = sh.size();
      g.insert(g.end(), q.gamma, q.gamma + d + 1);
      gr.insert(gr.end(), q.gs_re, q.gs_re + (size_t)(d + 1) * C);
      gi.insert(gi.end(), q.gs_im, q.gs_im + (size_t)(d + 1) * C);
      w.insert(w.end(), q.wts, q.wts + (size_t)2 * C * R);
      sh.insert(sh.end(), q.shifts, q.shifts + (size_t)2 * m * C * R);
      if (se != 0) {
        for (int i = 0; i <= d; ++i) {
          g[g0 + i] = std::ldexp(g[g0 + i], se * (d - i));
          for (int j = 0; j < C; ++j) {
            gr[gr0 + i + (size_t)(d + 1) * j] = std::ldexp(gr[gr0 + i + (size_t)(d + 1) * j], se * (d - i));
            gi[gr0 + i + (size_t)(d + 1) * j] = std::ldexp(gi[gr0 + i + (size_t)(d + 1) * j], se * (d - i));
          }
        }
        for (size_t t = w0; t < w.size(); ++t) w[t] = std::ldexp(w[t], -se);
        for (size_t t = sh0; t < sh.size(); ++t) sh[t] = std::ldexp(sh[t], -se);
      }
    }
    if ((rc = dupload(e, &gam, g.data(), g.size()))) return rc;
    if ((rc = dupload(e, &gsr, gr.data(), gr.size()))) return rc;
    if ((rc = dupload(e, &gsi, gi.data(), gi.size()))) return rc;
    if ((rc = dupload(e, &wts, w.data(), w.size()))) return rc;
    if ((rc = dupload(e, &shf, sh.data(), sh.size()))) return rc;
  }
  if (k > 0) {
    if ((rc = dupload(e, &flam, a->flam, (size_t)k * R))) return rc;
    if ((rc = dupload(e, &Q, a->Q, (size_t)k * n))) return rc;
  }
  std::vector<double> ones;
  if (a->mass && np == 1) {
    if ((rc = dupload(e, &mass, a->mass, n))) return rc;
  } else {
    ones.assign(n, 1.0);
    if ((rc = dupload(e, &mass, ones.data(), n))) return rc;
  }
  if (a->ode && np == 1) {
    if ((rc = dupload(e, &ode, a->ode, n))) return rc;
  } else {
    if ((rc = dalloc(e, &ode, n))) return rc;
    GM_CUDA(e, cudaMemset(ode, 0, n * sizeof(double)));
  }
  std::vector<double> cs(R, 1.0);
  if (a->col_scale) {
    for (int r = 0; r < R; ++r) cs[r] = a->col_scale[r];
  } else if (R == 2) {
    cs[1] = a->dt;  // lanczos_impl.cu:79: U(:,1) *= dt
  }
  if ((rc = dupload(e, &e->col_scale, cs.data(), R))) return rc;
  kp.gamma = gam; kp.gs_re = gsr; kp.gs_im = gsi; kp.wts = wts; kp.shifts = shf;
  kp.flam = flam; kp.Q = Q; kp.mass = mass; kp.ode = ode;

  const size_t nR = (size_t)n * R;
  const size_t bsz = e->prec == GM_FP64 ? 8 : 4;
  const size_t PR = (size_t)np * R;   // (problem, right-hand side) pairs
  if ((rc = dalloc(e, &kp.U, nR))) return rc;
  if ((rc = dalloc(e, &kp.Usol, nR))) return rc;
  if ((rc = dalloc(e, &kp.upd, nR))) return rc;
  if ((rc = dalloc(e, &kp.X, nR))) return rc;
  if ((rc = dalloc(e, &kp.S, nR))) return rc;
  if ((rc = dalloc(e, &e->stage, nR))) return rc;
  char *V, *W0, *W1;
  double *H0, *H1, *P;
  if ((rc = dalloc(e, &V, (size_t)m * nR * bsz))) return rc;
  if ((rc = dalloc(e, &W0, nR * bsz))) return rc;
  if ((rc = dalloc(e, &W1, nR * bsz))) return rc;
  if ((rc = dalloc(e, &H0, nR))) return rc;
  if ((rc = dalloc(e, &H1, nR))) return rc;
  if ((rc = dalloc(e, &P, d > 0 ? (size_t)(d + 1) * nR : 1))) return rc;
  kp.V = V; kp.W0 = W0; kp.W1 = W1; kp.H0 = H0; kp.H1 = H1; kp.P = P;
  if ((rc = dalloc(e, &kp.aabb, (size_t)(m + 1) * 2 * PR))) return rc;
  if ((rc = dalloc(e, &kp.Yr, (size_t)m * PR * C))) return rc;
  if ((rc = dalloc(e, &kp.Yi, (size_t)m * PR * C))) return rc;
  if ((rc = dalloc(e, &kp.coef, PR * (d + 1) * m))) return rc;
  if ((rc = dalloc(e, &kp.coef_ff, PR * (d + 1) * m))) return rc;
  if ((rc = dalloc(e, &kp.tri, (size_t)4 * m * PR * C))) return rc;
  if ((rc = dalloc(e, &kp.Z, (size_t)(k + 4) * R))) return rc;
  if ((rc = dalloc(e, &kp.part, (size_t)(2 * R + (k + 4) * R) * e->G))) return rc;
  kp.reorth = a->reorth;
  if (kp.reorth > 0) {
    if ((rc = dalloc(e, &kp.hpart, (size_t)2 * (m + 8) * R * e->G))) return rc;
    if ((rc = dalloc(e, &kp.hblk, (size_t)e->G * (m + 1) * R))) return rc;
  }
  if ((rc = dalloc(e, &kp.bar, 2 + 2 * (size_t)np))) return rc;
  if ((rc = dalloc(e, &kp.status, 1))) return rc;
  if ((rc = dalloc(e, &kp.meff, PR))) return rc;
  GM_CUDA(e, cudaMemset(kp.bar, 0, (2 + 2 * (size_t)np) * sizeof(unsigned)));
  GM_CUDA(e, cudaMemset(kp.status, 0, sizeof(int)));
  GM_CUDA(e, cudaMemset(kp.aabb, 0, (size_t)(m + 1) * 2 * PR * sizeof(double)));
  GM_CUDA(e, cudaMemset(kp.X, 0, nR * sizeof(double)));
  GM_CUDA(e, cudaMemset(kp.Yr, 0, (size_t)m * PR * C * sizeof(double)));
  GM_CUDA(e, cudaMemset(kp.Yi, 0, (size_t)m * PR * C * sizeof(double)));
  {
    std::vector<int> me(PR, m);
    GM_CUDA(e, cudaMemcpy(kp.meff, me.data(), PR * sizeof(int), cudaMemcpyHostToDevice));
  }
  GM_CUDA(e, cudaDeviceSynchronize());

  // constructor: scale columns, Usol = U, deflate (lanczos_impl.cu:79-89);
  // a batch's right-hand sides are stacked problem after problem per column
  std::vector<double> Uall;
  const double* U0 = probs[0].U;
  if (np > 1) {
    Uall.resize(nR);
    for (int r = 0; r < R; ++r)
      for (int p = 0; p < np; ++p)
        std::memcpy(Uall.data() + (size_t)r * n + prow0[p], probs[p].U + (size_t)r * probs[p].n, sizeof(double) * probs[p].n);
    U0 = Uall.data();
  }
  if ((rc = set_usol(e, U0, false))) return rc;
  const int saved = e->sync_mode;
  e->sync_mode = 1;
  rc = launch(e, gm::PH_DEFLATE, 0);
  e->sync_mode = saved;
  return rc;
}

}  // namespace

namespace gm {
// Sets the message gm_last_error(NULL) returns (used by entry points that
// have no handle).
void set_global_error(const char* msg) { g_create_error = msg ? msg : ""; }
}  // namespace gm

// ====================================================================== C ABI
extern "C" {

void gm_default_args(gm_create_args* a) {
  if (!a) return;
  std::memset(a, 0, sizeof(*a));
  a->struct_version = GM_CREATE_ARGS_VERSION;
  a->format = GM_CSC;
  a->nrhs = 2;
  a->sync_mode = 1;
  a->dt = 1.0;
  a->vamp = 1.0;
}

int gm_lanczos_create(const gm_create_args* args, gm_handle* out) {
  g_create_error.clear();
  if (!args || !out) return fail(nullptr, GM_ERR_ARG, "lanczos_create:invalidNumInputs: null argument");
  *out = nullptr;
  gm_engine* e = new (std::nothrow) gm_engine();
  if (!e) return fail(nullptr, GM_ERR_OOM, "host allocation failed");
  if (!args->ptr || !args->ind || !args->values || args->n <= 0) {
    // report shape errors under the reference's identifiers before any device work
    delete e;
    if (args->n <= 0) return fail(nullptr, GM_ERR_ARG, "lanczos_create:inputNotSquare: n must be positive");
    return fail(nullptr, GM_ERR_ARG, "lanczos_create:inputNotSparse: null sparse array");
  }
  ProbIn q{args->n, args->nnz, args->format, reinterpret_cast<const long long*>(args->ptr),
           reinterpret_cast<const long long*>(args->ind), args->values, args->U, args->gamma,
           args->gamma_s_real, args->gamma_s_imag, args->wts, args->shifts};
  int rc = create_impl(args, std::vector<ProbIn>{q}, e);
  if (rc) {
    g_create_error = e->err;
    destroy(e);
    return rc;
  }
  *out = e;
  return GM_OK;
}

int gm_batch_create(int nprob, const gm_batch_problem* probs, const gm_create_args* common, gm_handle* out) {
  g_create_error.clear();
  if (!probs || !common || !out || nprob < 1) return fail(nullptr, GM_ERR_ARG, "batch_create: null argument or no problems");
  *out = nullptr;
  gm_engine* e = new (std::nothrow) gm_engine();
  if (!e) return fail(nullptr, GM_ERR_OOM, "host allocation failed");
  std::vector<ProbIn> v;
  for (int p = 0; p < nprob; ++p) {
    const gm_batch_problem& b = probs[p];
    v.push_back(ProbIn{b.n, 0, b.format, reinterpret_cast<const long long*>(b.ptr), reinterpret_cast<const long long*>(b.ind),
                       b.values, b.U, b.gamma, b.gamma_s_real, b.gamma_s_imag, b.wts, b.shifts});
  }
  int rc = create_impl(common, v, e);
  if (rc) {
    g_create_error = e->err;
    destroy(e);
    return rc;
  }
  *out = e;
  return GM_OK;
}

int gm_lanczos_delete(gm_handle h) {
  if (!h) return fail(nullptr, GM_ERR_ARG, "lanczos_delete:inputNotHandle: null handle");
  destroy(h);
  return GM_OK;
}

int gm_build_subspace(gm_handle h) {
  if (!h) return GM_ERR_ARG;
  int rc = launch(h, gm::PH_LANCZOS, 1);
  if (!rc) { h->have_V = true; h->have_y = false; h->have_coef = false; }
  return rc;
}

int gm_lin_sys_solves(gm_handle h) {
  if (!h) return GM_ERR_ARG;
  if (!h->have_V) return fail(h, GM_ERR_STATE, "lin_sys_solves before build_subspace");
  int rc = launch(h, gm::PH_TRISOLVE | gm::PH_COEF, 2);
  if (!rc) { h->have_y = true; h->have_coef = true; }
  return rc;
}

int gm_apply_V(gm_handle h) {
  if (!h) return GM_ERR_ARG;
  if (!h->have_V || !h->have_coef) return fail(h, GM_ERR_STATE, "apply_V before build_subspace and lin_sys_solves/set_y");
  return launch(h, gm::PH_APPLY, 3);
}

int gm_update_U(gm_handle h) {
  if (!h) return GM_ERR_ARG;
  if (h->R != 2) return fail(h, GM_ERR_ARG, "update_U needs nrhs = 2");
  return launch(h, gm::PH_UPDATE_FKPP | gm::PH_DEFLATE, 0);
}

int gm_update_U_monodomain(gm_handle h) {
  if (!h) return GM_ERR_ARG;
  if (h->R != 2) return fail(h, GM_ERR_ARG, "update_U_monodomain needs nrhs = 2");
  return launch(h, gm::PH_UPDATE_FHN | gm::PH_DEFLATE, 0);
}

int gm_get_U(gm_handle h, double* dst) {
  if (!h) return GM_ERR_ARG;
  int rc = copy_out(h, h->kp.Usol, dst);
  return rc ? rc : check_sync(h);
}

int gm_get_xsol(gm_handle h, double* dst) {
  if (!h) return GM_ERR_ARG;
  int rc = copy_out(h, h->kp.X, dst);
  return rc ? rc : check_sync(h);
}

int gm_get_update(gm_handle h, double* dst) {
  if (!h) return GM_ERR_ARG;
  int rc = copy_out(h, h->kp.upd, dst);
  return rc ? rc : check_sync(h);
}

int gm_get_solution(gm_handle h, double* dst) {
  if (!h) return GM_ERR_ARG;
  int rc = copy_out(h, h->kp.S, dst);
  return rc ? rc : check_sync(h);
}

int gm_get_solution_device(gm_handle h, double* dst_dev) {
  if (!h || !dst_dev) return GM_ERR_ARG;
  const long long total = h->n * h->R;
  k_pack_out<<<(unsigned)((total + 255) / 256), 256, 0, h->stream>>>(h->kp.S, dst_dev, h->n, h->R);
  GM_CUDA(h, cudaGetLastError());
  h->launches++;
  return h->sync_mode ? check_sync(h) : GM_OK;
}

int gm_get_aabb(gm_handle h, double* dst) {
  if (!h || !dst) return GM_ERR_ARG;
  GM_CUDA(h, cudaMemcpyAsync(dst, h->kp.aabb, (size_t)(h->m + 1) * 2 * h->R * h->nprob * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  int rc = check_sync(h);
  if (h->scale_exp != 0) {
    // alpha_j and beta_{j>=1} of the scaled operator are those of A over 2^e
    const size_t ld = h->m + 1;
    for (int p = 0; p < h->nprob; ++p)
      for (int r = 0; r < 2 * h->R; ++r)
        for (size_t q = 0; q < ld; ++q)
          if (r < h->R || q > 0) {
            double& v = dst[((size_t)p * 2 * h->R + r) * ld + q];
            v = std::ldexp(v, h->scale_exp);
          }
  }
  return rc;
}

int gm_get_basis(gm_handle h, double* dst) {
  if (!h || !dst) return GM_ERR_ARG;
  const size_t n = (size_t)h->n, m = (size_t)h->m, R = (size_t)h->R;
  const size_t bsz = h->prec == GM_FP64 ? 8 : 4;
  std::vector<unsigned char> raw(m * n * R * bsz);
  GM_CUDA(h, cudaMemcpyAsync(raw.data(), h->kp.V, raw.size(), cudaMemcpyDeviceToHost, h->stream));
  int rc = check_sync(h);
  if (rc) return rc;
  // device [m][n][R] in the storage type -> host n x m per right-hand side
  for (size_t j = 0; j < m; ++j)
    for (size_t i = 0; i < n; ++i)
      for (size_t r = 0; r < R; ++r) {
        const size_t q = (j * n + i) * R + r;
        double v;
        if (bsz == 8) {
          std::memcpy(&v, raw.data() + q * 8, 8);
        } else {
          float f;
          std::memcpy(&f, raw.data() + q * 4, 4);
          v = (double)f;
        }
        dst[(r * m + j) * n + i] = v;
      }
  return GM_OK;
}

int gm_get_y(gm_handle h, double* yr, double* yi) {
  if (!h) return GM_ERR_ARG;
  const size_t cnt = (size_t)h->m * h->R * h->C * h->nprob;
  if (yr) GM_CUDA(h, cudaMemcpyAsync(yr, h->kp.Yr, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (yi) GM_CUDA(h, cudaMemcpyAsync(yi, h->kp.Yi, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return check_sync(h);
}

int gm_set_y(gm_handle h, const double* yr, const double* yi) {
  if (!h || !yr || !yi) return fail(h, GM_ERR_ARG, "set_y: null argument");
  const size_t cnt = (size_t)h->m * h->R * h->C * h->nprob;
  GM_CUDA(h, cudaMemcpyAsync(h->kp.Yr, yr, cnt * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  GM_CUDA(h, cudaMemcpyAsync(h->kp.Yi, yi, cnt * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int rc = launch(h, gm::PH_COEF, 2);
  if (!rc) { h->have_y = true; h->have_coef = true; }
  return rc;
}

int gm_get_meff(gm_handle h, int* meff) {
  if (!h || !meff) return GM_ERR_ARG;
  int rc = check_sync(h);
  for (int r = 0; r < h->R * h->nprob; ++r) meff[r] = h->h_status[1 + r];
  return rc;
}

static int set_U_common(gm_handle h, const double* U, bool on_device) {
  if (!h) return GM_ERR_ARG;
  int rc = set_usol(h, U, on_device);
  if (rc) return rc;
  if (h->fe_cur == 0) h->fe_fwd_ok = false;   // the stored forward state is being replaced
  GM_CUDA(h, cudaMemsetAsync(h->kp.status, 0, sizeof(int), h->stream));
  GM_CUDA(h, cudaMemsetAsync(h->kp.bar, 0, (2 + 2 * (size_t)h->nprob) * sizeof(unsigned), h->stream));
  h->have_V = h->have_y = h->have_coef = false;
  return launch(h, gm::PH_DEFLATE, 0);
}

int gm_set_U(gm_handle h, const double* U_host) { return set_U_common(h, U_host, false); }

int gm_get_ode(gm_handle h, double* ode_host) {
  if (!h || !ode_host) return GM_ERR_ARG;
  GM_CUDA(h, cudaMemcpyAsync(ode_host, h->kp.ode, (size_t)h->n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return check_sync(h);
}

int gm_set_state(gm_handle h, const double* Usol_host, const double* ode_host) {
  if (!h || !Usol_host) return GM_ERR_ARG;
  if (ode_host)
    GM_CUDA(h, cudaMemcpyAsync(h->kp.ode, ode_host, (size_t)h->n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int rc = set_usol(h, Usol_host, false, false);   // Usol as gm_get_U returned it: no column scaling
  if (rc) return rc;
  if (h->fe_cur == 0) h->fe_fwd_ok = false;
  GM_CUDA(h, cudaMemsetAsync(h->kp.status, 0, sizeof(int), h->stream));
  GM_CUDA(h, cudaMemsetAsync(h->kp.bar, 0, (2 + 2 * (size_t)h->nprob) * sizeof(unsigned), h->stream));
  h->have_V = h->have_y = h->have_coef = false;
  return launch(h, gm::PH_DEFLATE, 0);
}

int gm_set_U_device(gm_handle h, const double* U_dev) { return set_U_common(h, U_dev, true); }

int gm_solve(gm_handle h) {
  if (!h) return GM_ERR_ARG;
  int rc = launch(h, gm::PH_LANCZOS | gm::PH_TRISOLVE | gm::PH_COEF | gm::PH_APPLY | gm::PH_APPLY_SET, 4);
  if (!rc) h->have_V = h->have_y = h->have_coef = true;
  return rc;
}

int gm_solve_host(gm_handle h, const double* b_host, double* x_host) {
  if (!h) return GM_ERR_ARG;
  int rc = gm_set_U(h, b_host);
  if (rc) return rc;
  rc = gm_solve(h);
  if (rc) return rc;
  return gm_get_solution(h, x_host);
}

int gm_fe_attach(gm_handle h, int64_t ntri, const int64_t* ent_ptr, const int32_t* ent_tri, const double* ent_coef,
                 const int64_t* tri_nodes, const double* tri_kc) {
  if (!h) return GM_ERR_ARG;
  if (!h->csr2sell) return fail(h, GM_ERR_STATE, "fe_attach: create the engine with keep_entry_map = 1");
  if (h->fe_ent_ptr) return fail(h, GM_ERR_STATE, "fe_attach: already attached");
  if (ntri <= 0 || ntri > INT32_MAX) return fail(h, GM_ERR_ARG, "fe_attach: ntri out of range");
  if (!ent_ptr || !ent_tri || !ent_coef || !tri_nodes || !tri_kc) return fail(h, GM_ERR_ARG, "fe_attach: null argument");
  const long long nnz = h->nnz;
  if (ent_ptr[0] != 0) return fail(h, GM_ERR_ARG, "fe_attach: ent_ptr[0] must be 0");
  for (long long t = 0; t < nnz; ++t)
    if (ent_ptr[t + 1] < ent_ptr[t]) return fail(h, GM_ERR_ARG, "fe_attach: ent_ptr not monotone");
  const long long nc = ent_ptr[nnz];
  for (long long p = 0; p < nc; ++p)
    if (ent_tri[p] < 0 || ent_tri[p] >= ntri) return fail(h, GM_ERR_ARG, "fe_attach: triangle index out of range");
  for (long long t = 0; t < 3 * ntri; ++t)
    if (tri_nodes[t] < -1 || tri_nodes[t] >= h->n) return fail(h, GM_ERR_ARG, "fe_attach: node index out of range");
  int rc;
  h->fe_ntri = ntri;
  if ((rc = dupload(h, &h->fe_ent_ptr, reinterpret_cast<const long long*>(ent_ptr), nnz + 1))) return rc;
  if ((rc = dupload(h, &h->fe_ent_tri, ent_tri, nc))) return rc;
  if ((rc = dupload(h, &h->fe_ent_coef, ent_coef, nc))) return rc;
  if ((rc = dupload(h, &h->fe_nodes, reinterpret_cast<const long long*>(tri_nodes), 3 * ntri))) return rc;
  if ((rc = dupload(h, &h->fe_kc, tri_kc, 9 * ntri))) return rc;
  if ((rc = dalloc(h, &h->fe_kappa, (size_t)ntri))) return rc;
  if ((rc = dalloc(h, &h->fe_dk, (size_t)ntri))) return rc;
  return GM_OK;
}

int gm_fe_assemble(gm_handle h, const double* kappa_dev) {
  if (!h || !kappa_dev) return GM_ERR_ARG;
  if (!h->fe_ent_ptr) return fail(h, GM_ERR_STATE, "fe_assemble before fe_attach");
  const long long nnz = h->nnz;
  const unsigned blocks = (unsigned)((nnz + 255) / 256);
  if (h->prec == GM_FP64)
    gm::k_fe_assemble<double><<<blocks, 256, 0, h->stream>>>(nnz, h->fe_ent_ptr, h->fe_ent_tri, h->fe_ent_coef, kappa_dev,
                                                             h->csr2sell, (double*)h->kp.val, h->scale_exp);
  else if (h->comp)
    gm::k_fe_assemble_rows<<<(unsigned)((h->n + 255) / 256), 256, 0, h->stream>>>(
        h->n, h->csr_ptr, h->kp.col, h->fe_ent_ptr, h->fe_ent_tri, h->fe_ent_coef, kappa_dev, h->csr2sell,
        (float*)h->kp.val, h->scale_exp, h->d_roww, h->row2slot, const_cast<float*>(h->kp.dlo));
  else
    gm::k_fe_assemble<float><<<blocks, 256, 0, h->stream>>>(nnz, h->fe_ent_ptr, h->fe_ent_tri, h->fe_ent_coef, kappa_dev,
                                                            h->csr2sell, (float*)h->kp.val, h->scale_exp);
  GM_CUDA(h, cudaGetLastError());
  h->launches++;
  h->have_V = h->have_y = h->have_coef = false;
  h->fe_fwd_ok = false;
  return h->sync_mode ? check_sync(h) : GM_OK;
}

}  // extern "C"

namespace {
// Y -> the lift coefficients of the gradient: yb'[j][q] = y_b,j[q] / w_j
// (w_j the true weight: the stored one times 2^se) and yg[j][q] = y_g,j[q];
// column j of each side's Y (m x C, column-major).
__global__ void k_fe_prep_y(int C, int m, const double* __restrict__ Yrb, const double* __restrict__ Yib,
                            const double* __restrict__ Yrg, const double* __restrict__ Yig,
                            const double* __restrict__ wts, int se, double2* __restrict__ yb, double2* __restrict__ yg) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= C * m) return;
  const int j = t / m, q = t % m;
  const double wr = ldexp(wts[j], se), wi = ldexp(wts[C + j], se);
  const double ar = Yrb[(long long)j * m + q], ai = Yib[(long long)j * m + q];
  const double den = wr * wr + wi * wi;
  yb[t] = make_double2((ar * wr + ai * wi) / den, (ai * wr - ar * wi) / den);
  yg[t] = make_double2(Yrg[(long long)j * m + q], Yig[(long long)j * m + q]);
}
}  // namespace

extern "C" {

// The gradient from the two Krylov states: Y of b (divided by the weights)
// and of g, the bases Vb, Vg (element (q, i) at V[(q n + i) vstride]) and
// their m_eff; then the shifted-polynomial Horner and the per-triangle sum.
static int fe_gradient_core(gm_handle h, const double* Yrb, const double* Yib, const double* Yrg, const double* Yig,
                            const void* Vb, const void* Vg, int vstride, const int* meff_b, const int* meff_g,
                            double* dkappa_dev) {
  const long long n = h->n;
  const int C = h->C, m = h->m, d = h->d;
  int rc;
  if (!h->fe_buf[0]) {
    // Zb, Zg (lifts) and two Horner ping-pong pairs, each n x C complex
    for (int t = 0; t < 6; ++t)
      if ((rc = dalloc(h, &h->fe_buf[t], (size_t)n * C))) return rc;
    if ((rc = dalloc(h, &h->fe_yb, (size_t)m * C))) return rc;
    if ((rc = dalloc(h, &h->fe_yg, (size_t)m * C))) return rc;
  }
  double2 *Zb = h->fe_buf[0], *Zg = h->fe_buf[1];
  double2 *Xb[2] = {h->fe_buf[2], h->fe_buf[3]}, *Xg[2] = {h->fe_buf[4], h->fe_buf[5]};
  k_fe_prep_y<<<(C * m + 255) / 256, 256, 0, h->stream>>>(C, m, Yrb, Yib, Yrg, Yig, h->kp.wts, h->scale_exp,
                                                           h->fe_yb, h->fe_yg);
  const unsigned lblocks = (unsigned)std::min<long long>((n + 255) / 256, 2LL * h->nsm);
  if (h->prec == GM_FP64)
    gm::k_fe_lift_ff<double><<<lblocks, 256, 0, h->stream>>>(n, m, C, (const double*)Vb, (const double*)Vg, vstride,
                                                             h->fe_yb, h->fe_yg, Zb, Zg, meff_b, meff_g);
  else
    gm::k_fe_lift_ff<float><<<lblocks, 256, 0, h->stream>>>(n, m, C, (const float*)Vb, (const float*)Vg, vstride,
                                                            h->fe_yb, h->fe_yg, Zb, Zg, meff_b, meff_g);
  h->launches += 2;
  // X = gs(0, j) Z; X = A X + gs(i, j) Z for i = 1..d  ->  R_j, S_j
  const unsigned hblocks = (unsigned)std::min<long long>((n + 7) / 8, 32LL * h->nsm);
  for (int i = 0; i <= d; ++i) {
    const int in = (i + 1) & 1, out = i & 1;
    if (h->prec == GM_FP64)
      gm::k_fe_horner<double><<<hblocks, 256, 0, h->stream>>>(n, C, d + 1, i, h->csr_ptr, h->csr2sell, h->kp.col,
                                                              (const double*)h->kp.val, h->kp.gs_re, h->kp.gs_im, Zb, Zg,
                                                              Xb[in], Xg[in], Xb[out], Xg[out], i == 0);
    else
      gm::k_fe_horner<float><<<hblocks, 256, 0, h->stream>>>(n, C, d + 1, i, h->csr_ptr, h->csr2sell, h->kp.col,
                                                             (const float*)h->kp.val, h->kp.gs_re, h->kp.gs_im, Zb, Zg,
                                                             Xb[in], Xg[in], Xb[out], Xg[out], i == 0);
    h->launches++;
  }
  gm::k_fe_grad<<<(unsigned)((h->fe_ntri + 127) / 128), 128, 0, h->stream>>>(h->fe_ntri, C, h->fe_nodes, h->fe_kc,
                                                                              Xb[d & 1], Xg[d & 1], dkappa_dev);
  GM_CUDA(h, cudaGetLastError());
  h->launches++;
  return GM_OK;
}

int gm_fe_gradient(gm_handle h, double* dkappa_dev) {
  if (!h || !dkappa_dev) return GM_ERR_ARG;
  if (!h->fe_nodes) return fail(h, GM_ERR_STATE, "fe_gradient before fe_attach");
  if (h->R != 2 || h->k != 0 || h->nprob != 1)
    return fail(h, GM_ERR_UNSUPPORTED, "fe_gradient needs nrhs = 2 (b, g) and no deflation");
  if (!h->have_y) return fail(h, GM_ERR_STATE, "fe_gradient needs build_subspace and lin_sys_solves for [b, g] first");
  const int C = h->C, m = h->m;
  int rc = fe_gradient_core(h, h->kp.Yr, h->kp.Yi, h->kp.Yr + (size_t)C * m, h->kp.Yi + (size_t)C * m, h->kp.V,
                            static_cast<const char*>(h->kp.V) + (h->prec == GM_FP64 ? sizeof(double) : sizeof(float)),
                            2, h->kp.meff, h->kp.meff + 1, dkappa_dev);
  if (rc) return rc;
  return h->sync_mode ? check_sync(h) : GM_OK;
}

// host (pageable or pinned) or device pointer: cudaMemcpyDefault resolves it
static bool host_memory(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged;
}

// U = [b, g] (g = 0 when null) from host or device memory, via the stage buffer
// nrhs = 1 adjoint engines: Krylov state slot s (basis, shifted solutions,
// alpha/beta, m_eff).  Slot 1 is allocated on first use.
static int fe_use_slot(gm_handle h, int s) {
  if (!h->fe_slot[0].V) h->fe_slot[0] = {h->kp.V, h->kp.Yr, h->kp.Yi, h->kp.aabb, h->kp.meff};
  if (s == 1 && !h->fe_slot[1].V) {
    const size_t bsz = h->prec == GM_FP64 ? sizeof(double) : sizeof(float);
    unsigned char* V;
    gm_engine::FeSlot t{};
    int rc;
    if ((rc = dalloc(h, &V, (size_t)h->m * h->n * bsz))) return rc;
    t.V = V;
    if ((rc = dalloc(h, &t.Yr, (size_t)h->m * h->C))) return rc;
    if ((rc = dalloc(h, &t.Yi, (size_t)h->m * h->C))) return rc;
    if ((rc = dalloc(h, &t.aabb, (size_t)(h->m + 1) * 2))) return rc;
    if ((rc = dalloc(h, &t.meff, 1))) return rc;
    h->fe_slot[1] = t;
  }
  const gm_engine::FeSlot& t = h->fe_slot[s];
  h->kp.V = t.V; h->kp.Yr = t.Yr; h->kp.Yi = t.Yi; h->kp.aabb = t.aabb; h->kp.meff = t.meff;
  h->fe_cur = s;
  return GM_OK;
}

// kappa -> A(kappa), then a solve for U (nrhs = 1: b or g into the current
// slot; nrhs = 2: [b, g], g = 0 when null)
static int fe_assemble_from(gm_handle h, const double* kappa) {
  if (!h->fe_kappa) return fail(h, GM_ERR_STATE, "fe_forward/fe_backward before fe_attach");
  if (!kappa) return fail(h, GM_ERR_ARG, "fe_forward/fe_backward: null kappa");
  GM_CUDA(h, cudaMemcpyAsync(h->fe_kappa, kappa, (size_t)h->fe_ntri * sizeof(double), cudaMemcpyDefault, h->stream));
  h->fe_fwd_ok = false;
  return gm_fe_assemble(h, h->fe_kappa);
}

static int fe_solve_for(gm_handle h, const double* b, const double* g) {
  if (!b) return fail(h, GM_ERR_ARG, "fe_forward/fe_backward: null right-hand side");
  const size_t nb = (size_t)h->n * sizeof(double);
  GM_CUDA(h, cudaMemcpyAsync(h->stage, b, nb, cudaMemcpyDefault, h->stream));
  if (h->R == 2) {
    if (g)
      GM_CUDA(h, cudaMemcpyAsync(h->stage + h->n, g, nb, cudaMemcpyDefault, h->stream));
    else
      GM_CUDA(h, cudaMemsetAsync(h->stage + h->n, 0, nb, h->stream));
  }
  int rc = set_U_common(h, h->stage, true);
  return rc ? rc : gm_solve(h);
}

// column c of the solution (interleaved [n][R]) to dst (host or device)
static int fe_store_col(gm_handle h, int c, double* dst) {
  const long long total = h->n * h->R;
  k_pack_out<<<(unsigned)((total + 255) / 256), 256, 0, h->stream>>>(h->kp.S, h->stage, h->n, h->R);
  GM_CUDA(h, cudaGetLastError());
  h->launches++;
  GM_CUDA(h, cudaMemcpyAsync(dst, h->stage + (size_t)c * h->n, (size_t)h->n * sizeof(double), cudaMemcpyDefault,
                             h->stream));
  return GM_OK;
}

static int fe_check(gm_handle h) {
  if (!h->fe_kappa) return fail(h, GM_ERR_STATE, "fe_forward/fe_backward before fe_attach");
  if (h->R != 1 && h->R != 2) return fail(h, GM_ERR_UNSUPPORTED, "fe_forward/fe_backward need nrhs = 1 or 2");
  if (h->k != 0 || h->nprob != 1) return fail(h, GM_ERR_UNSUPPORTED, "fe adjoint: no deflation, one problem");
  return GM_OK;
}

int gm_fe_forward(gm_handle h, const double* kappa, const double* b, double* x) {
  if (!h) return GM_ERR_ARG;
  if (!x) return fail(h, GM_ERR_ARG, "fe_forward: null x");
  int rc = fe_check(h);
  if (!rc && h->R == 1) rc = fe_use_slot(h, 0);
  if (!rc) rc = fe_assemble_from(h, kappa);
  if (!rc) rc = fe_solve_for(h, b, nullptr);
  if (!rc) rc = fe_store_col(h, 0, x);
  if (rc) return rc;
  h->fe_fwd_ok = h->R == 1;
  return (h->sync_mode || host_memory(x)) ? check_sync(h) : GM_OK;
}

// backward with the b state in slot 0 (nrhs = 1) or recomputed with g (nrhs = 2)
static int fe_backward_impl(gm_handle h, bool reuse, const double* kappa, const double* b, const double* g,
                            double* dkappa, double* db) {
  if (!g || !dkappa) return fail(h, GM_ERR_ARG, "fe_backward: null g or dkappa");
  int rc = fe_check(h);
  if (rc) return rc;
  const int saved = h->sync_mode;
  h->sync_mode = 0;
  if (h->R == 2) {
    if (!(rc = fe_assemble_from(h, kappa)) && !(rc = fe_solve_for(h, b, g))) rc = gm_fe_gradient(h, h->fe_dk);
    if (!rc && db) rc = fe_store_col(h, 1, db);
  } else {
    if (!reuse || !h->fe_fwd_ok) {
      // recompute b's Krylov state into slot 0
      if (!(rc = fe_use_slot(h, 0)) && !(rc = fe_assemble_from(h, kappa))) rc = fe_solve_for(h, b, nullptr);
      if (!rc) h->fe_fwd_ok = true;
    }
    if (!rc) rc = fe_use_slot(h, 1);
    if (!rc) rc = fe_solve_for(h, g, nullptr);
    if (!rc && db) rc = fe_store_col(h, 0, db);
    if (!rc) {
      const gm_engine::FeSlot &sb = h->fe_slot[0], &sg = h->fe_slot[1];
      rc = fe_gradient_core(h, sb.Yr, sb.Yi, sg.Yr, sg.Yi, sb.V, sg.V, 1, sb.meff, sg.meff, h->fe_dk);
    }
    const int rc2 = fe_use_slot(h, 0);
    if (!rc) rc = rc2;
  }
  h->sync_mode = saved;
  if (rc) return rc;
  GM_CUDA(h, cudaMemcpyAsync(dkappa, h->fe_dk, (size_t)h->fe_ntri * sizeof(double), cudaMemcpyDefault, h->stream));
  return (h->sync_mode || host_memory(dkappa) || (db && host_memory(db))) ? check_sync(h) : GM_OK;
}

int gm_fe_backward(gm_handle h, const double* kappa, const double* b, const double* g, double* dkappa, double* db) {
  if (!h) return GM_ERR_ARG;
  return fe_backward_impl(h, false, kappa, b, g, dkappa, db);
}

int gm_fe_backward_stored(gm_handle h, const double* g, double* dkappa, double* db) {
  if (!h) return GM_ERR_ARG;
  if (h->R != 1) return fail(h, GM_ERR_UNSUPPORTED, "fe_backward_stored needs an nrhs = 1 engine");
  if (!h->fe_fwd_ok) return fail(h, GM_ERR_STATE, "fe_backward_stored without a preceding fe_forward");
  return fe_backward_impl(h, true, nullptr, nullptr, g, dkappa, db);
}

int gm_time_loop(gm_handle h, int nsteps, int mode, int use_graph) {
  if (!h) return GM_ERR_ARG;
  if (nsteps < 0 || (mode != 0 && mode != 1)) return fail(h, GM_ERR_ARG, "time_loop: nsteps >= 0 and mode 0 or 1");
  if (h->R != 2) return fail(h, GM_ERR_ARG, "time_loop needs nrhs = 2 (solution and reaction columns)");
  // Stream capture is not possible on the legacy default stream nor on the
  // per-thread default stream: refuse before any state changes.
  if (use_graph && (h->stream == cudaStreamLegacy || h->stream == cudaStreamPerThread))
    return fail(h, GM_ERR_ARG, "time_loop: a CUDA graph needs a created stream (gm_set_stream with the legacy or "
                               "per-thread default stream cannot be captured)");
  const int solve = gm::PH_LANCZOS | gm::PH_TRISOLVE | gm::PH_COEF | gm::PH_APPLY | gm::PH_APPLY_SET;
  const int upd = (mode == 0 ? gm::PH_UPDATE_FKPP : gm::PH_UPDATE_FHN) | gm::PH_DEFLATE;
  // launches inside the loop do not synchronise; the caller's sync mode is
  // restored on every exit below
  const int saved = h->sync_mode;
  h->sync_mode = 0;
  int rc = GM_OK;
  cudaError_t st = cudaSuccess;
  if (!use_graph) {
    for (int t = 0; t < nsteps && rc == GM_OK; ++t) {
      rc = launch(h, solve, 4);
      if (rc == GM_OK) rc = launch(h, upd, 0);
    }
  } else {
    if (!h->loop_exec || h->loop_steps != nsteps || h->loop_mode != mode) {
      if (h->loop_exec) {
        cudaGraphExecDestroy(h->loop_exec);
        h->loop_exec = nullptr;
      }
      cudaGraph_t graph = nullptr;
      st = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
      if (st != cudaSuccess) rc = cuda_fail(h, st, "cudaStreamBeginCapture");
      if (rc == GM_OK) {
        h->capturing = true;
        for (int t = 0; t < nsteps && rc == GM_OK; ++t) {
          rc = launch(h, solve, 4);
          if (rc == GM_OK) rc = launch(h, upd, 0);
        }
        h->capturing = false;
        st = cudaStreamEndCapture(h->stream, &graph);
        if (rc == GM_OK && st != cudaSuccess) rc = cuda_fail(h, st, "cudaStreamEndCapture");
        if (rc == GM_OK) {
          st = cudaGraphInstantiate(&h->loop_exec, graph, 0);
          if (st != cudaSuccess) rc = cuda_fail(h, st, "cudaGraphInstantiate");
        }
        if (graph) cudaGraphDestroy(graph);
      }
      if (rc == GM_OK) {
        h->loop_steps = nsteps;
        h->loop_mode = mode;
      } else {
        h->loop_exec = nullptr;
        h->loop_steps = h->loop_mode = -1;
      }
    }
    if (rc == GM_OK && (st = cudaEventRecord(h->ev[4][0], h->stream)) != cudaSuccess) rc = cuda_fail(h, st, "cudaEventRecord");
    if (rc == GM_OK && (st = cudaGraphLaunch(h->loop_exec, h->stream)) != cudaSuccess) rc = cuda_fail(h, st, "cudaGraphLaunch");
    if (rc == GM_OK && (st = cudaEventRecord(h->ev[4][1], h->stream)) != cudaSuccess) rc = cuda_fail(h, st, "cudaEventRecord");
    if (rc == GM_OK) h->ev_used[4] = true;
  }
  h->sync_mode = saved;
  if (rc != GM_OK) return rc;
  h->have_V = h->have_y = h->have_coef = true;
  if (saved) rc = check_sync(h);
  return rc;
}

int gm_sync(gm_handle h) {
  if (!h) return GM_ERR_ARG;
  return check_sync(h);
}

int gm_set_stream(gm_handle h, void* stream) {
  if (!h) return GM_ERR_ARG;
  GM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->stream = stream ? reinterpret_cast<cudaStream_t>(stream) : h->own_stream;
  return GM_OK;
}

int gm_phase_times(gm_handle h, float* ms) {
  if (!h || !ms) return GM_ERR_ARG;
  GM_CUDA(h, cudaStreamSynchronize(h->stream));
  for (int s = 0; s < 5; ++s) {
    ms[s] = 0.f;
    if (h->ev_used[s]) GM_CUDA(h, cudaEventElapsedTime(&ms[s], h->ev[s][0], h->ev[s][1]));
  }
  return GM_OK;
}

int gm_info(gm_handle h, int64_t* info) {
  if (!h || !info) return GM_ERR_ARG;
  info[0] = h->n; info[1] = h->R; info[2] = h->m; info[3] = h->d; info[4] = h->C; info[5] = h->k;
  info[6] = h->prec; info[7] = h->G; info[8] = h->threads; info[9] = h->padded;
  info[10] = (int64_t)h->bytes; info[11] = h->launches;
  info[12] = h->nprob;
  info[13] = h->kp.mpk;
  info[14] = h->kp.pf_vals;
  info[15] = h->kp.reorth;
  return GM_OK;
}

int gm_info_ex(gm_handle h, int64_t* info, int count) {
  if (!h || !info || count < 0) return GM_ERR_ARG;
  int64_t v[GM_INFO_EX_COUNT];
  if (int rc = gm_info(h, v)) return rc;
  v[16] = h->l2_window ? (int64_t)h->window.num_bytes : 0;
  v[17] = h->kp.stage_cap;
  v[18] = h->kp.dep_mode;
  for (int i = 0; i < count && i < GM_INFO_EX_COUNT; ++i) info[i] = v[i];
  return GM_OK;
}

const char* gm_last_error(gm_handle h) {
  return h ? h->err.c_str() : g_create_error.c_str();
}

const char* gm_version(void) { return "gpumatfun-gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
