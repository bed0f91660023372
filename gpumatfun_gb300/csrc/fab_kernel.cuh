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
//   hpart, hblk  (Gram-Schmidt only) per-block partial dots [2][m+8][R][G]
//                and each block's totals [G][m+1][R]
#pragma once
#include "fab_common.cuh"

namespace gm {

enum Phase : int {
  PH_LANCZOS = 1, PH_TRISOLVE = 2, PH_COEF = 4, PH_APPLY = 8,
  PH_UPDATE_FKPP = 16, PH_UPDATE_FHN = 32, PH_DEFLATE = 64,
  PH_APPLY_SET = 128,  // apply writes X = lift (fused solve) instead of X += lift
  PH_MPK = 256,        // compile-time only: entry points with matrix-powers Horner passes
  PH_REORTH = 512      // compile-time only: entry points with Gram-Schmidt reorthogonalisation
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
  const float* dlo;     // mixed: per-slot-row diagonal compensation (slot order), or null
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
  unsigned* bar;    // 64-bit barrier arrival counters: [0,1] whole grid, [2+2p, 3+2p] group p
  const int* blk_slice;       // [G+1] slice range owned by each block
  const int* dep_ptr;         // [G+1] neighbour list of each block
  const int* dep_idx;
  unsigned long long* prog;   // [G] pass progress flags
  unsigned long long epoch;   // launch counter
  int dep_mode;               // 1: neighbour waits between SpMV passes, 0: grid barriers
  int nprob;                  // independent problems in this launch (0 or 1: one problem)
  const int* blk_prob;        // [G] problem of each block
  const int* prob_blk0;       // [nprob+1] first block of each problem
  const long long* prob_row0; // [nprob+1] first row of each problem
  int stage_cap;              // >0: stage each slice's column indices in shared memory by TMA
  int pf_vals;                // >0: L2 bulk prefetch of the next slice's values (bytes per value)
  // Two Horner levels per pass (matrix powers): per block, the rows its rows
  // reference outside its own range (halo), the SELL column indices in block-
  // local numbering (own rows first, then the halo), and the offset of the
  // local vector in dynamic shared memory.  Enabled only without a row perm.
  int mpk;
  long long su_off;
  const long long* halo_ptr;  // [G + 1]
  const int* halo_rows;
  const int* lcol;            // per SELL slot
  // Gram-Schmidt reorthogonalisation of each Lanczos vector against the
  // stored basis: 0 = none (the reference's recurrence), 1 = CGS, 2 = CGS2
  int reorth;
  double* hpart;    // [2][m + 8][R][G] per-block partial dots
  double* hblk;     // [G][m + 1][R] each block's totals
  int* status;
  int* meff;        // [R]
  unsigned long long timeout_ns;
};

// ------------------------------------------------------------------ helpers
// Thread coordinates, recomputed from the special registers on use rather
// than held in registers across the passes (the kernel is register-bound).
struct Ctx {
  int G;
  __device__ explicit Ctx(int G_) : G(G_) {}
  __device__ __forceinline__ int b() const { return blockIdx.x; }
  __device__ __forceinline__ int tid() const { return threadIdx.x; }
  __device__ __forceinline__ int nt() const { return blockDim.x; }
  __device__ __forceinline__ int lane() const { return threadIdx.x & 31; }
  __device__ __forceinline__ int warp() const { return threadIdx.x >> 5; }
  __device__ __forceinline__ int nw() const { return blockDim.x >> 5; }
  __device__ __forceinline__ long long gw() const { return (long long)blockIdx.x * nw() + warp(); }
  __device__ __forceinline__ long long tw() const { return (long long)G * nw(); }
  __device__ __forceinline__ long long gt() const { return (long long)blockIdx.x * blockDim.x + threadIdx.x; }
  __device__ __forceinline__ long long tt() const { return (long long)G * blockDim.x; }
};

__device__ __forceinline__ DepSync make_dep(const KParams& kp) {
  return DepSync{kp.prog, kp.dep_ptr, kp.dep_idx, kp.status, kp.epoch << 20, kp.timeout_ns};
}

// Orders consecutive SpMV passes: after pass pc (published), the next
// gathering pass waits for the neighbours' pass pc (or a grid barrier).  One
// PassSync lives for the whole launch and is shared by all phases, so pass
// numbers keep increasing across phases: a phase that restarted at 0 would
// find its waits already satisfied by flags published earlier in the launch.
struct PassSync {
  int mode;
  int p;        // problem (group) whose barrier orders the passes without waits
  unsigned pc;
  __device__ void done(const KParams& kp) {
    ++pc;
    if (mode) make_dep(kp).publish(pc);
  }
  __device__ bool before_next(const KParams& kp);
};

// Arrival counter of problem group p's barrier (words 2 + 2p, 3 + 2p of
// kp.bar), or of the whole grid's (words 0, 1) for p = -1.
__device__ __forceinline__ unsigned long long* bar_word(const KParams& kp, int p) {
  return reinterpret_cast<unsigned long long*>(kp.bar + 2 + 2 * p);
}

// The block's problem group.  A launch can carry several independent
// problems (a batch); each owns a contiguous range of blocks, rows and SELL
// slices, its own barrier and its own reductions.  One problem is the
// single-group case.
struct Grp {
  int p, gb, Gp, bl;
  __device__ Grp(const KParams& kp, const Ctx& c) {
    if (kp.nprob > 0) {
      p = kp.blk_prob[c.b()];
      gb = kp.prob_blk0[p];
      Gp = kp.prob_blk0[p + 1] - gb;
    } else {
      p = 0; gb = 0; Gp = c.G;
    }
    bl = c.b() - gb;
  }
  // rows of this problem and the group-strided row loop (recomputed on use)
  __device__ __forceinline__ long long r0(const KParams& kp) const { return kp.nprob > 0 ? kp.prob_row0[p] : 0; }
  __device__ __forceinline__ long long r1(const KParams& kp) const { return kp.nprob > 0 ? kp.prob_row0[p + 1] : kp.n; }
  __device__ __forceinline__ long long gt(const KParams& kp) const {
    return r0(kp) + (long long)bl * blockDim.x + threadIdx.x;
  }
  __device__ __forceinline__ long long tt() const { return (long long)Gp * blockDim.x; }
  // barrier over this group's blocks (words 2 + 2p, 3 + 2p of kp.bar)
  __device__ GridBar bar(const KParams& kp) const {
    return GridBar{bar_word(kp, p), kp.status, (unsigned)Gp, kp.timeout_ns};
  }
};

__device__ __forceinline__ GridBar group_bar(const KParams& kp, int p) {
  const unsigned Gp = kp.nprob > 0 ? (unsigned)(kp.prob_blk0[p + 1] - kp.prob_blk0[p]) : (unsigned)kp.G;
  return GridBar{bar_word(kp, p), kp.status, Gp, kp.timeout_ns};
}

__device__ __forceinline__ bool PassSync::before_next(const KParams& kp) {
  return mode ? make_dep(kp).wait(pc) : group_bar(kp, p).sync();
}

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
// Chunk width: one column index, one value and R gathered entries are live
// per chunk element across the gathers.  What the SpMV needs is loads in
// flight per SM, and resident warps supply them more cheaply than wide
// chunks: every right-hand-side count runs its kernels at the residency
// below with the chunk width that fits it.
//   R = 1: three 512-thread blocks per SM (GM_MINB1, 42 registers), one entry
//          per chunk; against two blocks with four entries: 3D 256^3 mixed
//          40.6 vs 51.0 ms per solve, FP64 50.0 vs 63.6 ms, 1M-node FE disk
//          FP64 21.2 vs 22.1 ms, mixed equal (16.5 ms), despite the spills at
//          42 registers.  The matrix-powers and Gram-Schmidt entry points,
//          whose passes hold more state, stay at two blocks (GM_MINB1X): the
//          250k-node adjoint 288 vs 325 ms per gradient with three.
//   R = 2: two blocks per SM (GM_MINB, 64 registers), two entries per chunk,
//          the widest without spills there.
//   R = 4: two blocks per SM (GM_MINB4), one entry per chunk; against one
//          block with three entries at 128 registers (1M-node FE disk: mixed
//          40.0 vs 48.7 ms per launch, FP64 58.6 vs 64.9 ms).  The mixed
//          policy's Lanczos entry points run three blocks (GM_MINB4M): 1M-node
//          disk 39.0 vs 40.5 ms, 64-problem batch 19.0 vs 20.3 ms, where FP64
//          at three blocks is slower (63.1 vs 58.8 ms).
#ifndef GM_CH1
#define GM_CH1 1
#endif
#ifndef GM_CH2
#define GM_CH2 2
#endif
#ifndef GM_CH4
#define GM_CH4 1
#endif
#ifndef GM_CH4F
#define GM_CH4F 1
#endif
template <class VT, class XT, int R>
struct ChunkWidth {
  static constexpr int value = R == 1 ? GM_CH1 : (R == 2 ? GM_CH2 : (sizeof(VT) == 8 ? GM_CH4 : GM_CH4F));
};

// acc[r] += aa[u] * xv[u][r] for u < N, in order.
template <class Pol, int R, class XT, int N, int CH>
__device__ __forceinline__ void acc_first(typename Pol::AT (&acc)[R], const typename Pol::VT (&aa)[CH],
                                          const XT (&xv)[CH][R]) {
#pragma unroll
  for (int u = 0; u < N; ++u)
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = Pol::acc(acc[r], aa[u], xv[u][r]);
}

// One entry per step over a slice row: column index, value, gather, product.
// The column source (shared-memory stage or global memory) is fixed for the
// whole row, addresses advance by a slot column (32 entries) per step, and the
// mixed engine's diagonal compensation (entry 0 is the diagonal) is peeled
// out of the loop: the kernel is issue-bound, and these are the per-entry
// instructions that are not the product itself.
template <class Pol, int R, class XT, bool kStaged>
__device__ __forceinline__ void row_entries1(const int* __restrict__ cp, const typename Pol::VT* __restrict__ vp,
                                             int len, const XT* __restrict__ x, float dl,
                                             typename Pol::AT (&acc)[R]) {
  if (len <= 0) return;
  XT xv[R];
  int cc = kStaged ? cp[0] : __ldg(cp);
  typename Pol::VT a = ld_val(vp);
  VecIO<R>::ld(x + (long long)cc * R, xv);
  if constexpr (Pol::kMixed) {
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = Pol::acc(acc[r], dl, xv[r]);
  }
#pragma unroll
  for (int r = 0; r < R; ++r) acc[r] = Pol::acc(acc[r], a, xv[r]);
  for (int jj = 1; jj < len; ++jj) {
    cp += 32;
    vp += 32;
    cc = kStaged ? cp[0] : __ldg(cp);
    a = ld_val(vp);
    VecIO<R>::ld(x + (long long)cc * R, xv);
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = Pol::acc(acc[r], a, xv[r]);
  }
}

template <class Pol, int R, class XT>
__device__ __forceinline__ void spmv_slot(const KParams& kp, long long s, int lane, const XT* __restrict__ x,
                                          typename Pol::AT (&acc)[R], const int* scol = nullptr,
                                          const int* colarr = nullptr) {
  using VT = typename Pol::VT;
  constexpr int CH = ChunkWidth<VT, XT, R>::value;
  const long long base = kp.slice_off[s];
  const int len = (int)((kp.slice_off[s + 1] - base) >> 5);
  if constexpr (CH == 1) {
    // same products in the same order as the chunked loop below
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = Pol::zero();
    float dl = 0.f;
    if constexpr (Pol::kMixed) {
      if (kp.dlo) dl = __ldg(kp.dlo + s * 32 + lane);
    }
    const VT* vp = reinterpret_cast<const VT*>(kp.val) + base + lane;
    if (scol)
      row_entries1<Pol, R, XT, true>(scol + lane, vp, len, x, dl, acc);
    else
      row_entries1<Pol, R, XT, false>((colarr ? colarr : kp.col) + base + lane, vp, len, x, dl, acc);
    return;
  }
  // Chunks of two or more entries (two right-hand sides; tuning builds).
  // Column indices from the shared-memory stage when the slice is staged,
  // else from global memory, chosen by a warp-uniform branch per chunk;
  // values from global memory (read-only path; with value prefetch they are
  // already on their way into L2).  Measured against the two other shapes of
  // this loop (a per-load select of the source, and one generic pointer for
  // both): 1M FE disk FP64 44.6 vs 42.8 / 42.4 solves/s, mixed 57.1 vs 55.7;
  // the generic pointer is faster only for FP64 on the HBM-streamed 3D
  // matrix (17.2 vs 15.8), whose reference precision is the mixed engine
  // (19.6 vs 19.3 here).
  const int* gcp = (colarr ? colarr : kp.col) + base + lane;
  const VT* vp = reinterpret_cast<const VT*>(kp.val) + base + lane;
#pragma unroll
  for (int r = 0; r < R; ++r) acc[r] = Pol::zero();
  // Mixed engine: diagonal compensation of the FP32-stored values, c_r x_r.
  // The engine stores every row's diagonal entry first (slice column 0), so
  // x_r is the first chunk's first gather; pad lanes carry dl = 0.
  float dl = 0.f;
  if constexpr (Pol::kMixed) {
    if (kp.dlo) dl = __ldg(kp.dlo + s * 32 + lane);
  }
  for (int jj = 0; jj < len; jj += CH) {
    int cc[CH];
    VT aa[CH];
    if (scol) {
#pragma unroll
      for (int u = 0; u < CH; ++u) cc[u] = jj + u < len ? scol[(jj + u) * 32 + lane] : 0;
    } else {
#pragma unroll
      for (int u = 0; u < CH; ++u) cc[u] = jj + u < len ? __ldg(gcp + (long long)(jj + u) * 32) : 0;
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) aa[u] = jj + u < len ? ld_val(vp + (long long)(jj + u) * 32) : (VT)0;
    XT xv[CH][R];
#pragma unroll
    for (int u = 0; u < CH; ++u)
      if (jj + u < len) VecIO<R>::ld(x + (long long)cc[u] * R, xv[u]);
    if constexpr (Pol::kMixed) {
      if (jj == 0) {
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] = Pol::acc(acc[r], dl, xv[0][r]);
      }
    }
    // The chunk's valid products, in order.  In the guarded loop (FP64) the
    // compiler turns the guard into a select and issues the missing products
    // with a zero value: on a 7-column slice 8/7 of the FMAs (ncu DFMA count),
    // which measured faster than branching to exact counts (1M FE disk 41.5
    // vs 40.0 solves/s, 3D 17.0 vs 16.1).  The mixed engine's float-float
    // products cost ~10 instructions each on an issue-bound kernel, so it
    // branches to exactly the valid ones (+2-4%).
    if constexpr (!Pol::kMixed) {
#pragma unroll
      for (int u = 0; u < CH; ++u)
        if (jj + u < len) {
#pragma unroll
          for (int r = 0; r < R; ++r) acc[r] = Pol::acc(acc[r], aa[u], xv[u][r]);
        }
      continue;
    }
    const int cnt = len - jj;
    if (cnt >= CH) {
      acc_first<Pol, R, XT, CH>(acc, aa, xv);
    } else {
      if constexpr (CH > 1) if (cnt == 1) acc_first<Pol, R, XT, 1>(acc, aa, xv);
      if constexpr (CH > 2) if (cnt == 2) acc_first<Pol, R, XT, 2>(acc, aa, xv);
      if constexpr (CH > 3) if (cnt == 3) acc_first<Pol, R, XT, 3>(acc, aa, xv);
      if constexpr (CH > 4) if (cnt >= 4) {
#pragma unroll
        for (int u = 0; u < CH; ++u)
          if (u < cnt) {
#pragma unroll
            for (int r = 0; r < R; ++r) acc[r] = Pol::acc(acc[r], aa[u], xv[u][r]);
          }
      }
    }
  }
}

// A Horner / lift buffer entry as the policy's accumulator.
template <class Pol> __device__ __forceinline__ typename Pol::AT h_load_at(const typename Pol::HT& h) {
  if constexpr (Pol::kMixed) {
    return {h.x, h.y};
  } else {
    return h;
  }
}

// Per-warp double-buffered staging of SELL column indices.  Lane 0 issues a
// TMA bulk copy of the next slice's column block (128 bytes per slice column,
// contiguous in the SELL layout) into shared memory while the warp computes
// the current slice, so a slice costs one global round trip (values and x
// gathers together) instead of two.  Dynamic shared memory holds, per warp,
// two mbarriers and two stages of stage_cap * 32 ints.
// After a timed-out wait, how long a warp still waits for its TMA copy in
// flight before leaving (independent of the configured wait limit, which
// may be short): a copy completes in microseconds unless the GPU is failing.
constexpr unsigned long long kDrainNs = 2000000000ull;

struct ColStage {
  unsigned st;   // bit k: parity of stage k's next completion; bit 2 + k: stage k holds a copy
  int cap;

  // stage k's mbarrier and buffer for this warp, derived from the warp index
  __device__ __forceinline__ static unsigned char* base() {
    extern __shared__ __align__(128) unsigned char dsm[];
    return dsm;
  }
  __device__ __forceinline__ unsigned long long* bar(int k) const {
    return reinterpret_cast<unsigned long long*>(base()) + 2 * (threadIdx.x >> 5) + k;
  }
  __device__ __forceinline__ int* buf(int k) const {
    int* bufs = reinterpret_cast<int*>(base() + 16 * (blockDim.x >> 5));
    return bufs + (long long)(2 * (threadIdx.x >> 5) + k) * cap * 32;
  }

  __device__ void init(const KParams& kp, const Ctx& c) {
    cap = kp.stage_cap;
    st = 0u;
    if (cap <= 0) return;
    if (c.lane() == 0) {
      mbar_init(bar(0), 1);
      mbar_init(bar(1), 1);
      mbar_init_fence();
    }
    __syncwarp();
  }

  // Per warp: the vector whose slice rows the current pass's row epilogue
  // reads and the gathers of x do not bring into cache (set by lane 0 at the
  // start of a pass, read by lane 0 when it issues a slice), or null.  Kept
  // in shared memory rather than a register: the SpMV loop is register-bound.
  __device__ __forceinline__ static const void** row_pf_slot() {
    __shared__ const void* s_row_pf[32];
    return s_row_pf + (threadIdx.x >> 5);
  }

  // stage k <- columns of slice s (lane 0 issues; warp-uniform bookkeeping).
  // With RowB > 0 (bytes per row of the epilogue's vector) and a vector set
  // in row_pf_slot(), that vector's 32 rows of the slice are prefetched into
  // L2 with the values, so the epilogue's load after the slice's SpMV is an
  // L2 hit instead of a full HBM round trip.  Rows of a slice are
  // consecutive only without a row perm.
  template <unsigned RowB = 0>
  __device__ void issue(const KParams& kp, int k, long long s, int lane) {
    if (cap <= 0) return;
    const long long base = kp.slice_off[s];
    const int len = (int)((kp.slice_off[s + 1] - base) >> 5);
    if (len <= 0 || len > cap) return;
    if (lane == 0) {
      unsigned long long* b = bar(k);
      const unsigned bytes = 128u * (unsigned)len;
      mbar_arrive_expect_tx(b, bytes);
      tma_bulk_g2s(buf(k), kp.col + base, bytes, b);
      // the slice's values, which the warp reads right after the columns,
      // start their way from HBM into L2 now
      if (kp.pf_vals) {
        tma_bulk_prefetch_l2(static_cast<const unsigned char*>(kp.val) + base * kp.pf_vals,
                             (unsigned)kp.pf_vals * 32u * (unsigned)len);
        if constexpr (RowB > 0) {
          const void* rp = *row_pf_slot();
          if (rp && !kp.perm) {
            // rows s*32 .. min(s*32 + 32, n) of an n-row buffer: the start is
            // a multiple of 32 rows (aligned), the length rounded down to
            // whole 16-byte units
            const long long r0 = s * 32;
            const long long nr = kp.n - r0 < 32 ? kp.n - r0 : 32;
            const unsigned pb = nr > 0 ? (unsigned)(nr * RowB) & ~15u : 0u;
            if (pb > 0) tma_bulk_prefetch_l2(static_cast<const unsigned char*>(rp) + r0 * RowB, pb);
          }
        }
      }
    }
    st |= 4u << k;
  }

  // Waits for stage k; returns its buffer, or nullptr when the slice is read
  // from global memory (not staged) or the wait ran out (status recorded).
  __device__ const int* ready(const KParams& kp, int k, int lane) {
    if (!(st & (4u << k))) return nullptr;
    unsigned long long* b = bar(k);
    const unsigned par = (st >> k) & 1u;
    unsigned long long start = 0;
    bool timed_out = false;
    while (!mbar_try_wait(b, par)) {
      const unsigned long long now = global_timer_ns();
      if (start == 0) {
        start = now;
      } else if (!timed_out && now - start > kp.timeout_ns) {
        if (lane == 0) atomicCAS(kp.status, 0, (int)ST_TIMEOUT);
        timed_out = true;
        start = now;  // keep waiting a bounded time for the copy in flight
      } else if (timed_out && now - start > kDrainNs) {
        break;
      }
    }
    st ^= 1u << k;
    st &= ~(4u << k);
    return timed_out ? nullptr : buf(k);
  }

  // all lanes are done reading stage k before a later copy overwrites it
  __device__ void release() {
    if (cap <= 0) return;
    fence_proxy_async_smem();
    __syncwarp();
  }
};

// One SpMV pass over the block's slices: z = A x for the slice rows, then
// epi(s, z) for the row epilogue.  rowpf: the [n][R] storage-precision
// vector the epilogue reads at the slice rows and that the gathers of x do
// not bring into cache (prefetched one slice ahead with the values when the
// matrix streams from HBM), or null.
template <class Pol, int R, class XT, class Epi>
__device__ __forceinline__ bool spmv_pass(const KParams& kp, const Ctx& c, ColStage& cs, const XT* x, Epi&& epi,
                                          PassSync* wait = nullptr, const typename Pol::BT* rowpf = nullptr) {
  using AT = typename Pol::AT;
  // (one and two right-hand sides: with four, the 1M-node FE disk's mixed
  // launch measured 2.5% slower with the row prefetch, 3D 256^3 mixed with one
  // right-hand side 2% faster)
  constexpr unsigned kRowB = R <= 2 ? (unsigned)(R * sizeof(typename Pol::BT)) : 0u;
  const long long sb = kp.blk_slice[c.b()], se = kp.blk_slice[c.b() + 1];
  long long s = sb + c.warp();
  if (kRowB > 0 && c.lane() == 0) *ColStage::row_pf_slot() = rowpf;
  if (s < se) cs.issue<kRowB>(kp, 0, s, c.lane());
  // the ordering wait on the previous pass comes after the first column copy
  // is issued: the matrix does not depend on it, so the copy overlaps the wait
  if (wait && !wait->before_next(kp)) {
    if (s < se) cs.ready(kp, 0, c.lane());   // bounded drain of the copy in flight
    return false;
  }
  int k = 0;
  for (; s < se; s += c.nw(), k ^= 1) {
    const long long sn = s + c.nw();
    if (sn < se) cs.issue<kRowB>(kp, k ^ 1, sn, c.lane());
    const int* scol = cs.ready(kp, k, c.lane());
    AT z[R];
    spmv_slot<Pol, R, XT>(kp, s, c.lane(), x, z, scol);
#pragma unroll
    for (int r = 0; r < R; ++r) z[r] = Pol::norm(z[r]);
    epi(s, z);
    cs.release();
  }
  return true;
}

// One row of A x read through the SELL layout without a row perm (row r is
// lane r % 32 of slice r / 32): the halo rows of a matrix-powers pass.
template <class Pol, int R, class XT>
__device__ __forceinline__ void row_spmv(const KParams& kp, long long r, const XT* __restrict__ x,
                                         typename Pol::AT (&acc)[R]) {
  using VT = typename Pol::VT;
  const long long s = r >> 5;
  const int l = (int)(r & 31);
  const long long base = kp.slice_off[s];
  const int len = (int)((kp.slice_off[s + 1] - base) >> 5);
  const VT* vp = reinterpret_cast<const VT*>(kp.val) + base + l;
  const int* cp = kp.col + base + l;
#pragma unroll
  for (int q = 0; q < R; ++q) acc[q] = Pol::zero();
  float dl = 0.f;
  if constexpr (Pol::kMixed) {
    if (kp.dlo) dl = __ldg(kp.dlo + s * 32 + l);
  }
  for (int jj = 0; jj < len; ++jj) {
    const int cc = __ldg(cp + (long long)jj * 32);
    const VT a = __ldg(vp + (long long)jj * 32);
    XT xv[R];
    VecIO<R>::ld(x + (long long)cc * R, xv);
    if constexpr (Pol::kMixed) {
      if (jj == 0) {
#pragma unroll
        for (int q = 0; q < R; ++q) acc[q] = Pol::acc(acc[q], dl, xv[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < R; ++q) acc[q] = Pol::acc(acc[q], a, xv[q]);
  }
#pragma unroll
  for (int q = 0; q < R; ++q) acc[q] = Pol::norm(acc[q]);
}

// Two Horner levels in one pass (matrix powers):
//   level 1  u1 = A hin + g1 w   on the block's rows and its halo rows,
//            kept in shared memory in block-local numbering;
//   level 2  hout = A u1 + g2 w  on the block's rows, A read with local
//            column indices against the shared-memory vector.
// The ordering wait before it covers two hops of the row graph (the halo
// rows' neighbours), as every wait does when these passes are enabled.
template <class Pol, int R>
__device__ __forceinline__ bool horner_pair(const KParams& kp, const Ctx& c, ColStage& cs, PassSync& ps,
                            const typename Pol::HT* hin, typename Pol::HT* hout, const typename Pol::BT* w,
                            const typename Pol::ST (&g1)[R], const typename Pol::ST (&g2)[R]) {
  using BT = typename Pol::BT;
  using HT = typename Pol::HT;
  using AT = typename Pol::AT;
  extern __shared__ __align__(128) unsigned char dsm[];
  HT* const su = reinterpret_cast<HT*>(dsm + kp.su_off);
  const long long sb = kp.blk_slice[c.b()], se = kp.blk_slice[c.b() + 1];
  const long long rb0 = sb * 32;
  const long long nown = (se * 32 < kp.n ? se * 32 : kp.n) - rb0;
  // level 1, own rows (the usual pass, results to shared memory)
  const bool ok = spmv_pass<Pol, R, HT>(kp, c, cs, hin, [&](long long s, AT (&z)[R]) {
    const long long row = s * 32 + c.lane();
    if (row >= kp.n) return;
    BT sv[R];
    VecIO<R>::ld(w + row * R, sv);
    HT u[R];
#pragma unroll
    for (int r = 0; r < R; ++r) u[r] = Pol::to_h(Pol::add_mul(z[r], g1[r], sv[r]));
    VecIO<R>::st(su + (row - rb0) * R, u);
  }, &ps);
  if (!ok) return false;
  // level 1, halo rows
  const long long h0 = kp.halo_ptr[c.b()], h1 = kp.halo_ptr[c.b() + 1];
  for (long long k = h0 + c.tid(); k < h1; k += c.nt()) {
    const long long r = kp.halo_rows[k];
    AT z[R];
    row_spmv<Pol, R, HT>(kp, r, hin, z);
    BT sv[R];
    VecIO<R>::ld(w + r * R, sv);
    HT u[R];
#pragma unroll
    for (int q = 0; q < R; ++q) u[q] = Pol::to_h(Pol::add_mul(z[q], g1[q], sv[q]));
    VecIO<R>::st(su + (nown + (k - h0)) * R, u);
  }
  __syncthreads();
  // level 2, own rows from the shared-memory vector: its gathers have
  // shared-memory latency, so one entry at a time (few live registers)
  using VT = typename Pol::VT;
  for (long long s = sb + c.warp(); s < se; s += c.nw()) {
    const long long base = kp.slice_off[s];
    const int len = (int)((kp.slice_off[s + 1] - base) >> 5);
    const int* lp = kp.lcol + base + c.lane();
    const VT* vp = reinterpret_cast<const VT*>(kp.val) + base + c.lane();
    AT z[R];
#pragma unroll
    for (int r = 0; r < R; ++r) z[r] = Pol::zero();
    float dl = 0.f;
    if constexpr (Pol::kMixed) {
      if (kp.dlo) dl = __ldg(kp.dlo + s * 32 + c.lane());
    }
    for (int jj = 0; jj < len; ++jj) {
      const int lc = __ldg(lp + (long long)jj * 32);
      const VT a = __ldg(vp + (long long)jj * 32);
      HT xv[R];
      VecIO<R>::ld(su + (long long)lc * R, xv);
      if constexpr (Pol::kMixed) {
        if (jj == 0) {
#pragma unroll
          for (int r = 0; r < R; ++r) z[r] = Pol::acc(z[r], dl, xv[r]);
        }
      }
#pragma unroll
      for (int r = 0; r < R; ++r) z[r] = Pol::acc(z[r], a, xv[r]);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) z[r] = Pol::norm(z[r]);
    const long long row = s * 32 + c.lane();
    if (row >= kp.n) continue;
    BT sv[R];
    VecIO<R>::ld(w + row * R, sv);
    HT u[R];
#pragma unroll
    for (int r = 0; r < R; ++r) u[r] = Pol::to_h(Pol::add_mul(z[r], g2[r], sv[r]));
    VecIO<R>::st(hout + row * R, u);
  }
  return true;
}

// ------------------------------------------------------------------ LANCZOS
// build_subspace.cu:5-89 with the three-term recurrence as two grid passes
// per step (A: SpMV + beta_j v_{j-1} + alpha partials; B: w -= alpha v_j +
// beta partials), plus d Horner passes for the polynomial preconditioner.
// v_{j+1} = w (1/beta_{j+1}) is formed on the fly in the next step's first
// pass, which also stores it in V.
// Block-uniform Lanczos scalars live in shared memory, not registers: with R
// right-hand sides they would otherwise occupy ~10R registers across every
// SpMV pass and push the passes into local-memory spills.
#ifndef GM_MAX_DEG
#define GM_MAX_DEG 32
#endif
template <class Pol, int R>
struct LanczosScalars {
  double beta[R], rbeta[R], rbp[R], alpha[R], tot[R];
  int broken[R];
  typename Pol::ST sc[R], rb[R], bj[R], al[R];
  typename Pol::ST gr[GM_MAX_DEG + 1][R];   // gamma_h rbeta_j of the current step
  int all_broken;
};

// Every block sums the G per-block partials (layout [R][G]) in one fixed
// order into dst (shared memory); deterministic and identical in all blocks.
template <int N>
__device__ __forceinline__ void grid_total_smem(const double* partials, int stride, int count, double* dst) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      double t = 0.0;
      for (int b = lane; b < count; b += 32) t += partials[(long long)j * stride + b];
      t = warp_sum(t);
      if (lane == 0) dst[j] = t;
    }
  }
  __syncthreads();
}

// The per-block Gram-Schmidt coefficient x as the policy's scalar: FP64, or
// the float-float pair stored in the same 8 bytes.
template <class Pol>
__device__ __forceinline__ typename Pol::ST reorth_scalar(const double* hb, int x) {
  if constexpr (Pol::kMixed) {
    const float2 f = reinterpret_cast<const float2*>(hb)[x];
    return ff{f.x, f.y};
  } else {
    return hb[x];
  }
}

// Classical Gram-Schmidt of the step's work vector w (unrounded, in Hw)
// against the stored basis V_0..V_j, kp.reorth times (1 = CGS, 2 = CGS2):
//   h_t = V_t^T w  (t = 0..j; per-block partials, then every block totals the
//                  group's partials in one fixed order: deterministic)
//   w  <- w - sum_t h_t V_t
// The dots run over tiles of TT basis vectors so that each V_t is read once
// per dot pass with TT*R accumulators per thread.  Between passes w stays in
// the accumulator precision in Hw; the last correction rounds it to storage
// once (Wout) and accumulates ||w||^2 into bpa.  Consecutive passes use
// alternate halves of hpart, so a block that runs ahead cannot overwrite
// partials another block is still summing.
template <class Pol, int R>
__device__ bool reorth_step(const KParams& kp, const Ctx& c, const Grp& g, int j, typename Pol::HT* Hw,
                            typename Pol::BT* Wout, typename Pol::AT (&bpa)[R]) {
  using BT = typename Pol::BT;
  using HT = typename Pol::HT;
  using AT = typename Pol::AT;
  constexpr int TT = 8 / R;
  const long long n = kp.n;
  const BT* const V = reinterpret_cast<const BT*>(kp.V);
  const int G = kp.G;
  double* const hb = kp.hblk + (long long)c.b() * (kp.m + 1) * R;   // this block's totals [t][r]
  for (int q = 0; q < kp.reorth; ++q) {
    double* const hp = kp.hpart + (long long)(q & 1) * (kp.m + TT) * R * G;   // [t][r][G]
    for (int t0 = 0; t0 <= j; t0 += TT) {
      AT acc[TT][R];
#pragma unroll
      for (int u = 0; u < TT; ++u)
#pragma unroll
        for (int r = 0; r < R; ++r) acc[u][r] = Pol::zero();
      for (long long i = g.gt(kp); i < g.r1(kp); i += g.tt()) {
        HT wh[R];
        VecIO<R>::ld(Hw + i * R, wh);
#pragma unroll
        for (int u = 0; u < TT; ++u) {
          if (t0 + u <= j) {
            BT v[R];
            VecIO<R>::ld(V + ((long long)(t0 + u) * n + i) * R, v);
#pragma unroll
            for (int r = 0; r < R; ++r) acc[u][r] = Pol::dot(acc[u][r], h_load_at<Pol>(wh[r]), v[r]);
          }
        }
      }
      double a[TT * R];
#pragma unroll
      for (int u = 0; u < TT; ++u)
#pragma unroll
        for (int r = 0; r < R; ++r) a[u * R + r] = Pol::to_d(acc[u][r]);
      block_sum_store<TT * R>(a, hp + (long long)t0 * R * G + c.b(), G);
    }
    if (!group_bar(kp, g.p).sync()) return false;
    for (int x = c.warp(); x < (j + 1) * R; x += c.nw()) {
      const double* pp = hp + (long long)x * G + g.gb;
      double t = 0.0;
      for (int b = c.lane(); b < g.Gp; b += 32) t += pp[b];
      t = warp_sum(t);
      if (c.lane() == 0) {
        // the correction's scalar, once per block: float-float for the
        // mixed engine (no double conversions per element)
        if constexpr (Pol::kMixed) {
          const ff hv = ff_from_double(t);
          reinterpret_cast<float2*>(hb)[x] = make_float2(hv.hi, hv.lo);
        } else {
          hb[x] = t;
        }
      }
    }
    __syncthreads();
    const bool last = q + 1 == kp.reorth;
    for (long long i = g.gt(kp); i < g.r1(kp); i += g.tt()) {
      HT wh[R];
      VecIO<R>::ld(Hw + i * R, wh);
      AT w[R];
#pragma unroll
      for (int r = 0; r < R; ++r) w[r] = h_load_at<Pol>(wh[r]);
      // TT basis entries loaded before they are used: TT loads in flight per row
      int t = 0;
      for (; t + TT <= j + 1; t += TT) {
        BT v[TT][R];
#pragma unroll
        for (int u = 0; u < TT; ++u) VecIO<R>::ld(V + ((long long)(t + u) * n + i) * R, v[u]);
#pragma unroll
        for (int u = 0; u < TT; ++u)
#pragma unroll
          for (int r = 0; r < R; ++r) w[r] = Pol::sub_mul(w[r], reorth_scalar<Pol>(hb, (t + u) * R + r), v[u][r]);
      }
      for (; t <= j; ++t) {
        BT v[R];
        VecIO<R>::ld(V + ((long long)t * n + i) * R, v);
#pragma unroll
        for (int r = 0; r < R; ++r) w[r] = Pol::sub_mul(w[r], reorth_scalar<Pol>(hb, t * R + r), v[r]);
      }
      if (last) {
        BT wb[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          wb[r] = Pol::to_b(w[r]);
          bpa[r] = Pol::dot_self(bpa[r], w[r]);
        }
        VecIO<R>::st(Wout + i * R, wb);
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) wh[r] = Pol::to_h(w[r]);
        VecIO<R>::st(Hw + i * R, wh);
      }
    }
    __syncthreads();
  }
  return true;
}

template <class Pol, int R, bool MPK, bool RO>
__device__ bool phase_lanczos(const KParams& kp, const Ctx& c, const Grp& g, PassSync& ps, ColStage& cs) {
  using BT = typename Pol::BT;
  using HT = typename Pol::HT;
  using AT = typename Pol::AT;
  const long long n = kp.n;
  const int m = kp.m, d = kp.d, G = kp.G;
  double* const aab = kp.aabb + (long long)(m + 1) * 2 * R * g.p;   // this problem's aabb
  int* const meff = kp.meff + (long long)R * g.p;
  const double* const gam = kp.gamma + (long long)(d + 1) * g.p;
  BT* V = reinterpret_cast<BT*>(kp.V);
  BT* const W0 = reinterpret_cast<BT*>(kp.W0);
  BT* const W1 = reinterpret_cast<BT*>(kp.W1);
  HT* const H0 = reinterpret_cast<HT*>(kp.H0);
  HT* const H1 = reinterpret_cast<HT*>(kp.H1);
  double* part_a = kp.part;
  double* part_b = kp.part + (long long)R * G;
  __shared__ LanczosScalars<Pol, R> sh;

  // prologue: W1 = U (storage precision), beta_0 = ||U_r||
  {
    double bp[R];
#pragma unroll
    for (int r = 0; r < R; ++r) bp[r] = 0.0;
    for (long long i = g.gt(kp); i < g.r1(kp); i += g.tt()) {
      double u[R];
      VecIO<R>::ld(kp.U + i * R, u);
      BT wb[R];
#pragma unroll
      for (int r = 0; r < R; ++r) { bp[r] = fma(u[r], u[r], bp[r]); wb[r] = (BT)u[r]; }
      VecIO<R>::st(W1 + i * R, wb);
    }
    block_sum_store<R>(bp, part_b + c.b(), G);
  }
  if (!group_bar(kp, g.p).sync()) return false;
  grid_total_smem<R>(part_b + g.gb, G, g.Gp, sh.tot);
  if (c.tid() == 0) {
    for (int r = 0; r < R; ++r) {
      sh.beta[r] = sqrt(sh.tot[r]);
      sh.broken[r] = !(sh.beta[r] > 0.0);
      sh.rbeta[r] = sh.broken[r] ? 0.0 : 1.0 / sh.beta[r];
      sh.rbp[r] = 0.0;
      if (g.bl == 0) {
        aab[(long long)(m + 1) * (R + r)] = sh.beta[r];
        meff[r] = sh.broken[r] ? 0 : m;
        if (!(sh.tot[r] == sh.tot[r]) || isinf(sh.tot[r])) atomicCAS(kp.status, 0, (int)ST_NONFINITE);
      }
    }
  }
  __syncthreads();
  // Inside the recurrence the Lanczos vector is v_j = rbeta_j w_j, formed
  // from the stored work vector w_j (src) in the accumulator precision in
  // every pass, so the polynomial's terms all act on the same vector: its
  // monomial terms cancel strongly, and mixing w_j-based and separately
  // rounded v_j terms would turn the storage rounding into an error of
  // p(B) v_j.  The rounded v_j is stored in V for the apply only.  v_{j-1}
  // is rbeta_{j-1} w_{j-1}, read from the work buffer this step overwrites.
  const BT* src = W1;
  for (int j = 0; j < m; ++j) {
    BT* Vj = V + (long long)j * n * R;
    BT* Wout = (j & 1) ? W1 : W0;
    // w = B v_j - beta_j v_{j-1} goes to the Horner buffer the last pass does
    // not read, in the accumulator precision; pass B subtracts alpha_j v_j and
    // rounds once to storage (rounding before the subtraction would make the
    // storage error relative to |w| instead of to beta_{j+1} << |w|).
    HT* Hw = (d & 1) ? H0 : H1;
    if (c.tid() == 0) {
      for (int r = 0; r < R; ++r) {
        sh.sc[r] = Pol::scalar(sh.rbeta[r] * gam[0]);
        sh.rb[r] = Pol::scalar(sh.rbeta[r]);
        sh.bj[r] = Pol::scalar(sh.beta[r] * sh.rbp[r]);
        for (int h = 1; h <= d; ++h) sh.gr[h][r] = Pol::scalar(gam[h] * sh.rbeta[r]);
      }
    }
    __syncthreads();
    AT apa[R];
#pragma unroll
    for (int r = 0; r < R; ++r) apa[r] = Pol::zero();
    if (d == 0) {
      spmv_pass<Pol, R, BT>(kp, c, cs, src, [&](long long s, AT (&z)[R]) {
        const long long row = slot_row(kp, s, c.lane());
        if (row < 0) return;
        BT sv[R], v[R];
        VecIO<R>::ld(src + row * R, sv);
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = Pol::scale_to_b(sv[r], sh.rb[r]);
        VecIO<R>::st(Vj + row * R, v);
        AT w[R];
#pragma unroll
        for (int r = 0; r < R; ++r) w[r] = Pol::mul(z[r], sh.sc[r]);
        if (j > 0) {
          BT wp[R];
          VecIO<R>::ld(Wout + row * R, wp);   // w_{j-1}
#pragma unroll
          for (int r = 0; r < R; ++r) w[r] = Pol::sub_mul(w[r], sh.bj[r], wp[r]);
        }
        HT wh[R];
#pragma unroll
        for (int r = 0; r < R; ++r) { wh[r] = Pol::to_h(w[r]); apa[r] = Pol::dot(apa[r], w[r], sv[r]); }
        VecIO<R>::st(Hw + row * R, wh);
      }, nullptr, j > 0 ? Wout : nullptr);
    } else {
      // Horner pass 1: u = gamma_1 v_j + A (gamma_0 v_j); stores v_j
      {
        spmv_pass<Pol, R, BT>(kp, c, cs, src, [&](long long s, AT (&z)[R]) {
          const long long row = slot_row(kp, s, c.lane());
          if (row < 0) return;
          BT sv[R], v[R];
          VecIO<R>::ld(src + row * R, sv);
#pragma unroll
          for (int r = 0; r < R; ++r) v[r] = Pol::scale_to_b(sv[r], sh.rb[r]);
          VecIO<R>::st(Vj + row * R, v);
          HT u[R];
#pragma unroll
          for (int r = 0; r < R; ++r) u[r] = Pol::to_h(Pol::add_mul(Pol::mul(z[r], sh.sc[r]), sh.gr[1][r], sv[r]));
          VecIO<R>::st(H1 + row * R, u);
        });
      }
      ps.done(kp);
      const HT* hin;
      if constexpr (MPK) {
        // Horner levels 2..d, pairs in one pass each, then single passes.
        // Pass k (0-based, after pass 1) reads H1 when k is even, H0 when odd,
        // and writes the other buffer.
        int k = 0, h = 2;
        for (; h + 1 <= d; h += 2, ++k) {
          if (!horner_pair<Pol, R>(kp, c, cs, ps, (k & 1) ? H0 : H1, (k & 1) ? H1 : H0, src, sh.gr[h],
                                   sh.gr[h + 1]))
            return false;
          ps.done(kp);
        }
        for (; h <= d; ++h, ++k) {
          HT* hout = (k & 1) ? H1 : H0;
          const bool ok = spmv_pass<Pol, R, HT>(kp, c, cs, (k & 1) ? H0 : H1, [&](long long s, AT (&z)[R]) {
            const long long row = slot_row(kp, s, c.lane());
            if (row < 0) return;
            BT sv[R];
            VecIO<R>::ld(src + row * R, sv);
            HT u[R];
#pragma unroll
            for (int r = 0; r < R; ++r) u[r] = Pol::to_h(Pol::add_mul(z[r], sh.gr[h][r], sv[r]));
            VecIO<R>::st(hout + row * R, u);
          }, &ps);
          if (!ok) return false;
          ps.done(kp);
        }
        hin = (k & 1) ? H0 : H1;
        Hw = (k & 1) ? H1 : H0;   // w goes to the buffer the final pass does not read
      } else {
        for (int h = 2; h <= d; ++h) {
          const HT* hin_h = (h & 1) ? H0 : H1;
          HT* hout = (h & 1) ? H1 : H0;
          const bool ok = spmv_pass<Pol, R, HT>(kp, c, cs, hin_h, [&](long long s, AT (&z)[R]) {
            const long long row = slot_row(kp, s, c.lane());
            if (row < 0) return;
            BT sv[R];
            VecIO<R>::ld(src + row * R, sv);
            HT u[R];
#pragma unroll
            for (int r = 0; r < R; ++r) u[r] = Pol::to_h(Pol::add_mul(z[r], sh.gr[h][r], sv[r]));
            VecIO<R>::st(hout + row * R, u);
          }, &ps, src);
          if (!ok) return false;
          ps.done(kp);
        }
        hin = (d & 1) ? H1 : H0;
      }
      // final pass: w = A u - beta_j v_{j-1}
      const bool ok = spmv_pass<Pol, R, HT>(kp, c, cs, hin, [&](long long s, AT (&z)[R]) {
        const long long row = slot_row(kp, s, c.lane());
        if (row < 0) return;
        BT sv[R];
        VecIO<R>::ld(src + row * R, sv);
        AT w[R];
#pragma unroll
        for (int r = 0; r < R; ++r) w[r] = z[r];
        if (j > 0) {
          BT wp[R];
          VecIO<R>::ld(Wout + row * R, wp);   // w_{j-1}
#pragma unroll
          for (int r = 0; r < R; ++r) w[r] = Pol::sub_mul(w[r], sh.bj[r], wp[r]);
        }
        HT wh[R];
#pragma unroll
        for (int r = 0; r < R; ++r) { wh[r] = Pol::to_h(w[r]); apa[r] = Pol::dot(apa[r], w[r], sv[r]); }
        VecIO<R>::st(Hw + row * R, wh);
      }, &ps, j > 0 ? Wout : src);
      if (!ok) return false;
    }
    {
      double ap[R];
#pragma unroll
      for (int r = 0; r < R; ++r) ap[r] = Pol::to_d(apa[r]);
      block_sum_store<R>(ap, part_a + c.b(), G);
    }
    ps.done(kp);
    if (!group_bar(kp, g.p).sync()) return false;
    grid_total_smem<R>(part_a + g.gb, G, g.Gp, sh.alpha);
    if (c.tid() == 0) {
      // alpha_j = w^T v_j = rbeta_j (w^T w_j); pass B subtracts alpha_j rbeta_j w_j
      for (int r = 0; r < R; ++r) {
        sh.alpha[r] *= sh.rbeta[r];
        sh.al[r] = Pol::scalar(sh.alpha[r] * sh.rbeta[r]);
      }
    }
    __syncthreads();
    // pass B: w -= alpha_j v_j; beta_{j+1} = ||w||  (after the optional
    // Gram-Schmidt against V_0..V_j)
    {
      AT bpa[R];
#pragma unroll
      for (int r = 0; r < R; ++r) bpa[r] = Pol::zero();
      const bool ro = RO && kp.reorth > 0;
      long long i = g.gt(kp);
      if (!ro) {
        // a pure stream (16-32 bytes per row): PB rows per thread per
        // iteration with all their loads issued before any store, so each
        // thread keeps PB rows in flight; rows and the ||w||^2 terms in the
        // same order as the one-row loop below (bit-identical sums)
        constexpr int PB = R == 1 ? 4 : (R == 2 ? 2 : 1);
        const long long i1 = g.r1(kp), step = g.tt();
        for (; PB > 1 && i + (PB - 1) * step < i1; i += PB * step) {
          HT wh[PB][R];
          BT v[PB][R];
#pragma unroll
          for (int u = 0; u < PB; ++u) {
            VecIO<R>::ld(Hw + (i + u * step) * R, wh[u]);
            VecIO<R>::ld(src + (i + u * step) * R, v[u]);
          }
#pragma unroll
          for (int u = 0; u < PB; ++u) {
            BT wb[R];
#pragma unroll
            for (int r = 0; r < R; ++r) {
              AT w = Pol::sub_mul(h_load_at<Pol>(wh[u][r]), sh.al[r], v[u][r]);
              wb[r] = Pol::to_b(w);
              bpa[r] = Pol::dot_self(bpa[r], w);
            }
            VecIO<R>::st(Wout + (i + u * step) * R, wb);
          }
        }
      }
      for (; i < g.r1(kp); i += g.tt()) {
        HT wh[R];
        BT wb[R], v[R];
        VecIO<R>::ld(Hw + i * R, wh);
        VecIO<R>::ld(src + i * R, v);   // w_j
        if (ro) {
#pragma unroll
          for (int r = 0; r < R; ++r) wh[r] = Pol::to_h(Pol::sub_mul(h_load_at<Pol>(wh[r]), sh.al[r], v[r]));
          VecIO<R>::st(Hw + i * R, wh);
          continue;
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
          AT w = Pol::sub_mul(h_load_at<Pol>(wh[r]), sh.al[r], v[r]);
          wb[r] = Pol::to_b(w);
          bpa[r] = Pol::dot_self(bpa[r], w);
        }
        VecIO<R>::st(Wout + i * R, wb);
      }
      if constexpr (RO) {
        if (ro && !reorth_step<Pol, R>(kp, c, g, j, Hw, Wout, bpa)) return false;
      }
      double bp[R];
#pragma unroll
      for (int r = 0; r < R; ++r) bp[r] = Pol::to_d(bpa[r]);
      block_sum_store<R>(bp, part_b + c.b(), G);
    }
    if (!group_bar(kp, g.p).sync()) return false;
    grid_total_smem<R>(part_b + g.gb, G, g.Gp, sh.tot);
    if (c.tid() == 0) {
      int all = 1;
      for (int r = 0; r < R; ++r) {
        const double bn = sqrt(sh.tot[r]);
        const double al = sh.alpha[r];
        if (g.bl == 0) {
          aab[j + (long long)(m + 1) * r] = sh.broken[r] ? 0.0 : al;
          aab[(j + 1) + (long long)(m + 1) * (R + r)] = sh.broken[r] ? 0.0 : bn;
          if (!(bn == bn) || isinf(bn) || !(al == al)) atomicCAS(kp.status, 0, (int)ST_NONFINITE);
        }
        const double scale = fabs(al) + (j > 0 ? sh.beta[r] : 0.0);
        if (!sh.broken[r] && j + 1 < m && !(bn > kp.bd_tol * scale)) {
          sh.broken[r] = 1;
          if (g.bl == 0) meff[r] = j + 1;
        }
        sh.rbp[r] = sh.rbeta[r];
        sh.beta[r] = sh.broken[r] ? 0.0 : bn;
        sh.rbeta[r] = sh.broken[r] ? 0.0 : 1.0 / bn;
        all = all && sh.broken[r];
      }
      sh.all_broken = all;
    }
    __syncthreads();
    src = Wout;
    if (sh.all_broken) break;
  }
  return true;
}

// ------------------------------------------------------------------ solves
// copyforsolve + linsyssolve + copyafter (lanczos_impl.cu:292-406,
// lin_sys_solves.cu:8-19): system (r, j) has diagonal alpha_r - shift,
// off-diagonals beta_r[1..meff-1] and right-hand side -beta0_r w_{r,j} e1.
// Because the right-hand side is a multiple of e1, the solution needs no
// back substitution of a general right-hand side: with the bottom-up Schur
// complements g_q = (alpha_q - s_q) - beta_{q+1} (beta_{q+1} / g_{q+1}), the
// solution is y_0 = rhs / g_0 and y_q = -beta_q y_{q-1} / g_q.
// One thread per system (the recurrence is serial in q; neighbouring lanes
// take neighbouring contour nodes of the same alpha/beta), complex FP64.
// Scaling: 1/g is Smith's complex reciprocal (R. L. Smith, "Algorithm 116:
// Complex division", CACM 5(8), 1962), which never forms |g|^2, and the
// Schur update multiplies beta by (beta / g) instead of forming beta^2, so
// entries of T up to ~1e300 and down to ~1e-300 neither overflow nor
// underflow.  The reciprocals 1/g_q are kept in the tri scratch for the
// top-down sweep.

// 1/(a + ib) by Smith's algorithm: the ratio of the smaller to the larger
// component keeps every intermediate within the range of the inputs.
__device__ __forceinline__ void smith_recip(double a, double b, double& rr, double& ri) {
  if (fabs(a) >= fabs(b)) {
    const double t = b / a;
    const double inv = 1.0 / (a + b * t);
    rr = inv;
    ri = -t * inv;
  } else {
    const double t = a / b;
    const double inv = 1.0 / (a * t + b);
    rr = t * inv;
    ri = -inv;
  }
}

template <int R>
__device__ void phase_trisolve(const KParams& kp, const Ctx& c) {
  const int m = kp.m, C = kp.C;
  const int np = kp.nprob > 0 ? kp.nprob : 1;
  for (long long sys = c.gt(); sys < (long long)np * R * C; sys += c.tt()) {
    // sys = (p R + r) C + j for problem p, right-hand side r, node j
    const long long rr = sys / C;
    const int j = (int)(sys % C);
    const long long p = rr / R;
    const int r = (int)(rr % R);
    const int me = kp.meff[rr];
    const double* __restrict__ al = kp.aabb + (long long)(m + 1) * (2 * R * p + r);
    const double* __restrict__ be = kp.aabb + (long long)(m + 1) * (2 * R * p + R + r);
    const double* __restrict__ sh = kp.shifts + 2LL * m * sys;
    double* __restrict__ ig = kp.tri + 4LL * m * sys;  // 1/g_q (re, im)
    double* __restrict__ yr = kp.Yr + (long long)m * sys;
    double* __restrict__ yi = kp.Yi + (long long)m * sys;
    const double b0 = be[0];
    const double wr = kp.wts[2LL * C * rr + j], wi = kp.wts[2LL * C * rr + C + j];
    double igr = 0.0, igi = 0.0;   // 1/g_{q+1}
#pragma unroll 4
    for (int q = me - 1; q >= 0; --q) {
      const double bq = q + 1 < me ? be[q + 1] : 0.0;
      // beta^2 / g_{q+1} as beta (beta / g_{q+1})
      const double gr = (al[q] - sh[2 * q]) - bq * (bq * igr);
      const double gi = -sh[2 * q + 1] - bq * (bq * igi);
      smith_recip(gr, gi, igr, igi);
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
#pragma unroll 4
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
  const int np = kp.nprob > 0 ? kp.nprob : 1;
  const long long total = (long long)np * R * d1 * m;
  for (long long t = c.gt(); t < total; t += c.tt()) {
    // t = (rr d1 + i) m + q with rr = p R + r
    const int q = (int)(t % m);
    const int i = (int)((t / m) % d1);
    const long long rr = t / ((long long)m * d1);
    const long long p = rr / R;
    const double* gr = kp.gs_re + (long long)d1 * C * p;
    const double* gi = kp.gs_im + (long long)d1 * C * p;
    double acc = 0.0;
    for (int j = 0; j < C; ++j) {
      const long long col = rr * C + j;
      acc = fma(gr[i + (long long)d1 * j], kp.Yi[col * m + q], acc);
      acc = fma(gi[i + (long long)d1 * j], kp.Yr[col * m + q], acc);
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
__device__ bool phase_apply(const KParams& kp, const Ctx& c, const Grp& g, bool overwrite, PassSync& ps,
                            ColStage& cs) {
  using BT = typename Pol::BT;
  using HT = typename Pol::HT;
  using AT = typename Pol::AT;
  const long long n = kp.n;
  const int m = kp.m, d = kp.d, d1 = d + 1;
  const BT* V = reinterpret_cast<const BT*>(kp.V);
  HT* P = reinterpret_cast<HT*>(kp.P);
  HT* const H0 = reinterpret_cast<HT*>(kp.H0);
  HT* const H1 = reinterpret_cast<HT*>(kp.H1);
  constexpr int IC = 3;
  const long long sb = kp.blk_slice[c.b()], se = kp.blk_slice[c.b() + 1];
  for (long long s = sb + c.warp(); s < se; s += c.nw()) {
    const long long i = slot_row(kp, s, c.lane());
    if (i < 0) continue;
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
              const long long ci = (((long long)R * g.p + r) * d1 + i0 + ii) * m + q;
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
  ps.done(kp);
  for (int h = 1; h <= d; ++h) {
    const HT* hin = h == 1 ? P : ((h & 1) ? H0 : H1);
    HT* hout = (h & 1) ? H1 : H0;
    const HT* Ph = P + (long long)h * n * R;
    const bool ok = spmv_pass<Pol, R, HT>(kp, c, cs, hin, [&](long long s, AT (&z)[R]) {
      const long long row = slot_row(kp, s, c.lane());
      if (row < 0) return;
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
    }, &ps);
    if (!ok) return false;
    if (h < d) ps.done(kp);
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
  GridBar bar{bar_word(kp, -1), kp.status, (unsigned)G, kp.timeout_ns};
  double* part_z = kp.part + 2LL * R * G;
  constexpr int KC = 4;
  if (mode != 0 && R == 2) {
    for (long long i = c.gt(); i < n; i += c.tt()) {
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
      for (long long i = c.gt(); i < n; i += c.tt()) {
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
      block_sum_store<KC * R>(zp, part_z + (long long)e0 * R * G + c.b(), G);
    }
    if (!bar.sync()) return false;
    // every block totals the k*R entries in the same fixed order
    __shared__ double s_z[256];
    const int kr = k * R;
    for (int t0 = 0; t0 < kr; t0 += 256) {
      for (int t = t0 + c.tid(); t < kr && t < t0 + 256; t += c.nt()) {
        double acc = 0.0;
        const double* p = part_z + (long long)t * G;
        for (int b = 0; b < G; ++b) acc += p[b];
        s_z[t - t0] = acc;
        if (c.b() == 0) kp.Z[t] = acc;
      }
      __syncthreads();
      // pass 2 over this chunk of Z entries (rows by thread stride)
      const int e_lo = t0 / R, e_hi = min(k, (t0 + 256) / R);
      for (long long i = c.gt(); i < n; i += c.tt()) {
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
    for (long long i = c.gt(); i < n; i += c.tt()) {
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
#ifndef GM_MINB
#define GM_MINB 2
#endif
template <class Pol, int R, int PH>
#ifndef GM_MAXT
#define GM_MAXT 512
#endif
#ifndef GM_MINB4
#define GM_MINB4 2   // resident 512-thread blocks per SM for four right-hand sides
#endif
#ifndef GM_MINB4M
#define GM_MINB4M 3   // four right-hand sides, mixed precision, Lanczos entry points
#endif
#ifndef GM_MINB1
#define GM_MINB1 3   // and for one right-hand side
#endif
#ifndef GM_MINB1X
#define GM_MINB1X 2   // one right-hand side, matrix-powers or Gram-Schmidt entry points
#endif
#ifndef GM_MINB1L2
#define GM_MINB1L2 2   // one right-hand side, mixed, matrix held in the L2 window (PolMixedL2)
#endif
__global__ void __launch_bounds__(GM_MAXT, (R >= 4 ? ((Pol::kMixed && !(PH & (PH_MPK | PH_REORTH))) ? GM_MINB4M : GM_MINB4)
                                            : (R == 1 ? ((PH & (PH_MPK | PH_REORTH)) ? GM_MINB1X
                                                                                     : (Pol::kL2 ? GM_MINB1L2 : GM_MINB1))
                                                      : GM_MINB))) fab_kernel(KParams kp) {
  const Ctx c(kp.G);
  if (*(volatile int*)kp.status != 0) return;
  const int ph = kp.phases & PH;
  const Grp g(kp, c);
  PassSync ps{kp.dep_mode, g.p, 0u};
  ColStage cs;
  if (PH & (PH_LANCZOS | PH_APPLY)) cs.init(kp, c);
  bool first = true;
  auto sep = [&]() -> bool {
    if (first) { first = false; return true; }
    return GridBar{bar_word(kp, -1), kp.status, (unsigned)kp.G, kp.timeout_ns}.sync();
  };
  if ((PH & PH_LANCZOS) && (ph & PH_LANCZOS)) {
    if (!sep()) return;
    if (!phase_lanczos<Pol, R, (PH & PH_MPK) != 0, (PH & PH_REORTH) != 0>(kp, c, g, ps, cs)) return;
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
    if (!phase_apply<Pol, R>(kp, c, g, (ph & PH_APPLY_SET) != 0, ps, cs)) return;
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
