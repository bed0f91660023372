// Common device layer of the f(A)b engine: status codes, float-float
// arithmetic, precision policies, vector loads, a bounded grid barrier and
// deterministic block/grid reductions.
//
// Precision policies
//   PolFP64  : matrix values, Krylov basis and work vectors in FP64, every
//              per-element operation in FP64 (the plain engine).
//   PolMixed : matrix values, Krylov basis V and Lanczos work vector W in FP32;
//              Horner and lift buffers as float-float pairs; every per-element
//              operation on the FP32 pipe with exact products (two_prod) and
//              compensated sums (float-float, ~48-bit significand).  FP64 is
//              used only for per-thread reduction totals and the scalar
//              recurrences (alpha, beta, tridiagonal solves, quadrature sum).
//              On GB300 the FP64 rate is ~1/64 of FP32, so this keeps the
//              mixed engine HBM-bound instead of FP64-bound.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gm {

enum Status : int {
  ST_OK = 0, ST_ARG = 1, ST_OOM = 2, ST_CUDA = 3, ST_BREAKDOWN = 4,
  ST_TIMEOUT = 5, ST_STATE = 6, ST_NONFINITE = 7, ST_UNSUPPORTED = 8
};

// ---------------------------------------------------------------- float-float
struct ff { float hi, lo; };

__device__ __forceinline__ ff two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = a + b;
  float e = b - (s - a);
  return {s, e};
}
__device__ __forceinline__ ff two_prod(float a, float b) {
  float p = a * b;
  float e = fmaf(a, b, -p);
  return {p, e};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  float e = s.lo + (a.lo + b.lo);
  return fast_two_sum(s.hi, e);
}
__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }
// a * b with b a single float
__device__ __forceinline__ ff ff_mulf(ff a, float b) {
  ff p = two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  ff p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
  return fast_two_sum(p.hi, p.lo);
}
// acc + a*b, a and b floats (exact product, compensated sum)
__device__ __forceinline__ ff ff_fma_ff(ff acc, float a, float b) {
  ff p = two_prod(a, b);
  ff s = two_sum(acc.hi, p.hi);
  float e = s.lo + (acc.lo + p.lo);
  return fast_two_sum(s.hi, e);
}
__device__ __forceinline__ ff ff_from_double(double x) {
  float h = (float)x;
  float l = (float)(x - (double)h);
  return {h, l};
}
__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

// Matrix values of the SpMV: read once per pass, through the read-only path
// without allocating in L1, which stays with the gathered vector entries
// (3D 256^3 FP64 47.1 vs 50.1 ms per solve, 1M-node FE disk FP64 21.06 vs
// 21.20 ms, mixed equal).  GM_VAL_L1 (tuning builds) restores plain loads.
#ifndef GM_VAL_L1
#define GM_VAL_NOALLOC 1
#endif
__device__ __forceinline__ float ld_val(const float* p) {
#ifdef GM_VAL_NOALLOC
  float v;
  asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
#else
  return __ldg(p);
#endif
}
__device__ __forceinline__ double ld_val(const double* p) {
#ifdef GM_VAL_NOALLOC
  double v;
  asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
#else
  return __ldg(p);
#endif
}

// L2 prefetch of one global address (no register result, never faults on a
// valid address; used for the next slice's SELL values).
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// ---------------------------------------------------------------- policies
struct PolFP64 {
  using VT = double;   // matrix values
  using BT = double;   // Krylov basis V and Lanczos work vector W
  using HT = double;   // Horner / lift buffers
  using AT = double;   // per-element accumulator
  using ST = double;   // scalar used in per-element operations
  static constexpr bool kMixed = false;
  static constexpr bool kL2 = false;
  __device__ static __forceinline__ AT zero() { return 0.0; }
  __device__ static __forceinline__ ST scalar(double s) { return s; }
  __device__ static __forceinline__ AT acc(AT a, VT v, double x) { return fma(v, x, a); }
  __device__ static __forceinline__ AT norm(AT a) { return a; }
  __device__ static __forceinline__ AT mul(AT z, ST s) { return z * s; }
  __device__ static __forceinline__ AT add_mul(AT w, ST s, double v) { return fma(s, v, w); }
  __device__ static __forceinline__ AT sub_mul(AT w, ST s, double v) { return fma(-s, v, w); }
  __device__ static __forceinline__ AT add(AT a, AT b) { return a + b; }
  __device__ static __forceinline__ AT dot(AT a, AT w, double v) { return fma(w, v, a); }
  __device__ static __forceinline__ AT dot_self(AT a, AT w) { return fma(w, w, a); }
  __device__ static __forceinline__ double to_d(AT a) { return a; }
  __device__ static __forceinline__ AT from_d(double a) { return a; }
  __device__ static __forceinline__ BT to_b(AT a) { return a; }
  __device__ static __forceinline__ HT to_h(AT a) { return a; }
  __device__ static __forceinline__ AT from_b(BT b) { return b; }
  // b * s rounded to storage: v = w * rbeta
  __device__ static __forceinline__ BT scale_to_b(BT b, ST s) { return b * s; }
};

struct PolMixed {
  using VT = float;
  using BT = float;
  using HT = float2;   // float-float pair (x = hi, y = lo)
  using AT = ff;
  using ST = ff;
  static constexpr bool kMixed = true;
  static constexpr bool kL2 = false;
  __device__ static __forceinline__ AT zero() { return {0.f, 0.f}; }
  __device__ static __forceinline__ ST scalar(double s) { return ff_from_double(s); }
  // SpMV row accumulation: hi gathers the exactly-split products (two_sum),
  // lo collects every rounding error and stays unnormalised along the row;
  // norm() renormalises once per row.  Over a row's few terms lo stays of
  // order 2^-24 of the terms, so the sum keeps the float-float accuracy.
  __device__ static __forceinline__ AT acc(AT a, VT v, float x) {
    const ff p = two_prod(v, x);
    const ff s = two_sum(a.hi, p.hi);
    return {s.hi, a.lo + (s.lo + p.lo)};
  }
  __device__ static __forceinline__ AT acc(AT a, VT v, float2 x) {
    // v * (x.hi + x.lo): exact v*x.hi plus the small v*x.lo term
    const ff p = two_prod(v, x.x);
    const float pe = fmaf(v, x.y, p.lo);
    const ff s = two_sum(a.hi, p.hi);
    return {s.hi, a.lo + (s.lo + pe)};
  }
  __device__ static __forceinline__ AT norm(AT a) { return fast_two_sum(a.hi, a.lo); }
  __device__ static __forceinline__ AT mul(AT z, ST s) { return ff_mul(z, s); }
  // w +- s v and the reduction terms as in Ogita, Rump and Oishi's Dot2
  // (SIAM J. Sci. Comput. 26(6), 2005): the exact product's high part enters
  // a TwoSum, every low-order term goes to the low word, renormalised once
  // (w +- s v) or only when the partial is converted (dot products).
  __device__ static __forceinline__ AT add_mul(AT w, ST s, float v) {
    const ff p = two_prod(s.hi, v);
    const float pe = fmaf(s.lo, v, p.lo);
    const ff t = two_sum(w.hi, p.hi);
    return fast_two_sum(t.hi, (w.lo + pe) + t.lo);
  }
  __device__ static __forceinline__ AT sub_mul(AT w, ST s, float v) {
    const ff p = two_prod(s.hi, v);
    const float pe = fmaf(s.lo, v, p.lo);
    const ff t = two_sum(w.hi, -p.hi);
    return fast_two_sum(t.hi, (w.lo - pe) + t.lo);
  }
  __device__ static __forceinline__ AT dot(AT a, AT w, float v) {
    const ff p = two_prod(w.hi, v);
    const float pe = fmaf(w.lo, v, p.lo);
    const ff t = two_sum(a.hi, p.hi);
    return {t.hi, a.lo + (t.lo + pe)};
  }
  __device__ static __forceinline__ AT dot_self(AT a, AT w) {
    const ff p = two_prod(w.hi, w.hi);
    const float pe = fmaf(w.hi + w.hi, w.lo, p.lo);
    const ff t = two_sum(a.hi, p.hi);
    return {t.hi, a.lo + (t.lo + pe)};
  }
  __device__ static __forceinline__ AT add(AT a, AT b) { return ff_add(a, b); }
  __device__ static __forceinline__ double to_d(AT a) { return ff_to_double(a); }
  __device__ static __forceinline__ AT from_d(double a) { return ff_from_double(a); }
  __device__ static __forceinline__ BT to_b(AT a) { return a.hi + a.lo; }
  __device__ static __forceinline__ HT to_h(AT a) { return make_float2(a.hi, a.lo); }
  __device__ static __forceinline__ AT from_b(BT b) { return {b, 0.f}; }
  __device__ static __forceinline__ AT from_h(HT h) { return {h.x, h.y}; }
  __device__ static __forceinline__ BT scale_to_b(BT b, ST s) {
    ff p = ff_mulf(s, b);
    return p.hi + p.lo;
  }
};

// The mixed arithmetic for one-right-hand-side kernels compiled at two
// resident 512-thread blocks per SM (64 registers, no spills) instead of
// three (40 registers).  Mixed engines whose matrix is held in the L2
// persisting window use them: there the spill frames of the 40-register build
// compete with the vectors for the L2 left beside the window (1M-node FE disk:
// 13.9 vs 14.5 ms per solve), while a matrix streamed from HBM wants the third
// block's loads in flight (3D 256^3: 44.6 vs 37.8 ms with two blocks).  The
// FP64 engine, which spills little at 40 registers, measured slower with two
// blocks on the same L2-held disk (21.2 vs 19.2 ms) and has no such variant.
struct PolMixedL2 : PolMixed { static constexpr bool kL2 = true; };

__device__ __forceinline__ double h_to_d(double h) { return h; }
__device__ __forceinline__ double h_to_d(float2 h) { return (double)h.x + (double)h.y; }
__device__ __forceinline__ float2 h_from_ff(ff a) { return make_float2(a.hi, a.lo); }

// ---------------------------------------------------------------- vector I/O
// R consecutive values (one row of an interleaved [n][R] vector).
template <int R> struct VecIO;
template <> struct VecIO<1> {
  template <class T> __device__ static __forceinline__ void ld(const T* p, T (&o)[1]) { o[0] = p[0]; }
  template <class T> __device__ static __forceinline__ void st(T* p, const T (&o)[1]) { p[0] = o[0]; }
};
template <> struct VecIO<2> {
  __device__ static __forceinline__ void ld(const double* p, double (&o)[2]) {
    double2 v = *reinterpret_cast<const double2*>(p); o[0] = v.x; o[1] = v.y;
  }
  __device__ static __forceinline__ void st(double* p, const double (&o)[2]) {
    *reinterpret_cast<double2*>(p) = make_double2(o[0], o[1]);
  }
  __device__ static __forceinline__ void ld(const float* p, float (&o)[2]) {
    float2 v = *reinterpret_cast<const float2*>(p); o[0] = v.x; o[1] = v.y;
  }
  __device__ static __forceinline__ void st(float* p, const float (&o)[2]) {
    *reinterpret_cast<float2*>(p) = make_float2(o[0], o[1]);
  }
  __device__ static __forceinline__ void ld(const float2* p, float2 (&o)[2]) {
    float4 v = *reinterpret_cast<const float4*>(p); o[0] = make_float2(v.x, v.y); o[1] = make_float2(v.z, v.w);
  }
  __device__ static __forceinline__ void st(float2* p, const float2 (&o)[2]) {
    *reinterpret_cast<float4*>(p) = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
  }
};
template <> struct VecIO<4> {
  __device__ static __forceinline__ void ld(const double* p, double (&o)[4]) {
    double2 a = reinterpret_cast<const double2*>(p)[0];
    double2 b = reinterpret_cast<const double2*>(p)[1];
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
  }
  __device__ static __forceinline__ void st(double* p, const double (&o)[4]) {
    reinterpret_cast<double2*>(p)[0] = make_double2(o[0], o[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(o[2], o[3]);
  }
  __device__ static __forceinline__ void ld(const float* p, float (&o)[4]) {
    float4 v = *reinterpret_cast<const float4*>(p); o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
  __device__ static __forceinline__ void st(float* p, const float (&o)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
  }
  __device__ static __forceinline__ void ld(const float2* p, float2 (&o)[4]) {
    float4 a = reinterpret_cast<const float4*>(p)[0];
    float4 b = reinterpret_cast<const float4*>(p)[1];
    o[0] = make_float2(a.x, a.y); o[1] = make_float2(a.z, a.w);
    o[2] = make_float2(b.x, b.y); o[3] = make_float2(b.z, b.w);
  }
  __device__ static __forceinline__ void st(float2* p, const float2 (&o)[4]) {
    reinterpret_cast<float4*>(p)[0] = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
    reinterpret_cast<float4*>(p)[1] = make_float4(o[2].x, o[2].y, o[3].x, o[3].y);
  }
};

// ---------------------------------------------------------------- grid barrier
__device__ __forceinline__ unsigned long long global_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Barrier over a group of co-resident blocks on one 64-bit arrival counter
// that only grows (two adjacent words of the engine's barrier array, zeroed
// when the engine is created and after an aborted launch): the barrier an
// arrival belongs to is its number / nblocks, so no block resets anything and
// the last arrival's add is itself the release.  Against a count + generation
// pair (last arrival: reset the count, fence, publish the generation): 256^2
// FD solve 1.09 -> 0.94 ms, 1M-node FE disk FP64 21.18 -> 20.91 ms.  Every
// group barrier keeps the same nblocks for the engine's lifetime.  Every wait
// is bounded: after timeout_ns the waiting block records ST_TIMEOUT in
// *status and all blocks leave at their next barrier.  Returns false when the
// kernel must stop (timeout or an error recorded by any block).
struct GridBar {
  unsigned long long* count;
  int* status;
  unsigned nblocks;
  unsigned long long timeout_ns;

  __device__ bool sync() const {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
      int ok = 1;
      if (nblocks > 1) {
        unsigned long long* c64 = count;
        __threadfence();
        const unsigned long long old = atomicAdd(c64, 1ull);
        const unsigned long long target = (old / nblocks + 1ull) * nblocks;
        if (old + 1ull != target) {
          unsigned long long t0 = global_timer_ns();
          unsigned spins = 0;
          while (ld_acquire_u64(c64) < target) {
            if ((++spins & 31u) == 0u) {
              if (*(volatile int*)status != 0) { ok = 0; break; }
              if (global_timer_ns() - t0 > timeout_ns) {
                atomicCAS(status, 0, (int)ST_TIMEOUT);
                ok = 0;
                break;
              }
            }
            __nanosleep(32);
          }
        }
        __threadfence();
      }
      if (*(volatile int*)status != 0) ok = 0;
      s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
  }
};


// Dependency-local ordering between consecutive SpMV passes.  Block b owns a
// contiguous range of SELL slices; dep_idx[dep_ptr[b]..dep_ptr[b+1]) lists the
// blocks owning any row that b's rows reference, closed under symmetry.  After
// a pass, a block publishes (epoch << 20) + pass in prog[b]; before the next
// gathering pass it waits only for its neighbours.  Symmetry also makes the
// ping-pong buffer reuse safe: a neighbour that finished pass k-1 has finished
// reading this block's rows of the buffer pass k overwrites.  The epoch is the
// launch counter, so values left by earlier launches never satisfy a wait.
// Waits are bounded like GridBar's.
struct DepSync {
  unsigned long long* prog;
  const int* dep_ptr;
  const int* dep_idx;
  int* status;
  unsigned long long base;   // epoch << 20
  unsigned long long timeout_ns;

  __device__ void publish(unsigned pass) const {
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      st_release_u64(prog + blockIdx.x, base + pass);
    }
  }

  __device__ bool wait(unsigned pass) const {
    __shared__ int s_ok;
    const unsigned long long want = base + pass;
    if (threadIdx.x < 32) {
      int ok = 1;
      const int t0 = dep_ptr[blockIdx.x], t1 = dep_ptr[blockIdx.x + 1];
      for (int t = t0 + (int)threadIdx.x; t < t1 && ok; t += 32) {
        const unsigned long long* p = prog + dep_idx[t];
        unsigned long long start = 0;
        unsigned spins = 0;
        while (ld_acquire_u64(p) < want) {
          if ((++spins & 31u) == 0) {
            if (*(volatile int*)status != 0) { ok = 0; break; }
            const unsigned long long now = global_timer_ns();
            if (start == 0) {
              start = now;
            } else if (now - start > timeout_ns) {
              atomicCAS(status, 0, (int)ST_TIMEOUT);
              ok = 0;
              break;
            }
          }
          __nanosleep(20);
        }
      }
      ok = __all_sync(0xffffffffu, ok);
      if (threadIdx.x == 0) s_ok = ok && (*(volatile int*)status == 0);
    }
    __syncthreads();
    return s_ok != 0;
  }
};

// ---------------------------------------------------------------- TMA bulk copies
// Untiled bulk copy global -> shared completed on an mbarrier (the Blackwell
// TMA engine; both addresses 16-byte aligned, size a multiple of 16 bytes).
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
// Bulk prefetch of [src, src + bytes) from global memory into L2 (TMA unit;
// src 16-byte aligned, bytes a multiple of 16); no completion to wait for.
__device__ __forceinline__ void tma_bulk_prefetch_l2(const void* src, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
  return ok != 0;
}

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-sum of N values per thread; thread 0 writes out[j * stride] for j < N.
// Fixed reduction tree, so the result does not depend on timing.
template <int N>
__device__ __forceinline__ void block_sum_store(double (&v)[N], double* out, long long stride) {
  __shared__ double red[32][N > 0 ? N : 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int j = 0; j < N; ++j) v[j] = warp_sum(v[j]);
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < N; ++j) red[warp][j] = v[j];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      double t = lane < nw ? red[lane][j] : 0.0;
      t = warp_sum(t);
      if (lane == 0) out[j * stride] = t;
    }
  }
  __syncthreads();
}

// Every block computes the same total of G per-block partials for N
// quantities (partials laid out [N][G]); deterministic fixed order.
template <int N>
__device__ __forceinline__ void grid_total(const double* partials, int G, double (&tot)[N]) {
  __shared__ double s_tot[N > 0 ? N : 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      double t = 0.0;
      for (int b = lane; b < G; b += 32) t += partials[(long long)j * G + b];
      t = warp_sum(t);
      if (lane == 0) s_tot[j] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < N; ++j) tot[j] = s_tot[j];
  __syncthreads();
}

}  // namespace gm
