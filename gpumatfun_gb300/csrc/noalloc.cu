// gm_lin_sys_solves_noalloc: the shifted tridiagonal solves of lin_sys_solves
// for callers that cannot allocate device memory.
//
// Who needs it: applications that own every byte of device memory through
// their own allocator (MATLAB's gpuArray manager, a framework's caching
// pool, an embedded solver with a fixed memory budget) and code on a
// latency-critical path where cudaMalloc's implicit device-wide
// synchronisation is not acceptable.  They hand over their own device
// buffers for the inputs and the outputs; the only extra memory the solve
// needs, the table of reciprocal Schur complements 1/g_q (strided by four
// doubles per system entry) and nrhs m_eff slots, lives in the file-scope
// array g_noalloc_scratch below, which every GPU that loads this library
// holds until the process exits.
//
// Sharing rules: all calls (from every handle and thread) share that one
// array and it keeps the last call's contents.  Nothing in it must start at
// zero: each call writes every entry of the table before reading it, and the
// m_eff slots are written at the start of every call (the caller's values
// clamped to [0, m], or m when the caller passes none).  Two calls whose kernels overlap on the GPU (different streams, or
// different host threads without ordering) race on the array and produce
// wrong results; order them on one stream or synchronise between them.
#include <cuda_runtime.h>

#include <cstdio>

#include "../../include/gpumatfun.h"
#include "fab_kernel.cuh"

namespace {

// Reciprocal table of the solve for up to GM_NOALLOC_MAX_ENTRIES system
// entries (m * nrhs * C; the solve strides it by 4 doubles per entry),
// followed by 8 ints of m_eff: 1 MiB + 32 bytes.
constexpr long long kMaxEntries = GM_NOALLOC_MAX_ENTRIES;
constexpr long long kScratchDoubles = 4 * kMaxEntries + 4;
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

}  // namespace

namespace gm {
void set_global_error(const char* msg);  // engine.cu: the text gm_last_error(NULL) returns
}  // namespace gm

namespace {

int noalloc_fail(int code, const char* msg) {
  gm::set_global_error(msg);
  return code;
}

// slots[r] = min(max(meff[r], 0), m), or m without meff: the solve indexes
// the caller's arrays up to m_eff, so out-of-range values never reach it.
__global__ void k_fill_meff(const int* meff, int* slots, int R, int m) {
  if ((int)threadIdx.x < R) {
    int v = meff ? meff[threadIdx.x] : m;
    slots[threadIdx.x] = v < 0 ? 0 : (v > m ? m : v);
  }
}

template <int R>
__global__ void k_trisolve_noalloc(gm::KParams kp) {
  const gm::Ctx c(kp.G);
  gm::phase_trisolve<R>(kp, c);
}

}  // namespace

extern "C" int gm_lin_sys_solves_noalloc(int m, int nrhs, int contour_size, const double* aabb, const int* meff,
                                         const double* wts, const double* shifts, double* yreal, double* yimag,
                                         void* stream) {
  if (m < 1 || contour_size < 1 || (nrhs != 1 && nrhs != 2 && nrhs != 4))
    return noalloc_fail(GM_ERR_ARG, "lin_sys_solves_noalloc: need m >= 1, C >= 1 and nrhs in {1, 2, 4}");
  if (!aabb || !wts || !shifts || !yreal || !yimag)
    return noalloc_fail(GM_ERR_ARG, "lin_sys_solves_noalloc: null device pointer");
  const long long entries = (long long)m * nrhs * contour_size;
  if (entries > kMaxEntries) {
    char msg[160];
    snprintf(msg, sizeof(msg), "lin_sys_solves_noalloc: m * nrhs * C = %lld exceeds the fixed scratch of %lld entries",
             entries, kMaxEntries);
    return noalloc_fail(GM_ERR_ARG, msg);
  }
  cudaError_t st = cudaSuccess;
  // The host-side name g_noalloc_scratch is only a stand-in: the device
  // address is looked up on every call, with the caller's device current.
  // The lookup allocates nothing, and a fresh lookup stays right after a
  // cudaDeviceReset, which reloads the module at a new address.
  void* p = nullptr;
  st = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (st != cudaSuccess) return noalloc_fail(GM_ERR_CUDA, cudaGetErrorString(st));
  double* scratch = static_cast<double*>(p);
  gm::set_global_error("");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  gm::KParams kp{};
  kp.m = m;
  kp.C = contour_size;
  kp.aabb = const_cast<double*>(aabb);
  kp.wts = wts;
  kp.shifts = shifts;
  kp.Yr = yreal;
  kp.Yi = yimag;
  kp.tri = scratch;
  int* meff_slots = reinterpret_cast<int*>(scratch + 4 * kMaxEntries);
  k_fill_meff<<<1, 32, 0, s>>>(meff, meff_slots, nrhs, m);
  kp.meff = meff_slots;
  // one thread per system, as in the engine's lin_sys_solves phase
  const int threads = 256;
  const long long systems = (long long)nrhs * contour_size;
  kp.G = (int)((systems + threads - 1) / threads);
  if (nrhs == 1) k_trisolve_noalloc<1><<<kp.G, threads, 0, s>>>(kp);
  if (nrhs == 2) k_trisolve_noalloc<2><<<kp.G, threads, 0, s>>>(kp);
  if (nrhs == 4) k_trisolve_noalloc<4><<<kp.G, threads, 0, s>>>(kp);
  st = cudaGetLastError();
  if (st != cudaSuccess) return noalloc_fail(GM_ERR_CUDA, cudaGetErrorString(st));
  return GM_OK;
}
