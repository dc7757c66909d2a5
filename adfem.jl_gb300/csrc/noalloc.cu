// Allocation-free variant of the FP64 Jacobi-CG solve, for callers that cannot
// allocate device memory.
//
// Who needs it: code that runs inside another framework's device-memory regime --
// a TensorFlow/ADCME custom-op kernel or a Julia CUDA.jl task -- where every byte of
// HBM belongs to that framework's pool.  There a cudaMalloc bypasses the pool, can
// fail because the pool has already reserved nearly all free memory, and (like
// cudaFree) may synchronise the whole device, stalling the framework's streams.
//
// This entry point therefore takes only caller-owned device buffers (CSR matrix,
// right-hand side, solution) and keeps all of its scratch -- the r, p, q and
// Jacobi vectors, the reduction partials and the CG scalars -- in one file-scope
// `static __device__` array of fixed size (kNoAllocMaxRows rows).  Every GPU that
// loads the library holds that array until the process exits.  Every call shares
// it: calls whose work overlaps on the GPU (different streams or host threads at
// the same time) race on it and must be serialised by the caller.  The array keeps
// the previous call's contents; the call clears what must start at zero.
//
// Host code cannot use the array's name as a device address (in host code it is a
// host-side stand-in).  The device address is obtained once per device with
// cudaGetSymbolAddress, with that device current, the first time the entry point is
// called on it -- so that first call should happen before any stream capture.
//
// The call is synchronous: every 16 iterations it reads the CG scalars back to the host
// and waits for its stream, so it returns only when the solve has ended.  Called on a
// stream that is being captured it returns ADFEM_ERR_UNSUPPORTED before enqueueing
// anything, so the caller's capture is left intact.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "adfem_internal.h"

namespace adfem {
namespace {

constexpr int64_t kNoAllocMaxRows = 131072;  // 2^17 rows: 4 MiB of vectors
constexpr int kNaT = 256;
constexpr int kNaBlocks = 512;
constexpr int kNaMaxDevices = 64;

struct NaState {
  double rho, alpha, beta, bb, rr;
  int done, iters;  // done: 0 running, 1 converged, 2 breakdown, 3 max_iter, 4 column out of range
  unsigned counter[2];
};

// r, p, q, dinv (n doubles each), partials (2 x kNaBlocks), state
constexpr size_t kNaVec = (size_t)kNoAllocMaxRows;
constexpr size_t kNaDoubles = 4 * kNaVec + 2 * kNaBlocks + (sizeof(NaState) + 7) / 8;
static __device__ __align__(256) double g_noalloc_scratch[kNaDoubles];

std::mutex g_na_mu;
double* g_na_ptr[kNaMaxDevices] = {nullptr};

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// deterministic two-value grid reduction; the last block stores the totals in tot
__device__ bool na_reduce(double a, double b, double* part, unsigned* counter, double* tot) {
  __shared__ double sh[2][kNaT / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  a = na_warp_sum(a);
  b = na_warp_sum(b);
  if (lane == 0) {
    sh[0][wid] = a;
    sh[1][wid] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int w = 0; w < kNaT / 32; w++) {
      s0 += sh[0][w];
      s1 += sh[1][w];
    }
    part[blockIdx.x] = s0;
    part[kNaBlocks + blockIdx.x] = s1;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  if (threadIdx.x == 0) {
    __threadfence();
    double s0 = 0.0, s1 = 0.0;
    for (unsigned k = 0; k < gridDim.x; k++) {
      s0 += __ldcg(part + k);
      s1 += __ldcg(part + kNaBlocks + k);
    }
    tot[0] = s0;
    tot[1] = s1;
    *counter = 0u;
  }
  return true;
}

struct NaPtrs {
  double *r, *p, *q, *dinv, *part;
  NaState* st;
};

__host__ __device__ inline NaPtrs na_ptrs(double* base) {
  NaPtrs P;
  P.r = base;
  P.p = base + kNaVec;
  P.q = base + 2 * kNaVec;
  P.dinv = base + 3 * kNaVec;
  P.part = base + 4 * kNaVec;
  P.st = reinterpret_cast<NaState*>(base + 4 * kNaVec + 2 * kNaBlocks);
  return P;
}

// u = 0, r = b, dinv = 1/A_ii, p = dinv r; rho = r.p, bb = b.b
__global__ void __launch_bounds__(kNaT) k_na_init(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                                  const double* __restrict__ val, const double* __restrict__ b,
                                                  double* __restrict__ u, double* scratch) {
  NaPtrs P = na_ptrs(scratch);
  double a0 = 0.0, a1 = 0.0;
  for (int i = blockIdx.x * kNaT + threadIdx.x; i < n; i += gridDim.x * kNaT) {
    double d = 0.0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
      const int c = col[k];
      if (c < 0 || c >= n) P.st->done = 4;  // rejected before any gather uses it
      if (c == i) d += val[k];
    }
    const double di = d != 0.0 ? 1.0 / d : 0.0;
    const double bi = b[i];
    u[i] = 0.0;
    P.r[i] = bi;
    P.dinv[i] = di;
    P.p[i] = di * bi;
    a0 = fma(bi, di * bi, a0);
    a1 = fma(bi, bi, a1);
  }
  double tot[2];
  if (na_reduce(a0, a1, P.part, &P.st->counter[0], tot) && threadIdx.x == 0) {
    P.st->rho = tot[0];
    P.st->bb = tot[1];
    P.st->rr = tot[1];
    if (P.st->done == 0 && !(tot[0] > 0.0)) P.st->done = tot[1] == 0.0 ? 1 : 2;
  }
}

// q = A p, alpha = rho / p.q
__global__ void __launch_bounds__(kNaT) k_na_spmv(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                                  const double* __restrict__ val, double* scratch) {
  NaPtrs P = na_ptrs(scratch);
  if (P.st->done) return;
  double a0 = 0.0;
  for (int i = blockIdx.x * kNaT + threadIdx.x; i < n; i += gridDim.x * kNaT) {
    double s = 0.0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) s = fma(val[k], P.p[col[k]], s);
    P.q[i] = s;
    a0 = fma(P.p[i], s, a0);
  }
  double tot[2];
  if (na_reduce(a0, 0.0, P.part, &P.st->counter[0], tot) && threadIdx.x == 0) {
    if (!(tot[0] > 0.0) || !isfinite(tot[0])) P.st->done = 2;
    else P.st->alpha = P.st->rho / tot[0];
  }
}

// u += alpha p, r -= alpha q; rho' = r.(dinv r), rr = r.r; beta; convergence
__global__ void __launch_bounds__(kNaT) k_na_update(int n, double* __restrict__ u, double* scratch, double rtol2,
                                                    int max_iter) {
  NaPtrs P = na_ptrs(scratch);
  if (P.st->done) return;
  const double a = P.st->alpha;
  double a0 = 0.0, a1 = 0.0;
  for (int i = blockIdx.x * kNaT + threadIdx.x; i < n; i += gridDim.x * kNaT) {
    u[i] = fma(a, P.p[i], u[i]);
    const double ri = fma(-a, P.q[i], P.r[i]);
    P.r[i] = ri;
    a0 = fma(ri, P.dinv[i] * ri, a0);
    a1 = fma(ri, ri, a1);
  }
  double tot[2];
  if (na_reduce(a0, a1, P.part, &P.st->counter[1], tot) && threadIdx.x == 0) {
    NaState* st = P.st;
    st->iters += 1;
    st->rr = tot[1];
    if (!isfinite(tot[0])) st->done = 2;
    else if (tot[1] <= rtol2 * st->bb) st->done = 1;
    else if (st->iters >= max_iter) st->done = 3;
    else {
      st->beta = tot[0] / st->rho;
      st->rho = tot[0];
    }
  }
}

// p = dinv r + beta p
__global__ void __launch_bounds__(kNaT) k_na_p(int n, double* scratch) {
  NaPtrs P = na_ptrs(scratch);
  if (P.st->done) return;
  const double bt = P.st->beta;
  for (int i = blockIdx.x * kNaT + threadIdx.x; i < n; i += gridDim.x * kNaT)
    P.p[i] = fma(bt, P.p[i], P.dinv[i] * P.r[i]);
}

// device address of the scratch array for the current device (set up once per device)
int na_scratch(double** out) {
  int dev = 0;
  ADFEM_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNaMaxDevices) return fail(ADFEM_ERR_UNSUPPORTED, "device ordinal beyond 64");
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_na_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_na_ptr[dev];
  return ADFEM_OK;
}

}  // namespace
}  // namespace adfem

using namespace adfem;

extern "C" int adfem_csr_pcg_noalloc_d(int n, const int* rowptr_d, const int* colind_d, const double* vals_d,
                                       const double* rhs_d, double* u_d, double rtol, int max_iter,
                                       int* iterations, double* relres, void* stream) {
  ADFEM_RANGE("adfem_csr_pcg_noalloc_d");
  if (n <= 0 || !rowptr_d || !colind_d || !vals_d || !rhs_d || !u_d)
    return fail(ADFEM_ERR_INVALID, "csr_pcg_noalloc: null pointer or n <= 0");
  if ((int64_t)n > kNoAllocMaxRows)
    return fail(ADFEM_ERR_INVALID, "csr_pcg_noalloc: n = " + std::to_string(n) + " exceeds the fixed scratch of " +
                                       std::to_string(kNoAllocMaxRows) + " rows");
  if (!(rtol > 0.0) || max_iter < 1) return fail(ADFEM_ERR_INVALID, "csr_pcg_noalloc: rtol > 0 and max_iter >= 1");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  ADFEM_CUDA(cudaStreamIsCapturing(st, &cap));
  if (cap != cudaStreamCaptureStatusNone)
    return fail(ADFEM_ERR_UNSUPPORTED, "csr_pcg_noalloc: the call waits for its stream (it reads the CG state back "
                                       "every 16 iterations); it cannot run on a stream that is being captured");
  double* scratch = nullptr;
  ADFEM_TRY(na_scratch(&scratch));
  NaPtrs P = na_ptrs(scratch);
  // the previous call's state stays in the array: clear the scalars and counters
  ADFEM_CUDA(cudaMemsetAsync(P.st, 0, sizeof(NaState), st));
  const int blocks = (int)std::min<int64_t>(kNaBlocks, ((int64_t)n + kNaT - 1) / kNaT);
  k_na_init<<<blocks, kNaT, 0, st>>>(n, rowptr_d, colind_d, vals_d, rhs_d, u_d, scratch);
  ADFEM_CUDA(cudaGetLastError());
  NaState h;
  for (int it = 0; it < max_iter; it += 16) {
    for (int k = 0; k < 16; k++) {
      k_na_spmv<<<blocks, kNaT, 0, st>>>(n, rowptr_d, colind_d, vals_d, scratch);
      k_na_update<<<blocks, kNaT, 0, st>>>(n, u_d, scratch, rtol * rtol, max_iter);
      k_na_p<<<blocks, kNaT, 0, st>>>(n, scratch);
    }
    ADFEM_CUDA(cudaGetLastError());
    ADFEM_CUDA(cudaMemcpyAsync(&h, P.st, sizeof(NaState), cudaMemcpyDeviceToHost, st));
    ADFEM_CUDA(cudaStreamSynchronize(st));
    if (h.done) break;
  }
  if (iterations) *iterations = h.iters;
  if (relres) *relres = h.bb > 0.0 ? std::sqrt(h.rr / h.bb) : 0.0;
  if (h.done == 4) return fail(ADFEM_ERR_INVALID, "csr_pcg_noalloc: a column index is outside [0, n)");
  if (h.done == 2) return fail(ADFEM_ERR_BREAKDOWN, "csr_pcg_noalloc: breakdown (matrix not SPD?)");
  if (h.done != 1) return fail(ADFEM_ERR_NOT_CONVERGED, "csr_pcg_noalloc: max_iter reached before rtol");
  return ADFEM_OK;
}
