// Packed solves of small systems: many independent Jacobi-scaled systems solved by one
// graph launch, one thread block per system of at most kPackBlockRows rows and one
// thread-block cluster per larger system, the whole mixed-precision solve inside the
// block or cluster.  The launch (descriptor upload, the two solve kernels, result
// download) is a CUDA graph captured once and relaunched for every pack (its kernel
// grids set to the pack's systems), so a pack of small requests costs one graph launch
// instead of a chain of per-iteration launches per request.
//
// Method per system (the block owns every row; no grid-wide synchronisation):
//   b~ = s * rhs, y = u0 / s or 0                                    (FP64)
//   repeat: r = b~ - K~ y in the difference form of k_scale_values   (FP64, outer)
//           stop when |r| <= rtol |b~|, or when a pass improved |r|^2 less than 4x
//           (attainable accuracy of the FP64 residual reached)
//           CG on K~ d = r with FP32 vectors and the FP32 difference-form copy,
//           FP32 accumulation, until |r_inner| <= 1e-4 |r|           (FP32, inner)
//           y += d                                                   (FP64)
//   u = s * y, Dirichlet rows set exactly
// This is iterative refinement with an FP32 inner CG: FP64 holds the assembled values,
// the outer residual, the solution update and the stopping test.  On GB300 an FP64
// instruction costs the FP64 pipe ~60x an FP32 one, so a block running its CG in FP64
// would spend ~30 us per iteration on a 16k-row system; in FP32 the inner iterations
// are limited by the latency of the matrix loads and of the block's barriers instead.
//
// Larger systems (above kPackBlockRows rows) are solved by a thread-block cluster of
// kCC blocks instead (k_pack_cluster): each block owns a contiguous slice of rows and
// keeps its part of the search vector in shared memory; neighbours in another block's
// slice are read through distributed shared memory, and dot products are reduced over
// the cluster in rank order (each block posts its partial, a cluster barrier, every block
// sums all partials in the same order), so all blocks take the same decisions.
//
// Each system's arithmetic depends only on its own block or cluster (fixed block size,
// row ownership and reduction order), so a system's result is bit-identical whatever it
// is packed with.  Every loop is bounded (iteration budget, pass cap); the cluster
// barriers are hardware barriers that every thread of the cluster reaches.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "cg_common.cuh"

namespace adfem {

namespace {

constexpr int kPBT = 512;                // threads per system
constexpr int kMaxPasses = 64;           // outer refinement passes
constexpr double kInner2 = 1e-8;         // inner CG stops at |r_inner|^2 <= 1e-8 |r|^2
constexpr int kU = 8;                    // row entries loaded together in the inner SpMV
// dynamic shared memory of the one-block kernel: p, r, d, q of every row (FP32)
constexpr size_t kPSmem = 4 * sizeof(float) * kPackBlockRows;

// Scalars of the inner CG, kept by thread 0 and read by every thread after a barrier.
// Only thread 0 does FP64 work per inner iteration: on GB300 an FP64 instruction of a
// warp occupies the FP64 pipe ~16 cycles, so FP64 block reductions and divisions by
// every warp would cost microseconds per iteration.
struct InnerScal {
  double rho, target;
  float af, bf;
  int go;
};

// FP32 block sum in warp order (red: one float per warp); the total is valid in warp 0
template <int BT>
__device__ __forceinline__ float bsumf(float v, float* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) red[wid] = v;
  __syncthreads();
  float t = 0.0f;
  if (wid == 0) t = warp_sum(lane < BT / 32 ? red[lane] : 0.0f);
  return t;
}

// thread 0, after p.q is known: the step length, or stop on breakdown
__device__ __forceinline__ void step_alpha(InnerScal& c, float pq) {
  const double pqd = (double)pq;
  c.go = (pqd > 0.0 && isfinite(pqd)) ? 1 : 0;
  c.af = c.go ? (float)(c.rho / pqd) : 0.0f;
}

// thread 0, after the new r.r is known: stop at the inner tolerance, else the direction update
__device__ __forceinline__ void step_beta(InnerScal& c, float rr) {
  const double rn = (double)rr;
  c.go = (rn <= c.target || !isfinite(rn)) ? 0 : 1;
  c.bf = (float)(rn / c.rho);
  c.rho = rn;
}

__device__ __forceinline__ void bsum2(double& a, double& b, double* shb) {
  double v[2] = {a, b};
  block_sum<double, 2, kPBT>(v);
  if (threadIdx.x == 0) {
    shb[0] = v[0];
    shb[1] = v[1];
  }
  __syncthreads();
  a = shb[0];
  b = shb[1];
  __syncthreads();  // shb is reused by the next reduction
}

template <bool D16>
__device__ void pack_body(const PackDesc& D, float* __restrict__ sp, double* shb, PackDesc* out) {
  __shared__ float red[kPBT / 32];
  __shared__ InnerScal sc;
  const int n = D.n;
  const int tid = threadIdx.x;
  const float* __restrict__ s = D.s;
  double* __restrict__ y = D.y;
  // r, d, q of the inner CG next to p in shared memory
  float* __restrict__ rv = sp + kPackBlockRows;
  float* __restrict__ dv = sp + 2 * kPackBlockRows;
  float* __restrict__ qv = sp + 3 * kPackBlockRows;
  // b~ and the start
  double bb = 0.0, dummy = 0.0;
  for (int r = tid; r < n; r += kPBT) {
    const double si = (double)s[r];
    const double bi = (D.zero_rows && D.zero_rows[r] == 1) ? 0.0 : si * D.rhs[r];
    bb = fma(bi, bi, bb);
    y[r] = D.u0 ? D.u0[r] / (double)s[r] : 0.0;  // inverse of u = s y up to one rounding
  }
  bsum2(bb, dummy, shb);
  const double bnorm2 = bb, stop2 = D.rtol2 * bnorm2;
  int it = 0, passes = 0, status = 4, floor_hit = 0;
  double rr = 0.0, last = 0.0;
  for (int pass = 0; pass < kMaxPasses; pass++) {
    // FP64 residual in difference form; r32 = (float) r; p = r32; d = 0
    double a0 = 0.0, a1 = 0.0;
    for (int r = tid; r < n; r += kPBT) {
      int64_t base;
      int w;
      sell_row(D.sptr, r, base, w);
      const double yr = y[r];
      const double zr = (double)s[r] * yr;
      double acc = 0.0;
      for (int k = 0; k < w; k++) {
        const int64_t idx = base + 32 * (int64_t)k;
        const int j = colof<D16>(D.col, idx, r);
        const double t = (j == r) ? yr : fma((double)s[j], y[j], -zr);
        acc = fma(D.valD[idx], t, acc);
      }
      const double bi = (D.zero_rows && D.zero_rows[r] == 1) ? 0.0 : (double)s[r] * D.rhs[r];
      const double ri = bi - acc;
      a0 = fma(ri, ri, a0);
      const float rf = (float)ri;
      a1 = fma((double)rf, (double)rf, a1);
      rv[r] = rf;
      sp[r] = rf;
      dv[r] = 0.0f;
    }
    bsum2(a0, a1, shb);
    rr = a0;
    passes = pass + 1;
    if (!isfinite(rr)) {
      status = 2;
      break;
    }
    if (rr <= stop2) {
      status = 1;
      break;
    }
    if (pass > 0 && rr > 0.25 * last) {
      status = 1;
      floor_hit = 1;
      break;
    }
    if (it >= D.max_iter) {
      status = 4;
      break;
    }
    last = rr;
    if (tid == 0) {
      sc.rho = a1;
      sc.target = kInner2 * a1;
    }
    while (it < D.max_iter) {
      // q = K~ p (FP32 difference form) and p.q; a row's entries are loaded kU at a
      // time before they are used, so their gathers overlap
      float acc = 0.0f;
      for (int r = tid; r < n; r += kPBT) {
        int64_t base;
        int w;
        sell_row(D.sptr, r, base, w);
        const float pr = sp[r];
        const float zr = __ldg(s + r) * pr;
        float q = 0.0f;
        for (int k0 = 0; k0 < w; k0 += kU) {
          float v[kU];
          int j[kU];
#pragma unroll
          for (int u = 0; u < kU; u++) {
            const int64_t idx = base + 32 * (int64_t)(k0 + u);
            v[u] = k0 + u < w ? __ldg(D.val32 + idx) : 0.0f;
            j[u] = k0 + u < w ? colof<D16>(D.col, idx, r) : r;
          }
          float sj[kU];
#pragma unroll
          for (int u = 0; u < kU; u++) sj[u] = __ldg(s + j[u]);
#pragma unroll
          for (int u = 0; u < kU; u++) {
            const float t = (j[u] == r) ? pr : fmaf(sj[u], sp[j[u]], -zr);
            q = fmaf(v[u], t, q);
          }
        }
        qv[r] = q;
        acc = fmaf(pr, q, acc);
      }
      const float pq = bsumf<kPBT>(acc, red);
      if (tid == 0) step_alpha(sc, pq);
      __syncthreads();
      if (!sc.go) break;  // breakdown: the correction so far is still applied
      const float af = sc.af;
      float acc2 = 0.0f;
      for (int r = tid; r < n; r += kPBT) {
        dv[r] = fmaf(af, sp[r], dv[r]);
        const float ri = fmaf(-af, qv[r], rv[r]);
        rv[r] = ri;
        acc2 = fmaf(ri, ri, acc2);
      }
      const float rn = bsumf<kPBT>(acc2, red);
      if (tid == 0) step_beta(sc, rn);
      __syncthreads();
      it++;
      if (!sc.go) break;
      const float bf = sc.bf;
      for (int r = tid; r < n; r += kPBT) sp[r] = fmaf(bf, sp[r], rv[r]);
      __syncthreads();
    }
    for (int r = tid; r < n; r += kPBT) y[r] += (double)dv[r];
    __syncthreads();
  }
  for (int r = tid; r < n; r += kPBT) {
    if (D.fix_rows && D.fix_rows[r] == 1) D.u[r] = D.fix_vals ? D.fix_vals[r] : 0.0;
    else D.u[r] = (double)s[r] * y[r];
  }
  if (tid == 0) {
    out->iters = it;
    out->passes = passes;
    out->status = status;
    out->floor_hit = floor_hit;
    out->rr64 = rr;
    out->bnorm2 = bnorm2;
  }
}

__global__ void __launch_bounds__(kPBT, 1) k_pack_solve(PackDesc* desc) {
  extern __shared__ float sp[];
  __shared__ PackDesc D;
  __shared__ double shb[2];
  if (threadIdx.x == 0) D = desc[blockIdx.x];
  __syncthreads();
  if (D.n <= 0) return;
  if (D.d16) pack_body<true>(D, sp, shb, desc + blockIdx.x);
  else pack_body<false>(D, sp, shb, desc + blockIdx.x);
}

// ---------------------------------------------------------------------------
// cluster variant
namespace cg = cooperative_groups;
#ifndef ADFEM_PACK_CBT
#define ADFEM_PACK_CBT 1024
#endif
constexpr int kCC = 8;                 // blocks per system
constexpr int kCBT = ADFEM_PACK_CBT;   // threads per block
constexpr int kCRows = 8192;           // rows per block at most
static_assert(kCC * kCRows == kPackMaxRows, "cluster rows");
// dynamic shared memory per block: p, r, q, d of the block's rows (FP32)
constexpr size_t kCSmem = 4 * sizeof(float) * kCRows;

template <bool D16>
__device__ void cluster_body(const PackDesc& D, float* __restrict__ sm, double* slots, PackDesc* out) {
  __shared__ double red[2][kCBT / 32];
  __shared__ double shb[2];
  __shared__ float redf[kCBT / 32];
  __shared__ float slotf[2];
  __shared__ InnerScal sc;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int n = D.n;
  const int R = ((n + kCC - 1) / kCC + 31) / 32 * 32;  // rows per block
  const int lo = min(rank * R, n), hi = min(lo + R, n);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const float* __restrict__ s = D.s;
  double* __restrict__ y = D.y;
  float* __restrict__ sp = sm;  // p (read by the other blocks of the cluster)
  float* __restrict__ rv = sm + kCRows;
  float* __restrict__ qv = sm + 2 * kCRows;
  float* __restrict__ dv = sm + 3 * kCRows;
  int rb = 0;  // reduction slot pair (alternates: one cluster barrier per reduction suffices)
  // (a, b) summed over the cluster: block partials in warp order, then the blocks' totals
  // in rank order, the same sums in every block
  auto creduce = [&](double& a, double& b) {
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
      red[0][wid] = a;
      red[1][wid] = b;
    }
    __syncthreads();
    if (wid == 0) {
      double x0 = lane < kCBT / 32 ? red[0][lane] : 0.0;
      double x1 = lane < kCBT / 32 ? red[1][lane] : 0.0;
      x0 = warp_sum(x0);
      x1 = warp_sum(x1);
      if (lane == 0) {
        slots[2 * rb] = x0;
        slots[2 * rb + 1] = x1;
      }
    }
    cl.sync();
    if (wid == 0) {
      double p0 = 0.0, p1 = 0.0;
      if (lane < kCC) {
        const double* rs = cl.map_shared_rank(slots, lane);
        p0 = rs[2 * rb];
        p1 = rs[2 * rb + 1];
      }
      double t0 = 0.0, t1 = 0.0;
#pragma unroll
      for (int k = 0; k < kCC; k++) {
        t0 += __shfl_sync(0xffffffffu, p0, k);
        t1 += __shfl_sync(0xffffffffu, p1, k);
      }
      if (lane == 0) {
        shb[0] = t0;
        shb[1] = t1;
      }
    }
    __syncthreads();
    a = shb[0];
    b = shb[1];
    rb ^= 1;
  };
  // FP32 sum over the cluster in the same order in every block; valid in thread 0
  int rbf = 0;
  auto creducef = [&](float v) -> float {
    const float t = bsumf<kCBT>(v, redf);
    if (tid == 0) slotf[rbf] = t;
    cl.sync();
    float tot = 0.0f;
    if (wid == 0) {
      const float pv = lane < kCC ? cl.map_shared_rank(slotf, lane)[rbf] : 0.0f;
#pragma unroll
      for (int k = 0; k < kCC; k++) tot += __shfl_sync(0xffffffffu, pv, k);
    }
    rbf ^= 1;
    return tot;
  };
  auto pval = [&](int j) -> float {
    if (j >= lo && j < hi) return sp[j - lo];
    const int o = j / R;
    return cl.map_shared_rank(sp, o)[j - o * R];
  };
  double bb = 0.0, dummy = 0.0;
  for (int r = lo + tid; r < hi; r += kCBT) {
    const double si = (double)s[r];
    const double bi = (D.zero_rows && D.zero_rows[r] == 1) ? 0.0 : si * D.rhs[r];
    bb = fma(bi, bi, bb);
    y[r] = D.u0 ? D.u0[r] / (double)s[r] : 0.0;  // inverse of u = s y up to one rounding
  }
  creduce(bb, dummy);  // (its cluster barrier also publishes y)
  const double bnorm2 = bb, stop2 = D.rtol2 * bnorm2;
  int it = 0, passes = 0, status = 4, floor_hit = 0;
  double rr = 0.0, last = 0.0;
  for (int pass = 0; pass < kMaxPasses; pass++) {
    // FP64 residual in difference form; r32 = (float) r; p = r32; d = 0
    double a0 = 0.0, a1 = 0.0;
    for (int r = lo + tid; r < hi; r += kCBT) {
      int64_t base;
      int w;
      sell_row(D.sptr, r, base, w);
      const double yr = y[r];
      const double zr = (double)s[r] * yr;
      double acc = 0.0;
      for (int k = 0; k < w; k++) {
        const int64_t idx = base + 32 * (int64_t)k;
        const int j = colof<D16>(D.col, idx, r);
        // y of another block's rows: written in this launch, read past L1
        const double t = (j == r) ? yr : fma((double)s[j], __ldcg(y + j), -zr);
        acc = fma(D.valD[idx], t, acc);
      }
      const double bi = (D.zero_rows && D.zero_rows[r] == 1) ? 0.0 : (double)s[r] * D.rhs[r];
      const double ri = bi - acc;
      a0 = fma(ri, ri, a0);
      const float rf = (float)ri;
      a1 = fma((double)rf, (double)rf, a1);
      rv[r - lo] = rf;
      sp[r - lo] = rf;
      dv[r - lo] = 0.0f;
    }
    creduce(a0, a1);  // (its cluster barrier also publishes p = r)
    rr = a0;
    passes = pass + 1;
    if (!isfinite(rr)) {
      status = 2;
      break;
    }
    if (rr <= stop2) {
      status = 1;
      break;
    }
    if (pass > 0 && rr > 0.25 * last) {
      status = 1;
      floor_hit = 1;
      break;
    }
    if (it >= D.max_iter) {
      status = 4;
      break;
    }
    last = rr;
    if (tid == 0) {
      sc.rho = a1;
      sc.target = kInner2 * a1;
    }
    while (it < D.max_iter) {
      float acc = 0.0f;
      for (int r = lo + tid; r < hi; r += kCBT) {
        int64_t base;
        int w;
        sell_row(D.sptr, r, base, w);
        const float pr = sp[r - lo];
        const float zr = __ldg(s + r) * pr;
        float q = 0.0f;
        for (int k0 = 0; k0 < w; k0 += kU) {
          float v[kU];
          int j[kU];
#pragma unroll
          for (int u = 0; u < kU; u++) {
            const int64_t idx = base + 32 * (int64_t)(k0 + u);
            v[u] = k0 + u < w ? __ldg(D.val32 + idx) : 0.0f;
            j[u] = k0 + u < w ? colof<D16>(D.col, idx, r) : r;
          }
#pragma unroll
          for (int u = 0; u < kU; u++) {
            const float t = (j[u] == r) ? pr : fmaf(__ldg(s + j[u]), pval(j[u]), -zr);
            q = fmaf(v[u], t, q);
          }
        }
        qv[r - lo] = q;
        acc = fmaf(pr, q, acc);
      }
      const float pq = creducef(acc);  // (its cluster barrier: every block is done reading p)
      if (tid == 0) step_alpha(sc, pq);
      __syncthreads();
      if (!sc.go) break;
      const float af = sc.af;
      float acc2 = 0.0f;
      for (int r = tid; r < hi - lo; r += kCBT) {
        dv[r] = fmaf(af, sp[r], dv[r]);
        const float ri = fmaf(-af, qv[r], rv[r]);
        rv[r] = ri;
        acc2 = fmaf(ri, ri, acc2);
      }
      const float rn = creducef(acc2);
      if (tid == 0) step_beta(sc, rn);
      __syncthreads();
      it++;
      if (!sc.go) break;
      const float bf = sc.bf;
      for (int r = tid; r < hi - lo; r += kCBT) sp[r] = fmaf(bf, sp[r], rv[r]);
      cl.sync();  // the new p is visible to the cluster
    }
    for (int r = lo + tid; r < hi; r += kCBT) y[r] += (double)dv[r - lo];
    cl.sync();  // y is read by the neighbours' residual rows
  }
  for (int r = lo + tid; r < hi; r += kCBT) {
    if (D.fix_rows && D.fix_rows[r] == 1) D.u[r] = D.fix_vals ? D.fix_vals[r] : 0.0;
    else D.u[r] = (double)s[r] * y[r];
  }
  if (rank == 0 && tid == 0) {
    out->iters = it;
    out->passes = passes;
    out->status = status;
    out->floor_hit = floor_hit;
    out->rr64 = rr;
    out->bnorm2 = bnorm2;
  }
  cl.sync();  // no block leaves while another may still read its shared memory
}

__global__ void __cluster_dims__(kCC, 1, 1) __launch_bounds__(kCBT, 1) k_pack_cluster(PackDesc* desc) {
  extern __shared__ float sm[];
  __shared__ PackDesc D;
  __shared__ double slots[4];
  const int sys = (int)(blockIdx.x / kCC);
  if (threadIdx.x == 0) D = desc[sys];
  __syncthreads();
  if (D.n <= 0) return;  // the whole cluster returns (same descriptor)
  if (D.d16) cluster_body<true>(D, sm, slots, desc + sys);
  else cluster_body<false>(D, sm, slots, desc + sys);
}

}  // namespace

struct PackSlot {
  std::mutex mu;
  PackDesc* h = nullptr;  // pinned descriptors of one pack: [0, kPackMaxSystems) one block
                          // per system, [kPackMaxSystems, 2 kPackMaxSystems) one cluster
  DevBuf d;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t g = nullptr;
  // the two kernel nodes; their grids are set to the pack's systems before each launch
  cudaGraphNode_t node_block = nullptr, node_cluster = nullptr;
  cudaKernelNodeParams par_block{}, par_cluster{};
  PackDesc* arg_block = nullptr;
  PackDesc* arg_cluster = nullptr;
};

PackSlot* pack_slot_create() { return new PackSlot(); }

void pack_slot_destroy(PackSlot* s) {
  if (!s) return;
  if (s->g) cudaGraphExecDestroy(s->g);
  if (s->graph) cudaGraphDestroy(s->graph);
  if (s->h) {
    std::lock_guard<std::mutex> lk(device_alloc_mutex());
    cudaFreeHost(s->h);
  }
  delete s;
}

namespace {

// process lifetime (never destroyed: its buffers would otherwise be released after the
// allocation mutex and the CUDA runtime have shut down)
PackSlot& default_slot() {
  static PackSlot* c = new PackSlot();
  return *c;
}

// graph: descriptors up, the one-block kernel and the cluster kernel side by side,
// results down; each kernel's grid is set per launch to the systems of its kind
// (at least one block or cluster, whose descriptor has n = 0 and returns at entry)
int pack_graph(PackSlot& c) {
  if (c.g) return ADFEM_OK;
  const size_t bytes = sizeof(PackDesc) * 2 * kPackMaxSystems;
  std::lock_guard<std::mutex> lk(device_alloc_mutex());
  if (!c.h) ADFEM_CUDA(cudaMallocHost((void**)&c.h, bytes));
  if (!c.d.p) {
    cudaError_t e = injected_alloc_failure() ? cudaErrorMemoryAllocation : cudaMalloc(&c.d.p, bytes);
    if (e != cudaSuccess) {
      c.d.p = nullptr;
      return cuda_fail(e, "cudaMalloc");
    }
    c.d.bytes = bytes;
  }
  ADFEM_CUDA(cudaFuncSetAttribute(k_pack_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kPSmem));
  ADFEM_CUDA(cudaFuncSetAttribute(k_pack_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCSmem));
  std::memset(c.h, 0, bytes);
  cudaStream_t cs, cs2;
  cudaEvent_t e0, e1;
  ADFEM_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  ADFEM_CUDA(cudaStreamCreateWithFlags(&cs2, cudaStreamNonBlocking));
  ADFEM_CUDA(cudaEventCreateWithFlags(&e0, cudaEventDisableTiming));
  ADFEM_CUDA(cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    // upload; the one-block and the cluster kernels on two branches; download
    cudaMemcpyAsync(c.d.p, c.h, bytes, cudaMemcpyHostToDevice, cs);
    cudaEventRecord(e0, cs);
    cudaStreamWaitEvent(cs2, e0, 0);
    k_pack_solve<<<kPackMaxSystems, kPBT, kPSmem, cs>>>(c.d.as<PackDesc>());
    k_pack_cluster<<<kPackMaxSystems * kCC, kCBT, kCSmem, cs2>>>(c.d.as<PackDesc>() +
                                                                                kPackMaxSystems);
    cudaEventRecord(e1, cs2);
    cudaStreamWaitEvent(cs, e1, 0);
    cudaMemcpyAsync(c.h, c.d.p, bytes, cudaMemcpyDeviceToHost, cs);
    e = cudaStreamEndCapture(cs, &graph);
  }
  if (e == cudaSuccess) {
    // the kernel nodes, told apart by their captured grids
    size_t nn = 0;
    e = cudaGraphGetNodes(graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (e == cudaSuccess) e = cudaGraphGetNodes(graph, nodes.data(), &nn);
    for (size_t i = 0; e == cudaSuccess && i < nn; i++) {
      cudaGraphNodeType t;
      e = cudaGraphNodeGetType(nodes[i], &t);
      if (e != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
      cudaKernelNodeParams kp;
      e = cudaGraphKernelNodeGetParams(nodes[i], &kp);
      if (e != cudaSuccess) break;
      if (kp.gridDim.x == (unsigned)kPackMaxSystems) {
        c.node_block = nodes[i];
        c.par_block = kp;
      } else if (kp.gridDim.x == (unsigned)(kPackMaxSystems * kCC)) {
        c.node_cluster = nodes[i];
        c.par_cluster = kp;
      }
    }
    if (e == cudaSuccess && (!c.node_block || !c.node_cluster)) e = cudaErrorInvalidValue;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&c.g, graph, 0);
  if (e == cudaSuccess) {
    c.graph = graph;
    c.arg_block = c.d.as<PackDesc>();
    c.arg_cluster = c.d.as<PackDesc>() + kPackMaxSystems;
    c.par_block.extra = nullptr;
    c.par_cluster.extra = nullptr;
  } else if (graph) {
    cudaGraphDestroy(graph);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(cs2);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    c.g = nullptr;
    return cuda_fail(e, "pack graph");
  }
  return ADFEM_OK;
}

}  // namespace

int pack_rows_limit() {
  // a cluster of kCC blocks of kCBT threads with kCSmem shared memory each must fit one
  // GPC of this device (not so on small partitions of a GPU); if the query itself fails,
  // the launch reports any problem
  static const int limit = [] {
    std::lock_guard<std::mutex> lk(device_alloc_mutex());  // (no graph capture meanwhile)
    if (cudaFuncSetAttribute(k_pack_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCSmem) !=
        cudaSuccess) {
      cudaGetLastError();
      return kPackBlockRows;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kCC);
    cfg.blockDim = dim3(kCBT);
    cfg.dynamicSmemBytes = kCSmem;
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, k_pack_cluster, &cfg) != cudaSuccess) {
      cudaGetLastError();
      return kPackMaxRows;
    }
    return nc >= 1 ? kPackMaxRows : kPackBlockRows;
  }();
  return limit;
}

int solve_packed(PackItem* items, int count, cudaStream_t st, PackSlot* slot) {
  const int limit = pack_rows_limit();
  for (int i = 0; i < count; i++) {
    Solver& S = *items[i].S;
    if (!S.prepared) return fail(ADFEM_ERR_INVALID, "packed solve: operator not prepared");
    ADFEM_TRY(solver_ensure_scaled(S, st));  // the packed kernels read the Jacobi-scaled copies
    if (S.n > limit) return fail(ADFEM_ERR_INVALID, "packed solve: system larger than the packed limit");
    if (!(items[i].rtol > 0.0) || items[i].max_iter < 1) return fail(ADFEM_ERR_INVALID, "packed solve: bad options");
  }
  PackSlot& c = slot ? *slot : default_slot();
  std::lock_guard<std::mutex> lk(c.mu);
  ADFEM_TRY(pack_graph(c));
  // systems up to kPackBlockRows rows: one block each; larger: one cluster each
  std::vector<int> small, large;
  for (int i = 0; i < count; i++) (items[i].S->n <= kPackBlockRows ? small : large).push_back(i);
  size_t is = 0, il = 0;
  while (is < small.size() || il < large.size()) {
    std::memset(c.h, 0, sizeof(PackDesc) * 2 * kPackMaxSystems);
    std::vector<std::pair<int, int>> slot_of;  // (descriptor slot, item)
    for (int k = 0; k < kPackMaxSystems && is < small.size(); k++) slot_of.emplace_back(k, small[is++]);
    for (int k = 0; k < kPackMaxSystems && il < large.size(); k++)
      slot_of.emplace_back(kPackMaxSystems + k, large[il++]);
    for (auto [k, i] : slot_of) {
      PackItem& it = items[i];
      Solver& S = *it.S;
      const Sell& A = *S.A;
      PackDesc& D = c.h[k];
      D.sptr = A.sptr.as<int32_t>();
      D.col = A.col.p;
      D.valD = A.valD64.as<double>();
      D.val32 = A.val32.as<float>();
      D.s = S.s32.as<float>();
      D.rhs = it.rhs;
      D.zero_rows = it.zero_rows;
      D.fix_rows = it.fix_rows;
      D.fix_vals = it.fix_vals;
      D.u0 = it.warm ? it.u : nullptr;
      D.u = it.u;
      D.y = S.y64.as<double>();
      D.rtol2 = it.rtol * it.rtol;
      D.n = (int)S.n;
      D.d16 = A.delta16 ? 1 : 0;
      D.max_iter = it.max_iter;
    }
    int nb = 0, nc = 0;
    for (auto [k, i] : slot_of) (k < kPackMaxSystems ? nb : nc)++;
    void* ab[] = {&c.arg_block};
    void* ac[] = {&c.arg_cluster};
    c.par_block.gridDim = dim3((unsigned)std::max(nb, 1));
    c.par_block.kernelParams = ab;
    c.par_cluster.gridDim = dim3((unsigned)(std::max(nc, 1) * kCC));
    c.par_cluster.kernelParams = ac;
    ADFEM_CUDA(cudaGraphExecKernelNodeSetParams(c.g, c.node_block, &c.par_block));
    ADFEM_CUDA(cudaGraphExecKernelNodeSetParams(c.g, c.node_cluster, &c.par_cluster));
    ADFEM_CUDA(cudaGraphLaunch(c.g, st));
    ADFEM_CUDA(cudaStreamSynchronize(st));
    for (auto [k, i] : slot_of) {
      const PackDesc& D = c.h[k];
      PackItem& it = items[i];
      it.iters = D.iters;
      it.passes = D.passes;
      it.relres = D.bnorm2 > 0.0 ? std::sqrt(D.rr64 / D.bnorm2) : 0.0;
      it.status = D.status == 1 ? ADFEM_OK : (D.status == 2 ? ADFEM_ERR_BREAKDOWN : ADFEM_ERR_NOT_CONVERGED);
    }
  }
  return ADFEM_OK;
}

}  // namespace adfem
