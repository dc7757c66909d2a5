// Packed solves of small systems: many independent Jacobi-scaled systems solved by one
// kernel launch, one thread block per system, the whole mixed-precision solve inside
// the block.  The launch (descriptor upload, solve kernel, result download) is a CUDA
// graph captured once and relaunched for every pack, so a pack of small requests costs
// one graph launch instead of a chain of per-iteration launches per request.
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
// are limited by the block's shared-memory and L1 traffic instead.
//
// Each block's arithmetic depends only on its own system (fixed block size, row
// ownership and reduction order), so a system's result is bit-identical whatever it is
// packed with.  Every loop is bounded (iteration budget, pass cap).
#include <cstring>
#include <mutex>

#include "cg_common.cuh"

namespace adfem {

namespace {

constexpr int kPBT = 512;                // threads per system
constexpr int kMaxPasses = 64;           // outer refinement passes
constexpr double kInner2 = 1e-8;         // inner CG stops at |r_inner|^2 <= 1e-8 |r|^2
constexpr int kU = 8;                    // row entries loaded together in the inner SpMV

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
  const int n = D.n;
  const int tid = threadIdx.x;
  const float* __restrict__ s = D.s;
  double* __restrict__ y = D.y;
  float* __restrict__ rv = D.r;
  float* __restrict__ dv = D.d;
  float* __restrict__ qv = D.q;
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
    double rho = a1;
    const double target = kInner2 * rho;
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
      double pq = (double)acc, z0 = 0.0;
      bsum2(pq, z0, shb);
      if (!(pq > 0.0) || !isfinite(pq)) break;  // the correction so far is still applied
      const float af = (float)(rho / pq);
      float acc2 = 0.0f;
      for (int r = tid; r < n; r += kPBT) {
        dv[r] = fmaf(af, sp[r], dv[r]);
        const float ri = fmaf(-af, qv[r], rv[r]);
        rv[r] = ri;
        acc2 = fmaf(ri, ri, acc2);
      }
      double rho_new = (double)acc2, z1 = 0.0;
      bsum2(rho_new, z1, shb);
      it++;
      if (rho_new <= target || !isfinite(rho_new)) break;
      const float bf = (float)(rho_new / rho);
      for (int r = tid; r < n; r += kPBT) sp[r] = fmaf(bf, sp[r], rv[r]);
      __syncthreads();
      rho = rho_new;
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

}  // namespace

struct PackSlot {
  std::mutex mu;
  PackDesc* h = nullptr;  // pinned descriptors of one pack
  DevBuf d;
  cudaGraphExec_t g = nullptr;
};

PackSlot* pack_slot_create() { return new PackSlot(); }

void pack_slot_destroy(PackSlot* s) {
  if (!s) return;
  if (s->g) cudaGraphExecDestroy(s->g);
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

// graph: descriptors up, one block per descriptor slot (unused slots have n = 0 and
// return at entry), results down
int pack_graph(PackSlot& c) {
  if (c.g) return ADFEM_OK;
  const size_t bytes = sizeof(PackDesc) * kPackMaxSystems;
  std::lock_guard<std::mutex> lk(device_alloc_mutex());
  if (!c.h) ADFEM_CUDA(cudaMallocHost((void**)&c.h, bytes));
  if (!c.d.p) {
    cudaError_t e = cudaMalloc(&c.d.p, bytes);
    if (e != cudaSuccess) {
      c.d.p = nullptr;
      return cuda_fail(e, "cudaMalloc");
    }
    c.d.bytes = bytes;
  }
  ADFEM_CUDA(cudaFuncSetAttribute(k_pack_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(sizeof(float) * kPackMaxRows)));
  std::memset(c.h, 0, bytes);
  cudaStream_t cs;
  ADFEM_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaMemcpyAsync(c.d.p, c.h, bytes, cudaMemcpyHostToDevice, cs);
    k_pack_solve<<<kPackMaxSystems, kPBT, sizeof(float) * kPackMaxRows, cs>>>(c.d.as<PackDesc>());
    cudaMemcpyAsync(c.h, c.d.p, bytes, cudaMemcpyDeviceToHost, cs);
    e = cudaStreamEndCapture(cs, &graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&c.g, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    c.g = nullptr;
    return cuda_fail(e, "pack graph");
  }
  return ADFEM_OK;
}

}  // namespace

int solve_packed(PackItem* items, int count, cudaStream_t st, PackSlot* slot) {
  for (int i = 0; i < count; i++) {
    const Solver& S = *items[i].S;
    if (!S.prepared) return fail(ADFEM_ERR_INVALID, "packed solve: operator not prepared");
    if (S.n > kPackMaxRows) return fail(ADFEM_ERR_INVALID, "packed solve: system larger than the packed limit");
    if (!(items[i].rtol > 0.0) || items[i].max_iter < 1) return fail(ADFEM_ERR_INVALID, "packed solve: bad options");
  }
  PackSlot& c = slot ? *slot : default_slot();
  std::lock_guard<std::mutex> lk(c.mu);
  ADFEM_TRY(pack_graph(c));
  for (int i0 = 0; i0 < count; i0 += kPackMaxSystems) {
    const int m = std::min(kPackMaxSystems, count - i0);
    std::memset(c.h, 0, sizeof(PackDesc) * kPackMaxSystems);
    for (int k = 0; k < m; k++) {
      PackItem& it = items[i0 + k];
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
      D.r = S.r32.as<float>();
      D.d = S.pa32.as<float>();
      D.q = S.q32.as<float>();
      D.rtol2 = it.rtol * it.rtol;
      D.n = (int)S.n;
      D.d16 = A.delta16 ? 1 : 0;
      D.max_iter = it.max_iter;
    }
    ADFEM_CUDA(cudaGraphLaunch(c.g, st));
    ADFEM_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < m; k++) {
      const PackDesc& D = c.h[k];
      PackItem& it = items[i0 + k];
      it.iters = D.iters;
      it.passes = D.passes;
      it.relres = D.bnorm2 > 0.0 ? std::sqrt(D.rr64 / D.bnorm2) : 0.0;
      it.status = D.status == 1 ? ADFEM_OK : (D.status == 2 ? ADFEM_ERR_BREAKDOWN : ADFEM_ERR_NOT_CONVERGED);
    }
  }
  return ADFEM_OK;
}

}  // namespace adfem
