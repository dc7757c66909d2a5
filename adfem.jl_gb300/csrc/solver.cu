// Jacobi-scaled conjugate gradients on a sliced-ELL operator (sm_103a).
//
//  * The operator is scaled once, K~ = S K S with S = diag(1/sqrt(K_ii)), so CG on
//    K~ is Jacobi-preconditioned CG on K with no preconditioner vector in the loop.
//  * FP64 path: three kernels per iteration (SpMV + p.q, update + r.r, p update).
//  * Mixed path: FP32 difference-form copy of K~, FP32 residual/direction vectors
//    and FP32 accumulation of the dot products in the inner iteration (two kernels:
//    SpMV with the p update folded into the gather, and the x/r update).  The
//    solution correction is accumulated as an FP32 hi+lo pair (about 48 bits, no
//    FP64 instructions in the loop) and folded into the FP64 solution whenever the
//    FP32 residual has dropped by ru_delta; the residual is then recomputed in FP64
//    on the device (reliable update, with the search direction re-orthogonalised
//    against the new residual).  The stopping test is on that FP64 residual.
//  * SpMV kernels unroll the entries of a row (sliced-ELL widths are at most 8 for
//    the scalar operator and 16 for elasticity) so that every load of a row is in
//    flight at once; a plain loop serves wider operators.
//  * Reductions are deterministic: a fixed grid, per-block partials, and the last
//    block to arrive sums the partials in block order.  No kernel ever waits on
//    another: every kernel reads a device flag at entry and returns early once the
//    solve has finished, so a chunk of iterations captured in a CUDA graph can be
//    replayed without a host round trip per iteration.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>

#include "cg_common.cuh"
#include "checks.cuh"

namespace adfem {

static constexpr int kMaxBlocksPerSM = 8;
// systems up to this many rows run their solver stream at the highest priority
static constexpr int64_t kSmallSystemRows = 1 << 17;

// ---------------------------------------------------------------------------
// setup kernels
__global__ void k_csr_to_sell(int64_t n, const int32_t* __restrict__ sptr, const int32_t* __restrict__ rowptr,
                              const double* __restrict__ csr, double* __restrict__ sell) {
  const int64_t r = gtid();
  if (r >= n) return;
  const int64_t base = (int64_t)sptr[r >> 5] + (r & 31);
  for (int32_t k = rowptr[r]; k < rowptr[r + 1]; k++) sell[base + 32 * (int64_t)(k - rowptr[r])] = csr[k];
}

cudaError_t launch_csr_to_sell(const Sell& A, int64_t n, const int32_t* rowptr, const double* csr, double* sell,
                               cudaStream_t st) {
  k_csr_to_sell<<<(unsigned)((n + kT - 1) / kT), kT, 0, st>>>(n, A.sptr.as<int32_t>(), rowptr, csr, sell);
  return cudaGetLastError();
}

// s_i = rsqrt(K_ii) in FP32; flags a non-positive or non-finite diagonal
__global__ void k_scale_diag(int64_t n, const int32_t* __restrict__ sptr, const double* __restrict__ val,
                             const int32_t* __restrict__ diagpos, float* __restrict__ s, int* __restrict__ bad) {
  const int64_t r = gtid();
  if (r >= n) return;
  const int64_t base = (int64_t)sptr[r >> 5] + (r & 31);
  const double d = val[base + 32 * (int64_t)diagpos[r]];
  const float df = (float)d;
  if (!(df > 0.0f) || !isfinite(df)) {
    atomicExch(bad, 1);
    s[r] = 1.0f;
    return;
  }
  s[r] = rsqrtf(df);
}

// val64 <- s_i K_ij s_j (FP64, in place, standard form).  The difference-form copies
// (FP64 valD for residuals, FP32 val32 for the inner iteration) hold w_ij = s_i K_ij
// in off-diagonal slots and d_i = s_i^2 sum_j K_ij (the row sum, zero for rows of a
// pure Laplacian) in the diagonal slot, so that
//     (K~ x)_i = d_i x_i + sum_{j != i} w_ij (s_j x_j - s_i x_i)
// rounds in proportion to the differences s_j x_j - s_i x_i.  Smooth error modes,
// whose eigenvalues are far below FP32 resolution relative to the diagonal, keep
// their accuracy; a plain FP32 copy of K~ loses them once cond(K~) * 2^-24 ~ 1.
template <bool D16>
__global__ void k_scale_values(int64_t n, const int32_t* __restrict__ sptr, const void* __restrict__ col,
                               double* __restrict__ val, double* __restrict__ valD, float* __restrict__ val32,
                               const float* __restrict__ s, const int32_t* __restrict__ diagpos) {
  const int64_t r = gtid();
  if (r >= n) return;
  int64_t base;
  int w;
  sell_row(sptr, r, base, w);
  const double si = (double)s[r];
  double rowsum = 0.0;
  for (int k = 0; k < w; k++) {
    const int64_t idx = base + 32 * (int64_t)k;
    const double v = val[idx];
    rowsum += v;
    const double t = si * v;
    int j = colof<D16>(col, idx, r);
    if (!ADFEM_DCHECK(j >= 0 && j < n)) j = (int)r;
    val[idx] = t * (double)s[j];
    valD[idx] = t;
    val32[idx] = (float)t;
  }
  const double d = si * si * rowsum;
  valD[base + 32 * (int64_t)diagpos[r]] = d;
  val32[base + 32 * (int64_t)diagpos[r]] = (float)d;
}

// ---------------------------------------------------------------------------
// solve set-up: b~ = s * rhs (rows tagged 1 in zero_rows get 0), y0 = u / s or 0,
// ||b~||^2 and the stopping threshold.
__global__ void __launch_bounds__(kT) k_init(int64_t n, const double* __restrict__ rhs, const uint8_t* zero_rows,
                                             const float* __restrict__ s, const double* __restrict__ u0,
                                             double* __restrict__ b, double* __restrict__ y, CgState* st,
                                             double* partials, double rtol2) {
  double acc = 0.0;
  for (int64_t i = gtid(); i < n; i += gstride()) {
    const double si = (double)s[i];
    const double bi = (zero_rows && zero_rows[i] == 1) ? 0.0 : si * rhs[i];
    b[i] = bi;
    y[i] = u0 ? u0[i] / (double)s[i] : 0.0;  // inverse of u = s y up to one rounding
    acc = fma(bi, bi, acc);
  }
  double v[1] = {acc}, tot[1];
  if (reduce_grid<double, 1>(v, partials, &st->counter[0], tot) && threadIdx.x == 0) {
    st->bnorm2 = tot[0];
    st->stop2 = rtol2 * tot[0];
  }
}

// FP64 residual r = b~ - K~ y, evaluated in difference form (see k_scale_values) so
// that its rounding follows the differences of the solution rather than its size.
// mode 0: FP64 CG start (r64 = p64 = r, rho = r.r);
// mode 1: mixed residual replacement (r32 = (float) r, re-orthogonalise p, new coefficients);
// mode 2: final check only (rr64);
// mode 3: FP64 CG residual replacement (r64 = r, p64 = r + beta p64 with the beta of the
//         recurrence, then replacement_step64 decides: converged, at the attainable floor,
//         out of iterations, or continue from the true residual);
// mode 4: banded FP64 CG replacement (r into the current buffer of its pair, the norm and
//         the product with the current direction for re-orthogonalisation, as mode 1).
template <bool D16>
__global__ void __launch_bounds__(kT) k_residual64(int64_t n, const int32_t* __restrict__ sptr,
                                                   const void* __restrict__ col, const double* __restrict__ valD,
                                                   const float* __restrict__ sc, const double* __restrict__ b,
                                                   const double* __restrict__ y, double* __restrict__ r64,
                                                   double* __restrict__ p64, float* __restrict__ r32,
                                                   const float* __restrict__ pa, const float* __restrict__ pb,
                                                   double* __restrict__ r64b, const double* __restrict__ p64b,
                                                   CgState* st, double* partials, int mode, int force) {
  if (!force && st->done != 3) return;
  const int it = st->iters;
  const float* plat = (it & 1) ? pb : pa;
  double* rcur = (it & 1) ? r64b : r64;           // mode 4: the r / p pair the next launch reads
  const double* pcur = (it & 1) ? p64b : p64;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for (int64_t r = gtid(); r < n; r += gstride()) {
    int64_t base;
    int w;
    sell_row(sptr, r, base, w);
    const double yr = y[r];
    const double zr = (double)sc[r] * yr;
    double s = 0.0;
    for (int k = 0; k < w; k++) {
      const int64_t idx = base + 32 * (int64_t)k;
      int j = colof<D16>(col, idx, r);
      if (!ADFEM_DCHECK(j >= 0 && j < n)) j = (int)r;
      const double t = (j == r) ? yr : fma((double)sc[j], y[j], -zr);
      s = fma(valD[idx], t, s);
    }
    const double ri = b[r] - s;
    a0 = fma(ri, ri, a0);
    if (mode == 0) {
      r64[r] = ri;
      p64[r] = ri;
    } else if (mode == 3) {
      r64[r] = ri;
      p64[r] = fma(st->beta, p64[r], ri);
    } else if (mode == 4) {
      rcur[r] = ri;
      a1 = fma(ri, ri, a1);
      a2 = fma(ri, pcur[r], a2);
    } else if (mode == 1) {
      const float rf = (float)ri;
      r32[r] = rf;
      a1 = fma((double)rf, (double)rf, a1);
      a2 = fma((double)rf, (double)plat[r], a2);
    }
  }
  double v[3] = {a0, a1, a2}, tot[3];
  if (reduce_grid<double, 3>(v, partials, &st->counter[1], tot) && threadIdx.x == 0) {
    const double rr = tot[0];
    if (mode == 3) {
      replacement_step64(st, rr);
      return;
    }
    if (mode != 0) {
      if (mode == 4) replacement_step(st, rr, tot[1], tot[2], 1, true);
      else replacement_step(st, rr, tot[1], tot[2], mode);
      return;
    }
    st->rr64 = rr;
    if (!isfinite(rr)) st->done = 2;
    else if (rr <= st->stop2) st->done = 1;
    else if (st->iters >= st->max_iter) st->done = 4;
    else {
      st->rho = rr;
      st->ru2 = st->delta2 * rr;
      st->last_rr64 = rr;
      st->done = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// FP64 CG iteration
// Column pattern access of a sliced-ELL operator (see Sell::spat).
struct SellPat {
  const int32_t* spat;
  const int16_t* pat;
  int period;
};

// Matrix entries of one sliced-ELL row held in registers.  In a slice with a
// uniform column pattern the gather indices come from the (warp-uniform, cached)
// slice pattern and do not wait for per-row column loads.
template <class V, bool D16, int MAXW>
struct RowRegs {
  V v[MAXW];
  int j[MAXW];
  int w;
  __device__ __forceinline__ void load(const int32_t* __restrict__ sptr, const void* __restrict__ col,
                                       const SellPat& sp, const V* __restrict__ val, int64_t r, int64_t n) {
    int64_t base = 0;
    w = 0;
    int32_t so = -1;
    if (r < n) {
      sell_row(sptr, r, base, w);
      so = __ldg(sp.spat + (r >> 5));
    }
    const int16_t* pp = sp.pat + (so < 0 ? 0 : so) + (sp.period == 2 ? (int)(r & 1) * w : 0);
#pragma unroll
    for (int k = 0; k < MAXW; k++) {
      v[k] = k < w ? __ldg(val + base + 32 * k) : V(0);
      int jk = (int)r;
      if (k < w) jk = so >= 0 ? (int)r + (int)__ldg(pp + k) : colof<D16>(col, base + 32 * k, r);
      if (!ADFEM_DCHECK(jk >= 0 && jk < n)) jk = (int)r;
      j[k] = jk;
    }
  }
};

// q = K~ p (FP64, standard form) and p.q.  PF: software pipelining (the next row's
// entries are loaded while the current row's gathers are in flight).
template <bool D16, int MAXW, bool PF>
__global__ void __launch_bounds__(kT, PF ? 4 : 1) k_cg64_spmv(int64_t n, const int32_t* __restrict__ sptr,
                                                              const void* __restrict__ col, SellPat sp,
                                                              const double* __restrict__ val,
                                                              const double* __restrict__ p, double* __restrict__ q,
                                                              CgState* st, double* partials) {
  if (st->done) return;
  double acc = 0.0;
  if constexpr (MAXW > 0) {
    RowRegs<double, D16, MAXW> cur, nxt;
    int64_t r = gtid();
    if (PF) cur.load(sptr, col, sp, val, r, n);
    for (; r < n; r += gstride()) {
      if (PF) nxt.load(sptr, col, sp, val, r + gstride(), n);
      else cur.load(sptr, col, sp, val, r, n);
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < MAXW; k++)
        if (k < cur.w) s = fma(cur.v[k], __ldg(p + cur.j[k]), s);
      q[r] = s;
      acc = fma(__ldg(p + r), s, acc);
      if (PF) cur = nxt;
    }
  } else {
    for (int64_t r = gtid(); r < n; r += gstride()) {
      int64_t base;
      int w;
      sell_row(sptr, r, base, w);
      double s = 0.0;
      for (int k = 0; k < w; k++) {
        const int64_t idx = base + 32 * (int64_t)k;
        int j = colof<D16>(col, idx, r);
        if (!ADFEM_DCHECK(j >= 0 && j < n)) j = (int)r;
        s = fma(val[idx], p[j], s);
      }
      q[r] = s;
      acc = fma(p[r], s, acc);
    }
  }
  double v1[1] = {acc}, tot[1];
  if (reduce_grid<double, 1>(v1, partials, &st->counter[0], tot) && threadIdx.x == 0) {
    const double pq = tot[0];
    if (!(pq > 0.0) || !isfinite(pq)) st->done = 2;
    else st->alpha = st->rho / pq;
  }
}

// y here is the group correction z (y64 += z at every residual replacement, k_fold64):
// each update adds rounding noise of the order 2^-53 |z| instead of 2^-53 |y|, and z is
// 10x smaller than y after the first replacement, so the iterate's attainable residual
// is not set by ~10^4 roundings of the full solution (measured at 4M DOF: updating y
// directly stalls the true residual at 1.3e-9 relative).
__global__ void __launch_bounds__(kT) k_cg64_update(int64_t n, double* __restrict__ y, double* __restrict__ r,
                                                    const double* __restrict__ p, const double* __restrict__ q,
                                                    CgState* st, double* partials) {
  if (st->done) return;
  const double a = st->alpha;
  double acc = 0.0;
  const int64_t n2 = n >> 1;
  for (int64_t v2 = gtid(); v2 < n2; v2 += gstride()) {
    const double2 pp = __ldg(reinterpret_cast<const double2*>(p) + v2);
    const double2 qq = __ldg(reinterpret_cast<const double2*>(q) + v2);
    double2 yy = reinterpret_cast<double2*>(y)[v2];
    double2 rr = reinterpret_cast<double2*>(r)[v2];
    yy.x = fma(a, pp.x, yy.x);
    yy.y = fma(a, pp.y, yy.y);
    rr.x = fma(-a, qq.x, rr.x);
    rr.y = fma(-a, qq.y, rr.y);
    reinterpret_cast<double2*>(y)[v2] = yy;
    reinterpret_cast<double2*>(r)[v2] = rr;
    acc = fma(rr.x, rr.x, acc);
    acc = fma(rr.y, rr.y, acc);
  }
  for (int64_t i = 2 * n2 + gtid(); i < n; i += gstride()) {
    y[i] = fma(a, p[i], y[i]);
    const double ri = fma(-a, q[i], r[i]);
    r[i] = ri;
    acc = fma(ri, ri, acc);
  }
  double v[1] = {acc}, tot[1];
  if (reduce_grid<double, 1>(v, partials + gridDim.x, &st->counter[2], tot) && threadIdx.x == 0) {
    const double rn = tot[0];
    st->iters += 1;
    st->rho_new = rn;
    if (!isfinite(rn)) {
      st->done = 2;
    } else {
      st->beta = rn / st->rho;  // the direction update also uses it after a replacement
      // The recurrence residual drifts from the true one (at 4M DOF by ~6e-9 relative
      // over a solve): a recurrence that meets rtol, has dropped by delta since the last
      // replacement, or runs out of iterations hands over to the true FP64 residual
      // (k_residual64 mode 3), which replaces r and decides.
      if (rn <= st->stop2) {
        st->final_req = 1;
        st->done = 3;
      } else if (rn <= st->ru2 || st->iters >= st->max_iter) {
        st->done = 3;
      } else {
        st->rho = rn;
      }
    }
  }
}

__global__ void __launch_bounds__(kT) k_cg64_p(int64_t n, const double* __restrict__ r, double* __restrict__ p,
                                               const CgState* st) {
  if (st->done) return;
  const double bt = st->beta;
  const int64_t n2 = n >> 1;
  for (int64_t v2 = gtid(); v2 < n2; v2 += gstride()) {
    const double2 rr = __ldg(reinterpret_cast<const double2*>(r) + v2);
    double2 pp = reinterpret_cast<double2*>(p)[v2];
    pp.x = fma(bt, pp.x, rr.x);
    pp.y = fma(bt, pp.y, rr.y);
    reinterpret_cast<double2*>(p)[v2] = pp;
  }
  for (int64_t i = 2 * n2 + gtid(); i < n; i += gstride()) p[i] = fma(bt, p[i], r[i]);
}

// ---------------------------------------------------------------------------
// FP32 inner iteration of the mixed solve.  The two p buffers alternate: the
// iteration with counter it reads p_old = P[it&1] and writes p_new = P[(it+1)&1],
// P = {pa, pb}.  The SpMV uses the difference form of k_scale_values: the diagonal
// slot (and zero padding, column = row) multiplies p_i, an off-diagonal slot
// multiplies s_j p_j - s_i p_i.
template <bool D16, int MAXW, bool PF>
__global__ void __launch_bounds__(kT, PF ? 4 : 1) k_cg32_spmv(int64_t n, const int32_t* __restrict__ sptr,
                                                              const void* __restrict__ col, SellPat sp,
                                                              const float* __restrict__ val,
                                                              const float* __restrict__ sc,
                                                              const float* __restrict__ r, float* pa, float* pb,
                                                              float* __restrict__ q, CgState* st, double* partials) {
  if (st->done) return;
  const int it = st->iters;
  const float* __restrict__ pold = (it & 1) ? pb : pa;
  float* __restrict__ pnew = (it & 1) ? pa : pb;
  const float ar = (float)st->ar, ap = (float)st->ap;
  float acc = 0.0f;
  if constexpr (MAXW > 0) {
    RowRegs<float, D16, MAXW> cur, nxt;
    int64_t row = gtid();
    if (PF) cur.load(sptr, col, sp, val, row, n);
    for (; row < n; row += gstride()) {
      if (PF) nxt.load(sptr, col, sp, val, row + gstride(), n);
      else cur.load(sptr, col, sp, val, row, n);
      const float pr = fmaf(ap, __ldg(pold + row), ar * __ldg(r + row));
      const float zr = __ldg(sc + row) * pr;
      float s = 0.0f;
#pragma unroll
      for (int k = 0; k < MAXW; k++) {
        if (k < cur.w) {
          const int j = cur.j[k];
          const float pj = fmaf(ap, __ldg(pold + j), ar * __ldg(r + j));
          const float t = (j == row) ? pr : fmaf(__ldg(sc + j), pj, -zr);
          s = fmaf(cur.v[k], t, s);
        }
      }
      pnew[row] = pr;
      q[row] = s;
      acc = fmaf(pr, s, acc);
      if (PF) cur = nxt;
    }
  } else {
    for (int64_t row = gtid(); row < n; row += gstride()) {
      int64_t base;
      int w;
      sell_row(sptr, row, base, w);
      const float pr = fmaf(ap, pold[row], ar * r[row]);
      const float zr = sc[row] * pr;
      float s = 0.0f;
      for (int k = 0; k < w; k++) {
        const int64_t idx = base + 32 * (int64_t)k;
        int j = colof<D16>(col, idx, row);
        if (!ADFEM_DCHECK(j >= 0 && j < n)) j = (int)row;
        const float pj = fmaf(ap, pold[j], ar * r[j]);
        const float t = (j == row) ? pr : fmaf(sc[j], pj, -zr);
        s = fmaf(val[idx], t, s);
      }
      pnew[row] = pr;
      q[row] = s;
      acc = fmaf(pr, s, acc);
    }
  }
  // per-thread partials in FP32, summed as FP32 pairs within warps and in FP64 by one warp
  // per block and across blocks
  float v1[1] = {acc};
  double tot[1];
  if (reduce_grid_w<1, kT, true>(v1, partials, &st->counter[0], tot) && threadIdx.x == 0) {
    const double pq = tot[0];
    if (!(pq > 0.0) || !isfinite(pq)) st->done = 2;
    else st->alpha = st->rho / pq;
  }
}

// x/r update of the mixed iteration: residual and its norm in FP32; the solution
// correction y += alpha p accumulated in an FP32 hi+lo pair with error-free
// transformations (two-product, two-sum), i.e. about 48 bits without FP64
// instructions.  A plain FP32 accumulator would add rounding noise of size
// 2^-24 |y| that the operator amplifies by its largest eigenvalue.
__global__ void __launch_bounds__(kT) k_cg32_update(int64_t n, float* __restrict__ yh, float* __restrict__ yl,
                                                    float* __restrict__ r, const float* pa, const float* pb,
                                                    const float* __restrict__ q, CgState* st, double* partials) {
  if (st->done) return;
  const int it = st->iters;
  const float* __restrict__ pnew = (it & 1) ? pa : pb;
  const float a = (float)st->alpha;
  float acc = 0.0f;
  // four entries per thread and step (16-byte loads and stores), then the tail
  const int64_t n4 = n >> 2;
  for (int64_t v4 = gtid(); v4 < n4; v4 += gstride()) {
    const float4 p = __ldg(reinterpret_cast<const float4*>(pnew) + v4);
    const float4 qq = __ldg(reinterpret_cast<const float4*>(q) + v4);
    float4 h = reinterpret_cast<float4*>(yh)[v4];
    float4 l = reinterpret_cast<float4*>(yl)[v4];
    float4 rr = reinterpret_cast<float4*>(r)[v4];
    df_axpy(h.x, l.x, a, p.x);
    df_axpy(h.y, l.y, a, p.y);
    df_axpy(h.z, l.z, a, p.z);
    df_axpy(h.w, l.w, a, p.w);
    rr.x = fmaf(-a, qq.x, rr.x);
    rr.y = fmaf(-a, qq.y, rr.y);
    rr.z = fmaf(-a, qq.z, rr.z);
    rr.w = fmaf(-a, qq.w, rr.w);
    reinterpret_cast<float4*>(yh)[v4] = h;
    reinterpret_cast<float4*>(yl)[v4] = l;
    reinterpret_cast<float4*>(r)[v4] = rr;
    acc = fmaf(rr.x, rr.x, acc);
    acc = fmaf(rr.y, rr.y, acc);
    acc = fmaf(rr.z, rr.z, acc);
    acc = fmaf(rr.w, rr.w, acc);
  }
  for (int64_t i = 4 * n4 + gtid(); i < n; i += gstride()) {
    float h = yh[i], l = yl[i];
    df_axpy(h, l, a, pnew[i]);
    yh[i] = h;
    yl[i] = l;
    const float ri = fmaf(-a, q[i], r[i]);
    r[i] = ri;
    acc = fmaf(ri, ri, acc);
  }
  float v[1] = {acc};
  double tot[1];
  if (reduce_grid_w<1, kT, true>(v, partials + gridDim.x, &st->counter[2], tot) && threadIdx.x == 0) {
    const double rn = tot[0];
    st->iters = it + 1;
    st->rho_new = rn;
    if (!isfinite(rn)) st->done = 2;
    else if (rn <= st->stop2) {
      st->final_req = 1;
      st->done = 3;
    } else if (rn <= st->ru2) st->done = 3;
    else if (st->iters >= st->max_iter) st->done = 3;  // the FP64 check decides
    else {
      const double beta = rn / st->rho;
      st->ar = 1.0;
      st->ap = beta;
      st->rho = rn;
    }
  }
}

// FP64 CG: fold the group correction into the solution, y64 += z, z = 0 (when a
// residual replacement is due, or forced at the end of the solve)
__global__ void __launch_bounds__(kT) k_fold64(int64_t n, double* __restrict__ y64, double* __restrict__ z,
                                               const CgState* st, int force) {
  if (!force && st->done != 3) return;
  for (int64_t i = gtid(); i < n; i += gstride()) {
    y64[i] += z[i];
    z[i] = 0.0;
  }
}

// fold the correction into the FP64 solution: y64 += hi + lo, hi = lo = 0
__global__ void __launch_bounds__(kT) k_fold(int64_t n, double* __restrict__ y64, float* __restrict__ yh,
                                             float* __restrict__ yl, const CgState* st, int force) {
  if (!force && st->done != 3) return;
  for (int64_t i = gtid(); i < n; i += gstride()) {
    y64[i] += (double)yh[i] + (double)yl[i];
    yh[i] = 0.0f;
    yl[i] = 0.0f;
  }
}

// u = S y; rows tagged 1 (Dirichlet) get their prescribed value exactly (or 0)
__global__ void k_unscale(int64_t n, const double* __restrict__ y, const float* __restrict__ s,
                          const uint8_t* __restrict__ fix, const double* __restrict__ fixval,
                          double* __restrict__ u) {
  const int64_t i = gtid();
  if (i >= n) return;
  if (fix && fix[i] == 1) u[i] = fixval ? fixval[i] : 0.0;
  else u[i] = (double)s[i] * y[i];
}

// y = K x = S^-1 K~ S^-1 x
template <bool D16>
__global__ void k_apply(int64_t n, const int32_t* __restrict__ sptr, const void* __restrict__ col,
                        const double* __restrict__ val, const float* __restrict__ s, const double* __restrict__ x,
                        double* __restrict__ y) {
  const int64_t r = gtid();
  if (r >= n) return;
  int64_t base;
  int w;
  sell_row(sptr, r, base, w);
  double acc = 0.0;
  for (int k = 0; k < w; k++) {
    const int64_t idx = base + 32 * (int64_t)k;
    int j = colof<D16>(col, idx, r);
    if (!ADFEM_DCHECK(j >= 0 && j < n)) j = (int)r;
    acc = fma(val[idx], x[j] / (double)s[j], acc);
  }
  y[r] = acc / (double)s[r];
}

// ---------------------------------------------------------------------------
// dispatch on the column format and the widest slice
#define ADFEM_SELL_DISPATCH_PF(A, KERNEL, PF, GRID, STREAM, ...)                           \
  do {                                                                                     \
    if ((A).delta16) {                                                                     \
      if ((A).maxw <= 8) KERNEL<true, 8, PF><<<GRID, kT, 0, STREAM>>>(__VA_ARGS__);        \
      else if ((A).maxw <= 16) KERNEL<true, 16, PF><<<GRID, kT, 0, STREAM>>>(__VA_ARGS__); \
      else KERNEL<true, 0, PF><<<GRID, kT, 0, STREAM>>>(__VA_ARGS__);                      \
    } else {                                                                               \
      if ((A).maxw <= 8) KERNEL<false, 8, PF><<<GRID, kT, 0, STREAM>>>(__VA_ARGS__);       \
      else if ((A).maxw <= 16) KERNEL<false, 16, PF><<<GRID, kT, 0, STREAM>>>(__VA_ARGS__); \
      else KERNEL<false, 0, PF><<<GRID, kT, 0, STREAM>>>(__VA_ARGS__);                     \
    }                                                                                      \
  } while (0)
#define ADFEM_SELL_DISPATCH(S, KERNEL, GRID, STREAM, ...)                                  \
  do {                                                                                     \
    if ((S).prefetch) ADFEM_SELL_DISPATCH_PF(*(S).A, KERNEL, true, GRID, STREAM, __VA_ARGS__); \
    else ADFEM_SELL_DISPATCH_PF(*(S).A, KERNEL, false, GRID, STREAM, __VA_ARGS__);         \
  } while (0)

static SellPat sell_pat(const Sell& A) {
  return SellPat{A.spat.as<int32_t>(), A.pat.as<int16_t>(), A.pat_period};
}

Solver::~Solver() {
  if (g64) cudaGraphExecDestroy(g64);
  if (gd) cudaGraphExecDestroy(gd);
  if (g32) cudaGraphExecDestroy(g32);
  if (gz) cudaGraphExecDestroy(gz);
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : pev) cudaEventDestroy(e);
  if (stream) cudaStreamDestroy(stream);
  if (h_state) {
    std::lock_guard<std::mutex> lk(device_alloc_mutex());
    cudaFreeHost(h_state);
  }
}

template <class F>
static int resident_grid(F kernel, int sms, int64_t need, int* grid) {
  int per = 0;
  ADFEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kT, 0));
  per = std::max(1, std::min(per, kMaxBlocksPerSM));
  *grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)sms * per));
  return ADFEM_OK;
}

int Solver::init(const Sell* A_, int64_t n_) {
  A = A_;
  n = n_;
  int dev = 0, sms = 0;
  ADFEM_CUDA(cudaGetDevice(&dev));
  ADFEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t need = (n + kT - 1) / kT;
  // one grid for all grid-stride vector kernels: the smallest resident grid among them
  {
    int g = 0;
    ADFEM_TRY(resident_grid(k_cg32_update, sms, need, &grid));
    ADFEM_TRY(resident_grid(k_cg64_update, sms, need, &g));
    grid = std::min(grid, g);
    ADFEM_TRY(resident_grid(k_cg64_p, sms, need, &g));
    grid = std::min(grid, g);
    ADFEM_TRY(resident_grid(k_fold, sms, need, &g));
    grid = std::min(grid, g);
    ADFEM_TRY(resident_grid(k_fold64, sms, need, &g));
    grid = std::min(grid, g);
    ADFEM_TRY(resident_grid(k_init, sms, need, &g));
    grid = std::min(grid, g);
    ADFEM_TRY(resident_grid(k_residual64<true>, sms, need, &g));
    grid = std::min(grid, g);
  }
  const char* pf = std::getenv("ADFEM_SPMV_PREFETCH");
  prefetch = pf && pf[0] == '1';
  int g2 = 0, g3 = 0;
  const bool w8 = A->maxw <= 8;
  if (prefetch) {
    ADFEM_TRY(resident_grid(w8 ? k_cg32_spmv<true, 8, true> : k_cg32_spmv<true, 16, true>, sms, need, &g2));
    ADFEM_TRY(resident_grid(w8 ? k_cg64_spmv<true, 8, true> : k_cg64_spmv<true, 16, true>, sms, need, &g3));
  } else {
    ADFEM_TRY(resident_grid(w8 ? k_cg32_spmv<true, 8, false> : k_cg32_spmv<true, 16, false>, sms, need, &g2));
    ADFEM_TRY(resident_grid(w8 ? k_cg64_spmv<true, 8, false> : k_cg64_spmv<true, 16, false>, sms, need, &g3));
  }
  grid_spmv = std::min(g2, g3);
  ADFEM_TRY(zcg_plan(*this, sms));
  ADFEM_TRY(state.alloc(sizeof(CgState)));
  ADFEM_CUDA(cudaMemset(state.p, 0, sizeof(CgState)));
  ADFEM_TRY(partials.alloc(sizeof(double) * 4 * (size_t)std::max(std::max(grid, grid_spmv), zgrid)));
  const size_t n8 = sizeof(double) * (size_t)n, n4 = sizeof(float) * (size_t)n;
  ADFEM_TRY(s32.alloc(n4));
  ADFEM_TRY(b.alloc(n8));
  ADFEM_TRY(y64.alloc(n8));
  ADFEM_TRY(r64.alloc(n8));
  ADFEM_TRY(p64.alloc(n8));
  ADFEM_TRY(q64.alloc(n8));
  ADFEM_TRY(z64.alloc(n8));
  ADFEM_TRY(r32.alloc(n4));
  ADFEM_TRY(pa32.alloc(n4));
  ADFEM_TRY(pb32.alloc(n4));
  ADFEM_TRY(q32.alloc(n4));
  ADFEM_TRY(yh32.alloc(n4));
  ADFEM_TRY(yl32.alloc(n4));
  ADFEM_TRY(dcg_plan(*this));
  if (!h_state) {
    std::lock_guard<std::mutex> lk(device_alloc_mutex());
    ADFEM_CUDA(cudaMallocHost(&h_state, 2 * sizeof(CgState)));
  }
  if (!stream) {
    // Small systems get the highest stream priority: when solves of different sizes run
    // concurrently (the request server), the block scheduler then starts a small solve's
    // short kernels as soon as SMs free up instead of queueing them behind the whole-GPU
    // kernels of large solves.  Priorities change scheduling only, never results.
    int least = 0, greatest = 0;
    ADFEM_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int prio = n <= kSmallSystemRows ? greatest : least;
    ADFEM_CUDA(cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking, prio));
  }
  for (auto& e : ev)
    if (!e) ADFEM_CUDA(cudaEventCreate(&e));
  return ADFEM_OK;
}

// After an assembly: the copies the system's default solve needs are made at once (the
// banded mixed copies when the band fits, else the Jacobi-scaled copies), which also
// checks the diagonal; the Jacobi-scaled copies of a banded system (FP64 solves, the
// scaled mixed path, packed solves, apply) are made on first use (solver_ensure_scaled),
// so an assembly followed by mixed solves does not pay for them.
int solver_prepare(Solver& S, const int32_t* diagpos_dev, cudaStream_t user) {
  S.prepared = false;
  S.prep_scaled = false;
  if (!diagpos_dev) return fail(ADFEM_ERR_INVALID, "solver_prepare: diagonal positions required");
  S.diagpos = diagpos_dev;
  if (!S.zcg) {
    ADFEM_TRY(solver_ensure_scaled(S, user));
    S.prepared = true;
    return ADFEM_OK;
  }
  DevBuf bad;
  ADFEM_TRY(bad.alloc(sizeof(int)));
  ADFEM_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), user));
  ADFEM_TRY(zcg_prepare(S, diagpos_dev, bad.as<int>(), user));  // reads the unscaled values
  int hbad = 0;
  ADFEM_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, user));
  ADFEM_CUDA(cudaStreamSynchronize(user));
  if (hbad) return fail(ADFEM_ERR_BREAKDOWN, "operator has a non-positive or non-finite diagonal entry");
  S.prepared = true;
  return ADFEM_OK;
}

// Jacobi-scaled copies: s_i = rsqrt(K_ii), val64 <- s_i K_ij s_j in place (standard form),
// valD64 / val32 the FP64 / FP32 difference forms (k_scale_values).  Once per assembly.
int solver_ensure_scaled(Solver& S, cudaStream_t user) {
  if (S.prep_scaled) return ADFEM_OK;
  if (!S.diagpos) return fail(ADFEM_ERR_INVALID, "solver: operator not prepared");
  const Sell& A = *S.A;
  DevBuf bad;
  ADFEM_TRY(bad.alloc(sizeof(int)));
  ADFEM_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), user));
  const unsigned nb = (unsigned)((S.n + kT - 1) / kT);
  k_scale_diag<<<nb, kT, 0, user>>>(S.n, A.sptr.as<int32_t>(), A.val64.as<double>(), S.diagpos, S.s32.as<float>(),
                                    bad.as<int>());
  if (A.delta16)
    k_scale_values<true><<<nb, kT, 0, user>>>(S.n, A.sptr.as<int32_t>(), A.col.p, A.val64.as<double>(),
                                              A.valD64.as<double>(), A.val32.as<float>(), S.s32.as<float>(),
                                              S.diagpos);
  else
    k_scale_values<false><<<nb, kT, 0, user>>>(S.n, A.sptr.as<int32_t>(), A.col.p, A.val64.as<double>(),
                                               A.valD64.as<double>(), A.val32.as<float>(), S.s32.as<float>(),
                                               S.diagpos);
  ADFEM_CUDA(cudaGetLastError());
  int hbad = 0;
  ADFEM_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, user));
  ADFEM_CUDA(cudaStreamSynchronize(user));
  if (hbad) return fail(ADFEM_ERR_BREAKDOWN, "operator has a non-positive or non-finite diagonal entry");
  S.prep_scaled = true;
  return ADFEM_OK;
}

// Optional per-launch timing (profiled solves only): a pair of events around each launch,
// or around a run of launches of one kernel (open, the launches, open_n = their number,
// close), whose time is shared by its launches.
struct Timer {
  struct Pending {
    int kind, ev, count;
  };
  Solver* S = nullptr;
  SolveProfile* prof = nullptr;
  std::vector<Pending> pending;
  int next = 0;
  int open_kind = -1, open_ev = 0, open_n = 0;
  void reserve() {
    if (next + 2 > (int)S->pev.size()) {
      for (int i = 0; i < 64; i++) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        S->pev.push_back(e);
      }
    }
  }
  template <class F>
  void run(int kind, cudaStream_t st, F&& launch) {
    if (!prof) {
      launch();
      return;
    }
    reserve();
    cudaEventRecord(S->pev[next], st);
    launch();
    cudaEventRecord(S->pev[next + 1], st);
    pending.push_back({kind, next, 1});
    next += 2;
  }
  // a run of launches of one kind: open, run_in per launch, close
  void open(int kind, cudaStream_t st) {
    if (!prof) return;
    reserve();
    open_kind = kind;
    open_ev = next;
    open_n = 0;
    cudaEventRecord(S->pev[next], st);
    next += 2;
  }
  void close(cudaStream_t st) {
    if (!prof || open_kind < 0) return;
    cudaEventRecord(S->pev[open_ev + 1], st);
    pending.push_back({open_kind, open_ev, open_n});
    open_kind = -1;
  }
  // after a stream sync: add the measured durations, recycle the events
  void collect() {
    for (auto& pk : pending) {
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, S->pev[pk.ev], S->pev[pk.ev + 1]);
      prof->ms[pk.kind] += ms;
      prof->n[pk.kind] += pk.count;
    }
    pending.clear();
    next = 0;
  }
};

// enqueue one FP64 CG iteration
static void enqueue_cg64(Solver& S, cudaStream_t st, Timer* tm = nullptr) {
  Timer none;
  if (!tm) tm = &none;
  const Sell& A = *S.A;
  auto* sp = A.sptr.as<int32_t>();
  auto* cs = S.state.as<CgState>();
  auto* part = S.partials.as<double>();
  tm->run(0, st, [&] {
    ADFEM_SELL_DISPATCH(S, k_cg64_spmv, S.grid_spmv, st, S.n, sp, A.col.p, sell_pat(A), A.val64.as<double>(),
                        S.p64.as<double>(), S.q64.as<double>(), cs, part);
  });
  tm->run(1, st, [&] {
    k_cg64_update<<<S.grid, kT, 0, st>>>(S.n, S.z64.as<double>(), S.r64.as<double>(), S.p64.as<double>(),
                                         S.q64.as<double>(), cs, part);
  });
  tm->run(2, st, [&] { k_cg64_p<<<S.grid, kT, 0, st>>>(S.n, S.r64.as<double>(), S.p64.as<double>(), cs); });
}

static void enqueue_residual(Solver& S, cudaStream_t st, int mode, int force, Timer* tm = nullptr) {
  Timer none;
  if (!tm) tm = &none;
  const Sell& A = *S.A;
  auto* sp = A.sptr.as<int32_t>();
  tm->run(3, st, [&] {
    if (A.delta16)
      k_residual64<true><<<S.grid, kT, 0, st>>>(S.n, sp, A.col.p, A.valD64.as<double>(), S.s32.as<float>(),
                                                S.b.as<double>(), S.y64.as<double>(), S.r64.as<double>(),
                                                S.p64.as<double>(), S.r32.as<float>(), S.pa32.as<float>(),
                                                S.pb32.as<float>(), S.dr1.as<double>(), S.dp1.as<double>(),
                                                S.state.as<CgState>(), S.partials.as<double>(), mode, force);
    else
      k_residual64<false><<<S.grid, kT, 0, st>>>(S.n, sp, A.col.p, A.valD64.as<double>(), S.s32.as<float>(),
                                                 S.b.as<double>(), S.y64.as<double>(), S.r64.as<double>(),
                                                 S.p64.as<double>(), S.r32.as<float>(), S.pa32.as<float>(),
                                                 S.pb32.as<float>(), S.dr1.as<double>(), S.dp1.as<double>(),
                                                 S.state.as<CgState>(), S.partials.as<double>(), mode, force);
  });
}

static void enqueue_cg32(Solver& S, cudaStream_t st, Timer* tm = nullptr) {
  Timer none;
  if (!tm) tm = &none;
  const Sell& A = *S.A;
  auto* sp = A.sptr.as<int32_t>();
  auto* cs = S.state.as<CgState>();
  auto* part = S.partials.as<double>();
  tm->run(0, st, [&] {
    ADFEM_SELL_DISPATCH(S, k_cg32_spmv, S.grid_spmv, st, S.n, sp, A.col.p, sell_pat(A), A.val32.as<float>(),
                        S.s32.as<float>(), S.r32.as<float>(), S.pa32.as<float>(), S.pb32.as<float>(),
                        S.q32.as<float>(), cs, part);
  });
  tm->run(1, st, [&] {
    k_cg32_update<<<S.grid, kT, 0, st>>>(S.n, S.yh32.as<float>(), S.yl32.as<float>(), S.r32.as<float>(),
                                         S.pa32.as<float>(), S.pb32.as<float>(), S.q32.as<float>(), cs, part);
  });
}

// fold + FP64 residual replacement of the mixed solve (both return at entry unless due)
static void enqueue_reliable_update(Solver& S, cudaStream_t st, int force, Timer* tm = nullptr) {
  Timer none;
  if (!tm) tm = &none;
  tm->run(2, st, [&] {
    k_fold<<<S.grid, kT, 0, st>>>(S.n, S.y64.as<double>(), S.yh32.as<float>(), S.yl32.as<float>(),
                                  S.state.as<CgState>(), force);
  });
  enqueue_residual(S, st, 1, force, tm);
}

// fold + true-residual replacement of the FP64 CG (both return at entry unless due)
static void enqueue_fp64_replacement(Solver& S, cudaStream_t st, int force, Timer* tm = nullptr) {
  Timer none;
  if (!tm) tm = &none;
  tm->run(2, st, [&] {
    k_fold64<<<S.grid, kT, 0, st>>>(S.n, S.y64.as<double>(), S.z64.as<double>(), S.state.as<CgState>(), force);
  });
  enqueue_residual(S, st, 3, force, tm);
}

// The four iteration schemes: FP64 CG (three kernels), the scaled two-kernel mixed
// iteration, and the banded one-kernel iterations (zcg.cu), mixed and FP64.
enum class Path { FP64, MIXED, BANDED, DBANDED };

// fold + true-residual replacement of the banded FP64 path (both return at entry unless due)
static void enqueue_dreliable_update(Solver& S, cudaStream_t st, int force, Timer* tm = nullptr) {
  Timer none;
  if (!tm) tm = &none;
  tm->run(2, st, [&] { dcg_enqueue_fold(S, st, force); });
  enqueue_residual(S, st, 4, force, tm);
}

// fold + FP64 residual replacement of the banded path (both return at entry unless due)
static void enqueue_zreliable_update(Solver& S, cudaStream_t st, int force, Timer* tm = nullptr) {
  Timer none;
  if (!tm) tm = &none;
  tm->run(2, st, [&] { zcg_enqueue_fold(S, st, force); });
  tm->run(3, st, [&] { zcg_enqueue_residual(S, st, 1, force); });
}

// iterations between two replacement checks of the mixed paths (each check is two
// launches that return at entry unless a replacement is due; 16 instead of 8: +1.5%
// solves/s at 4M DOF)
#ifndef ADFEM_CG_CHECK
#define ADFEM_CG_CHECK 16
#endif
constexpr int kCheck = ADFEM_CG_CHECK;

// iteration i of a chunk of `chunk` (the replacement check follows every kCheck-th and the last)
static void enqueue_iteration(Solver& S, Path path, int i, int chunk, cudaStream_t st, Timer* tm = nullptr) {
  const bool check = (i + 1) % kCheck == 0 || i + 1 == chunk;
  if (path == Path::FP64) {
    enqueue_cg64(S, st, tm);
    if (check) enqueue_fp64_replacement(S, st, 0, tm);
  } else if (path == Path::MIXED) {
    enqueue_cg32(S, st, tm);
    if (check) enqueue_reliable_update(S, st, 0, tm);
  } else if (path == Path::BANDED) {
    if (tm) tm->run(0, st, [&] { zcg_enqueue_iter(S, st); });
    else zcg_enqueue_iter(S, st);
    if (check) enqueue_zreliable_update(S, st, 0, tm);
  } else {
    if (tm) tm->run(0, st, [&] { dcg_enqueue_iter(S, st); });
    else dcg_enqueue_iter(S, st);
    if (check) enqueue_dreliable_update(S, st, 0, tm);
  }
}

static int chunk_launches(Path path, int chunk) {
  int ru = 0;
  for (int i = 0; i < chunk; i++)
    if ((i + 1) % kCheck == 0 || i + 1 == chunk) ru++;
  if (path == Path::FP64) return 3 * chunk + 2 * ru;
  return (path == Path::MIXED ? 2 : 1) * chunk + 2 * ru;  // (both banded paths: one launch)
}

// capture `chunk` iterations into a graph (kernels read all scalars from device state)
// A capture can be invalidated by work another host thread does at the same time that
// has to synchronise the device (allocations take device_alloc_mutex for that reason;
// first-use loading of kernel code is another such event); such a capture is retried.
template <class F>
static int capture_graph(Solver& S, cudaGraphExec_t* out, F&& body) {
  cudaError_t e = cudaSuccess;
  for (int attempt = 0; attempt < 8; attempt++) {
    cudaGraph_t g = nullptr;
    {
      std::lock_guard<std::mutex> lk(device_alloc_mutex());
      ADFEM_CUDA(cudaStreamBeginCapture(S.stream, cudaStreamCaptureModeThreadLocal));
      body();
      e = cudaStreamEndCapture(S.stream, &g);
    }
    if (e == cudaErrorStreamCaptureInvalidated || e == cudaErrorStreamCaptureUnjoined) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();  // the launches of the invalidated capture reported it too
      std::this_thread::yield();
      continue;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return ADFEM_OK;
  }
  return cuda_fail(e, "cudaStreamEndCapture (retried)");
}

static int capture_chunk(Solver& S, Path path, int chunk, cudaGraphExec_t* out) {
  return capture_graph(S, out, [&] {
    for (int i = 0; i < chunk; i++) enqueue_iteration(S, path, i, chunk, S.stream);
  });
}

// the solve's outcome is decided: converged, breakdown, max_iter or a kernel wait that gave up
static bool finished(int done) { return done == 1 || done == 2 || done == 4 || done == 5; }

struct GraphExecGuard {
  cudaGraphExec_t g = nullptr;
  ~GraphExecGuard() {
    if (g) cudaGraphExecDestroy(g);
  }
};

int solver_solve(Solver& S, const double* rhs, double* u, const uint8_t* zero_rows, const uint8_t* fix_rows,
                 const double* fix_vals, const adfem_solver_opts& o, adfem_solver_stats* stats, cudaStream_t user,
                 SolveProfile* prof) {
  if (!S.prepared) return fail(ADFEM_ERR_INVALID, "solver: operator not prepared");
  const bool mixed = o.precision == ADFEM_PREC_MIXED;
  if (o.precision != ADFEM_PREC_FP64 && !mixed) return fail(ADFEM_ERR_INVALID, "solver: unknown precision");
  if (!(o.rtol > 0.0) || o.max_iter < 1) return fail(ADFEM_ERR_INVALID, "solver: rtol must be > 0, max_iter >= 1");
  const int chunk = std::max(1, std::min(o.chunk > 0 ? o.chunk : 32, 512));
  const Path path = !mixed ? (S.dcg ? Path::DBANDED : Path::FP64) : (S.zcg ? Path::BANDED : Path::MIXED);
  if (path != Path::BANDED) ADFEM_TRY(solver_ensure_scaled(S, user));
  cudaStream_t st = S.stream;
  cudaGraphExec_t* gx = path == Path::FP64 ? &S.g64
                        : (path == Path::MIXED ? &S.g32 : (path == Path::BANDED ? &S.gz : &S.gd));
  int* gc = path == Path::FP64 ? &S.g64_chunk
            : (path == Path::MIXED ? &S.g32_chunk : (path == Path::BANDED ? &S.gz_chunk : &S.gd_chunk));
  if (!prof) {
    if (*gx && *gc != chunk) {
      cudaGraphExecDestroy(*gx);
      *gx = nullptr;
    }
    if (!*gx) {
      ADFEM_TRY(capture_chunk(S, path, chunk, gx));
      *gc = chunk;
    }
  }
  long long launches = 0;
  ADFEM_CUDA(cudaEventRecord(S.ev[0], user));
  ADFEM_CUDA(cudaStreamWaitEvent(st, S.ev[0], 0));
  ADFEM_CUDA(cudaEventRecord(S.ev[1], st));

  CgState init;
  std::memset(&init, 0, sizeof(init));
  init.max_iter = o.max_iter;
  const double dl = (o.ru_delta > 0.0 && o.ru_delta < 1.0) ? o.ru_delta : 0.1;
  init.delta2 = dl * dl;
  init.done = 3;  // lets the forced residual kernel run in mixed mode
  ADFEM_CUDA(cudaMemcpyAsync(S.state.p, &init, sizeof(CgState), cudaMemcpyHostToDevice, st));
  if (path == Path::BANDED) {
    ADFEM_TRY(zcg_clear(S, st));
    zcg_enqueue_init(S, st, rhs, zero_rows, o.warm_start ? u : nullptr, o.rtol * o.rtol);
    zcg_enqueue_residual(S, st, 1, 1);
  } else {
    k_init<<<S.grid, kT, 0, st>>>(S.n, rhs, zero_rows, S.s32.as<float>(), o.warm_start ? u : nullptr,
                                  S.b.as<double>(), S.y64.as<double>(), S.state.as<CgState>(), S.partials.as<double>(),
                                  o.rtol * o.rtol);
    ADFEM_CUDA(cudaGetLastError());
    if (mixed) {
      ADFEM_CUDA(cudaMemsetAsync(S.pa32.p, 0, sizeof(float) * S.n, st));
      ADFEM_CUDA(cudaMemsetAsync(S.pb32.p, 0, sizeof(float) * S.n, st));
      ADFEM_CUDA(cudaMemsetAsync(S.yh32.p, 0, sizeof(float) * S.n, st));
      ADFEM_CUDA(cudaMemsetAsync(S.yl32.p, 0, sizeof(float) * S.n, st));
      enqueue_residual(S, st, 1, 1);
    } else if (path == Path::DBANDED) {
      ADFEM_TRY(dcg_clear(S, st));
      enqueue_residual(S, st, 4, 1);
    } else {
      ADFEM_CUDA(cudaMemsetAsync(S.z64.p, 0, sizeof(double) * S.n, st));
      enqueue_residual(S, st, 0, 1);
    }
  }
  ADFEM_CUDA(cudaGetLastError());
  launches += 2;

  CgState cur;
  if (prof && (path == Path::BANDED || path == Path::DBANDED)) {
    // runs of kCheck iterations as a captured graph (as in the solve) with an event pair
    // around each run, the fold and residual checks with an event pair around each launch
    Timer tm;
    tm.S = &S;
    tm.prof = prof;
    GraphExecGuard runk;
    ADFEM_TRY(capture_graph(S, &runk.g, [&] {
      for (int i = 0; i < kCheck; i++) {
        if (path == Path::BANDED) zcg_enqueue_iter(S, S.stream);
        else dcg_enqueue_iter(S, S.stream);
      }
    }));
    for (;;) {
      for (int r = 0; r < 4; r++) {
        tm.open(0, st);
        tm.open_n = kCheck;
        ADFEM_CUDA(cudaGraphLaunch(runk.g, st));
        tm.close(st);
        if (path == Path::BANDED) enqueue_zreliable_update(S, st, 0, &tm);
        else enqueue_dreliable_update(S, st, 0, &tm);
      }
      launches += 4 * (kCheck + 2);
      ADFEM_CUDA(cudaGetLastError());
      ADFEM_CUDA(cudaMemcpyAsync(&S.h_state[0], S.state.p, sizeof(CgState), cudaMemcpyDeviceToHost, st));
      ADFEM_CUDA(cudaStreamSynchronize(st));
      tm.collect();
      cur = S.h_state[0];
      if (finished(cur.done)) break;
    }
  } else if (prof) {
    // kernel-by-kernel loop with an event pair around every launch
    Timer tm;
    tm.S = &S;
    tm.prof = prof;
    for (;;) {
      for (int i = 0; i < chunk; i++) enqueue_iteration(S, path, i, chunk, st, &tm);
      launches += chunk_launches(path, chunk);
      ADFEM_CUDA(cudaGetLastError());
      ADFEM_CUDA(cudaMemcpyAsync(&S.h_state[0], S.state.p, sizeof(CgState), cudaMemcpyDeviceToHost, st));
      ADFEM_CUDA(cudaStreamSynchronize(st));
      tm.collect();
      cur = S.h_state[0];
      if (finished(cur.done)) break;
    }
  } else {
    // pipelined host loop: keep one chunk in flight beyond the one being checked
    int slot = 0;
    ADFEM_CUDA(cudaGraphLaunch(*gx, st));
    ADFEM_CUDA(cudaMemcpyAsync(&S.h_state[0], S.state.p, sizeof(CgState), cudaMemcpyDeviceToHost, st));
    ADFEM_CUDA(cudaEventRecord(S.ev[2], st));
    launches += chunk_launches(path, chunk);
    for (;;) {
      ADFEM_CUDA(cudaGraphLaunch(*gx, st));
      launches += chunk_launches(path, chunk);
      ADFEM_CUDA(cudaMemcpyAsync(&S.h_state[1 - slot], S.state.p, sizeof(CgState), cudaMemcpyDeviceToHost, st));
      ADFEM_CUDA(cudaEventRecord(S.ev[2 + (1 - slot)], st));
      ADFEM_CUDA(cudaEventSynchronize(S.ev[2 + slot]));
      cur = S.h_state[slot];
      if (finished(cur.done)) break;
      slot = 1 - slot;
    }
  }
  // final fold (mixed), FP64 residual (difference form) for the report, then u = S y
  // with the Dirichlet rows set exactly
  if (path == Path::BANDED) {
    zcg_enqueue_fold(S, st, 1);
    launches += 1;
  } else if (path == Path::DBANDED) {
    dcg_enqueue_fold(S, st, 1);
    launches += 1;
  } else if (mixed) {
    k_fold<<<S.grid, kT, 0, st>>>(S.n, S.y64.as<double>(), S.yh32.as<float>(), S.yl32.as<float>(),
                                  S.state.as<CgState>(), 1);
    launches += 1;
  } else {
    k_fold64<<<S.grid, kT, 0, st>>>(S.n, S.y64.as<double>(), S.z64.as<double>(), S.state.as<CgState>(), 1);
    launches += 1;
  }
  if (path == Path::BANDED) {
    zcg_enqueue_residual(S, st, 2, 1);
    zcg_enqueue_unscale(S, st, fix_rows, fix_vals, u);
  } else {
    enqueue_residual(S, st, 2, 1);
    k_unscale<<<(unsigned)((S.n + kT - 1) / kT), kT, 0, st>>>(S.n, S.y64.as<double>(), S.s32.as<float>(), fix_rows,
                                                             fix_vals, u);
  }
  ADFEM_CUDA(cudaGetLastError());
  launches += 2;
  ADFEM_CUDA(cudaMemcpyAsync(&S.h_state[0], S.state.p, sizeof(CgState), cudaMemcpyDeviceToHost, st));
  ADFEM_CUDA(cudaEventRecord(S.ev[3], st));
  ADFEM_CUDA(cudaEventSynchronize(S.ev[3]));
  CgState fin = S.h_state[0];
  ADFEM_CUDA(cudaStreamWaitEvent(user, S.ev[3], 0));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, S.ev[1], S.ev[3]);
  int status = ADFEM_OK;
  if (cur.done == 2) status = ADFEM_ERR_BREAKDOWN;
  else if (cur.done == 4) status = ADFEM_ERR_NOT_CONVERGED;
  else if (cur.done == 5) status = ADFEM_ERR_CUDA;
  const double relres = fin.bnorm2 > 0.0 ? std::sqrt(fin.rr64 / fin.bnorm2) : 0.0;
  if (stats) {
    stats->iterations = fin.iters;
    stats->updates = fin.updates;
    stats->relres = relres;
    stats->ms = ms;
    stats->status = status;
    stats->launches = launches;
  }
  if (status == ADFEM_ERR_BREAKDOWN) return fail(status, "CG breakdown: p.Ap <= 0 or non-finite (operator not SPD?)");
  if (status == ADFEM_ERR_CUDA) return fail(status, "banded CG: a wait on the shared-memory matrix ring timed out");
  if (status == ADFEM_ERR_NOT_CONVERGED)
    return fail(status, "CG did not reach rtol within max_iter (relres " + std::to_string(relres) + ")");
  return ADFEM_OK;
}

int solver_apply(Solver& S, const double* x, double* y, cudaStream_t user) {
  ADFEM_TRY(solver_ensure_scaled(S, user));
  const Sell& A = *S.A;
  const unsigned nb = (unsigned)((S.n + kT - 1) / kT);
  if (A.delta16)
    k_apply<true><<<nb, kT, 0, user>>>(S.n, A.sptr.as<int32_t>(), A.col.p, A.val64.as<double>(), S.s32.as<float>(), x,
                                       y);
  else
    k_apply<false><<<nb, kT, 0, user>>>(S.n, A.sptr.as<int32_t>(), A.col.p, A.val64.as<double>(), S.s32.as<float>(),
                                        x, y);
  ADFEM_CUDA(cudaGetLastError());
  return ADFEM_OK;
}

ADFEM_CHECK_READER(check_line_solver)

}  // namespace adfem
