// Device helpers shared by the CG kernels (solver.cu, zcg.cu): thread indexing,
// sliced-ELL row access, deterministic block/grid reductions, the FP32 hi+lo axpy
// and the residual-replacement bookkeeping of the mixed solves.
#pragma once
#include "pairs.cuh"
#include "solver.cuh"

namespace adfem {

static constexpr int kT = 256;

__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t gstride() { return (int64_t)gridDim.x * blockDim.x; }

template <bool D16>
__device__ __forceinline__ int colof(const void* c, int64_t idx, int64_t r) {
  if constexpr (D16) return (int)(r + (int64_t)__ldg(reinterpret_cast<const int16_t*>(c) + idx));
  else return __ldg(reinterpret_cast<const int32_t*>(c) + idx);
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic block sum of NV values over a block of BT threads; the totals end up
// in thread 0.
template <class T, int NV, int BT = kT>
__device__ __forceinline__ void block_sum(T (&v)[NV]) {
  static_assert(BT % 32 == 0 && BT <= 1024, "block size");
  __shared__ T sh[NV][BT / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; j++) v[j] = warp_sum(v[j]);
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < NV; j++) sh[j][wid] = v[j];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int j = 0; j < NV; j++) {
      T x = lane < (BT / 32) ? sh[j][lane] : T(0);
      v[j] = warp_sum(x);
    }
  }
  __syncthreads();
}

// Grid sum of FP32 per-thread partials with the FP64 work confined to one warp per
// block: FP32 within each warp, FP64 across the block's warps (warp 0) and across the
// blocks (warp 0 of the last block to arrive, in block order).  On GB300 an FP64 warp
// instruction holds the FP64 pipe ~16 cycles, so FP64 shuffle-adds by every warp of two
// 512-thread blocks per SM would cost microseconds at the end of every launch.  Returns
// true in the last block (block-uniform); tot is valid in thread 0.
// Warp sum of FP32 values as an unevaluated FP32 pair (h + l): each butterfly step adds
// the partner's pair with an error-free two-sum, so the result carries ~48 bits.
__device__ __forceinline__ float2 warp_sum_pair(float v) {
  float h = v, l = 0.0f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, h, o), l2 = __shfl_xor_sync(0xffffffffu, l, o);
    const float s = __fadd_rn(h, h2);
    const float bb = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(h2, bb));
    l = __fadd_rn(__fadd_rn(l, l2), e);
    h = s;
  }
  return make_float2(h, l);
}

// Sum of two FP32 pairs with an error-free two-sum of the high parts (the butterfly step of
// warp_sum_pair); symmetric in its arguments, so both lanes of a butterfly get one result.
__device__ __forceinline__ float2 pair_add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  const float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  return make_float2(s, __fadd_rn(__fadd_rn(a.y, b.y), e));
}
__device__ __forceinline__ float2 shfl_pair(float2 a, int o) {
  return make_float2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
}

// Warp sums of four quantities as FP32 pairs, transposed: at the first two butterfly
// levels each lane sends the quantities it does not keep (half of them, then one), so
// the warp spends 12 shuffles instead of 40; lane L ends with the total of quantity
// 2 ((L >> 4) & 1) + ((L >> 3) & 1) (lanes 0, 8, 16, 24 hold quantities 0..3).  After a
// phase of global stores the shuffles queue behind the stores in the memory pipe, so their
// number sets the time of the block reduction.
__device__ __forceinline__ float2 warp_sum_pair4(const float2 (&x)[4]) {
  const int lane = threadIdx.x & 31;
  const bool b4 = (lane & 16) != 0, b3 = (lane & 8) != 0;
  float2 k0 = b4 ? x[2] : x[0], k1 = b4 ? x[3] : x[1];
  const float2 r0 = shfl_pair(b4 ? x[0] : x[2], 16), r1 = shfl_pair(b4 ? x[1] : x[3], 16);
  k0 = pair_add(k0, r0);
  k1 = pair_add(k1, r1);
  float2 k = pair_add(b3 ? k1 : k0, shfl_pair(b3 ? k0 : k1, 8));
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) k = pair_add(k, shfl_pair(k, o));
  return k;
}

// Grid sum of four FP32 per-thread values as FP32 pairs (the reduction of the banded mixed
// iteration), in two parts so that the caller can issue work between them.
// reduce4_arrive: transposed warp sums, the block's warps summed by warp 0 the same way,
// the block's partials stored and the block counted in; returns true in the last block to
// arrive (block-uniform).  reduce4_finish (last block, warp 0): the blocks' partials summed,
// each lane over its blocks in block order, then across lanes; tot valid in lane 0.
// Deterministic; no FP64 instruction.  partials: 4 * gridDim.x pairs.
template <int BT>
__device__ __forceinline__ bool reduce4_arrive(const float (&v)[4], float2* partials, unsigned* counter) {
  static_assert(BT % 32 == 0 && BT <= 1024, "block size");
  __shared__ float2 sh[4][BT / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int q = lane >> 3;  // the quantity a lane holds after warp_sum_pair4 (lanes 0, 8, 16, 24)
  {
    const float2 x[4] = {make_float2(v[0], 0.0f), make_float2(v[1], 0.0f), make_float2(v[2], 0.0f),
                         make_float2(v[3], 0.0f)};
    const float2 w = warp_sum_pair4(x);
    if ((lane & 7) == 0) sh[q][wid] = w;
  }
  __syncthreads();
  if (wid == 0) {
    float2 x[4];
#pragma unroll
    for (int j = 0; j < 4; j++) x[j] = lane < BT / 32 ? sh[j][lane] : make_float2(0.0f, 0.0f);
    const float2 w = warp_sum_pair4(x);
    if ((lane & 7) == 0) partials[q * gridDim.x + blockIdx.x] = w;
    __threadfence();
    __syncwarp();
    if (lane == 0) {
      const unsigned prev = atomicAdd(counter, 1u);
      last = (prev == gridDim.x - 1);
    }
  }
  __syncthreads();
  return last;
}

template <int BT>
__device__ __forceinline__ void reduce4_finish(float2* partials, unsigned* counter, float2 (&tot)[4]) {
  const int lane = threadIdx.x & 31;
  __threadfence();
  // up to 160 blocks: each lane loads all of its partials before adding (one L2 round
  // trip), then the rest, if any, in the plain loop
  constexpr int kB = 5;
  float2 pl[kB][4];
#pragma unroll
  for (int b5 = 0; b5 < kB; b5++) {
    const int b = lane + 32 * b5;
#pragma unroll
    for (int j = 0; j < 4; j++)
      pl[b5][j] = b < (int)gridDim.x ? __ldcg(partials + j * gridDim.x + b) : make_float2(0.0f, 0.0f);
  }
  float2 s[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    s[j] = pl[0][j];
#pragma unroll
    for (int b5 = 1; b5 < kB; b5++) s[j] = pair_add(s[j], pl[b5][j]);
  }
  for (int b = lane + 32 * kB; b < (int)gridDim.x; b += 32)
#pragma unroll
    for (int j = 0; j < 4; j++) s[j] = pair_add(s[j], __ldcg(partials + j * gridDim.x + b));
  const float2 r = warp_sum_pair4(s);
  // lane 0 collects the four totals (normalised pairs for the step-length arithmetic)
  const float2 r1 = make_float2(__shfl_sync(0xffffffffu, r.x, 8), __shfl_sync(0xffffffffu, r.y, 8));
  const float2 r2 = make_float2(__shfl_sync(0xffffffffu, r.x, 16), __shfl_sync(0xffffffffu, r.y, 16));
  const float2 r3 = make_float2(__shfl_sync(0xffffffffu, r.x, 24), __shfl_sync(0xffffffffu, r.y, 24));
  if (lane == 0) {
    tot[0] = df_norm(r.x, r.y);
    tot[1] = df_norm(r1.x, r1.y);
    tot[2] = df_norm(r2.x, r2.y);
    tot[3] = df_norm(r3.x, r3.y);
    *counter = 0u;
  }
}

// Grid sum of FP32 per-thread partials kept as FP32 pairs all the way: pair sums within
// each warp, across the block's warps (warp 0) and across the blocks (warp 0 of the last
// block to arrive, in block order); no FP64 instruction.  partials: NV * gridDim.x pairs.
// Returns true in the last block (block-uniform); tot is valid in thread 0.
template <int NV, int BT>
__device__ __forceinline__ bool reduce_grid_pair(float (&v)[NV], float2* partials, unsigned* counter,
                                                 float2 (&tot)[NV]) {
  static_assert(BT % 32 == 0 && BT <= 1024, "block size");
  __shared__ float2 sh[NV][BT / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2 w[NV];
#pragma unroll
  for (int j = 0; j < NV; j++) w[j] = warp_sum_pair(v[j]);
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < NV; j++) sh[j][wid] = w[j];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int j = 0; j < NV; j++) {
      float2 x = lane < BT / 32 ? sh[j][lane] : make_float2(0.0f, 0.0f);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        x = df_add(x, make_float2(__shfl_xor_sync(0xffffffffu, x.x, o), __shfl_xor_sync(0xffffffffu, x.y, o)));
      w[j] = x;
    }
    if (lane == 0) {
#pragma unroll
      for (int j = 0; j < NV; j++) partials[j * gridDim.x + blockIdx.x] = w[j];
      __threadfence();
      const unsigned prev = atomicAdd(counter, 1u);
      last = (prev == gridDim.x - 1);
    }
  }
  __syncthreads();
  if (!last) return false;
  if (wid == 0) {
    __threadfence();
    float2 s[NV];
#pragma unroll
    for (int j = 0; j < NV; j++) s[j] = make_float2(0.0f, 0.0f);
    // up to 160 blocks: each lane loads all of its partials before adding (one L2 round
    // trip instead of one per 32 blocks), then the rest, if any, in the plain loop
    constexpr int kB = 5;
    float2 pl[kB][NV];
#pragma unroll
    for (int q = 0; q < kB; q++) {
      const int b = lane + 32 * q;
#pragma unroll
      for (int j = 0; j < NV; j++)
        pl[q][j] = b < (int)gridDim.x ? __ldcg(partials + j * gridDim.x + b) : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int q = 0; q < kB; q++)
#pragma unroll
      for (int j = 0; j < NV; j++) s[j] = df_add(s[j], pl[q][j]);
    for (int b = lane + 32 * kB; b < (int)gridDim.x; b += 32)
#pragma unroll
      for (int j = 0; j < NV; j++) {
        const float2 pv = __ldcg(partials + j * gridDim.x + b);
        s[j] = df_add(s[j], pv);
      }
#pragma unroll
    for (int j = 0; j < NV; j++)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        s[j] = df_add(s[j], make_float2(__shfl_xor_sync(0xffffffffu, s[j].x, o),
                                        __shfl_xor_sync(0xffffffffu, s[j].y, o)));
    if (lane == 0) {
#pragma unroll
      for (int j = 0; j < NV; j++) tot[j] = s[j];
      *counter = 0u;
    }
  }
  return true;
}

template <int NV, int BT, bool PAIR = false>
__device__ __forceinline__ bool reduce_grid_w(float (&v)[NV], double* partials, unsigned* counter, double (&tot)[NV]) {
  static_assert(BT % 32 == 0 && BT <= 1024, "block size");
  __shared__ double sh[NV][BT / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2 w[NV];
#pragma unroll
  for (int j = 0; j < NV; j++) w[j] = PAIR ? warp_sum_pair(v[j]) : make_float2(warp_sum(v[j]), 0.0f);
  if (lane == 0)  // (FP64 conversions by one lane only)
#pragma unroll
    for (int j = 0; j < NV; j++) sh[j][wid] = PAIR ? (double)w[j].x + (double)w[j].y : (double)w[j].x;
  __syncthreads();
  if (wid == 0) {
    double x[NV];
#pragma unroll
    for (int j = 0; j < NV; j++) x[j] = warp_sum(lane < BT / 32 ? sh[j][lane] : 0.0);
    if (lane == 0) {
#pragma unroll
      for (int j = 0; j < NV; j++) partials[j * gridDim.x + blockIdx.x] = x[j];
      __threadfence();
      const unsigned prev = atomicAdd(counter, 1u);
      last = (prev == gridDim.x - 1);
    }
  }
  __syncthreads();
  if (!last) return false;
  if (wid == 0) {
    __threadfence();
    double s[NV];
#pragma unroll
    for (int j = 0; j < NV; j++) s[j] = 0.0;
#pragma unroll 4
    for (int b = lane; b < (int)gridDim.x; b += 32)
#pragma unroll
      for (int j = 0; j < NV; j++) s[j] += __ldcg(partials + j * gridDim.x + b);
#pragma unroll
    for (int j = 0; j < NV; j++) s[j] = warp_sum(s[j]);
    if (lane == 0) {
#pragma unroll
      for (int j = 0; j < NV; j++) tot[j] = s[j];
      *counter = 0u;
    }
  }
  return true;
}

// Publish this block's partial sums; the last block to arrive sums all partials in
// block order into tot (valid in thread 0) and returns true (block-uniform).
template <class T, int NV, int BT = kT>
__device__ __forceinline__ bool reduce_grid(T (&v)[NV], T* partials, unsigned* counter, T (&tot)[NV]) {
  __shared__ bool last;
  block_sum<T, NV, BT>(v);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; j++) partials[j * gridDim.x + blockIdx.x] = v[j];
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  T s[NV];
#pragma unroll
  for (int j = 0; j < NV; j++) s[j] = T(0);
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
    for (int j = 0; j < NV; j++) s[j] += __ldcg(partials + j * gridDim.x + b);
  block_sum<T, NV, BT>(s);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; j++) tot[j] = s[j];
    *counter = 0u;
  }
  return true;
}

// row geometry in sliced-ELL: first entry of row r and the slice width
__device__ __forceinline__ void sell_row(const int32_t* __restrict__ sptr, int64_t r, int64_t& base, int& w) {
  const int32_t s0 = __ldg(sptr + (r >> 5)), s1 = __ldg(sptr + (r >> 5) + 1);
  base = (int64_t)s0 + (r & 31);
  w = (s1 - s0) >> 5;
}

// (h, l) += a * p as an unevaluated FP32 pair: two-product of a*p, two-sum with h,
// renormalisation.  Explicitly rounded intrinsics keep the compiler from fusing
// or reassociating the error terms.
__device__ __forceinline__ void df_axpy(float& h, float& l, float a, float p) {
  const float ph = __fmul_rn(a, p);
  const float pl = fmaf(a, p, -ph);
  const float s = __fadd_rn(h, ph);
  const float bb = __fsub_rn(s, h);
  float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(ph, bb));
  e = __fadd_rn(e, __fadd_rn(l, pl));
  const float hi = __fadd_rn(s, e);
  l = __fsub_rn(e, __fsub_rn(hi, s));
  h = hi;
}

// Bookkeeping after an FP64 residual evaluation of a mixed solve, or of the banded FP64
// solve (thread 0 of the last block).  rr: FP64 residual norm^2 (scaled), rn: norm^2 of
// its copy in the iteration's precision, rp: (that copy, current direction) in the same
// inner product.  mode 1 replaces the recurrence residual; mode 2 only records rr.
// st->rho_new: the recurrence's value that requested the replacement.
__device__ __forceinline__ void replacement_step(CgState* st, double rr, double rn, double rp, int mode,
                                                 bool fp64_recurrence = false) {
  const double prev = st->last_rr64;
  st->rr64 = rr;
  if (mode == 2) return;
  // the solution correction has just been folded: no update term is pending any more
  st->alpha = 0.0;
  st->alpha_prev = 0.0;
  if (!isfinite(rr)) {
    st->done = 2;
    return;
  }
  if (rr <= st->stop2) {
    st->done = 1;
    return;
  }
  // The FP64 residual of an FP64 iterate cannot fall below about 2^-53 |K| |y|
  // (rounding of y itself, amplified by the largest eigenvalues).  A replacement whose
  // FP64 residual improved less than 4x on the previous one, although the recurrence
  // dropped 10x in between, means the iterate is at that attainable accuracy: stop there.
  // An FP32 recurrence can also stall for its own reasons (the inner iteration's
  // attainable accuracy), so for the mixed solves the test applies only after a
  // replacement requested by rtol has failed; an FP64 recurrence tracks the true residual
  // until the floor, so for the banded FP64 solve it also applies after a 10x drop.  (A
  // floor less than 10x above rtol is only seen through a failed rtol replacement: the
  // recurrence reaches rtol again without dropping 10x.)
  const bool stalled = prev > 0.0 && rr > 0.0625 * prev;
  const bool floor =
      stalled && (st->final_seen || (fp64_recurrence && st->rho_new <= st->delta2 * prev));
  if (floor) {
    st->floor_hit = 1;
    st->done = 1;
    return;
  }
  if (st->iters >= st->max_iter) {
    st->done = 4;
    return;
  }
  if (st->final_req) st->final_seen = 1;
  if (fp64_recurrence || st->final_seen) st->last_rr64 = rr;
  st->final_req = 0;
  if (st->updates == 0) {
    st->ar = 1.0;
    st->ap = 0.0;
  } else {
    // re-orthogonalise the direction against the new residual: p <- p - c r, folded
    // into the next direction update p_new = r + beta p = (1 - beta c) r + beta p
    const double c = rp / rn;
    const double beta = rn / st->rho;
    st->ar = 1.0 - beta * c;
    st->ap = beta;
  }
  st->updates += 1;
  st->rho = rn;
  st->ru2 = st->delta2 * rn;
  st->done = 0;
}

// Bookkeeping after the true FP64 residual of an FP64 CG solve (thread 0 of the last
// block; mode 3 of k_residual64, which has already replaced r and updated p).  rr: true
// residual norm^2 (scaled); st->rho_new: the recurrence's value that requested it.  The
// FP64 iterate has an attainable accuracy: its residual cannot fall below the rounding
// of y itself (~2^-53 |K| |y|).  The FP64 recurrence tracks the true residual closely
// until then, so a replacement after a 10x drop of the recurrence whose true residual
// improved less than 4x on the previous replacement's means the iterate is at that
// floor: the solve stops there.
__device__ __forceinline__ void replacement_step64(CgState* st, double rr) {
  const double prev = st->last_rr64;
  st->rr64 = rr;
  st->last_rr64 = rr;
  if (!isfinite(rr)) {
    st->done = 2;
    return;
  }
  if (rr <= st->stop2) {
    st->done = 1;
    return;
  }
  // (after a failed rtol replacement the recurrence may reach rtol again without a 10x
  // drop, when the floor is less than 10x above rtol: then the second stall decides)
  const bool dropped = st->rho_new <= st->delta2 * prev;
  if (prev > 0.0 && rr > 0.0625 * prev && (dropped || st->final_seen)) {
    st->floor_hit = 1;
    st->done = 1;
    return;
  }
  if (st->iters >= st->max_iter) {
    st->done = 4;
    return;
  }
  if (st->final_req) st->final_seen = 1;
  st->final_req = 0;
  st->updates += 1;
  st->rho = rr;
  st->ru2 = st->delta2 * rr;
  st->done = 0;
}

}  // namespace adfem
