// Mixed-precision Jacobi-PCG for banded operators, one kernel per iteration (sm_103a).
//
// Vectors are kept in the physical space of K (the operator is not Jacobi-scaled):
//   Z  = D^-1 r   preconditioned residual (FP32),
//   P             search direction (FP32),
//   q^ = D^-1 K P (FP32),
//   Y             solution correction since the last fold (FP32 hi+lo pair),
//   D  = fp32(diag K), used as the Jacobi preconditioner everywhere (also by the FP64
//        residual), so the preconditioner is exactly consistent across precisions.
// K P is evaluated in difference form, (K P)_i = rowsum_i P_i + sum_{j!=i} K_ij (P_j - P_i),
// from an FP32 copy whose diagonal slot holds the FP64 row sum rounded once.
//
// Launch k of the iteration, for the rows of each block's contiguous range:
//   Z_k = Z_{k-1} - a_{k-1} q^_{k-1}   (lagged update),
//   Y += a_{k-2} P_{k-2} + a_{k-1} P_{k-1}   on even k only (P_{k-2} is still in the buffer
//        launch k overwrites; a fold after an odd k adds the pending a_{k-1} P_{k-1}),
//   P_k = ar Z_k + ap P_{k-1}          (ar = 1, ap = beta_{k-1}; other values after a
//                                       residual replacement re-orthogonalise P),
//   q_k = K P_k,  q^_k = q_k / D,
//   rho_k = sum D Z_k^2,  P_k.q_k,  Z_k.q_k,  q_k.q^_k   (one grid reduction).
// The last block sets a_k = rho_k / P.q and beta_k from the one-step estimate
//   rho_{k+1} ~ rho_k - 2 a_k Z.q + a_k^2 q.q^   (the algebra of Z_{k+1} = Z_k - a_k q^).
// rho_{k+1} is then computed directly by launch k+1, so the estimate never compounds.
// Z.q = P.q - ap P_{k-1}.q; with ar = 1 the second term vanishes by the conjugacy of
// successive directions and is not formed; after a residual replacement (ar != 1) it is.
// When rho_k meets the replacement or stopping threshold, launch k's direction work is
// discarded (the iteration counter does not advance): Y and Z_k are consistent, the
// FP64 residual replaces Z_k, and the iteration is redone from there with a = 0.
//
// Gathers: the columns of row i lie in [i - H, i + H] (H = matrix band).  A block owns a
// contiguous row range and works through it in super-tiles of at most S rows (one for
// the usual sizes).  Phase 1 streams the positions [lo - H, hi + H) of the super-tile
// (Z, q^, P of the previous iteration), forms P_k into shared memory and updates Z, P
// and Y of its own rows; after one barrier, phase 2 streams the matrix rows of the
// super-tile and gathers P_k from shared memory.  Neither phase has a barrier inside,
// so every warp keeps its loads in flight independently.  Halo positions belong to
// neighbouring blocks and are recomputed there bit-identically; the Z, P and q^ buffers
// are ping-pong pairs, so halos always read the previous iteration's values.
//
// Variants: 8-wide rows (P1 Poisson; an opt-in RING form streams the matrix through
// shared memory), 16-wide rows (plain, or the node-block form B2 of interleaved 2-DOF
// elasticity), 24-wide rows in 768-thread blocks reading the sliced layout with per-slice
// widths (P2).  The four dot products are reduced by reduce4_arrive / reduce4_finish; each
// thread's last q^ stores are issued after its block is counted in.  Launches are
// programmatic dependent launches (griddepcontrol) in the solver's graphs.
#include <cstdlib>
#include <mutex>
#include <vector>

#include "cg_common.cuh"
#include "checks.cuh"

namespace adfem {

struct ZcgArgs {
  int64_t n;
  int64_t L;          // rows per block (multiple of 32)
  int S;              // rows per super-tile (multiple of 32)
  int H;              // band: |col - row| <= H
  int period;         // slice pattern period
  int zw;             // fixed slice width of the banded layout
  const int32_t* zpid;  // per slice: id of its column pattern in `pool`, or -1 (per-entry deltas in colz)
  const int32_t* pool;  // [pattern id][period][MAXW] column deltas, padded with 0 (copied to shared memory)
  int npool;            // ints in pool
  const int16_t* colz;  // column deltas (fixed-width layout; 24-wide: the sliced layout)
  const float* val;   // FP32 difference-form values, physical scale (same layout as colz)
  const float* dz;    // fp32(K_ii)
  const float2* bz;   // B2: per row {K_ii, K_(i,i^1)} in FP32, the row of its node's 2x2 block
  float* z[2];
  float* p[2];
  float* q[2];
  float* yh;
  float* yl;
  CgState* st;
  double* partials;
  const int32_t* sptr;  // 24-wide variant: slice offsets of the sliced layout (entries), variable widths
  int ns;      // stages of the matrix ring (RING variants; 0 otherwise)
  int refill;  // RING: 1 the ring is refilled through phase 2, 0 only the first ns stages come through it
};

// Lanes of the current node pair (rows 2a, 2a+1 sit in lanes 2j, 2j+1 of a warp): the
// block-Jacobi shuffles name exactly these two lanes, which always execute them together.
__device__ __forceinline__ unsigned pair_mask() { return 3u << (threadIdx.x & 30); }

// L2 policies.  The matrix is read once per iteration: it is streamed with evict-first,
// so that the vectors the next iteration reads again (Z, P, q^, Y, D, about as large as
// L2) stay cached, and those vectors are stored with evict-last (ADFEM_ZCG_KEEP_STORES=0
// at build time turns that off).
// The iteration's dot products: ADFEM_ZCG_WRED=3 (default) sums them as FP32 pairs
// (error-free two-sums, ~48 bits) within warps, across warps and across blocks, and the
// last block computes the step lengths in the same double-float arithmetic
// (reduce_grid_pair); 2: FP32 pairs within each warp, FP64 across warps and blocks and in
// the step lengths (reduce_grid_w); 1: plain FP32 within warps; 0: FP64 block sums by every
// warp.  Measured on GB300 at 4M DOF (per iteration): 0 -> 62.3 us, 1 -> 57.6 us but 3.4%
// more iterations (the rounding of the residual estimate), 2 -> 60.2 us with the iterates
// of 0 (52.9 us with the later 1024-thread blocks); with 2, the end-of-launch reduction --
// chains of dependent FP64 additions, shuffles and divisions in one warp and one thread,
// while every other SM waits -- took ~10 us of each iteration (per-block timestamps).
#ifndef ADFEM_ZCG_WRED
#define ADFEM_ZCG_WRED 3
#endif
#ifndef ADFEM_ZCG_KEEP_STORES
#define ADFEM_ZCG_KEEP_STORES 1
#endif
// With WRED 3: 1 (default) sums the four dot products with the transposed warp reduction
// (reduce4_arrive / reduce4_finish, 12 shuffles per warp) and issues the q^ stores of each
// thread's last rows after its block's partials are out; 0 with one butterfly per quantity
// (40 shuffles) after all stores.  After phase 2 the reduction's shuffles wait behind the
// SM's queued global stores: per-block timestamps at 4M DOF gave 2.4 us from the end of
// phase 2 to the warp sums with 40 shuffles, 1.8 us with 12.
#ifndef ADFEM_ZCG_RED4
#define ADFEM_ZCG_RED4 1
#endif
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_evict_last_policy() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void st_keep(float* a, float v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(a), "f"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ float ld_stream(const float* a, uint64_t pol) {
  float v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
  return v;
}

// Programmatic dependent launch (launches with the programmatic-serialization attribute):
// wait for the previous grid in the stream to complete with its memory visible (a no-op
// when launched without the attribute), and let the next grid be scheduled.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// ---- the matrix ring of the RING variants: each stage holds the fixed-width values of
// BT consecutive rows (contiguous in global memory), copied by the bulk-copy engine
// (cp.async.bulk, this GPU's memory into this CTA's shared memory) and tracked by a
// full and an empty mbarrier per stage.
static constexpr int kZMaxStages = 4;
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
// makes the initialised barriers visible to the bulk-copy engine (async proxy)
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the phase of the given parity to complete; gives up after 2^31 SM cycles
// (about a second) and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity) {
  if (mbar_try_wait(b, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(b, parity))
    if (clock64() - t0 > (1ll << 31)) return false;
  return true;
}
// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16) completing
// on the mbarrier, with an L2 cache policy
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
      : "memory");
}

// Positions and row indices are 32-bit (the plan requires n and the fixed-width layout
// to stay below 2^31).  A warp's 32 rows are one slice (block ranges and super-tiles are
// multiples of 32 rows), so the pattern/no-pattern branch is warp-uniform.
// B2: block difference form of an interleaved 2-DOF operator (rows 2a, 2a+1 are the x, y
// DOFs of node a): each neighbour is differenced against the value of the same component
// at row i's node, the same-component row sum sits in the diagonal slot and the
// other-component row sum in the slot of the partner DOF i^1 (see k_zprep).  The
// preconditioner is then the node-block Jacobi M = blockdiag(K_aa) (2x2 per node): a row
// and its partner are neighbouring lanes of one warp (block ranges, windows and tiles
// start at even rows), so M and M^-1 are applied with one lane shuffle.
//
// RING: phase 2 reads the matrix values from a shared-memory ring of A.ns stages of BT
// rows each, filled by bulk copies that thread 0 issues; the first stages are issued at
// kernel entry (the values do not depend on the iteration), so they load during phase 1
// and the phase barrier.  A row's diagonal and slice pattern id are loaded one stage
// ahead into registers.  Thread 0 refills a stage once every warp has released it.
// The arithmetic and its order are those of the plain variant, so the iterates are
// bit-identical.
template <int MAXW, int BT, int U1, int U2, bool B2, bool RING>
__global__ void __launch_bounds__(BT, 1024 / BT) k_zcg_iter(ZcgArgs A) {
  static_assert(MAXW % 4 == 0, "pattern rows are loaded as int4");
  constexpr int kNDP = MAXW > 16 ? MAXW / 2 : 1;  // words of prefetched column deltas (24-wide rows)
  extern __shared__ __align__(128) float zsm[];
  const int stagef = RING ? BT * A.zw : 0;                        // floats per ring stage
  float* ring = zsm;                                              // RING: A.ns stages (16-byte aligned)
  int* spool = reinterpret_cast<int*>(zsm + (RING ? A.ns * stagef : 0));  // column patterns
  float* sP = reinterpret_cast<float*>(spool) + ((A.npool + 3) & ~3);    // P_k of the super-tile's positions
  // (the column patterns are fixed for the solve: copied while the previous launch may
  // still be finishing)
  for (int j = threadIdx.x; j < A.npool; j += BT) spool[j] = __ldg(A.pool + j);
  // programmatic dependent launch: this launch's blocks start as the previous launch's
  // blocks exit; the state and the vectors are read only after it has completed
  pdl_wait();
  pdl_trigger();
  CgState* st = A.st;
  if (st->done) return;
  const int it = st->iters;
  const int cur = it & 1, nxt = cur ^ 1;
  const float* __restrict__ zprev = A.z[cur];
  const float* __restrict__ pprev = A.p[cur];
  const float* __restrict__ qprev = A.q[cur];
  float* __restrict__ znew = A.z[nxt];
  float* __restrict__ pnew = A.p[nxt];
  float* __restrict__ qnew = A.q[nxt];
  float* __restrict__ yh = A.yh;
  float* __restrict__ yl = A.yl;
  const float a = (float)st->alpha, ar = (float)st->ar, ap = (float)st->ap;
  const float a2 = (float)st->alpha_prev;
#if ADFEM_ZCG_WRED == 3
  // the scalars the last block's step-length code reads, fetched now by thread 0 (the one
  // thread that uses them): after the reduction they would be a chain of dependent global
  // loads on the critical path between two launches
  __shared__ double s_sc[3];
  __shared__ float2 s_th[2];  // the stopping and replacement thresholds as FP32 pairs
  __shared__ int s_maxit;
  if (threadIdx.x == 0) {
    s_sc[0] = st->alpha;
    s_sc[1] = st->ar;
    s_sc[2] = st->ap;
    s_th[0] = d_to_df(st->stop2);
    s_th[1] = d_to_df(st->ru2);
    s_maxit = st->max_iter;
  }
#endif
  const bool ydo = (it & 1) == 0;   // the two-step solution update runs on even iterations
  const bool full_zq = ar != 1.0f;  // uniform
  const uint64_t pol = l2_evict_first_policy();
  const uint64_t keep = ADFEM_ZCG_KEEP_STORES ? l2_evict_last_policy() : 0;
  const int tid = threadIdx.x;
  const int zw = A.zw;
  const int n = (int)A.n;
  const int blo = (int)blockIdx.x * (int)A.L;
  const int bhi = min(blo + (int)A.L, n);
  float pq = 0.f, pkq = 0.f, qq = 0.f, rr = 0.f;

  // ---- RING: stage t covers chunk c of super-tile j (t = j * cs + c, cs chunks of BT rows
  // per full super-tile); the copy is rounded up to whole 32-row slices (the fixed-width
  // layout holds every slice in full, padding included)
  __shared__ uint64_t s_full[RING ? kZMaxStages : 1], s_empty[RING ? kZMaxStages : 1];
  __shared__ int s_fault;
  int nstage = 0, t = 0;
  bool fault = false;
  auto issue = [&](int ts) {
    const int cs = (A.S + BT - 1) / BT;
    const int j = ts / cs;
    const int r0 = blo + j * A.S + (ts - j * cs) * BT;
    const int r1 = min(min(r0 + BT, blo + (j + 1) * A.S), bhi);
    const int slot = ts % A.ns;
    const unsigned bytes = (unsigned)(((r1 - r0 + 31) & ~31) * zw) * (unsigned)sizeof(float);
    mbar_expect_tx(&s_full[slot], bytes);
    bulk_load(ring + slot * stagef, A.val + (size_t)r0 * zw, bytes, &s_full[slot], pol);
  };
  if constexpr (RING) {
    const int cs = (A.S + BT - 1) / BT;
    const int nsup = (bhi - blo + A.S - 1) / A.S;
    nstage = (nsup - 1) * cs + (bhi - blo - (nsup - 1) * A.S + BT - 1) / BT;
    if (tid == 0) {
      s_fault = 0;
      for (int s = 0; s < A.ns; s++) {
        mbar_init(&s_full[s], 1);
        mbar_init(&s_empty[s], BT / 32);
      }
      mbar_init_fence();
      for (int ts = 0; ts < min(A.ns, nstage); ts++) issue(ts);
    }
    if (!A.refill) nstage = min(A.ns, nstage);  // stages that go through the ring
  }
  // q^ of the rows of this thread's last trip, not yet stored: rows dbase + u BT, u < dcnt
  float dq[U2];
  int dbase = 0, dcnt = 0;
  auto put = [&](int i, float qh) {
    if constexpr (ADFEM_ZCG_KEEP_STORES) st_keep(qnew + i, qh, keep);
    else qnew[i] = qh;
  };
  auto flush = [&]() {
#pragma unroll
    for (int u = 0; u < U2; u++)
      if (u < dcnt) put(dbase + u * BT, dq[u]);
    dcnt = 0;
  };
  // RING: diagonal (block row) and slice pattern id of this thread's row in the next stage
  float nd = 0.f, nc = 0.f;
  int npid = -1;
  auto fetch_dc = [&](int i, float& d, float& c, int& pid) {
    if constexpr (B2) {
      const float2 b = __ldg(A.bz + i);
      d = b.x;
      c = b.y;
    } else {
      d = __ldg(A.dz + i);
      c = 0.f;
    }
    pid = __ldg(A.zpid + (i >> 5));
  };

  for (int lo = blo; lo < bhi; lo += A.S) {
    const int hi = min(lo + A.S, bhi);
    // (B2: the window starts and ends at even positions, so lane pairs hold node pairs)
    const int wlo = B2 ? (max(lo - A.H, 0) & ~1) : max(lo - A.H, 0);
    const int whi = B2 ? min((hi + A.H + 1) & ~1, n) : min(hi + A.H, n);
    if (lo != blo) __syncthreads();  // the previous super-tile's gathers are done
    if (RING && lo + tid < hi) fetch_dc(lo + tid, nd, nc, npid);
    // ---- phase 1: P_k for [wlo, whi) into shared memory; Z, P, Y of own rows.  All loads
    // of a trip (U1 positions per thread) are issued before any store.
    struct In {
      float zp, qp, pp, p2, h, l, d, c;
      bool own;
    };
    auto fetch1 = [&](int pos, In& x) {
      x.own = pos >= lo && pos < hi;
      x.zp = __ldg(zprev + pos);
      x.qp = __ldg(qprev + pos);
      x.pp = __ldg(pprev + pos);
      const bool yupd = x.own && ydo;
      x.p2 = yupd ? pnew[pos] : 0.f;  // P_{k-2}, read before this thread overwrites it with P_k
      x.h = yupd ? yh[pos] : 0.f;
      x.l = yupd ? yl[pos] : 0.f;
      if constexpr (B2) {
        const float2 b = x.own ? __ldg(A.bz + pos) : make_float2(0.f, 0.f);
        x.d = b.x;
        x.c = b.y;
      } else {
        x.d = x.own ? __ldg(A.dz + pos) : 0.f;
        x.c = 0.f;
      }
    };
    auto commit = [&](int pos, In& x) {
      const float zk = fmaf(-a, x.qp, x.zp);
      const float pk = fmaf(ap, x.pp, __fmul_rn(ar, zk));
      // B2: the partner DOF's Z_k (lane pairs move together through the window)
      const float zpart = B2 ? __shfl_xor_sync(pair_mask(), zk, 1) : 0.f;
      sP[pos - wlo] = pk;
      if (x.own) {
        if constexpr (ADFEM_ZCG_KEEP_STORES) {
          st_keep(znew + pos, zk, keep);
          st_keep(pnew + pos, pk, keep);
        } else {
          znew[pos] = zk;
          pnew[pos] = pk;
        }
        if (ydo) {
          df_axpy(x.h, x.l, a2, x.p2);
          df_axpy(x.h, x.l, a, x.pp);
          if constexpr (ADFEM_ZCG_KEEP_STORES) {
            st_keep(yh + pos, x.h, keep);
            st_keep(yl + pos, x.l, keep);
          } else {
            yh[pos] = x.h;
            yl[pos] = x.l;
          }
        }
        // rho_k = Z_k . M Z_k
        rr = B2 ? fmaf(fmaf(x.d, zk, __fmul_rn(x.c, zpart)), zk, rr) : fmaf(__fmul_rn(x.d, zk), zk, rr);
      }
    };
    int pos = wlo + tid;
    for (; pos + (U1 - 1) * BT < whi; pos += U1 * BT) {
      In x[U1];
#pragma unroll
      for (int u = 0; u < U1; u++) fetch1(pos + u * BT, x[u]);
#pragma unroll
      for (int u = 0; u < U1; u++) commit(pos + u * BT, x[u]);
    }
    // (a partial last trip with all of a thread's remaining positions issued at once, the
    // positions past the window clamped and not committed, needed more than the 64 registers
    // and measured slower: 4M-DOF Poisson 50.9 against 50.4 us, 2M-DOF elasticity 53.3
    // against 48.9 us)
    for (; pos < whi; pos += BT) {
      In x0;
      fetch1(pos, x0);
      commit(pos, x0);
    }
    __syncthreads();
    // ---- phase 2: q = K P_k for the rows [lo, hi)
    // 24-wide rows: slice offsets of the sliced layout for this thread's row of the trip
    // (sp0, sp1), loaded one trip ahead (nsp0, nsp1) so that the value loads do not wait for them
    int sp0 = 0, sp1 = 0, nsp0 = 0, nsp1 = 0;
    auto row = [&](int i, const float (&v)[MAXW], float d, float c, int pid, const unsigned (&dpk)[kNDP]) -> float {
      const float Pi = sP[i - wlo];
      const float Pp = B2 ? sP[(i ^ 1) - wlo] : Pi;  // partner DOF (B2: rows come in even/odd pairs)
      const int dpart = (i & 1) ? -1 : 1;            // column delta of the partner DOF
      // (24-wide rows: the column deltas were loaded with the values, two int16 per word, and
      // are unpacked as they are used)
      int dl[MAXW > 16 ? 1 : MAXW];
      if constexpr (MAXW > 16) {
        dl[0] = 0;
      } else if (pid >= 0) {
        // the slice's column pattern (int32, padded with 0 to MAXW per row parity)
        const int4* pv = reinterpret_cast<const int4*>(spool) + (pid * A.period + (A.period == 2 ? (i & 1) : 0)) *
                                                                     (MAXW / 4);
#pragma unroll
        for (int h = 0; h < MAXW / 4; h++) {
          const int4 x = pv[h];
          dl[4 * h] = x.x;
          dl[4 * h + 1] = x.y;
          dl[4 * h + 2] = x.z;
          dl[4 * h + 3] = x.w;
        }
      } else {
        const int base = (i >> 5) * (32 * zw) + (i & 31);
#pragma unroll
        for (int k = 0; k < MAXW; k++) dl[k] = k < zw ? (int)__ldg(A.colz + base + 32 * k) : 0;
      }
      // (24-wide rows: the slice's own width, uniform over the warp, ends the row: a 9-entry
      // edge row does not spend the instructions of 24)
      const int wrow = MAXW > 16 ? (sp1 - sp0) >> 5 : MAXW;
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < MAXW; k++) {
        if (k >= wrow) break;
        const int dk = MAXW > 16 ? (int)(short)(dpk[k >> 1] >> (16 * (k & 1))) : dl[MAXW > 16 ? 0 : k];
        float tv;
        if (dk == 0) tv = Pi;
        else if (B2 && dk == dpart) tv = Pp;
        else {
          int w_ = i + dk - wlo;
          if (!ADFEM_DCHECK(w_ >= 0 && w_ < whi - wlo)) w_ = i - wlo;
          tv = __fsub_rn(sP[w_], (B2 && (dk & 1)) ? Pp : Pi);
        }
        s = fmaf(v[k], tv, s);
      }
      float qh;
      if constexpr (B2) {
        // q^ = M^-1 q with the node's 2x2 block [d c; c dp] (partner row in the next lane)
        const unsigned msk = pair_mask();
        const float qpart = __shfl_xor_sync(msk, s, 1);
        const float dp = __shfl_xor_sync(msk, d, 1);
        const float det = __fsub_rn(__fmul_rn(d, dp), __fmul_rn(c, c));
        qh = __fdiv_rn(__fsub_rn(__fmul_rn(dp, s), __fmul_rn(c, qpart)), det);
      } else {
        qh = __fdiv_rn(s, d);
      }
      pq = fmaf(Pi, s, pq);
      qq = fmaf(s, qh, qq);
      if (full_zq) pkq = fmaf(__ldg(pprev + i), s, pkq);
      return qh;
    };
    // fixed-width layout: entry k of row i at (i>>5)*32*zw + 32k + (i&31) (padding: value 0,
    // delta 0), so the loads of a row depend on nothing but i
    auto slice_of = [&](int i, int& a, int& b) {
      if constexpr (MAXW > 16) {
        a = __ldg(A.sptr + (i >> 5));
        b = __ldg(A.sptr + (i >> 5) + 1);
      }
    };
    auto fetch = [&](int i, float (&v)[MAXW], float& d, float& c, int& pid, unsigned (&dpk)[kNDP]) {
      // (24-wide: the slice's own width, entry k of row i at sptr[i/32] + 32k + i%32)
      const int base = MAXW > 16 ? sp0 + (i & 31) : (i >> 5) * (32 * zw) + (i & 31);
      const int wr = MAXW > 16 ? (sp1 - sp0) >> 5 : zw;
#pragma unroll
      for (int k = 0; k < MAXW; k++) v[k] = k < wr ? ld_stream(A.val + base + 32 * k, pol) : 0.f;
      if constexpr (MAXW > 16) {
#pragma unroll
        for (int k = 0; k < MAXW; k += 2) {
          const unsigned a0 = k < wr ? (unsigned)(unsigned short)__ldg(A.colz + base + 32 * k) : 0u;
          const unsigned a1 = k + 1 < wr ? (unsigned)(unsigned short)__ldg(A.colz + base + 32 * (k + 1)) : 0u;
          dpk[k >> 1] = a0 | (a1 << 16);
        }
      } else {
        dpk[0] = 0u;
      }
      if constexpr (B2) {
        const float2 b = __ldg(A.bz + i);
        d = b.x;
        c = b.y;
      } else {
        d = __ldg(A.dz + i);
        c = 0.f;
      }
      pid = MAXW > 16 ? -1 : __ldg(A.zpid + (i >> 5));
    };
    int c0 = lo;
    if constexpr (RING) {
      // one row per thread and stage; the stage's local layout is the global one (slice
      // tid/32, entry k of lane tid%32 at 32k)
      for (; c0 < hi && (A.refill || t < A.ns); c0 += BT, t++) {
        const int i = c0 + tid;
        const float d = nd, c = nc;
        const int pid = npid;
        if (i + BT < hi) fetch_dc(i + BT, nd, nc, npid);
        const int slot = t % A.ns;
        const unsigned par = (unsigned)(t / A.ns) & 1u;
        if (!mbar_wait(&s_full[slot], par)) fault = true;
        if (i < hi) {
          const float* sv = ring + slot * stagef + (tid >> 5) * (32 * zw) + (tid & 31);
          float v[MAXW];
#pragma unroll
          for (int k = 0; k < MAXW; k++) v[k] = k < zw ? sv[32 * k] : 0.f;
          const unsigned dpk[kNDP] = {};
          put(i, row(i, v, d, c, pid, dpk));
        }
        __syncwarp();
        if ((tid & 31) == 0) mbar_arrive(&s_empty[slot]);
        if (tid == 0 && A.refill && t + A.ns < nstage) {
          if (!mbar_wait(&s_empty[slot], par)) fault = true;
          issue(t + A.ns);
        }
      }
    }
    // rows not served by the ring: loaded by the threads; the q^ of a trip is stored after
    // the next trip's loads are issued (or at the end of the launch)
    int i = c0 + tid;
    static_assert(MAXW <= 16 || U2 == 1, "24-wide rows: one row per thread and trip");
    if constexpr (MAXW > 16) {
      // 24-wide rows are grouped by length within windows of 8 slices, so the slice width
      // depends on the slice's position in its window; with a fixed warp -> slice map and a
      // multiple of 8 warps, warp w would take the slice at position w mod 8 on every trip
      // and the warps of the widest positions would finish last.  The warp's slice of the
      // trip rotates by one per trip: each warp meets every position, and the rows of a trip
      // are still the BT rows from the trip's first row (a thread's rows increase, so it stops
      // at its first row past hi)
      constexpr int kNW = BT / 32;
      int slot = tid >> 5;
      int tb = c0;  // the trip's first row
      if (i < hi) slice_of(i, sp0, sp1);
      while (i < hi) {
        float v0[MAXW], d0, cc0;
        int g0;
        unsigned dp0[kNDP];
        fetch(i, v0, d0, cc0, g0, dp0);
        tb += BT;
        slot = slot + 1 == kNW ? 0 : slot + 1;
        const int ni = tb + 32 * slot + (tid & 31);
        if (ni < hi) slice_of(ni, nsp0, nsp1);
        flush();
        dq[0] = row(i, v0, d0, cc0, g0, dp0);
        dbase = i;
        dcnt = 1;
        sp0 = nsp0;
        sp1 = nsp1;
        i = ni;
      }
    }
    for (; MAXW <= 16 && i + (U2 - 1) * BT < hi; i += U2 * BT) {  // U2 rows per thread and trip, loads first
      float v[U2][MAXW], d[U2], c[U2];
      int pid[U2];
      unsigned dpk[U2][kNDP];
#pragma unroll
      for (int u = 0; u < U2; u++) fetch(i + u * BT, v[u], d[u], c[u], pid[u], dpk[u]);
      if (MAXW > 16 && i + BT < hi) slice_of(i + BT, nsp0, nsp1);
      flush();
#pragma unroll
      for (int u = 0; u < U2; u++) dq[u] = row(i + u * BT, v[u], d[u], c[u], pid[u], dpk[u]);
      dbase = i;
      dcnt = U2;
      sp0 = nsp0;
      sp1 = nsp1;
    }
    for (; MAXW <= 16 && i < hi; i += BT) {
      float v0[MAXW], d0, cc0;
      int g0;
      unsigned dp0[kNDP];
      fetch(i, v0, d0, cc0, g0, dp0);
      flush();
      dq[0] = row(i, v0, d0, cc0, g0, dp0);
      dbase = i;
      dcnt = 1;
    }
  }
  if constexpr (RING) {
    // a wait that gave up: the stages still in flight are waited for (again bounded), so no
    // copy lands in the shared memory of a finished block, and the solve stops with done = 5
    if (fault) s_fault = 1;
    __syncthreads();
    if (s_fault && tid == 0) {
      for (int ts = max(0, nstage - A.ns); ts < nstage; ts++) mbar_wait(&s_full[ts % A.ns], (unsigned)(ts / A.ns) & 1u);
      atomicExch(&st->fault, 1);
    }
  }

#if ADFEM_ZCG_WRED == 3
  // FP32 pairs end to end (the default): the reduction and the step-length arithmetic of the
  // last block spend no FP64 instruction on the critical path between two launches
  float v[4] = {pq, pkq, qq, rr};
  float2 tot2[4];
#if ADFEM_ZCG_RED4
  const bool lastb = reduce4_arrive<BT>(v, reinterpret_cast<float2*>(A.partials), &st->counter[0]);
  // the deferred q^ stores go out once the block is counted in; warp 0 of the last block
  // stores after the step lengths (the fence of reduce4_finish would wait for them)
  const bool w0last = lastb && (threadIdx.x >> 5) == 0;
  if (!w0last) flush();
  if (w0last) reduce4_finish<BT>(reinterpret_cast<float2*>(A.partials), &st->counter[0], tot2);
#else
  flush();
  const bool lastb = reduce_grid_pair<4, BT>(v, reinterpret_cast<float2*>(A.partials), &st->counter[0], tot2);
#endif
  if (lastb && threadIdx.x == 0) {
    const float2 pq2 = tot2[0], qq2 = tot2[2], rho2 = tot2[3];
    // decisions in pair arithmetic against the thresholds prepared at entry: no dependent
    // FP64 instruction before the branch
    float2 zq2 = pq2;
    if (full_zq && s_sc[1] != 0.0)
      zq2 = d_to_df((df_to_d(pq2) - s_sc[2] * df_to_d(tot2[1])) / s_sc[1]);  // after a replacement only
    if (RING && *reinterpret_cast<volatile int*>(&st->fault)) {
      st->done = 5;
    } else if (!isfinite(rho2.x) || !isfinite(pq2.x)) {
      st->done = 2;
    } else if (df_le(rho2, s_th[0])) {
      st->final_req = 1;
      st->done = 3;
    } else if (df_le(rho2, s_th[1]) || it >= s_maxit) {
      st->done = 3;  // the FP64 residual decides
    } else if (!(pq2.x > 0.0f)) {
      st->done = 2;
    } else {
      const float2 al = df_div(rho2, pq2);
      const float2 az = df_mul(al, zq2);
      const float2 est = df_add(df_add(rho2, df_neg(make_float2(2.0f * az.x, 2.0f * az.y))),
                                df_mul(df_mul(al, al), qq2));
      const float2 apf = est.x > 0.0f ? df_div(est, rho2) : make_float2(0.0f, 0.0f);
      st->alpha_prev = s_sc[0];
      st->alpha = df_to_d(al);
      st->ar = 1.0;
      st->ap = df_to_d(apf);
      st->rho = df_to_d(rho2);
      st->iters = it + 1;
    }
  }
#if ADFEM_ZCG_RED4
  if (w0last) flush();
#endif
#else
  flush();
  double tot[4];
  bool lastb;
  if constexpr (ADFEM_ZCG_WRED) {
    float v[4] = {pq, pkq, qq, rr};
    lastb = reduce_grid_w<4, BT, (ADFEM_ZCG_WRED == 2)>(v, A.partials, &st->counter[0], tot);
  } else {
    double v[4] = {(double)pq, (double)pkq, (double)qq, (double)rr};
    lastb = reduce_grid<double, 4, BT>(v, A.partials, &st->counter[0], tot);
  }
  if (lastb && threadIdx.x == 0) {
    const double pqd = tot[0], qqd = tot[2], rho = tot[3];
    const double zqd = (full_zq && st->ar != 0.0) ? (pqd - st->ap * tot[1]) / st->ar : pqd;
    if (RING && *reinterpret_cast<volatile int*>(&st->fault)) {
      st->done = 5;
    } else if (!isfinite(rho) || !isfinite(pqd)) {
      st->done = 2;
    } else if (rho <= st->stop2) {
      st->final_req = 1;
      st->done = 3;
    } else if (rho <= st->ru2 || it >= st->max_iter) {
      st->done = 3;  // the FP64 residual decides
    } else if (!(pqd > 0.0)) {
      st->done = 2;
    } else {
      const double al = rho / pqd;
      const double est = rho - 2.0 * al * zqd + al * al * qqd;
      st->alpha_prev = st->alpha;
      st->alpha = al;
      st->ar = 1.0;
      st->ap = fmax(est, 0.0) / rho;
      st->rho = rho;
      st->iters = it + 1;
    }
  }
#endif
}

// Operator copies for the banded path from the unscaled FP64 sliced-ELL values:
// difference form (off-diagonal K_ij, diagonal slot = row sum) in FP64 (sliced-ELL
// layout, for the FP64 residual) and FP32 (fixed-width layout of width zw, whose
// padding stays 0), and the FP32 diagonal.  With block2 (interleaved 2-DOF operator)
// the diagonal slot holds the row sum over same-component columns and the partner
// slot (column i^1) the sum over other-component columns: the two sums vanish in
// interior rows (rigid translations), which keeps FP32 rounding relative to the
// component-wise differences.  Flags a non-positive or non-finite diagonal.
__global__ void k_zprep(int64_t n, const int32_t* __restrict__ sptr, const int16_t* __restrict__ col,
                        const double* __restrict__ val, const int32_t* __restrict__ diagpos, int zw, int block2,
                        double* __restrict__ valz64, float* __restrict__ valz32, float* __restrict__ dz,
                        float2* __restrict__ bz, int* __restrict__ bad) {
  const int64_t r = gtid();
  if (r >= n) return;
  int64_t base;
  int w;
  sell_row(sptr, r, base, w);
  const int64_t fbase = zw > 0 ? ((r >> 5) * 32) * zw + (r & 31) : base;  // (zw 0: the sliced layout itself)
  const int dpart = (r & 1) ? -1 : 1;
  double rs = 0.0, ro = 0.0;  // same-component / other-component row sums
  for (int k = 0; k < w; k++) {
    const double v = val[base + 32 * (int64_t)k];
    if (block2 && (col[base + 32 * (int64_t)k] & 1)) ro += v;
    else rs += v;
  }
  const int dp = diagpos[r];
  for (int k = 0; k < w; k++) {
    const int64_t idx = base + 32 * (int64_t)k;
    const double v = k == dp ? rs : ((block2 && col[idx] == dpart) ? ro : val[idx]);
    valz64[idx] = v;
    valz32[fbase + 32 * (int64_t)k] = (float)v;
  }
  float d = (float)val[base + 32 * (int64_t)dp];
  if (!(d > 0.0f) || !isfinite(d)) {
    atomicExch(bad, 1);
    d = 1.0f;
  }
  dz[r] = d;
  if (block2) {
    // the row of the node's 2x2 block: {K_ii, K_(i,i^1)}; the partner row is the next
    // lane (n is even), so the block's determinant is checked here too
    float c = 0.0f;
    for (int k = 0; k < w; k++)
      if (col[base + 32 * (int64_t)k] == dpart) c = (float)val[base + 32 * (int64_t)k];
    const unsigned pm = pair_mask();
    const float dpp = __shfl_xor_sync(pm, d, 1);
    c = __shfl_sync(pm, c, threadIdx.x & 30);  // both rows take K_(2a,2a+1): an exactly symmetric block
    if (!(__fsub_rn(__fmul_rn(d, dpp), __fmul_rn(c, c)) > 0.0f) || !isfinite(c)) atomicExch(bad, 1);
    bz[r] = make_float2(d, c);
  }
}

// b = rhs (rows tagged 1 in zero_rows get 0), y0 = u0 or 0, ||b||_{D^-1}^2 and the
// stopping threshold.
__global__ void __launch_bounds__(kT) k_zinit(int64_t n, const double* __restrict__ rhs, const uint8_t* zero_rows,
                                              const float* __restrict__ dz, const float2* __restrict__ bz,
                                              const double* __restrict__ u0, double* __restrict__ b,
                                              double* __restrict__ y, CgState* st, double* partials, double rtol2) {
  double acc = 0.0;
  for (int64_t i = gtid(); i < n; i += gstride()) {
    const double bi = (zero_rows && zero_rows[i] == 1) ? 0.0 : rhs[i];
    b[i] = bi;
    y[i] = u0 ? u0[i] : 0.0;
    if (bz) {  // node-block preconditioner: b . M^-1 b (the partner row is the next lane)
      const unsigned msk = pair_mask();
      const float2 m = bz[i];
      const double d = m.x, c = m.y, dp = __shfl_xor_sync(msk, d, 1), bp = __shfl_xor_sync(msk, bi, 1);
      acc = fma(bi, (dp * bi - c * bp) / (d * dp - c * c), acc);
    } else {
      acc = fma(bi, bi / (double)dz[i], acc);
    }
  }
  double v[1] = {acc}, tot[1];
  if (reduce_grid<double, 1>(v, partials, &st->counter[0], tot) && threadIdx.x == 0) {
    st->bnorm2 = tot[0];
    st->stop2 = rtol2 * tot[0];
  }
}

// FP64 residual r = b - K y in difference form; mode 1 also replaces Z (the buffer the
// next iteration reads) by fp32(r / D) and supplies the re-orthogonalisation dot with
// the direction that iteration starts from; mode 2 only records ||r||_{D^-1}^2.
__global__ void __launch_bounds__(kT) k_zres64(int64_t n, const int32_t* __restrict__ sptr,
                                               const int16_t* __restrict__ col, const double* __restrict__ valz,
                                               int block2, const float* __restrict__ dz,
                                               const float2* __restrict__ bz, const double* __restrict__ b,
                                               const double* __restrict__ y, float* z0, float* z1, const float* p0,
                                               const float* p1, CgState* st, double* partials, int mode, int force) {
  if (!force && st->done != 3) return;
  const int it = st->iters;
  float* zc = (it & 1) ? z1 : z0;
  const float* pc = (it & 1) ? p1 : p0;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for (int64_t r = gtid(); r < n; r += gstride()) {
    int64_t base;
    int w;
    sell_row(sptr, r, base, w);
    const double yr = y[r];
    const int dpart = (r & 1) ? -1 : 1;
    const double yp = block2 ? y[r ^ 1] : yr;
    double s = 0.0;
    for (int k = 0; k < w; k++) {
      const int64_t idx = base + 32 * (int64_t)k;
      const int dl = (int)__ldg(col + idx);
      double t;
      if (dl == 0) t = yr;
      else if (block2 && dl == dpart) t = yp;
      else {
        int64_t j = r + dl;
        if (!ADFEM_DCHECK(j >= 0 && j < n)) j = r;
        t = y[j] - ((block2 && (dl & 1)) ? yp : yr);
      }
      s = fma(valz[idx], t, s);
    }
    const double ri = b[r] - s;
    if (block2) {
      // node-block preconditioner: z = M^-1 r with the FP32 block the iteration uses (the
      // partner row is the next lane; both rows of a node are in range together)
      const unsigned msk = pair_mask();
      const float2 m = bz[r];
      const double d = m.x, c = m.y, dp = __shfl_xor_sync(msk, d, 1), rp = __shfl_xor_sync(msk, ri, 1);
      const double zt = (dp * ri - c * rp) / (d * dp - c * c);
      a0 = fma(ri, zt, a0);
      if (mode == 1) {
        const float zf = (float)zt;
        zc[r] = zf;
        const double zd = (double)zf, zp = __shfl_xor_sync(msk, zd, 1);
        const double mz = fma(d, zd, c * zp);  // (M Z)_r
        a1 = fma(mz, zd, a1);
        a2 = fma(mz, (double)pc[r], a2);
      }
    } else {
      const double di = (double)dz[r];
      const double zt = ri / di;
      a0 = fma(ri, zt, a0);
      if (mode == 1) {
        const float zf = (float)zt;
        zc[r] = zf;
        const double dzf = di * (double)zf;
        a1 = fma(dzf, (double)zf, a1);
        a2 = fma(dzf, (double)pc[r], a2);
      }
    }
  }
  double v[3] = {a0, a1, a2}, tot[3];
  if (reduce_grid<double, 3>(v, partials, &st->counter[1], tot) && threadIdx.x == 0)
    replacement_step(st, tot[0], tot[1], tot[2], mode);
}

// Per-entry column deltas of the fixed-width layout (once per operator pattern);
// padding stays 0.  no_partner is set when a row lacks the entry of its partner DOF
// (column r^1), which the block difference form of 2-DOF operators needs.
__global__ void k_zlayout(int64_t n, const int32_t* __restrict__ sptr, const int16_t* __restrict__ col, int zw,
                          int16_t* __restrict__ colz, int* __restrict__ no_partner) {
  const int64_t r = gtid();
  if (r >= n) return;
  int64_t base;
  int w;
  sell_row(sptr, r, base, w);
  const int64_t fbase = zw > 0 ? ((r >> 5) * 32) * zw + (r & 31) : base;  // (zw 0: the sliced layout itself)
  const int dpart = (r & 1) ? -1 : 1;
  bool found = false;
  for (int k = 0; k < w; k++) {
    const int16_t d = col[base + 32 * (int64_t)k];
    colz[fbase + 32 * (int64_t)k] = d;
    found |= d == dpart;
  }
  if (!found || (r ^ 1) >= n) atomicExch(no_partner, 1);
}

// Fold the FP32 hi+lo correction into the FP64 solution: y += Yh + Yl, plus the update
// term a_{k-1} P_{k-1} that is still pending when the last launch had an odd iteration
// counter (the two-step update of Y runs on even ones); Yh = Yl = 0.  Runs when a
// residual replacement is due (done == 3) or when forced.
__global__ void __launch_bounds__(kT) k_zfold(int64_t n, double* __restrict__ y64, float* __restrict__ yh,
                                              float* __restrict__ yl, const float* __restrict__ p0,
                                              const float* __restrict__ p1, const CgState* st, int force) {
  if (!force && st->done != 3) return;
  const int it = st->iters;
  const double a = (it & 1) ? (double)(float)st->alpha : 0.0;  // the FP32 alpha the iteration used
  const float* __restrict__ pp = (it & 1) ? p1 : p0;
  for (int64_t i = gtid(); i < n; i += gstride()) {
    y64[i] += (double)yh[i] + (double)yl[i] + a * (double)pp[i];
    yh[i] = 0.0f;
    yl[i] = 0.0f;
  }
}

// u = y; rows tagged 1 get their prescribed value exactly (or 0)
__global__ void k_zunscale(int64_t n, const double* __restrict__ y, const uint8_t* __restrict__ fix,
                           const double* __restrict__ fixval, double* __restrict__ u) {
  const int64_t i = gtid();
  if (i >= n) return;
  u[i] = (fix && fix[i] == 1) ? (fixval ? fixval[i] : 0.0) : y[i];
}

// ---------------------------------------------------------------------------
// One 1024-thread block per SM: half the blocks of a 2 x 512 launch, so half the halo
// positions each block recomputes in phase 1.  Measured on GB300 (with the one-warp FP64
// reductions; per launch, graph-launched runs): 4M-DOF Poisson 52.9 vs 54.6 us, 1M-DOF
// Poisson 19.8 vs 20.8 us, 2M-DOF elasticity +7.7% solves/s.  (With FP64 shuffle-adds by
// every warp at the end of a launch the 1024-thread block had been the slower one.)
#ifndef ADFEM_ZCG_BT
#define ADFEM_ZCG_BT 1024
#endif
static constexpr int kZBT = ADFEM_ZCG_BT;            // threads per block
static constexpr int kZPerSM = 1024 / kZBT;          // resident blocks per SM (1024 threads)
#ifndef ADFEM_ZCG_U1
#define ADFEM_ZCG_U1 4
#endif
#ifndef ADFEM_ZCG_U2
#define ADFEM_ZCG_U2 2
#endif
static constexpr int kZU1 = ADFEM_ZCG_U1;            // phase-1 positions per thread and trip
static constexpr int kZU2 = ADFEM_ZCG_U2;            // phase-2 matrix rows per thread and trip
#ifndef ADFEM_ZCG_U1_RING
#define ADFEM_ZCG_U1_RING 3
#endif
static constexpr int kZU1R = ADFEM_ZCG_U1_RING;      // phase-1 positions per thread and trip, ring variant
#ifndef ADFEM_ZCG_U2_WIDE
#define ADFEM_ZCG_U2_WIDE 1
#endif
// rows per trip of the 16-wide variants: two rows of 16 entries do not fit in 64 registers
// per thread (they spill); 768-thread blocks with two rows per trip (79 registers, no
// spills) measured 49.5 against 48.9 us per iteration at 2M-DOF elasticity
static constexpr int kZU2W = ADFEM_ZCG_U2_WIDE;
static constexpr size_t kZSmemBlock = (kZPerSM >= 2 ? 100 : 200) * 1024;  // shared memory per block
// ring variants: window + pattern pool + ring stages (the static shared memory of the
// kernel -- reductions, scalars, mbarriers, ~1.2 KB -- comes on top, within the 227 KB a
// block may hold)
static constexpr size_t kZSmemRing = 225 * 1024;

// Distinct slice column patterns (at most kZMaxPatterns; further slices use their
// per-entry deltas), padded to the kernel's unrolled width per row parity, and the
// pattern id of every slice.  Built on the host from the operator's pattern pool.
static constexpr int kZMaxPatterns = 32;

template <class T>
static int zupload(DevBuf& b, const T* src, size_t count) {
  ADFEM_TRY(b.alloc(sizeof(T) * count));
  ADFEM_CUDA(cudaMemcpy(b.p, src, sizeof(T) * count, cudaMemcpyHostToDevice));
  return ADFEM_OK;
}

static int zcg_build_pool(Solver& S) {
  const Sell& A = *S.A;
  const int64_t ns = A.nslices;
  const int period = A.pat_period;
  std::vector<int32_t> spat(std::max<int64_t>(ns, 1)), sptr(ns + 1);
  std::vector<int16_t> pat(A.pat.bytes / sizeof(int16_t));
  ADFEM_CUDA(cudaMemcpy(spat.data(), A.spat.p, sizeof(int32_t) * spat.size(), cudaMemcpyDeviceToHost));
  ADFEM_CUDA(cudaMemcpy(sptr.data(), A.sptr.p, sizeof(int32_t) * sptr.size(), cudaMemcpyDeviceToHost));
  if (!pat.empty()) ADFEM_CUDA(cudaMemcpy(pat.data(), A.pat.p, A.pat.bytes, cudaMemcpyDeviceToHost));
  std::vector<int32_t> zpid(std::max<int64_t>(ns, 1), -1), pool;
  std::vector<int32_t> offs;  // pool offset of each pattern id
  for (int64_t sl = 0; sl < ns; sl++) {
    const int32_t so = spat[sl];
    if (so < 0) continue;
    const int w = (sptr[sl + 1] - sptr[sl]) / 32;
    int id = -1;
    for (size_t j = 0; j < offs.size(); j++)
      if (offs[j] == so) id = (int)j;
    if (id < 0) {
      if ((int)offs.size() >= kZMaxPatterns || (size_t)so + (size_t)period * w > pat.size()) continue;
      id = (int)offs.size();
      offs.push_back(so);
      for (int q = 0; q < period; q++)
        for (int k = 0; k < S.zps; k++) pool.push_back(k < w ? (int32_t)pat[so + q * w + k] : 0);
    }
    zpid[sl] = id;
  }
  if (pool.empty()) pool.assign(4, 0);
  S.znpool = (int)pool.size();
  ADFEM_TRY(zupload(S.zpid32, zpid.data(), zpid.size()));
  ADFEM_TRY(zupload(S.zpool32, pool.data(), pool.size()));
  return ADFEM_OK;
}

// threads per block of a variant: 24-wide rows hold 24 values and 12 words of column
// deltas per thread, which do not fit in the 64 registers of a 1024-thread block (512-thread
// blocks with two rows per thread and trip, 125 registers, measured 156 against 125 us per
// iteration at 4M-DOF P2)
template <int MAXW>
constexpr int zbt() {
  return MAXW > 16 ? 768 : kZBT;
}

template <int MAXW, bool B2, bool RING = false>
static int zcg_configure(Solver& S, int sms) {
  constexpr int BT = zbt<MAXW>();
  auto kern = k_zcg_iter<MAXW, BT, (RING ? kZU1R : kZU1), (MAXW > 8 ? kZU2W : kZU2), B2, RING>;
  const size_t limit = RING ? kZSmemRing : kZSmemBlock;
  // The shared-memory limit is raised once per process to the most any plan uses:
  // changing a kernel's attributes while another thread captures a graph with that
  // kernel invalidates the capture.
  static std::once_flag once;
  static cudaError_t set_err = cudaSuccess;
  std::call_once(once, [&] {
    std::lock_guard<std::mutex> lk(device_alloc_mutex());
    set_err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit);
  });
  if (set_err != cudaSuccess) return cuda_fail(set_err, "cudaFuncSetAttribute");
  if (S.zsmem > limit) return fail(ADFEM_ERR_INVALID, "banded CG plan exceeds its shared-memory limit");
  int per = 0;
  ADFEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, BT, S.zsmem));
  if (per < 1) return fail(ADFEM_ERR_CUDA, "banded CG kernel cannot be resident");
  S.zbt = BT;
  const int64_t want = (int64_t)sms * per;
  // at least one band width of rows per block, so that halos stay below twice the rows
  int64_t L = (S.n + want - 1) / want;
  L = std::max<int64_t>(std::max<int64_t>(L, S.zH), 32);
  L = (L + 31) / 32 * 32;
  S.zL = L;
  S.zgrid = (int)((S.n + L - 1) / L);
  S.zK = (int)((L + S.zS - 1) / S.zS);
  return ADFEM_OK;
}

int zcg_plan(Solver& S, int sms) {
  const Sell& A = *S.A;
  S.zcg = false;
  const char* env = std::getenv("ADFEM_ZCG");
  if (env && env[0] == '0') return ADFEM_OK;
  if (!A.delta16 || A.maxw > 24 || A.maxw < 1 || A.band > 32767 || S.n < 1) return ADFEM_OK;
  // 32-bit positions and fixed-width indices
  if (A.nslices * 32 * (int64_t)A.maxw >= INT32_MAX || S.n + A.band >= INT32_MAX) return ADFEM_OK;
  const int H = (int)A.band;
  S.zw = A.maxw;
  S.zps = S.zw <= 8 ? 8 : (S.zw <= 16 ? 16 : 24);
  ADFEM_TRY(zcg_build_pool(S));
  const size_t pool_bytes = sizeof(int32_t) * (size_t)((S.znpool + 3) & ~3);
  // super-tile rows: the whole per-block range when it fits beside its 2H halo, else the
  // largest multiple of 32 that does; a halo larger than the rows it serves is not worth it
  const int64_t per_block = ((S.n + kZPerSM * (int64_t)sms - 1) / (kZPerSM * (int64_t)sms) + 31) / 32 * 32;
  const int64_t room = (int64_t)((kZSmemBlock - pool_bytes) / sizeof(float)) - 2 * (int64_t)H - 2;
  int64_t smax = room / 32 * 32;
  if (smax < std::max<int64_t>(1024, 2 * (int64_t)H)) return ADFEM_OK;  // scaled two-kernel path
  // ADFEM_ZCG_SMAX caps the super-tile rows (a test hook for ranges split into several)
  if (const char* cap = std::getenv("ADFEM_ZCG_SMAX")) {
    const int64_t c = std::atoll(cap) / 32 * 32;
    if (c >= 32) smax = std::min(smax, c);
  }
  S.zS = (int)std::min<int64_t>(std::max<int64_t>(per_block, ((int64_t)H + 31) / 32 * 32), smax);
  S.zH = H;
  S.zW = S.zS + 2 * H + 2;  // (+2: windows of 2-DOF operators are widened to even ends)
  S.zsmem = pool_bytes + sizeof(float) * (size_t)S.zW;
  // the matrix ring (8-wide operators, opt-in with ADFEM_ZCG_RING=2..4: at most that many
  // stages of kZBT rows, as many as fit beside the window, at least 2).  Measured slower on
  // GB300 at 4M DOF (71 us per iteration with 3 stages, 69 with 2, against 50 for the
  // plain variant; only the first stages through the ring: 64 / 55 us): the larger shared-
  // memory footprint leaves less L1 for the loads in flight of phase 1 and of the rows the
  // threads load (phase 1 19 -> 29 us with 3 stages), and one refill per stage after every
  // warp released it keeps too few bytes in flight in phase 2.
  S.zns = 0;
  const char* renv = std::getenv("ADFEM_ZCG_RING");
  if (A.maxw <= 8 && renv && renv[0] >= '2' && renv[0] <= '9') {
    const int cap = std::min(kZMaxStages, std::atoi(renv));
    const size_t stage = sizeof(float) * (size_t)kZBT * (size_t)S.zw;
    for (int ns = cap; ns >= 2; ns--)
      if (S.zsmem + ns * stage <= kZSmemRing) {
        S.zns = ns;
        break;
      }
    S.zsmem += S.zns * stage;
    const char* fenv = std::getenv("ADFEM_ZCG_RING_REFILL");
    S.zrefill = !(fenv && fenv[0] == '0');
  }
  const char* penv = std::getenv("ADFEM_ZCG_PDL");
  S.zpdl = !(penv && penv[0] == '0');
  // (the block form is decided after the layout pass below; both 16-wide variants have
  // the same resources, so the plan is made with the plain one)
  if (A.maxw <= 8 && S.zns) ADFEM_TRY((zcg_configure<8, false, true>(S, sms)));
  else if (A.maxw <= 8) ADFEM_TRY((zcg_configure<8, false>(S, sms)));
  else if (A.maxw <= 16) ADFEM_TRY((zcg_configure<16, false>(S, sms)));
  else ADFEM_TRY((zcg_configure<24, false>(S, sms)));
  if (A.maxw > 8 && A.maxw <= 16) ADFEM_TRY((zcg_configure<16, true>(S, sms)));
  const size_t n4 = sizeof(float) * (size_t)S.n;
  ADFEM_TRY(S.z1.alloc(n4));
  ADFEM_TRY(S.zq1.alloc(n4));
  ADFEM_TRY(S.dz32.alloc(n4));
  // FP64 copy in the sliced-ELL layout; FP32 copy and column deltas in the fixed-width layout
  const size_t ne = (size_t)std::max<int64_t>(A.nent, 1);
  // 24-wide rows (P2): the FP32 copy and the column deltas keep the sliced layout's variable
  // slice widths (rows of one length are grouped into slices when the system is built);
  // narrower rows: the fixed-width layout
  S.zvarw = A.maxw > 16;
  const size_t nf = S.zvarw ? ne : (size_t)std::max<int64_t>(A.nslices, 1) * 32 * (size_t)S.zw;
  ADFEM_TRY(S.valz64.alloc(sizeof(double) * ne));
  ADFEM_TRY(S.valz32.alloc(sizeof(float) * nf));
  ADFEM_TRY(S.colz16.alloc(sizeof(int16_t) * nf));
  ADFEM_CUDA(cudaMemset(S.valz64.p, 0, sizeof(double) * ne));
  ADFEM_CUDA(cudaMemset(S.valz32.p, 0, sizeof(float) * nf));
  ADFEM_CUDA(cudaMemset(S.colz16.p, 0, sizeof(int16_t) * nf));
  DevBuf flag;
  ADFEM_TRY(flag.alloc(sizeof(int)));
  ADFEM_CUDA(cudaMemset(flag.p, 0, sizeof(int)));
  k_zlayout<<<(unsigned)((S.n + kT - 1) / kT), kT>>>(S.n, A.sptr.as<int32_t>(), A.col.as<int16_t>(), S.zvarw ? 0 : S.zw,
                                                     S.colz16.as<int16_t>(), flag.as<int>());
  ADFEM_CUDA(cudaGetLastError());
  // legacy-stream sync, not a device-wide one: other threads may be capturing graphs on
  // their (non-blocking) solver streams
  ADFEM_CUDA(cudaStreamSynchronize(0));
  int no_partner = 0;
  ADFEM_CUDA(cudaMemcpy(&no_partner, flag.p, sizeof(int), cudaMemcpyDeviceToHost));
  S.zblock2 = A.pat_period == 2 && !no_partner && A.maxw > 8 && A.maxw <= 16;
  if (S.zblock2) ADFEM_TRY(S.bz32.alloc(sizeof(float2) * (size_t)S.n));

  S.zcg = true;
  return ADFEM_OK;
}

int zcg_prepare(Solver& S, const int32_t* diagpos_dev, int* bad_dev, cudaStream_t st) {
  const Sell& A = *S.A;
  const unsigned nb = (unsigned)((S.n + kT - 1) / kT);
  k_zprep<<<nb, kT, 0, st>>>(S.n, A.sptr.as<int32_t>(), A.col.as<int16_t>(), A.val64.as<double>(), diagpos_dev,
                             S.zvarw ? 0 : S.zw, S.zblock2 ? 1 : 0, S.valz64.as<double>(), S.valz32.as<float>(),
                             S.dz32.as<float>(), S.zblock2 ? S.bz32.as<float2>() : nullptr, bad_dev);
  ADFEM_CUDA(cudaGetLastError());
  return ADFEM_OK;
}

static ZcgArgs zcg_args(Solver& S) {
  const Sell& A = *S.A;
  ZcgArgs z;
  z.n = S.n;
  z.L = S.zL;
  z.S = S.zS;
  z.H = S.zH;
  z.period = A.pat_period;
  z.zw = S.zw;
  z.zpid = S.zpid32.as<int32_t>();
  z.pool = S.zpool32.as<int32_t>();
  z.npool = S.znpool;
  z.colz = S.colz16.as<int16_t>();
  z.val = S.valz32.as<float>();
  z.dz = S.dz32.as<float>();
  z.bz = S.zblock2 ? S.bz32.as<float2>() : nullptr;
  z.z[0] = S.r32.as<float>();
  z.z[1] = S.z1.as<float>();
  z.p[0] = S.pa32.as<float>();
  z.p[1] = S.pb32.as<float>();
  z.q[0] = S.q32.as<float>();
  z.q[1] = S.zq1.as<float>();
  z.yh = S.yh32.as<float>();
  z.yl = S.yl32.as<float>();
  z.st = S.state.as<CgState>();
  z.partials = S.partials.as<double>();
  z.ns = S.zns;
  z.sptr = A.sptr.as<int32_t>();
  z.refill = S.zrefill ? 1 : 0;
  return z;
}

// Launch with the programmatic-serialization attribute (S.zpdl): in a stream or a captured
// graph, the next iteration's blocks are scheduled as this one's exit and wait inside the
// kernel (griddepcontrol.wait) for its completion, which hides the launch latency between
// two iterations.
template <class Kern>
static void zlaunch(Kern kern, const Solver& S, cudaStream_t st, const ZcgArgs& z) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)S.zgrid);
  cfg.blockDim = dim3((unsigned)S.zbt);
  cfg.dynamicSmemBytes = S.zsmem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = S.zpdl ? 1 : 0;
  if (cudaLaunchKernelEx(&cfg, kern, z) != cudaSuccess && S.zpdl) {
    // without the attribute (the launch then reports its own error, if any, to the caller's
    // cudaGetLastError)
    (void)cudaGetLastError();
    cfg.numAttrs = 0;
    cudaLaunchKernelEx(&cfg, kern, z);
  }
}

void zcg_enqueue_iter(Solver& S, cudaStream_t st) {
  const ZcgArgs z = zcg_args(S);
  if (S.A->maxw <= 8 && S.zns) zlaunch(k_zcg_iter<8, kZBT, kZU1R, kZU2, false, true>, S, st, z);
  else if (S.A->maxw <= 8) zlaunch(k_zcg_iter<8, kZBT, kZU1, kZU2, false, false>, S, st, z);
  else if (S.A->maxw > 16) zlaunch(k_zcg_iter<24, zbt<24>(), kZU1, kZU2W, false, false>, S, st, z);
  else if (S.zblock2) zlaunch(k_zcg_iter<16, kZBT, kZU1, kZU2W, true, false>, S, st, z);
  else zlaunch(k_zcg_iter<16, kZBT, kZU1, kZU2W, false, false>, S, st, z);
}

void zcg_enqueue_init(Solver& S, cudaStream_t st, const double* rhs, const uint8_t* zero_rows, const double* u0,
                      double rtol2) {
  k_zinit<<<S.grid, kT, 0, st>>>(S.n, rhs, zero_rows, S.dz32.as<float>(), S.zblock2 ? S.bz32.as<float2>() : nullptr,
                                 u0, S.b.as<double>(), S.y64.as<double>(), S.state.as<CgState>(),
                                 S.partials.as<double>(), rtol2);
}

void zcg_enqueue_residual(Solver& S, cudaStream_t st, int mode, int force) {
  const Sell& A = *S.A;
  k_zres64<<<S.grid, kT, 0, st>>>(S.n, A.sptr.as<int32_t>(), A.col.as<int16_t>(), S.valz64.as<double>(),
                                  S.zblock2 ? 1 : 0, S.dz32.as<float>(), S.zblock2 ? S.bz32.as<float2>() : nullptr, S.b.as<double>(), S.y64.as<double>(), S.r32.as<float>(),
                                  S.z1.as<float>(), S.pa32.as<float>(), S.pb32.as<float>(), S.state.as<CgState>(),
                                  S.partials.as<double>(), mode, force);
}

void zcg_enqueue_fold(Solver& S, cudaStream_t st, int force) {
  k_zfold<<<S.grid, kT, 0, st>>>(S.n, S.y64.as<double>(), S.yh32.as<float>(), S.yl32.as<float>(),
                                 S.pa32.as<float>(), S.pb32.as<float>(), S.state.as<CgState>(), force);
}

void zcg_enqueue_unscale(Solver& S, cudaStream_t st, const uint8_t* fix, const double* fixval, double* u) {
  k_zunscale<<<(unsigned)((S.n + kT - 1) / kT), kT, 0, st>>>(S.n, S.y64.as<double>(), fix, fixval, u);
}

// ---------------------------------------------------------------------------
// Banded FP64 CG: the same one-kernel iteration in FP64 -- same banded row ranges,
// shared-memory window, column patterns and lagged vector updates -- for the Jacobi-
// scaled operator K~ = S K S (unit diagonal) in standard form, so it is Jacobi-PCG on K
// with every value, vector and dot product in FP64.  It is the like-for-like FP64
// counterpart of k_zcg_iter (selected with ADFEM_ZCG64=1, see dcg_plan).  Per launch k:
//   r_k = r_{k-1} - a_{k-1} q_{k-1},  p_k = ar r_k + ap p_{k-1},  q_k = K~ p_k,
//   z += a_{k-2} p_{k-2} + a_{k-1} p_{k-1} on even k (the solution correction since the
//   last fold, as in the mixed kernel), and the dot products r_k.r_k, p_k.q_k, q_k.q_k
//   (p_{k-1}.q_k after a residual replacement) in one grid reduction; the last block sets
//   a_k = rho_k / p.q and beta_k from rho_{k+1} ~ rho_k - 2 a_k r.q + a_k^2 q.q.
// The window holds p_k in FP64 (twice the bytes of the mixed window), so at 4M DOF a
// block's rows are split into two super-tiles, each with its own halo.  The values are
// read from the scaled sliced-ELL operator (entry k of row i at sptr[i/32] + 32k + i%32).
struct DcgArgs {
  int64_t n;
  int64_t L;
  int S, H, period, zw;
  const int32_t* zpid;
  const int32_t* pool;
  int npool;
  const int16_t* colz;
  const int32_t* sptr;
  const double* val;
  double* r[2];
  double* p[2];
  double* q[2];
  double* z;
  CgState* st;
  double* partials;
};

template <int MAXW, int BT, int U1, int U2>
__global__ void __launch_bounds__(BT, 1) k_dcg_iter(DcgArgs A) {
  static_assert(MAXW % 4 == 0, "pattern rows are loaded as int4");
  CgState* st = A.st;
  if (st->done) return;
  extern __shared__ double dsm[];
  int* spool = reinterpret_cast<int*>(dsm);
  double* sP = dsm + ((A.npool + 3) & ~3) / 2;  // (pool padded to 16 bytes)
  for (int j = threadIdx.x; j < A.npool; j += BT) spool[j] = __ldg(A.pool + j);
  const int it = st->iters;
  const int cur = it & 1, nxt = cur ^ 1;
  const double* __restrict__ rprev = A.r[cur];
  const double* __restrict__ pprev = A.p[cur];
  const double* __restrict__ qprev = A.q[cur];
  double* __restrict__ rnew = A.r[nxt];
  double* __restrict__ pnew = A.p[nxt];
  double* __restrict__ qnew = A.q[nxt];
  double* __restrict__ z = A.z;
  const double a = st->alpha, ar = st->ar, ap = st->ap, a2 = st->alpha_prev;
  const bool ydo = (it & 1) == 0;
  const bool plain = ar == 1.0;   // uniform
  const bool full_zq = !plain;
  const int tid = threadIdx.x;
  const int zw = A.zw;
  const int n = (int)A.n;
  const int blo = (int)blockIdx.x * (int)A.L;
  const int bhi = min(blo + (int)A.L, n);
  double pq = 0.0, pkq = 0.0, qq = 0.0, rr = 0.0;

  for (int lo = blo; lo < bhi; lo += A.S) {
    const int hi = min(lo + A.S, bhi);
    const int wlo = max(lo - A.H, 0);
    const int whi = min(hi + A.H, n);
    if (lo != blo) __syncthreads();
    struct In {
      double rp, qp, pp, p2, y;
      bool own;
    };
    auto fetch1 = [&](int pos, In& x) {
      x.own = pos >= lo && pos < hi;
      x.rp = __ldg(rprev + pos);
      x.qp = __ldg(qprev + pos);
      x.pp = __ldg(pprev + pos);
      const bool yupd = x.own && ydo;
      x.p2 = yupd ? pnew[pos] : 0.0;  // p_{k-2}, read before this thread overwrites it with p_k
      x.y = yupd ? z[pos] : 0.0;
    };
    auto commit = [&](int pos, In& x) {
      const double rk = fma(-a, x.qp, x.rp);
      const double pk = plain ? fma(ap, x.pp, rk) : fma(ap, x.pp, ar * rk);
      sP[pos - wlo] = pk;
      if (x.own) {
        rnew[pos] = rk;
        pnew[pos] = pk;
        if (ydo) z[pos] = fma(a, x.pp, fma(a2, x.p2, x.y));
        rr = fma(rk, rk, rr);
      }
    };
    int pos = wlo + tid;
    for (; pos + (U1 - 1) * BT < whi; pos += U1 * BT) {
      In x[U1];
#pragma unroll
      for (int u = 0; u < U1; u++) fetch1(pos + u * BT, x[u]);
#pragma unroll
      for (int u = 0; u < U1; u++) commit(pos + u * BT, x[u]);
    }
    for (; pos < whi; pos += BT) {
      In x0;
      fetch1(pos, x0);
      commit(pos, x0);
    }
    __syncthreads();
    // ---- phase 2: q = K~ p_k for the rows [lo, hi)
    auto fetch = [&](int i, double (&v)[MAXW], int& pid) {
      const int s0 = __ldg(A.sptr + (i >> 5)), s1 = __ldg(A.sptr + (i >> 5) + 1);
      const int w = (s1 - s0) >> 5;
      const int base = s0 + (i & 31);
#pragma unroll
      for (int k = 0; k < MAXW; k++) v[k] = k < w ? __ldg(A.val + base + 32 * k) : 0.0;
      pid = __ldg(A.zpid + (i >> 5));
    };
    auto row = [&](int i, const double (&v)[MAXW], int pid) {
      // column deltas are read as they are used (no register copy of the row's pattern:
      // the 16-wide variant would spill)
      double s = 0.0;
      if (pid >= 0) {
        const int4* pv = reinterpret_cast<const int4*>(spool) + (pid * A.period + (A.period == 2 ? (i & 1) : 0)) *
                                                                     (MAXW / 4);
        const double* sPi = sP + (i - wlo);
        // (slots at and beyond the fixed width zw are padding: no FP64 FMA is spent on them)
#pragma unroll
        for (int h = 0; h < MAXW / 4; h++) {
          const int4 x = pv[h];
#ifdef ADFEM_CHECKS
          if (!ADFEM_DCHECK(i - wlo + min(min(x.x, x.y), min(x.z, x.w)) >= 0 &&
                            i - wlo + max(max(x.x, x.y), max(x.z, x.w)) < whi - wlo))
            continue;
#endif
          if (4 * h < zw) s = fma(v[4 * h], sPi[x.x], s);
          if (4 * h + 1 < zw) s = fma(v[4 * h + 1], sPi[x.y], s);
          if (4 * h + 2 < zw) s = fma(v[4 * h + 2], sPi[x.z], s);
          if (4 * h + 3 < zw) s = fma(v[4 * h + 3], sPi[x.w], s);
        }
      } else {
        const int base = (i >> 5) * (32 * zw) + (i & 31);
#pragma unroll
        for (int k = 0; k < MAXW; k++) {
          const int dk = k < zw ? (int)__ldg(A.colz + base + 32 * k) : 0;
          int w_ = i + dk - wlo;
          if (!ADFEM_DCHECK(w_ >= 0 && w_ < whi - wlo)) w_ = i - wlo;
          s = fma(v[k], sP[w_], s);
        }
      }
      qnew[i] = s;
      const double Pi = sP[i - wlo];
      pq = fma(Pi, s, pq);
      qq = fma(s, s, qq);
      if (full_zq) pkq = fma(__ldg(pprev + i), s, pkq);
    };
    int i = lo + tid;
    for (; i + (U2 - 1) * BT < hi; i += U2 * BT) {
      double v[U2][MAXW];
      int pid[U2];
#pragma unroll
      for (int u = 0; u < U2; u++) fetch(i + u * BT, v[u], pid[u]);
#pragma unroll
      for (int u = 0; u < U2; u++) row(i + u * BT, v[u], pid[u]);
    }
    for (; i < hi; i += BT) {
      double v0[MAXW];
      int g0;
      fetch(i, v0, g0);
      row(i, v0, g0);
    }
  }

  double v[4] = {pq, pkq, qq, rr}, tot[4];
  if (reduce_grid<double, 4, BT>(v, A.partials, &st->counter[0], tot) && threadIdx.x == 0) {
    const double pqd = tot[0], qqd = tot[2], rho = tot[3];
    const double zqd = (full_zq && st->ar != 0.0) ? (pqd - st->ap * tot[1]) / st->ar : pqd;
    if (!isfinite(rho) || !isfinite(pqd)) {
      st->done = 2;
    } else if (rho <= st->stop2) {
      st->rho_new = rho;
      st->final_req = 1;
      st->done = 3;
    } else if (rho <= st->ru2 || it >= st->max_iter) {
      st->rho_new = rho;
      st->done = 3;
    } else if (!(pqd > 0.0)) {
      st->done = 2;
    } else {
      const double al = rho / pqd;
      const double est = rho - 2.0 * al * zqd + al * al * qqd;
      st->alpha_prev = st->alpha;
      st->alpha = al;
      st->ar = 1.0;
      st->ap = fmax(est, 0.0) / rho;
      st->rho = rho;
      st->iters = it + 1;
    }
  }
}

// Fold of the banded FP64 path: y += z plus the update a_{k-1} p_{k-1} still pending
// after an odd iteration counter; z = 0.  Runs when a replacement is due or when forced.
__global__ void __launch_bounds__(kT) k_dfold(int64_t n, double* __restrict__ y64, double* __restrict__ z,
                                              const double* __restrict__ p0, const double* __restrict__ p1,
                                              const CgState* st, int force) {
  if (!force && st->done != 3) return;
  const int it = st->iters;
  const double a = (it & 1) ? st->alpha : 0.0;
  const double* __restrict__ pp = (it & 1) ? p1 : p0;
  for (int64_t i = gtid(); i < n; i += gstride()) {
    y64[i] += z[i] + a * pp[i];
    z[i] = 0.0;
  }
}

#ifndef ADFEM_DCG_U1
#define ADFEM_DCG_U1 2
#endif
static constexpr int kDU1 = ADFEM_DCG_U1;  // phase-1 positions per thread and trip
static constexpr int kDU2W8 = 1;           // phase-2 rows per thread and trip

// Plan of the banded FP64 path (after zcg_plan succeeded): FP64 window super-tiles of
// equal size within each block's rows, and the second buffers of the r, p, q pairs.
//
// Measured on GB300 (Poisson, 4M DOF): 148 us per iteration against 69 + 28 + 13 us for
// the three FP64 kernels -- the FP64 pipe, not memory, bounds both (0.70 TFLOP/s here),
// and the fused form does more FP64 work per row (the halo rows of the two super-tiles the
// FP64 window needs, the extra dot product of the one-step beta estimate).  So FP64
// solves keep the three-kernel iteration, and this path is selected only with
// ADFEM_ZCG64=1 at system creation, as the like-for-like FP64 counterpart of the mixed
// kernel.
int dcg_plan(Solver& S) {
  S.dcg = false;
  const char* env = std::getenv("ADFEM_ZCG64");
  if (!env || env[0] != '1') return ADFEM_OK;
  if (!S.zcg || S.A->maxw > 16) return ADFEM_OK;
  const size_t pool_bytes = sizeof(int32_t) * (size_t)((S.znpool + 3) & ~3);
  const int64_t room = (int64_t)((kZSmemBlock - pool_bytes) / sizeof(double)) - 2 * (int64_t)S.zH - 2;
  const int64_t smax = room / 32 * 32;
  if (smax < std::max<int64_t>(512, (int64_t)S.zH)) return ADFEM_OK;
  const int64_t L = S.zL;
  const int64_t tiles = (L + smax - 1) / smax;
  int64_t St = (L + tiles - 1) / tiles;
  St = (St + 31) / 32 * 32;
  if (const char* cap = std::getenv("ADFEM_ZCG_SMAX")) {
    const int64_t c = std::atoll(cap) / 32 * 32;
    if (c >= 32) St = std::min(St, c);
  }
  S.dS = (int)St;
  S.dsmem = pool_bytes + sizeof(double) * (size_t)(St + 2 * S.zH + 2);
  if (S.dsmem > kZSmemBlock) return ADFEM_OK;
  auto kern8 = k_dcg_iter<8, kZBT, kDU1, kDU2W8>;
  auto kern16 = k_dcg_iter<16, kZBT, 1, 1>;
  static std::once_flag once;
  static cudaError_t set_err = cudaSuccess;
  std::call_once(once, [&] {
    std::lock_guard<std::mutex> lk(device_alloc_mutex());
    set_err = cudaFuncSetAttribute(kern8, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZSmemBlock);
    if (set_err == cudaSuccess)
      set_err = cudaFuncSetAttribute(kern16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZSmemBlock);
  });
  if (set_err != cudaSuccess) return cuda_fail(set_err, "cudaFuncSetAttribute");
  int per = 0;
  ADFEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, S.A->maxw <= 8 ? kern8 : kern16, kZBT, S.dsmem));
  if (per < 1) return ADFEM_OK;
  const size_t n8 = sizeof(double) * (size_t)S.n;
  ADFEM_TRY(S.dr1.alloc(n8));
  ADFEM_TRY(S.dp1.alloc(n8));
  ADFEM_TRY(S.dq1.alloc(n8));
  S.dcg = true;
  return ADFEM_OK;
}

static DcgArgs dcg_args(Solver& S) {
  const Sell& A = *S.A;
  DcgArgs d;
  d.n = S.n;
  d.L = S.zL;
  d.S = S.dS;
  d.H = S.zH;
  d.period = A.pat_period;
  d.zw = S.zw;
  d.zpid = S.zpid32.as<int32_t>();
  d.pool = S.zpool32.as<int32_t>();
  d.npool = S.znpool;
  d.colz = S.colz16.as<int16_t>();
  d.sptr = A.sptr.as<int32_t>();
  d.val = A.val64.as<double>();
  d.r[0] = S.r64.as<double>();
  d.r[1] = S.dr1.as<double>();
  d.p[0] = S.p64.as<double>();
  d.p[1] = S.dp1.as<double>();
  d.q[0] = S.q64.as<double>();
  d.q[1] = S.dq1.as<double>();
  d.z = S.z64.as<double>();
  d.st = S.state.as<CgState>();
  d.partials = S.partials.as<double>();
  return d;
}

void dcg_enqueue_iter(Solver& S, cudaStream_t st) {
  const DcgArgs d = dcg_args(S);
  if (S.A->maxw <= 8) k_dcg_iter<8, kZBT, kDU1, kDU2W8><<<S.zgrid, kZBT, S.dsmem, st>>>(d);
  else k_dcg_iter<16, kZBT, 1, 1><<<S.zgrid, kZBT, S.dsmem, st>>>(d);
}

void dcg_enqueue_fold(Solver& S, cudaStream_t st, int force) {
  k_dfold<<<S.grid, kT, 0, st>>>(S.n, S.y64.as<double>(), S.z64.as<double>(), S.p64.as<double>(),
                                 S.dp1.as<double>(), S.state.as<CgState>(), force);
}

// buffers the banded FP64 path zeroes before a solve (r, p, q pairs and the correction)
int dcg_clear(Solver& S, cudaStream_t st) {
  const size_t n8 = sizeof(double) * (size_t)S.n;
  for (DevBuf* b : {&S.r64, &S.dr1, &S.p64, &S.dp1, &S.q64, &S.dq1, &S.z64})
    ADFEM_CUDA(cudaMemsetAsync(b->p, 0, n8, st));
  return ADFEM_OK;
}

// buffers the banded path zeroes before a solve
int zcg_clear(Solver& S, cudaStream_t st) {
  const size_t n4 = sizeof(float) * (size_t)S.n;
  for (DevBuf* b : {&S.r32, &S.z1, &S.pa32, &S.pb32, &S.q32, &S.zq1, &S.yh32, &S.yl32})
    ADFEM_CUDA(cudaMemsetAsync(b->p, 0, n4, st));
  return ADFEM_OK;
}

ADFEM_CHECK_READER(check_line_zcg)

}  // namespace adfem
