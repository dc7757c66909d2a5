// Solver internals shared by solver.cu and capi.cpp.
#pragma once
#include "adfem_internal.h"

namespace adfem {

// Device-resident CG scalars.  Written only by the last block of a reduction
// kernel (or by single-thread kernels), read by every kernel of the next step.
struct CgState {
  double rho;          // current (recursive) r.r
  double rho_new;      // r.r computed by the last update step
  double alpha, beta;  // CG coefficients
  double alpha_prev;   // banded mixed path: alpha of the iteration before (two-step solution update)
  double ar, ap;       // mixed: p_new = ar*r + ap*p_old
  double bnorm2;       // ||b~||^2
  double stop2;        // stop when ||r||^2 <= stop2 (= rtol^2 ||b~||^2)
  double ru2;          // mixed: replace the residual when rho_new <= ru2
  double delta2;       // mixed: reliable-update factor squared
  double rr64;         // last FP64 true-residual norm^2 (mixed) / final check
  int iters;           // inner iterations done
  int max_iter;
  int done;            // 0 running, 1 converged, 2 breakdown, 3 residual replacement due, 4 max_iter,
                       // 5 a bounded wait inside a kernel gave up (see fault)
  int updates;         // residual replacements done (mixed)
  int final_req;       // the last replacement was requested because the recurrence residual met rtol
  int floor_hit;       // stopped at the attainable accuracy of the FP64 residual
  int final_seen;      // mixed: a replacement requested by rtol has already failed the true-residual test
  double last_rr64;    // FP64 residual norm^2 at the previous replacement (mixed: once final_seen)
  int fault;           // banded ring variant: a wait on a shared-memory stage timed out
  unsigned counter[4]; // last-block arrival counters (returned to 0 by the last block)
};

struct Solver {
  int64_t n = 0;
  int grid = 0;            // blocks of the grid-stride kernels (resident blocks per SM x SMs)
  int grid_spmv = 0;       // same for the unrolled SpMV kernels (higher register use)
  bool prefetch = false;   // SpMV software pipelining (ADFEM_SPMV_PREFETCH=1)
  const Sell* A = nullptr; // sliced-ELL operator (val64 scaled in place, val32 scaled copy)
  DevBuf s32;              // Jacobi scaling s_i = 1/sqrt(K_ii) (float, exact in double)
  DevBuf state;            // CgState
  DevBuf partials;         // 4 * grid doubles
  DevBuf b;                // scaled rhs (FP64)
  DevBuf y64, r64, p64, q64;
  DevBuf z64;              // FP64 CG: solution correction since the last residual replacement
  DevBuf r32, pa32, pb32, q32;
  DevBuf yh32, yl32;       // mixed: solution correction since the last fold, as an FP32 hi+lo pair
  CgState* h_state = nullptr;  // pinned, 2 slots
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaGraphExec_t g64 = nullptr, g32 = nullptr;
  std::vector<cudaEvent_t> pev;  // event pool of profiled solves
  int g64_chunk = 0, g32_chunk = 0;
  bool prepared = false;
  bool prep_scaled = false;        // the Jacobi-scaled copies are current (see solver_ensure_scaled)
  const int32_t* diagpos = nullptr; // device: entry index of the diagonal in each row
  // banded mixed path (zcg.cu): used by mixed solves when the band fits the ring
  bool zcg = false;
  int zH = 0, zgrid = 0;
  int zS = 0;              // rows per super-tile
  int zK = 0;              // super-tiles per block
  int zW = 0;              // shared-memory positions per super-tile (zS + 2 zH)
  int zns = 0;             // stages of the shared-memory matrix ring (0: the plain variant)
  int zbt = 1024;          // threads per block of the variant in use
  bool zvarw = false;      // FP32 copy in the sliced layout (variable slice widths), 24-wide rows
  bool zrefill = true;     // the ring serves every row (else only the first zns stages)
  bool zpdl = true;        // iterations launched as programmatic dependent launches
  int64_t zL = 0;
  size_t zsmem = 0;
  DevBuf z1, zq1;          // second buffers of the Z and q^ ping-pong pairs (first: r32, q32)
  DevBuf dz32;             // fp32(K_ii)
  DevBuf valz64, valz32;   // difference-form copies of K (physical scale; FP32 in the fixed-width layout)
  DevBuf colz16;           // per-entry column deltas of the fixed-width layout
  DevBuf zpid32, zpool32;  // per-slice pattern id, distinct padded column patterns
  int znpool = 0;          // ints in zpool32
  int zw = 0;              // fixed slice width (widest slice)
  int zps = 0;             // pattern row stride (8 or 16, the kernel's unrolled width)
  bool zblock2 = false;    // interleaved 2-DOF operator: block difference form, node-block Jacobi
  DevBuf bz32;             // zblock2: per row {K_ii, K_(i,i^1)} (FP32)
  cudaGraphExec_t gz = nullptr;
  int gz_chunk = 0;
  // banded FP64 path (zcg.cu, k_dcg_iter): FP64 solves when the band fits
  bool dcg = false;
  int dS = 0;              // rows per FP64 super-tile
  size_t dsmem = 0;
  DevBuf dr1, dp1, dq1;    // second buffers of the r, p, q pairs (first: r64, p64, q64)
  cudaGraphExec_t gd = nullptr;
  int gd_chunk = 0;
  ~Solver();
  int init(const Sell* A, int64_t n);
};

// After an assembly (diagpos: entry index k of the diagonal in row i): makes the copies
// the default solve needs now and marks the others for first use.
int solver_prepare(Solver& S, const int32_t* diagpos_dev, cudaStream_t user);
// The Jacobi-scaled copies: s_i = rsqrt(K_ii) (FP32), val64 <- s_i K_ij s_j, valD64 / val32
// the FP64 / FP32 difference-form copies (see k_scale_values); no-op when current.
int solver_ensure_scaled(Solver& S, cudaStream_t user);
// Per-kernel timing of a profiled solve: 0 SpMV+dot, 1 update+dot, 2 p update / fold,
// 3 FP64 residual.
struct SolveProfile {
  double ms[4] = {0, 0, 0, 0};
  long long n[4] = {0, 0, 0, 0};
};
// Solve K u = rhs (rhs, u unscaled, device).  zero_rows (optional, uint8 tags == 1): rows
// whose rhs is replaced by 0 (adjoint solves).  With prof != null every kernel is launched
// on its own between two CUDA events (no graph) and timed.
// fix_rows (optional, tags == 1) get u = fix_vals (or 0 when fix_vals is null) exactly.
int solver_solve(Solver& S, const double* rhs, double* u, const uint8_t* zero_rows, const uint8_t* fix_rows,
                 const double* fix_vals, const adfem_solver_opts& o, adfem_solver_stats* stats, cudaStream_t user,
                 SolveProfile* prof = nullptr);
// y = K x with the unscaled operator (via the scaled copy)
int solver_apply(Solver& S, const double* x, double* y, cudaStream_t user);

// Banded mixed path (zcg.cu).  zcg_plan decides whether the operator's band fits
// the shared-memory ring and allocates the path's buffers; zcg_prepare derives its
// operator copies from the unscaled FP64 values (before they are scaled in place).
int zcg_plan(Solver& S, int sms);
int zcg_prepare(Solver& S, const int32_t* diagpos_dev, int* bad_dev, cudaStream_t st);
int zcg_clear(Solver& S, cudaStream_t st);
void zcg_enqueue_init(Solver& S, cudaStream_t st, const double* rhs, const uint8_t* zero_rows, const double* u0,
                      double rtol2);
void zcg_enqueue_iter(Solver& S, cudaStream_t st);
void zcg_enqueue_residual(Solver& S, cudaStream_t st, int mode, int force);
void zcg_enqueue_fold(Solver& S, cudaStream_t st, int force);
void zcg_enqueue_unscale(Solver& S, cudaStream_t st, const uint8_t* fix, const double* fixval, double* u);
// Banded FP64 path (zcg.cu): planned after zcg_plan; iteration, fold, clear.
int dcg_plan(Solver& S);
void dcg_enqueue_iter(Solver& S, cudaStream_t st);
void dcg_enqueue_fold(Solver& S, cudaStream_t st, int force);
int dcg_clear(Solver& S, cudaStream_t st);

// Fill sliced-ELL values from CSR values (same pattern).
// ---- packed solves of small systems (pack.cu)
#ifndef ADFEM_PACK_BLOCK_ROWS
#define ADFEM_PACK_BLOCK_ROWS 3072
#endif
constexpr int kPackBlockRows = ADFEM_PACK_BLOCK_ROWS;  // rows of a system solved by one thread block
constexpr int kPackMaxRows = 65536;    // rows of a packed system (larger ones: a cluster of 8 blocks)
constexpr int kPackMaxSystems = 128;   // systems of each kind per packed launch
// one system of a packed launch (device-side descriptor; outputs filled by the kernel)
struct PackDesc {
  const int32_t* sptr;
  const void* col;
  const double* valD;     // FP64 difference form (outer residual)
  const float* val32;     // FP32 difference form (inner CG)
  const float* s;         // Jacobi scaling
  const double* rhs;
  const uint8_t* zero_rows;
  const uint8_t* fix_rows;
  const double* fix_vals;
  const double* u0;       // warm start (may alias u) or NULL
  double* u;
  double* y;              // scratch: scaled solution (FP64); the FP32 inner-CG vectors live in
                          // shared memory
  double rtol2;
  int n, d16, max_iter;
  int iters, passes, status, floor_hit;
  double rr64, bnorm2;
};
struct PackItem {
  Solver* S = nullptr;
  const double* rhs = nullptr;
  double* u = nullptr;
  const uint8_t* zero_rows = nullptr;
  const uint8_t* fix_rows = nullptr;
  const double* fix_vals = nullptr;
  bool warm = false;
  double rtol = 1e-12;
  int max_iter = 200000;
  // results
  int iters = 0, passes = 0, status = 0;
  double relres = 0.0;
};
// Descriptor buffers and the captured graph of packed launches; one pack at a time runs
// on a slot (packs on different slots run concurrently).
struct PackSlot;
PackSlot* pack_slot_create();
void pack_slot_destroy(PackSlot* s);
// Solves every item in one launch per kPackMaxSystems items (one block per system;
// the systems must be prepared and have at most kPackMaxRows rows) on the given slot
// (NULL: a process-wide slot).  Synchronises st.
int solve_packed(PackItem* items, int count, cudaStream_t st, PackSlot* slot = nullptr);
// largest packed system on this device: kPackMaxRows, or kPackBlockRows where a cluster
// of the packed solver cannot be scheduled
int pack_rows_limit();

cudaError_t launch_csr_to_sell(const Sell& A, int64_t n, const int32_t* rowptr, const double* csr, double* sell,
                               cudaStream_t st);
int sell_build_pattern(int64_t n, const int32_t* rowptr, const int32_t* colind, Sell& s, int period);

}  // namespace adfem
