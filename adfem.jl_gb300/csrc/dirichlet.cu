// Algebraic Dirichlet imposition on user-supplied sparse matrices (sm_103a).
//
//  * SparseMatrixCSC arm (src/MFEM/MUtils.jl:184-199): per-column compaction of
//    the kept entries (row and column outside bd; entries equal to 0.0 dropped
//    unless keep_zeros), unit diagonal on bd columns.
//  * SparseTensor/COO arm (deps/MFEM/ImposeDirichlet/ImposeDirichlet.h:27-93):
//    order-preserving compaction of the kept COO entries and the list of entries
//    that feed the right-hand-side lift; the backward pass of the same op.
// The compactions use a deterministic multi-level exclusive scan.
#include "dirichlet.cuh"

namespace adfem {

static constexpr int kT = 256;
static constexpr int kItems = 16;
static constexpr int kTile = kT * kItems;
__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
static inline unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

// ---------------------------------------------------------------------------
// exclusive scan of int64 counts (in place allowed: out may equal in)
__global__ void __launch_bounds__(kT) k_tile_sums(int64_t n, const int64_t* __restrict__ in,
                                                  int64_t* __restrict__ sums) {
  __shared__ int64_t sh[kT];
  const int64_t base = (int64_t)blockIdx.x * kTile;
  int64_t s = 0;
  for (int j = 0; j < kItems; j++) {
    const int64_t i = base + (int64_t)j * kT + threadIdx.x;
    if (i < n) s += in[i];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = kT / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = sh[0];
}

// scan one tile per block with a starting offset taken from offs (may be null)
__global__ void __launch_bounds__(kT) k_tile_scan(int64_t n, const int64_t* in, int64_t* out,
                                                  const int64_t* __restrict__ offs) {
  __shared__ int64_t sh[kT];
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
  int64_t v[kItems];
  int64_t s = 0;
  for (int j = 0; j < kItems; j++) {
    const int64_t i = base + j;
    v[j] = i < n ? in[i] : 0;
    s += v[j];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  // Hillis-Steele inclusive scan over the per-thread totals
  for (int o = 1; o < kT; o <<= 1) {
    const int64_t x = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += x;
    __syncthreads();
  }
  int64_t run = (threadIdx.x ? sh[threadIdx.x - 1] : 0) + (offs ? offs[blockIdx.x] : 0);
  for (int j = 0; j < kItems; j++) {
    const int64_t i = base + j;
    if (i < n) out[i] = run;
    run += v[j];
  }
}

int exclusive_scan(int64_t n, const int64_t* in, int64_t* out, cudaStream_t st) {
  if (n <= 0) return ADFEM_OK;
  const int64_t tiles = (n + kTile - 1) / kTile;
  if (tiles == 1) {
    k_tile_scan<<<1, kT, 0, st>>>(n, in, out, nullptr);
  } else {
    DevBuf sums;
    ADFEM_TRY(sums.alloc(sizeof(int64_t) * (size_t)tiles));
    k_tile_sums<<<(unsigned)tiles, kT, 0, st>>>(n, in, sums.as<int64_t>());
    ADFEM_CUDA(cudaGetLastError());
    ADFEM_TRY(exclusive_scan(tiles, sums.as<int64_t>(), sums.as<int64_t>(), st));
    k_tile_scan<<<(unsigned)tiles, kT, 0, st>>>(n, in, out, sums.as<int64_t>());
    ADFEM_CUDA(cudaGetLastError());
    // sums is freed on return; make sure the kernels that read it have finished
    ADFEM_CUDA(cudaStreamSynchronize(st));
  }
  ADFEM_CUDA(cudaGetLastError());
  return ADFEM_OK;
}

// scan of counts with the total: keeps a copy of the last count
int scan_counts(int64_t n, int64_t* counts, int64_t* total, cudaStream_t st) {
  if (n <= 0) {
    *total = 0;
    return ADFEM_OK;
  }
  int64_t lastc = 0;
  ADFEM_CUDA(cudaMemcpyAsync(&lastc, counts + (n - 1), sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  ADFEM_CUDA(cudaStreamSynchronize(st));
  ADFEM_TRY(exclusive_scan(n, counts, counts, st));
  int64_t lastx = 0;
  ADFEM_CUDA(cudaMemcpyAsync(&lastx, counts + (n - 1), sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  ADFEM_CUDA(cudaStreamSynchronize(st));
  *total = lastx + lastc;
  return ADFEM_OK;
}

// ---------------------------------------------------------------------------
// CSC arm.  colptr/rowval 0-based int64 on the device.
__global__ void k_csc_count(int64_t n, const int64_t* __restrict__ colptr, const int64_t* __restrict__ rowval,
                            const double* __restrict__ nzval, const uint8_t* __restrict__ isbd, int keep_zeros,
                            int64_t* __restrict__ cnt) {
  const int64_t j = gtid();
  if (j >= n) return;
  int64_t c = 0;
  if (isbd[j]) {
    c = 1;  // only the unit diagonal
  } else {
    for (int64_t p = colptr[j]; p < colptr[j + 1]; p++) {
      const int64_t i = rowval[p];
      if (!isbd[i] && (keep_zeros || nzval[p] != 0.0)) c++;
    }
  }
  cnt[j] = c;
}

__global__ void k_csc_write(int64_t n, const int64_t* __restrict__ colptr, const int64_t* __restrict__ rowval,
                            const double* __restrict__ nzval, const uint8_t* __restrict__ isbd, int keep_zeros,
                            const int64_t* __restrict__ ocolptr, int64_t* __restrict__ orowval1,
                            double* __restrict__ onzval) {
  const int64_t j = gtid();
  if (j >= n) return;
  int64_t z = ocolptr[j];
  if (isbd[j]) {
    orowval1[z] = j + 1;
    onzval[z] = 1.0;
    return;
  }
  for (int64_t p = colptr[j]; p < colptr[j + 1]; p++) {
    const int64_t i = rowval[p];
    const double v = nzval[p];
    if (!isbd[i] && (keep_zeros || v != 0.0)) {
      orowval1[z] = i + 1;
      onzval[z] = v;
      z++;
    }
  }
}

__global__ void k_to0(int64_t n, const int64_t* __restrict__ a1, int64_t* __restrict__ a0) {
  const int64_t i = gtid();
  if (i < n) a0[i] = a1[i] - 1;
}
__global__ void k_to1(int64_t n, const int64_t* __restrict__ a0, int64_t* __restrict__ a1, int64_t add) {
  const int64_t i = gtid();
  if (i < n) a1[i] = a0[i] + add;
}

int dirichlet_csc_device(int64_t n, int64_t nnz, const int64_t* colptr0, const int64_t* rowval0,
                         const double* nzval, const uint8_t* isbd, int keep_zeros, DevBuf& ocolptr,
                         int64_t* out_nnz, DevBuf& orowval1, DevBuf& onzval, bool count_only, cudaStream_t st) {
  (void)nnz;
  ADFEM_TRY(ocolptr.alloc(sizeof(int64_t) * (size_t)(n + 1)));
  k_csc_count<<<nblk(n, kT), kT, 0, st>>>(n, colptr0, rowval0, nzval, isbd, keep_zeros, ocolptr.as<int64_t>());
  ADFEM_CUDA(cudaGetLastError());
  int64_t tot = 0;
  ADFEM_TRY(scan_counts(n, ocolptr.as<int64_t>(), &tot, st));
  ADFEM_CUDA(cudaMemcpyAsync(ocolptr.as<int64_t>() + n, &tot, sizeof(int64_t), cudaMemcpyHostToDevice, st));
  *out_nnz = tot;
  if (count_only) return ADFEM_OK;
  ADFEM_TRY(orowval1.alloc(sizeof(int64_t) * (size_t)std::max<int64_t>(tot, 1)));
  ADFEM_TRY(onzval.alloc(sizeof(double) * (size_t)std::max<int64_t>(tot, 1)));
  k_csc_write<<<nblk(n, kT), kT, 0, st>>>(n, colptr0, rowval0, nzval, isbd, keep_zeros, ocolptr.as<int64_t>(),
                                          orowval1.as<int64_t>(), onzval.as<double>());
  ADFEM_CUDA(cudaGetLastError());
  return ADFEM_OK;
}

// ---------------------------------------------------------------------------
// COO arm.  indices 0-based (row, col) pairs; isbd dense over [0, N).
// keep[k] = row and col outside bd; lift[k] = row outside bd, col inside.
__global__ void k_coo_flags(int64_t sN, const longlong2* __restrict__ idx, const uint8_t* __restrict__ isbd,
                            int64_t N, int64_t* __restrict__ keep, int64_t* __restrict__ lift, int* __restrict__ bad) {
  const int64_t k = gtid();
  if (k >= sN) return;
  const longlong2 ij = idx[k];
  if (ij.x < 0 || ij.x >= N || ij.y < 0 || ij.y >= N) {
    atomicExch(bad, 1);
    keep[k] = 0;
    lift[k] = 0;
    return;
  }
  const bool bi = isbd[ij.x] != 0, bj = isbd[ij.y] != 0;
  keep[k] = (!bi && !bj) ? 1 : 0;
  lift[k] = (!bi && bj) ? 1 : 0;
}

__global__ void k_coo_compact(int64_t sN, const longlong2* __restrict__ idx, const double* __restrict__ vv,
                              const int64_t* __restrict__ keep_pos, const int64_t* __restrict__ lift_pos,
                              const uint8_t* __restrict__ isbd, int64_t sNk, longlong2* __restrict__ oidx,
                              double* __restrict__ ov, int64_t* __restrict__ lift_k) {
  const int64_t k = gtid();
  if (k >= sN) return;
  const longlong2 ij = idx[k];
  const bool bi = isbd[ij.x] != 0, bj = isbd[ij.y] != 0;
  if (!bi && !bj) {
    const int64_t z = keep_pos[k];
    oidx[z] = ij;
    ov[z] = vv[k];
  } else if (!bi && bj) {
    lift_k[lift_pos[k]] = k;
  }
  (void)sNk;
}

int dirichlet_coo_device(int64_t sN, const long long* idx, const double* vv, const uint8_t* isbd, int64_t N,
                         int64_t* nkeep, DevBuf& oidx, DevBuf& ov, int64_t* nlift, DevBuf& lift_k, bool count_only,
                         cudaStream_t st) {
  DevBuf keep, lift, bad;
  ADFEM_TRY(keep.alloc(sizeof(int64_t) * (size_t)std::max<int64_t>(sN, 1)));
  ADFEM_TRY(lift.alloc(sizeof(int64_t) * (size_t)std::max<int64_t>(sN, 1)));
  ADFEM_TRY(bad.alloc(sizeof(int)));
  ADFEM_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  const auto* ij = reinterpret_cast<const longlong2*>(idx);
  k_coo_flags<<<nblk(sN, kT), kT, 0, st>>>(sN, ij, isbd, N, keep.as<int64_t>(), lift.as<int64_t>(), bad.as<int>());
  ADFEM_CUDA(cudaGetLastError());
  int hbad = 0;
  ADFEM_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  ADFEM_CUDA(cudaStreamSynchronize(st));
  if (hbad) return fail(ADFEM_ERR_INVALID, "impose Dirichlet: a COO index is outside [0, N)");
  ADFEM_TRY(scan_counts(sN, keep.as<int64_t>(), nkeep, st));
  ADFEM_TRY(scan_counts(sN, lift.as<int64_t>(), nlift, st));
  if (count_only) return ADFEM_OK;
  ADFEM_TRY(oidx.alloc(sizeof(longlong2) * (size_t)std::max<int64_t>(*nkeep, 1)));
  ADFEM_TRY(ov.alloc(sizeof(double) * (size_t)std::max<int64_t>(*nkeep, 1)));
  ADFEM_TRY(lift_k.alloc(sizeof(int64_t) * (size_t)std::max<int64_t>(*nlift, 1)));
  k_coo_compact<<<nblk(sN, kT), kT, 0, st>>>(sN, ij, vv, keep.as<int64_t>(), lift.as<int64_t>(), isbd, *nkeep,
                                             oidx.as<longlong2>(), ov.as<double>(), lift_k.as<int64_t>());
  ADFEM_CUDA(cudaGetLastError());
  return ADFEM_OK;
}

// backward: grad_vv_in[k] = keep ? grad_vv[z_k] : 0, minus bdval_j grad_rhs_i on lift entries
// pcl_ImposeDirichlet (deps/MFEM/ImposeDirichlet/ImposeDirichlet.h:97-111): output
// position of every input entry the COO arm keeps (its exclusive keep-scan), -1 for the
// dropped ones.
__global__ void k_pcl_positions(int64_t sN, const longlong2* __restrict__ idx, const uint8_t* __restrict__ isbd,
                                const int64_t* __restrict__ keep_pos, int64_t* __restrict__ pos) {
  const int64_t k = gtid();
  if (k >= sN) return;
  const longlong2 ij = idx[k];
  pos[k] = (isbd[ij.x] == 0 && isbd[ij.y] == 0) ? keep_pos[k] : -1;
}

int pcl_dirichlet_device(int64_t sN, const long long* idx, const uint8_t* isbd, int64_t N, int64_t* pos,
                         int64_t* nkeep, cudaStream_t st) {
  DevBuf keep, lift, bad;
  ADFEM_TRY(keep.alloc(sizeof(int64_t) * (size_t)std::max<int64_t>(sN, 1)));
  ADFEM_TRY(lift.alloc(sizeof(int64_t) * (size_t)std::max<int64_t>(sN, 1)));
  ADFEM_TRY(bad.alloc(sizeof(int)));
  ADFEM_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  const auto* ij = reinterpret_cast<const longlong2*>(idx);
  k_coo_flags<<<nblk(sN, kT), kT, 0, st>>>(sN, ij, isbd, N, keep.as<int64_t>(), lift.as<int64_t>(), bad.as<int>());
  ADFEM_CUDA(cudaGetLastError());
  int hbad = 0;
  ADFEM_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  ADFEM_CUDA(cudaStreamSynchronize(st));
  if (hbad) return fail(ADFEM_ERR_INVALID, "pcl_ImposeDirichlet: a COO index is outside [0, N)");
  ADFEM_TRY(scan_counts(sN, keep.as<int64_t>(), nkeep, st));
  if (sN > 0) {
    k_pcl_positions<<<nblk(sN, kT), kT, 0, st>>>(sN, ij, isbd, keep.as<int64_t>(), pos);
    ADFEM_CUDA(cudaGetLastError());
  }
  ADFEM_CUDA(cudaStreamSynchronize(st));
  return ADFEM_OK;
}

__global__ void k_coo_backward(int64_t sN, const longlong2* __restrict__ idx, const uint8_t* __restrict__ isbd,
                               const int64_t* __restrict__ keep_pos, const double* __restrict__ gvv,
                               const double* __restrict__ bdval_dense, const double* __restrict__ grhs,
                               double* __restrict__ gvv_in) {
  const int64_t k = gtid();
  if (k >= sN) return;
  const longlong2 ij = idx[k];
  const bool bi = isbd[ij.x] != 0, bj = isbd[ij.y] != 0;
  double g = 0.0;
  if (!bi && !bj) g = gvv[keep_pos[k]];
  if (!bi && bj) g -= bdval_dense[ij.y] * grhs[ij.x];
  gvv_in[k] = g;
}

int dirichlet_coo_backward_device(int64_t sN, const long long* idx, const uint8_t* isbd, int64_t N,
                                  const double* gvv, const double* bdval_dense, const double* grhs, double* gvv_in,
                                  cudaStream_t st) {
  DevBuf keep, lift, bad;
  ADFEM_TRY(keep.alloc(sizeof(int64_t) * (size_t)std::max<int64_t>(sN, 1)));
  ADFEM_TRY(lift.alloc(sizeof(int64_t) * (size_t)std::max<int64_t>(sN, 1)));
  ADFEM_TRY(bad.alloc(sizeof(int)));
  ADFEM_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  const auto* ij = reinterpret_cast<const longlong2*>(idx);
  k_coo_flags<<<nblk(sN, kT), kT, 0, st>>>(sN, ij, isbd, N, keep.as<int64_t>(), lift.as<int64_t>(), bad.as<int>());
  ADFEM_CUDA(cudaGetLastError());
  int hbad = 0;
  ADFEM_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  ADFEM_CUDA(cudaStreamSynchronize(st));
  if (hbad) return fail(ADFEM_ERR_INVALID, "impose Dirichlet backward: a COO index is outside [0, N)");
  int64_t nk = 0;
  ADFEM_TRY(scan_counts(sN, keep.as<int64_t>(), &nk, st));
  k_coo_backward<<<nblk(sN, kT), kT, 0, st>>>(sN, ij, isbd, keep.as<int64_t>(), gvv, bdval_dense, grhs, gvv_in);
  ADFEM_CUDA(cudaGetLastError());
  return ADFEM_OK;
}

cudaError_t launch_to0(int64_t n, const int64_t* a1, int64_t* a0, cudaStream_t st) {
  k_to0<<<nblk(n, kT), kT, 0, st>>>(n, a1, a0);
  return cudaGetLastError();
}
cudaError_t launch_to1(int64_t n, const int64_t* a0, int64_t* a1, int64_t add, cudaStream_t st) {
  k_to1<<<nblk(n, kT), kT, 0, st>>>(n, a0, a1, add);
  return cudaGetLastError();
}

}  // namespace adfem
