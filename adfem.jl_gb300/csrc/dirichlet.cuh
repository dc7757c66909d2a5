// Dirichlet-imposition helpers used by the C API (see dirichlet.cu).
#pragma once
#include "adfem_internal.h"

namespace adfem {
int exclusive_scan(int64_t n, const int64_t* in, int64_t* out, cudaStream_t st);
int scan_counts(int64_t n, int64_t* counts, int64_t* total, cudaStream_t st);
int dirichlet_csc_device(int64_t n, int64_t nnz, const int64_t* colptr0, const int64_t* rowval0,
                         const double* nzval, const uint8_t* isbd, int keep_zeros, DevBuf& ocolptr,
                         int64_t* out_nnz, DevBuf& orowval1, DevBuf& onzval, bool count_only, cudaStream_t st);
int dirichlet_coo_device(int64_t sN, const long long* idx, const double* vv, const uint8_t* isbd, int64_t N,
                         int64_t* nkeep, DevBuf& oidx, DevBuf& ov, int64_t* nlift, DevBuf& lift_k, bool count_only,
                         cudaStream_t st);
int dirichlet_coo_backward_device(int64_t sN, const long long* idx, const uint8_t* isbd, int64_t N,
                                  const double* gvv, const double* bdval_dense, const double* grhs, double* gvv_in,
                                  cudaStream_t st);
// positions of the kept COO entries in the output of the COO arm (-1: dropped)
int pcl_dirichlet_device(int64_t sN, const long long* idx, const uint8_t* isbd, int64_t N, int64_t* pos,
                         int64_t* nkeep, cudaStream_t st);
cudaError_t launch_to0(int64_t n, const int64_t* a1, int64_t* a0, cudaStream_t st);
cudaError_t launch_to1(int64_t n, const int64_t* a0, int64_t* a1, int64_t add, cudaStream_t st);
}  // namespace adfem
