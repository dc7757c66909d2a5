// Elasticity launchers used by the C API (see elastic.cu).
#pragma once
#include "adfem_internal.h"

namespace adfem {
// nperm / kperm: node renumbering of the system (NULL: none), see k_elastic_system
cudaError_t launch_elastic_system(const Mesh& m, const double* Dbar, const double* srcx, const double* srcy,
                                  const int32_t* sptr2, const uint8_t* isbd2, const double* bdval2, double* vals,
                                  double* rhs, const int32_t* nperm, const uint8_t* kperm, cudaStream_t st);
cudaError_t launch_elastic_grad_E(const Mesh& m, const double* u2, const double* lam2, const uint8_t* isbd2,
                                  const double* nu, double* gE, cudaStream_t st);
// reference order <-> solver order through a DOF map (sol[map[d]] = ref[d])
cudaError_t launch_to_solver(int64_t n, const int32_t* map, const double* ref, double* sol, cudaStream_t st);
cudaError_t launch_from_solver(int64_t n, const int32_t* map, const double* sol, double* ref, cudaStream_t st);
cudaError_t launch_to_interleaved(int64_t nv, const double* ref, double* il, cudaStream_t st);
cudaError_t launch_from_interleaved(int64_t nv, const double* il, double* ref, cudaStream_t st);
}  // namespace adfem
