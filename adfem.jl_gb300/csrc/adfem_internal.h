// Internal declarations shared by the host runtime and the CUDA kernels of
// libadfem_gpu.  Nothing here is part of the C ABI (see include/adfem_gpu.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/adfem_gpu.h"

namespace adfem {

// ---------------------------------------------------------------------------
// errors: every entry point returns an adfem status; the message of the last
// failure on the calling thread is kept for adfem_last_error().
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define ADFEM_CUDA(call)                                   \
  do {                                                     \
    cudaError_t _e = (call);                               \
    if (_e != cudaSuccess) return ::adfem::cuda_fail(_e, #call); \
  } while (0)

#define ADFEM_TRY(call)                  \
  do {                                   \
    int _s = (call);                     \
    if (_s != ADFEM_OK) return _s;       \
  } while (0)

// NVTX range around a C-ABI call: the library's calls appear by name on an Nsight
// timeline beside their kernels (a push/pop pair costs nanoseconds when no tool is
// attached; nvtx3 is header-only).
struct NvtxRange {
  explicit NvtxRange(const char* name);
  ~NvtxRange();
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define ADFEM_RANGE(name) ::adfem::NvtxRange _adfem_range_(name)

// Armed by adfem_debug_fail_alloc: true when this device allocation is to fail (once).
// Debug build (-DADFEM_CHECKS): the first failed index check of each translation unit, as
// a source line (0: none; release builds always 0); reading clears it.
int check_line_solver();
int check_line_zcg();
int check_line_assemble();
int check_line_generic();

bool injected_alloc_failure();
void arm_alloc_failure(long long k);

// ---------------------------------------------------------------------------
// device buffer with RAII ownership (cudaMalloc / cudaFree)
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release();
  int alloc(size_t nbytes);  // (re)allocates only when larger storage is needed
  template <class T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

// cudaMalloc and cudaFree may synchronize the device, which invalidates a CUDA-graph
// capture running in another thread; the library's allocations and its graph captures
// therefore take this lock (held briefly: a capture records a few dozen launches).
std::mutex& device_alloc_mutex();

// ---------------------------------------------------------------------------
// Packed node->element incidence record.  For node i, each incident element e in
// ascending element order contributes one record:
//   x = e
//   y = a | off0 << 2 | off1 << 12 | off2 << 22
// where a is i's local vertex index in e and off_b is the position (within row i
// of the scalar CSR pattern) of the column of e's local vertex b.  Rows are
// limited to 1024 entries by the 10-bit fields.
__host__ __device__ inline unsigned inc_a(unsigned y) { return y & 3u; }
__host__ __device__ inline unsigned inc_off(unsigned y, unsigned b) { return (y >> (2 + 10 * b)) & 1023u; }

// Sliced-ELL layout (slices of 32 consecutive rows, entries stored column-major
// within a slice so that one warp reads 32 consecutive values per step).
// Entry k of row r sits at sptr[r>>5] + 32*k + (r&31); a slice is as wide as its
// longest row, padding entries have value 0 and delta 0 (column = row).
struct Sell {
  int64_t n = 0;        // rows
  int64_t nslices = 0;  // ceil(n / 32)
  int64_t nent = 0;     // stored entries incl. padding
  int maxw = 0;         // widest slice
  int64_t band = 0;     // max |col - row| over all stored entries
  bool delta16 = false; // column stored as int16 delta to the row, else int32 column
  DevBuf sptr;          // int32 [nslices + 1]  (units of entries)
  DevBuf col;           // int16 [nent] (delta) or int32 [nent]
  // Slice-uniform column patterns: when every row r of a slice has the same column
  // offsets col - r (for period 2: the same per row parity, as for interleaved x/y
  // DOFs), they are stored once in `pat` and spat[slice] points at them (int16
  // units; pattern for parity q at pat[spat + q*w]); spat = -1 keeps the per-row
  // columns of `col`.  Kernels then issue the gathers of a row without waiting for
  // its column loads, and the column bytes of uniform slices are never read.
  DevBuf spat;          // int32 [nslices]
  DevBuf pat;           // int16 pool
  int pat_period = 1;
  int64_t uniform_slices = 0;
  int64_t uniform_entries = 0;  // stored entries of the uniform slices
  DevBuf val64;         // double [nent]  (Jacobi-scaled, standard form)
  DevBuf valD64;        // double [nent]  (Jacobi-scaled, difference form, for FP64 residuals)
  DevBuf val32;         // float  [nent]
};

// Degree-generic Lagrange space on a triangle mesh (P1 or P2), used by the generic
// element kernels (generic.cu): element DOFs, the DOF graph pattern and the
// DOF->element incidence.  P2 DOFs are the vertices, then nv + edge for the edge
// midpoints; an element lists its vertices, then its local edges (0,1), (1,2), (2,0).
// Incidence record s of DOF i (ascending element order) is {e, a, o0 | o1 << 10 |
// o2 << 20, o3 | o4 << 10 | o5 << 20}: element, local index of i in e, and the
// position within row i of the column of each local DOF b of e.
struct Space {
  int degree = 1;
  int nd = 3;            // DOFs per element
  int ng = 3;            // Gauss points per element
  int64_t ndof = 0, nnz = 0;
  int maxrow = 0;
  std::vector<int32_t> dof;      // nd * ne
  std::vector<int32_t> rowptr;   // ndof + 1
  std::vector<int32_t> colind;   // nnz
  DevBuf d_dof;      // int32 [nd * ne]
  DevBuf d_area;     // double [ne]
  DevBuf d_rowptr;   // int32 [ndof + 1]
  DevBuf d_colind;   // int32 [nnz]
  DevBuf d_inc_ptr;  // int32 [ndof + 1]
  DevBuf d_inc;      // uint4 [nd * ne]
  DevBuf d_ke;       // element matrices (scratch of the summed-operator kernels)
};
__host__ __device__ inline unsigned space_off(uint4 r, int b) {
  return ((b < 3 ? r.z : r.w) >> (10 * (b % 3))) & 1023u;
}

// Device-resident triangle mesh: P1 geometry, incidence, scalar CSR pattern and the
// sliced-ELL copy of that pattern; degree-2 meshes add a P2 space.
struct Mesh {
  int64_t nv = 0, ne = 0;
  int degree = 1;       // element degree the mesh was created with (1 or 2)
  int64_t nnz = 0;      // scalar CSR pattern entries
  int maxrow = 0;       // longest scalar row
  int maxinc = 0;       // largest node valence (incident elements)
  int flipped = 0;      // elements reoriented

  // host copies (needed by the getters and by the legacy API)
  std::vector<double> xy;        // 2*nv
  std::vector<int32_t> elem;     // 3*ne vertex ids after the orientation fix
  std::vector<double> area;      // ne (Heron)
  std::vector<double> grad;      // 6*ne: hx0 hy0 hx1 hy1 hx2 hy2
  std::vector<int32_t> rowptr;   // nv+1
  std::vector<int32_t> colind;   // nnz
  std::vector<int32_t> inc_ptr;  // nv+1
  std::vector<uint32_t> inc;     // 2 * 3ne (x,y pairs)
  std::vector<int64_t> edges;    // 2*nedges, 1-based (min block then max block); filled lazily
  std::vector<int32_t> eedge;    // 3*ne edge of each local edge (0,1), (1,2), (2,0); with edges
  int64_t nedges = -1;
  std::unique_ptr<Space> space[3];  // [degree], built on first use

  // device copies
  DevBuf d_xy;       // double2 [nv]
  DevBuf d_conn;     // int4 [ne] {v0,v1,v2,0}
  DevBuf d_geo;      // double4 [ne] {g01, g02, g12, w}; g_ab = w * grad_a . grad_b
  DevBuf d_grad;     // double2 [3*ne] {hx_a, hy_a}
  DevBuf d_inc_ptr;  // int32 [nv+1]
  DevBuf d_inc;      // uint2 [3*ne]
  DevBuf d_rowptr;   // int32 [nv+1]
  DevBuf d_colind;   // int32 [nnz]
  DevBuf d_diagpos;  // int32 [nv] position of the diagonal within its row
  // geometry as FP32 pairs for the pair-arithmetic Poisson system kernel (built on first
  // use, mesh_geo_pairs): gpa {g01, g02}, gpb {g12, w/6}, gpc {w/2}
  DevBuf d_gpa, d_gpb, d_gpc;

  Sell sell;         // scalar pattern in sliced-ELL (values unused here)
  DevBuf d_sell2;    // (built lazily) interleaved 2-dof pattern: see Elasticity

  // per-mesh scratch reused by the host-pointer entry points (mu also guards space[])
  std::mutex mu;
  DevBuf s_in0, s_in1, s_out0, s_out1, s_el0, s_el1;
};

// Build a mesh from xyz triples (z ignored) and 0-based triangles.  Host work
// (orientation fix, geometry, incidence, pattern) then upload.
int mesh_build(const double* xyz, int64_t nv, const int32_t* elems0, int64_t ne, Mesh** out);
int mesh_edges(Mesh* m);  // fills m->edges / eedge / nedges (first-appearance numbering)
// Boundary DOFs, 1-based: ascending boundary vertices; for degree-2 meshes followed by
// the ascending DOFs of boundary edges
int64_t mesh_bcnode(Mesh* m, int64_t* out1);
// Reverse Cuthill-McKee renumbering of the mesh nodes (pi[node] = new index); returns
// the bandwidth of the renumbered pattern.
int64_t mesh_rcm(const Mesh& m, std::vector<int32_t>& pi);
int64_t graph_rcm(int64_t n, const std::vector<int32_t>& rowptr, const std::vector<int32_t>& colind,
                  std::vector<int32_t>& pi);
// Gauss points per element (3 for the order-2 rule of P1, 6 for the order-4 rule of P2)
inline int mesh_ng(const Mesh& m) { return m.degree == 2 ? 6 : 3; }
inline int64_t mesh_ngauss(const Mesh& m) { return (int64_t)mesh_ng(m) * m.ne; }
// DOFs of the mesh's own space (nv, or nv + nedges for P2)
int64_t mesh_ndof(Mesh* m);
void mesh_gauss(const Mesh* m, double* x, double* y);      // mesh_ng points per element
void mesh_gauss_weights(const Mesh* m, double* w);          // ip.weight * area / 0.5
// The space of the given degree on m, built on first use (host work + upload); the
// caller holds m->mu.
int mesh_space(Mesh* m, int degree, Space** out);
// Triangle rules: reference coordinates and weights of point k (order 2 or 4)
void rule_point(int degree, int k, double* xi, double* eta, double* w);

// ---------------------------------------------------------------------------
// kernels (launchers; every launcher returns cudaError_t from cudaGetLastError)
enum class Layout { CSR = 0, CSRT = 1, SELL = 2 };

// per-element prepass: sigma_e = kappa_e0 + kappa_e1 + kappa_e2 (may be null),
// src_e[r] = w * sum_k f_k phi_r(x_k) (may be null)
cudaError_t launch_element_prepass(const Mesh& m, const double* kappa, const double* f, double* sigma,
                                   double* src3, cudaStream_t st);
// the same with src_e[r] = sum_k f_k phi_r(x_k), without the weight w (the input of
// launch_poisson_system, whose rows apply w)
cudaError_t launch_element_prepass_unweighted(const Mesh& m, const double* kappa, const double* f, double* sigma,
                                              double* src3, cudaStream_t st);
// Laplace values into the scalar pattern (CSR or sliced-ELL), no Dirichlet
cudaError_t launch_laplace_rows(const Mesh& m, const double* sigma, double* vals, Layout lay, cudaStream_t st);
// load vector: rhs[i] (+)= sum over incident elements of src_e[a]
cudaError_t launch_source_rows(const Mesh& m, const double* src3, double* rhs, bool accumulate, cudaStream_t st);
// unsummed COO of the reference op (FemLaplaceScalar_forward): 9 entries per Gauss point
cudaError_t launch_laplace_coo(const Mesh& m, const double* kappa, long long* indices, double* vv, cudaStream_t st);
cudaError_t launch_laplace_coo_backward(const Mesh& m, const double* grad_vv, double* grad_kappa, cudaStream_t st);
cudaError_t launch_source_backward(const Mesh& m, const double* grad_rhs, double* grad_f, cudaStream_t st);
// fused Poisson system: Laplace + load + Dirichlet (bd rows -> identity, bd columns
// dropped into the rhs lift), values into the system's sliced-ELL (sptr; full pattern,
// dropped entries 0); src3 from launch_element_prepass_unweighted.  diagpos_mesh: diagonal
// slot of each mesh pattern row.  nperm / kperm (NULL: no renumbering): solver row of each
// node and rank of each pattern slot in its renumbered row; isbd, bdval and rhs are in
// solver order.  Rows of up to 64 entries.
cudaError_t launch_poisson_system(const Mesh& m, const double* sigma, const double* src3, const uint8_t* isbd,
                                  const double* bdval_dense, double* sell_vals, double* rhs, const int32_t* sptr,
                                  const int32_t* diagpos_mesh, const int32_t* nperm, const uint8_t* kperm,
                                  cudaStream_t st);
// the same system in FP32-pair arithmetic (rows of up to 16 entries; the geometry pairs must
// exist: mesh_geo_pairs): element pass (sigma_e and the load terms as pairs), then the rows
int mesh_geo_pairs(Mesh& m);
cudaError_t launch_element_prepass_pairs(const Mesh& m, const double* kappa, const double* f, float2* sigma,
                                         float2* src3, cudaStream_t st);
cudaError_t launch_poisson_system_pairs(const Mesh& m, const float2* sigma, const float2* src3, const uint8_t* isbd,
                                        const double* bdval_dense, double* sell_vals, double* rhs,
                                        const int32_t* sptr, const int32_t* diagpos_mesh, const int32_t* nperm,
                                        const uint8_t* kperm, cudaStream_t st);
// adjoint element kernel: grad_kappa[3e+k] = -w_e (grad lam_e).(grad u_e), lam zero on bd
cudaError_t launch_poisson_kappa_grad(const Mesh& m, const double* u, const double* lam, const uint8_t* isbd,
                                      double* grad_kappa, cudaStream_t st);

// elasticity
cudaError_t launch_plane_strain(int mode, int64_t n, const double* E, const double* nu, double* D, cudaStream_t st);
cudaError_t launch_plane_strain_backward(int mode, int64_t n, const double* g, const double* E, const double* nu,
                                         double* gE, double* gnu, cudaStream_t st);
// Dbar_e = w_e * sum_k D_k (9 per element)
cudaError_t launch_stiffness_prepass(const Mesh& m, const double* D, double* Dbar, cudaStream_t st);
// Dbar_e from E (plane strain, reference formula) -- fused material path
cudaError_t launch_stiffness_prepass_E(const Mesh& m, const double* E, const double* nu, double* Dbar,
                                       cudaStream_t st);
// block-ordered [x; y] CSR rows (reference ordering); transpose => CSC values
cudaError_t launch_stiffness_rows(const Mesh& m, const double* Dbar, double* vals, bool transpose,
                                  cudaStream_t st);
cudaError_t launch_stiffness_coo(const Mesh& m, const double* D, long long* indices, double* vv, cudaStream_t st);
cudaError_t launch_stiffness_coo_backward(const Mesh& m, const double* grad_vv, double* grad_D, cudaStream_t st);

// degree-generic element kernels (generic.cu), on a Space of degree 1 or 2.  Per-point
// inputs hold sp.ng values per element (9 per point for D), element-major.
enum class GenOp { LAPLACE = 0, MASS = 1 };
// unsummed COO of the reference op: nd*nd entries per Gauss point (Laplace, mass)
cudaError_t launch_gen_coo(const Mesh& m, const Space& sp, GenOp op, const double* coef, long long* indices,
                           double* vv, cudaStream_t st);
cudaError_t launch_gen_coo_backward(const Mesh& m, const Space& sp, GenOp op, const double* grad_vv, double* grad_coef,
                                    cudaStream_t st);
// 4 nd^2 entries per Gauss point, DOFs [dof; dof + ndof]
cudaError_t launch_gen_stiffness_coo(const Mesh& m, const Space& sp, const double* D, long long* indices, double* vv,
                                     cudaStream_t st);
cudaError_t launch_gen_stiffness_coo_backward(const Mesh& m, const Space& sp, const double* grad_vv, double* grad_D,
                                              cudaStream_t st);
// summed operator values in the space's CSR pattern (transpose: CSC of the same
// symmetric pattern); ke: scratch of nd*nd doubles per element
cudaError_t launch_gen_matrix(const Mesh& m, const Space& sp, GenOp op, const double* coef, double* ke, double* vals,
                              bool transpose, cudaStream_t st);
// summed elasticity operator in the [x; y] block pattern (rows 2 ndof, 4 nnz entries);
// ke: scratch of 4 nd^2 doubles per element
cudaError_t launch_gen_stiffness_matrix(const Mesh& m, const Space& sp, const double* D, double* ke, double* vals,
                                        bool transpose, cudaStream_t st);
cudaError_t launch_gen_source(const Mesh& m, const Space& sp, const double* f, double* rhs, bool accumulate,
                              cudaStream_t st);
// resident P2 (or P1) Poisson system from the space sp: element matrices into ke (nd^2
// per element), then Laplace rows + load + Dirichlet into the system's sliced-ELL values
// (sptr; nperm / kperm as for launch_poisson_system; diagpos_space: diagonal slot of each
// space pattern row); isbd, bdval, rhs in solver order
cudaError_t launch_gen_poisson_system(const Mesh& m, const Space& sp, const double* kappa, const double* f, double* ke,
                                      const uint8_t* isbd, const double* bdval, double* sell_vals, double* rhs,
                                      const int32_t* sptr, const int32_t* diagpos_space, const int32_t* nperm,
                                      const uint8_t* kperm, cudaStream_t st);
// dL/dkappa per Gauss point of sp's rule: -w_k grad(lam).grad(u), lam zero where
// isbd_space == 1 (u, lam in space order)
cudaError_t launch_gen_kappa_grad(const Mesh& m, const Space& sp, const double* u, const double* lam,
                                  const uint8_t* isbd_space, double* grad_kappa, cudaStream_t st);
cudaError_t launch_gen_source_backward(const Mesh& m, const Space& sp, const double* grad_rhs, double* grad_f,
                                       cudaStream_t st);
// values at the Gauss points of the mesh's rule: through the P1 shape of the vertices
// (vertex_only, fem_to_gauss_points) or through all DOFs of sp (dof_to_gauss_points)
cudaError_t launch_gen_to_gauss(const Mesh& m, const Space& sp, bool vertex_only, const double* u, double* out,
                                cudaStream_t st);
// transposes of the above: grad_u (+)= ...; vertex_only writes entries [0, nv) only
cudaError_t launch_gen_to_gauss_backward(const Mesh& m, const Space& sp, bool vertex_only, const double* grad_out,
                                         double* grad_u, bool accumulate, cudaStream_t st);

cudaError_t launch_fill(int64_t n, double v, double* out, cudaStream_t st);
// dense column-major Jacobian of the unsummed Laplace COO values with respect to kappa:
// H[gp + nz * ng] = vv[nz] (vv: COO values at kappa = 1, nd2 per Gauss point)
cudaError_t launch_pcl_scatter(int64_t N, int nd2, int64_t ng, const double* vv, double* H, cudaStream_t st);

// Packed forward (g == NULL) or adjoint solves of resident systems on a pack slot
// (adfem_system_solve_packed_d / adfem_system_adjoint_packed_d with an explicit slot).
struct PackSlot;
int system_solve_packed(adfem_system** sys, int count, double** out, const double* const* g,
                        const adfem_solver_opts* opts, adfem_solver_stats* stats, void* stream, bool adjoint,
                        PackSlot* slot);

// Device bytes held by a resident system (operator copies, Dirichlet data, solver
// vectors) -- what the serving loop counts against its HBM budget.
size_t system_device_bytes(const adfem_system* s);
// Mesh behind a handle (sizes for admission estimates).
const Mesh* mesh_of(const adfem_mesh* h);

}  // namespace adfem
