/*
 * adfem_gpu.h -- C ABI of libadfem_gpu.so, a GB300 (sm_103a) implementation of
 * AdFem.jl's P1-triangle forward and adjoint path:
 *   compute_fem_laplace_matrix1, compute_fem_source_term1,
 *   compute_fem_stiffness_matrix, impose_Dirichlet_boundary_conditions, K\F.
 *
 * Two layers:
 *   1. The symbols AdFem's Julia code already ccalls from libadmfem
 *      (src/MFEM/MFEM.jl, src/MFEM/MCore.jl), with the same names, argument
 *      order, 0/1-based conventions and "current mesh" global state, so that
 *      AdFem's LIBMFEM constant can point at this library unchanged.  They
 *      return void like the originals; a failure is recorded and can be read
 *      with adfem_last_error().
 *   2. New entry points (prefix adfem_) returning an int status, with explicit
 *      mesh handles, explicit lengths, caller-owned buffers and, for the
 *      "_d" variants, device pointers plus a CUDA stream (passed as void*).
 *
 * All pointers are plain host or device pointers; no framework types appear.
 * Indices: long long = int64 (Julia Int64), int = int32.
 */
#ifndef ADFEM_GPU_H
#define ADFEM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define ADFEM_API __attribute__((visibility("default")))
#else
#define ADFEM_API
#endif

/* ---------------------------------------------------------------- status */
enum {
  ADFEM_OK = 0,
  ADFEM_ERR_INVALID = 1,       /* bad argument: size, index out of range, duplicate ... */
  ADFEM_ERR_CUDA = 2,          /* a CUDA call failed (message has the CUDA error string) */
  ADFEM_ERR_NOMEM = 3,         /* device or host allocation failed */
  ADFEM_ERR_NOT_CONVERGED = 4, /* iterative solve hit max_iter before rtol */
  ADFEM_ERR_BREAKDOWN = 5,     /* CG breakdown: p.Ap <= 0 or non-finite (matrix not SPD) */
  ADFEM_ERR_NO_MESH = 6,       /* legacy call without a current mesh */
  ADFEM_ERR_NONFINITE = 7,     /* NaN/Inf found in an input field */
  ADFEM_ERR_UNSUPPORTED = 8,   /* valid request outside what this build implements */
  ADFEM_ERR_BUSY = 9,          /* server: request does not fit the HBM budget now */
  ADFEM_ERR_TIMEOUT = 10       /* server: request exceeded its deadline */
};

ADFEM_API const char *adfem_status_string(int status);
/* Message of the last failure on the calling thread ("" if none). */
ADFEM_API const char *adfem_last_error(void);
ADFEM_API const char *adfem_version(void);
/* Testing hook, no counterpart in the reference: makes the k-th following device
 * allocation of the library (k = 0: the next one) fail once, exactly as if cudaMalloc
 * had returned cudaErrorMemoryAllocation, so callers can check that every entry point
 * reports ADFEM_ERR_NOMEM and the library stays usable.  k < 0 disarms it.  Returns
 * ADFEM_OK. */
ADFEM_API int adfem_debug_fail_alloc(long long k);
/* Testing hook, no counterpart in the reference: in the debug build (-DADFEM_CHECKS, a
 * second library built by build.py --checks) kernels check the indices they compute before
 * using them and record the first failure instead of faulting; this returns it as
 * 100000 * unit + source line (unit 1: solver.cu, 2: zcg.cu, 3: assemble.cu, 4: generic.cu), 0 when no check
 * failed (always 0 in release builds), -1 if the flags cannot be read, and clears it. */
ADFEM_API int adfem_debug_check_code(void);

/* ====================================================================
 * Layer 1: libadmfem-compatible symbols (current-mesh global state)
 * ==================================================================== */

/* deps/MFEM/API.cpp:4-14 (init_nnfem_mesh); caller src/MFEM/MFEM.jl:95-97.
 * vertices: 3*num_vertices xyz triples (z ignored); element_indices: 3*num_elements
 * 0-based vertex ids.  Implemented: degree 1 (P1) with order 2 and degree 2 (P2) with
 * order 4 (order -1 selects these defaults, MFEM.jl:71-77); other degrees (BDM1) and
 * orders record ADFEM_ERR_UNSUPPORTED and return NULL.  Builds a new mesh,
 * makes it current (replacing the previous current mesh, with the same warning the
 * reference prints), writes the edge count and returns a malloc'ed array of
 * 2*nedges 1-based vertex ids (all minimum endpoints, then all maximum endpoints)
 * that the caller releases with free() (Julia: unsafe_wrap(..., own=true)). */
ADFEM_API long long *init_nnfem_mesh(double *vertices, int num_vertices, int *element_indices, int num_elements,
                                     int order, int lorder, int degree, long long *nedges);
/* deps/MFEM/API.cpp:17-65 -- getters on the current mesh.  For P2 meshes: 6 Gauss
 * points per element, elem_ndof 6, ndof = nnode + nedges, connectivity rows list the
 * vertices, then nnode + edge of the local edges (0,1), (1,2), (2,0) (Common.cpp:62-71). */
ADFEM_API int mfem_get_ngauss(void);
ADFEM_API void mfem_get_gauss(double *x, double *y);
ADFEM_API void mfem_get_gauss_weights(double *w);
ADFEM_API void mfem_get_area(double *a);
ADFEM_API int mfem_get_elem_ndof(void);
ADFEM_API int mfem_get_ndof(void);
ADFEM_API void mfem_get_connectivity(long long *conn);
ADFEM_API void mfem_get_element_to_vertices(long long *elems);

/* deps/MFEM/FemLaplace1/FemLaplaceScalar.h:59-61 (caller src/MFEM/MCore.jl:117).
 * Unsummed COO: elem_ndof^2 entries per Gauss point (9 for P1, 36 for P2), indices
 * 0-based (row,col) pairs. */
ADFEM_API void FemLaplaceScalar_forward_Julia(long long *indices, double *vv, const double *kappa);
/* deps/MFEM/FemSource1/FemSourceScalar.h:35-37 (caller MCore.jl:80).  Accumulates
 * into rhs, which the caller pre-zeroes (MCore.jl:79). */
ADFEM_API void FemSourceScalar_forward_Julia(double *rhs, const double *f);
/* deps/MFEM/ComputeFemStiffnessMatrixMfem/ComputeFemStiffnessMatrixMfem.h:84-87
 * (caller MCore.jl:311-312).  hmat: 9 row-major entries per Gauss point; 4 elem_ndof^2
 * entries per Gauss point, DOFs [dof; dof + ndof]. */
ADFEM_API void ComputeFemStiffnessMatrixMfem_forward_Julia(long long *indices, double *vv, const double *hmat);
/* deps/MFEM/FemToGaussPoints/FemToGaussPointsMfem.h:36-49 (caller src/MFEM/MUtils.jl:241-246):
 * out[ngauss] = nodal values u[nnode] through the P1 shape of the vertices. */
ADFEM_API void FemToGaussPointsMfem_Julia(double *out, const double *u);
/* deps/MFEM/DofToGaussPoints/DofToGaussPointsMfem.h:35-37 (caller MUtils.jl:264-270):
 * out[ngauss] = DOF values u[ndof] through all element basis functions. */
ADFEM_API void DofToGaussPointsMfem_forward_Julia(double *out, const double *u);

/* Compute functions behind AdFem's TensorFlow custom ops, same argument order as
 * the reference MFEM:: functions, on the current mesh, host pointers. */
/* FemLaplaceScalar.h:28-54 (grad op FemLaplaceScalarGrad, FemLaplaceScalar.cpp:88-144) */
ADFEM_API void FemLaplaceScalar_backward(double *grad_kappa, const double *grad_vv, const long long *indices,
                                         const double *vv, const double *kappa);
/* FemSourceScalar.h:17-32 */
ADFEM_API void FemSourceScalar_backward(double *grad_f, const double *grad_rhs, const double *rhs, const double *f);
/* ComputeFemStiffnessMatrixMfem.h:50-81 */
ADFEM_API void ComputeFemStiffnessMatrixMfem_backward(double *grad_hmat, const double *grad_vv);
/* deps/MFEM/ComputeFemMassMatrix1/ComputeFemMassMatrixMfem.h:4-55 (op compute_fem_mass_matrix_mfem,
 * caller src/MFEM/MCore.jl:170-177): elem_ndof^2 COO entries per Gauss point of
 * phi_l phi_s rho w; the backward overwrites grad_rho. */
ADFEM_API void ComputeFemMassMatrix1_forward(long long *indices, double *vv, const double *rho);
ADFEM_API void ComputeFemMassMatrix1_backward(double *grad_rho, const double *grad_vv, const double *vv,
                                              const double *rho);
/* FemToGaussPointsMfem.h:5-34, DofToGaussPointsMfem.h:5-35 (ops fem_to_gauss_points_mfem,
 * dof_to_gauss_points_mfem); the backward functions add into grad_u (nnode or ndof
 * entries), as the reference loops do into a zeroed tensor. */
ADFEM_API void FemToGaussPointsMfem_forward(double *out, const double *u);
ADFEM_API void FemToGaussPointsMfem_backward(double *grad_u, const double *grad_out, const double *out,
                                             const double *u);
ADFEM_API void DofToGaussPointsMfem_forward(double *out, const double *u);
ADFEM_API void DofToGaussPointsMfem_backward(double *grad_u, const double *grad_out, const double *out,
                                             const double *u);
/* PCL helpers (src/pcl.jl:1-39).  FemLaplaceScalar.h:63-91: H = d vv / d kappa of the
 * unsummed Laplace COO, column-major ngauss x elem_ndof^2 ngauss, only nonzeros written.
 * ImposeDirichlet.h:97-111: J = d v_B / d v_A of the COO Dirichlet arm, column-major
 * sN x outdof; indices 1-based sN x 2 column-major; only the ones are written. */
ADFEM_API void pcl_FemLaplaceScalar_Jacobian(double *H);
ADFEM_API void pcl_ImposeDirichlet(double *J, const long long *indices, const long long *bd, int bdN, int sN);
/* deps/MFEM/PlaneStrainAndStress/PlaneStrainAndStress.h:5-78 (op plane_strain_and_stress,
 * mode 0 = strain with the reference's all-nine-entries formula, mode 1 = stress) */
ADFEM_API void PlaneStrainMatrix_forward(double *out, const double *E, const double *nu, int N);
ADFEM_API void PlaneStrainMatrix_backward(double *grad_nu, double *grad_E, const double *grad_out, const double *E,
                                          const double *nu, int N);
ADFEM_API void PlaneStressMatrix_forward(double *out, const double *E, const double *nu, int N);
ADFEM_API void PlaneStressMatrix_backward(double *grad_nu, double *grad_E, const double *grad_out, const double *E,
                                          const double *nu, int N);

/* ====================================================================
 * Layer 2: handle-based API (int status)
 * ==================================================================== */
typedef struct adfem_mesh adfem_mesh;
typedef struct adfem_system adfem_system;

/* Same inputs as init_nnfem_mesh (src/MFEM/MFEM.jl:60-119).  degree 1 (P1, order-2
 * rule) or 2 (P2, order-4 rule). */
ADFEM_API int adfem_mesh_create(const double *xyz, long long num_vertices, const int *elems0, long long num_elements,
                                int degree, adfem_mesh **out);
ADFEM_API int adfem_mesh_destroy(adfem_mesh *mesh);
/* nv, ne, ngauss (3 ne for P1, 6 ne for P2), nnz of the scalar DOF pattern */
ADFEM_API int adfem_mesh_sizes(const adfem_mesh *mesh, long long *nv, long long *ne, long long *ngauss,
                               long long *nnz);
/* Element degree, DOFs per element, Gauss points per element, DOF count (nnode, or
 * nnode + nedges for P2) and scalar pattern nnz of the mesh's own space. */
ADFEM_API int adfem_mesh_space(const adfem_mesh *mesh, int *degree, int *elem_ndof, int *ngauss_elem,
                               long long *ndof, long long *nnz);
/* mfem_get_connectivity: ne x elem_ndof DOFs, 1-based, row-major */
ADFEM_API int adfem_mesh_connectivity(const adfem_mesh *mesh, long long *conn1);
/* mfem_get_gauss_weights: ip.weight * area / 0.5 per Gauss point (Common.cpp:116) */
ADFEM_API int adfem_mesh_gauss_weights(const adfem_mesh *mesh, double *w);
/* Make a handle the "current mesh" of layer 1 (NULL clears it).  The library keeps
 * one current mesh like the reference's global mmesh (deps/MFEM/Common.cpp:7). */
ADFEM_API int adfem_set_current_mesh(adfem_mesh *mesh);
ADFEM_API adfem_mesh *adfem_current_mesh(void);
/* 1-based CSC pattern of the scalar operator (Julia SparseMatrixCSC colptr/rowval).
 * Equal to the pattern of sparse(I,J,V) on the unsummed COO (src/MFEM/MCore.jl:119):
 * the full DOF graph, stored zeros included.  colptr: ndof+1, rowval: nnz. */
ADFEM_API int adfem_mesh_pattern(const adfem_mesh *mesh, long long *colptr1, long long *rowval1);
/* Same for the 2 ndof x 2 ndof elasticity operator in the reference's [x block; y block]
 * ordering (MCore.jl:314): colptr 2ndof+1, rowval 4 nnz. */
ADFEM_API int adfem_mesh_pattern_elasticity(const adfem_mesh *mesh, long long *colptr1, long long *rowval1);
/* bcnode (src/MFEM/MCore.jl:439-450): nodes on edges used by exactly one element, 1-based,
 * ascending (the reference returns Julia Set order); for P2 meshes followed by the DOFs
 * of those edges (nnode + edge, ascending).  With out == NULL only *count is set. */
ADFEM_API int adfem_mesh_bcnode(const adfem_mesh *mesh, long long *out, long long *count);
/* gauss_nodes (src/MFEM/MFEM.jl:226-232): 3 (P1) or 6 (P2) points per element, element-major */
ADFEM_API int adfem_mesh_gauss_nodes(const adfem_mesh *mesh, double *x, double *y);
/* Element vertices after the orientation fix, 1-based, row-major ne x 3 (the content
 * mfem_get_element_to_vertices writes back into Julia's mesh.elems, API.cpp:57-64). */
ADFEM_API int adfem_mesh_elements(const adfem_mesh *mesh, long long *elems1);
/* get_area (src/MFEM/MFEM.jl:216-220 / API.cpp:36-39): Heron area per element */
ADFEM_API int adfem_mesh_area(const adfem_mesh *mesh, double *area);
/* Edge list as returned by init_nnfem_mesh (Common.cpp:133-139): 2*nedges 1-based ids,
 * minimum endpoints then maximum endpoints.  With out == NULL only *nedges is set. */
ADFEM_API int adfem_mesh_edges(const adfem_mesh *mesh, long long *out, long long *nedges);

/* ---- compute_fem_mass_matrix1 (src/MFEM/MCore.jl:170-181), ComputeFemMassMatrixMfem.h:4-55 ----
 * rho: one value per Gauss point.  Summed operator in the adfem_mesh_pattern order
 * (CSC, host) or its CSR rows on the device; unsummed COO (elem_ndof^2 per Gauss point)
 * and its backward (grad_rho overwritten) on the device.  Every degree. */
ADFEM_API int adfem_mass_csc(adfem_mesh *mesh, const double *rho, long long nrho, double *nzval);
ADFEM_API int adfem_mass_csr_d(adfem_mesh *mesh, const double *rho_d, double *vals_d, void *stream);
ADFEM_API int adfem_mass_coo_d(adfem_mesh *mesh, const double *rho_d, long long *indices_d, double *vv_d,
                               void *stream);
ADFEM_API int adfem_mass_coo_backward_d(adfem_mesh *mesh, const double *grad_vv_d, double *grad_rho_d, void *stream);

/* ---- PCL Jacobians (src/pcl.jl:1-39) ----
 * pcl_compute_fem_laplace_matrix1: H[gp, nz] = d vv_nz / d kappa_gp, dense column-major
 * ngauss x (elem_ndof^2 ngauss) (host: only nonzeros written; device: the caller zeroes H).
 * pcl_impose_Dirichlet_boundary_conditions: pos[k] = output position of input COO entry
 * k (0-based (row, col) pairs, bd 1-based) in the COO Dirichlet arm, -1 if dropped; J is
 * then J[k, pos[k]] = 1. */
ADFEM_API int adfem_pcl_laplace_jacobian(adfem_mesh *mesh, double *H);
ADFEM_API int adfem_pcl_laplace_jacobian_d(adfem_mesh *mesh, double *H_d, void *stream);
ADFEM_API int adfem_pcl_dirichlet(const long long *indices, long long sN, const long long *bd, long long nbd,
                                  long long N, long long *pos, long long *nkeep);

/* ---- fem_to_gauss_points / dof_to_gauss_points (src/MFEM/MUtils.jl:231-275) ----
 * fem: u holds nodal values (nu >= nnode; P1 shape of the vertices); dof: u holds DOF
 * values (nu >= ndof; all basis functions).  out: ngauss values.  The backward of
 * either writes (accumulate = 0; entries past the values used are zeroed) or adds
 * (accumulate = 1) grad_u, nu entries. */
ADFEM_API int adfem_fem_to_gauss(adfem_mesh *mesh, const double *u, long long nu, double *out);
ADFEM_API int adfem_dof_to_gauss(adfem_mesh *mesh, const double *u, long long nu, double *out);
ADFEM_API int adfem_fem_to_gauss_d(adfem_mesh *mesh, const double *u_d, double *out_d, void *stream);
ADFEM_API int adfem_fem_to_gauss_backward_d(adfem_mesh *mesh, const double *grad_out_d, double *grad_u_d,
                                            long long nu, int accumulate, void *stream);
ADFEM_API int adfem_dof_to_gauss_d(adfem_mesh *mesh, const double *u_d, double *out_d, void *stream);
ADFEM_API int adfem_dof_to_gauss_backward_d(adfem_mesh *mesh, const double *grad_out_d, double *grad_u_d,
                                            long long nu, int accumulate, void *stream);

/* ---- compute_fem_laplace_matrix1 (src/MFEM/MCore.jl:112-120), Array arm ----
 * kappa: ngauss values (host).  nzval: nnz values in the adfem_mesh_pattern order,
 * i.e. the nzval of the SparseMatrixCSC the reference returns. */
ADFEM_API int adfem_laplace_csc(adfem_mesh *mesh, const double *kappa, long long nkappa, double *nzval);
/* device variant: values in 0-based CSR order of the same pattern (symmetric, so equal) */
ADFEM_API int adfem_laplace_csr_d(adfem_mesh *mesh, const double *kappa_d, double *vals_d, void *stream);
/* graph-op arm (FemLaplaceScalar.h:3-26): unsummed COO on the device */
ADFEM_API int adfem_laplace_coo_d(adfem_mesh *mesh, const double *kappa_d, long long *indices_d, double *vv_d,
                                  void *stream);
/* FemLaplaceScalar.h:28-54 on the device */
ADFEM_API int adfem_laplace_coo_backward_d(adfem_mesh *mesh, const double *grad_vv_d, double *grad_kappa_d,
                                           void *stream);

/* ---- compute_fem_source_term1 (MCore.jl:77-82) ----
 * f: ngauss values.  accumulate = 1 adds into rhs (FemSourceScalar_forward_Julia
 * semantics), 0 overwrites it. */
ADFEM_API int adfem_source(adfem_mesh *mesh, const double *f, long long nf, double *rhs, int accumulate);
ADFEM_API int adfem_source_d(adfem_mesh *mesh, const double *f_d, double *rhs_d, int accumulate, void *stream);
/* FemSourceScalar.h:17-32 on the device */
ADFEM_API int adfem_source_backward_d(adfem_mesh *mesh, const double *grad_rhs_d, double *grad_f_d, void *stream);

/* ---- compute_fem_stiffness_matrix (MCore.jl:296-315), Array arm ----
 * D: ngauss row-major 3x3 blocks (the flattening of MCore.jl:298-307).
 * nzval: 4 nnz values in adfem_mesh_pattern_elasticity order. */
ADFEM_API int adfem_stiffness_csc(adfem_mesh *mesh, const double *D, long long nD, double *nzval);
/* device variant: 0-based CSR values of the same pattern (transpose of the CSC values) */
ADFEM_API int adfem_stiffness_csr_d(adfem_mesh *mesh, const double *D_d, double *vals_d, void *stream);
/* graph-op arm (ComputeFemStiffnessMatrixMfem.h:4-48): unsummed COO, 4 elem_ndof^2 per Gauss point */
ADFEM_API int adfem_stiffness_coo_d(adfem_mesh *mesh, const double *D_d, long long *indices_d, double *vv_d,
                                    void *stream);
ADFEM_API int adfem_stiffness_coo_backward_d(adfem_mesh *mesh, const double *grad_vv_d, double *grad_D_d,
                                             void *stream);
/* compute_plane_strain_matrix(E, nu) (src/Core.jl:777-785) / plane stress, on the device */
ADFEM_API int adfem_plane_strain_d(int mode, long long n, const double *E_d, const double *nu_d, double *D_d,
                                   void *stream);
ADFEM_API int adfem_plane_strain_backward_d(int mode, long long n, const double *grad_D_d, const double *E_d,
                                            const double *nu_d, double *grad_E_d, double *grad_nu_d, void *stream);

/* ---- impose_Dirichlet_boundary_conditions ----
 * SparseMatrixCSC arm (src/MFEM/MUtils.jl:184-199), host pointers, 1-based CSC in and out.
 * B = [A_II 0; 0 I], r_I = rhs_I - A_IB * bdval, r_B = bdval.  Entries of A_II equal to
 * 0.0 are not stored unless keep_zeros != 0 (Julia's sparse setindex! into spzeros does
 * not insert zeros).  bd: 1-based, no duplicates.  Two calls: with out_colptr1 == NULL
 * only *out_nnz is set. */
ADFEM_API int adfem_dirichlet_csc(long long n, const long long *colptr1, const long long *rowval1,
                                  const double *nzval, const double *rhs, const long long *bd, long long nbd,
                                  const double *bdval, int keep_zeros, long long *out_colptr1,
                                  long long *out_rowval1, double *out_nzval, long long *out_nnz, double *out_rhs);
/* SparseTensor arm (deps/MFEM/ImposeDirichlet/ImposeDirichlet.h:27-60), host pointers:
 * keeps COO entries with row and column outside bd in input order, lifts the rhs,
 * appends (b,b,1.0) for each distinct bd node in ascending order.  indices 0-based
 * (row,col) pairs; bd 1-based (duplicates allowed, last bdval wins).  Returns the
 * output entry count in *out_n; with oindices == NULL only counts. */
ADFEM_API int adfem_dirichlet_coo(const long long *indices, const double *vv, long long sN, const long long *bd,
                                  long long nbd, const double *rhs, const double *bdval, long long N,
                                  long long *oindices, double *ov, double *orhs, long long *out_n);
/* ImposeDirichlet.h:63-93 */
ADFEM_API int adfem_dirichlet_coo_backward(const double *grad_vv, const double *grad_rhs, const long long *indices,
                                           const double *vv, long long sN, const long long *bd, long long nbd,
                                           const double *bdval, long long N, double *grad_vv_in,
                                           double *grad_rhs_in, double *grad_bdval);

/* ---- K \ F ---- */
enum { ADFEM_PREC_FP64 = 0, ADFEM_PREC_MIXED = 1 };
typedef struct {
  double rtol;     /* stop when ||b~ - K~ y|| <= rtol ||b~|| in the Jacobi-scaled system (default 1e-12) */
  int max_iter;    /* cap on CG iterations (default 200000) */
  int precision;   /* ADFEM_PREC_FP64: FP64 Jacobi-CG; ADFEM_PREC_MIXED: FP32 inner CG with FP64
                      reliable updates (FP64 residual r = F - K u, FP64 solution, FP64 stop test) */
  double ru_delta; /* mixed: replace the FP32 residual by the FP64 one when it dropped by this factor
                      since the last replacement (default 0.1) */
  int chunk;       /* iterations per device-resident chunk between host checks (default 32) */
  int warm_start;  /* 1: start from the u passed in; 0: from zero */
} adfem_solver_opts;

typedef struct {
  int iterations;      /* inner CG iterations */
  int updates;         /* FP64 residual replacements (mixed) */
  double relres;       /* final scaled residual ||b~ - K~ y|| / ||b~||, FP64 */
  double ms;           /* wall time of the solve on the stream (CUDA events) */
  int status;
  long long launches;  /* kernels launched by the solve (graph-resident ones included) */
} adfem_solver_stats;

ADFEM_API void adfem_solver_opts_default(adfem_solver_opts *opts);

/* K\F for a symmetric positive definite 1-based CSC matrix (e.g. the output of the
 * Dirichlet entry), host pointers.  Replaces Julia SparseArrays' `\` on this path
 * (README.md:54) with a GPU Jacobi-CG; u receives the solution. */
ADFEM_API int adfem_csc_solve(long long n, const long long *colptr1, const long long *rowval1, const double *nzval,
                              const double *rhs, double *u, const adfem_solver_opts *opts,
                              adfem_solver_stats *stats);

/* ---- resident solver systems (device pointers) ----
 * A system keeps the assembled, Dirichlet-imposed operator of one mesh resident in
 * sliced-ELL form (FP64 and FP32 Jacobi-scaled copies) with its right-hand side and
 * CG work vectors, so repeated solves and adjoint solves reuse them. */
enum { ADFEM_SYS_POISSON = 0, ADFEM_SYS_ELASTICITY = 1 };
/* Poisson systems on P1 or P2 meshes (P2: the vertex-then-edge DOFs of the mesh's space,
 * kappa and f at the 6 points per element of the order-4 rule; DOFs renumbered for the
 * solver by reverse Cuthill-McKee, inputs and outputs in the reference order); elasticity
 * systems on P1 meshes (a P2 mesh gives ADFEM_ERR_UNSUPPORTED: assemble its stiffness
 * operator and use adfem_csc_solve). */
ADFEM_API int adfem_system_create(adfem_mesh *mesh, int kind, adfem_system **out);
ADFEM_API int adfem_system_destroy(adfem_system *sys);
/* Dirichlet data: bd 1-based DOF ids (for elasticity DOF ids in the [x; y] ordering,
 * 1..2nv), host arrays, no duplicates; bdval may be NULL (all zero). */
ADFEM_API int adfem_system_set_dirichlet(adfem_system *sys, const long long *bd, long long nbd, const double *bdval);
/* Poisson: K(kappa), F(f), Dirichlet imposed -- one fused pass.  kappa_d, f_d: ngauss. */
ADFEM_API int adfem_system_assemble_poisson_d(adfem_system *sys, const double *kappa_d, const double *f_d,
                                              void *stream);
/* Elasticity with plane-strain D(E, nu) (reference formula) at each Gauss point and
 * body force (fx, fy) at the Gauss points. */
/* Same as adfem_system_assemble_poisson_d, and ms[0..2] receive the device time of its
 * three phases (CUDA events): element pass (sigma, element loads), fused Laplace + load +
 * Dirichlet rows, operator conversion for the solver (Jacobi scaling, FP32 and banded copies).
 * Synchronises the stream. */
ADFEM_API int adfem_system_assemble_poisson_profiled_d(adfem_system *sys, const double *kappa_d, const double *f_d,
                                                       double *ms, void *stream);
ADFEM_API int adfem_system_assemble_elasticity_d(adfem_system *sys, const double *E_d, const double *nu_d,
                                                 const double *fx_d, const double *fy_d, void *stream);
/* Solve the assembled system; u_d: ndof (nv or 2nv, reference DOF ordering). */
ADFEM_API int adfem_system_solve_d(adfem_system *sys, double *u_d, const adfem_solver_opts *opts,
                                   adfem_solver_stats *stats, void *stream);
/* Adjoint solve K lambda = g (K symmetric); lambda is zero on Dirichlet DOFs. */
ADFEM_API int adfem_system_adjoint_d(adfem_system *sys, const double *g_d, double *lam_d,
                                     const adfem_solver_opts *opts, adfem_solver_stats *stats, void *stream);
/* dL/dkappa at every Gauss point: -w (grad lam).(grad u) at the point (P1: equal for the 3
 * points of an element; P2: the quadratic fields' gradients at each of the 6 points), lam
 * zero on the Dirichlet DOFs; the composition of the reference's FemLaplaceScalar,
 * ImposeDirichlet and sparse-solve gradients. */
ADFEM_API int adfem_system_grad_kappa_d(adfem_system *sys, const double *u_d, const double *lam_d,
                                        double *grad_kappa_d, void *stream);
/* dL/dE at every Gauss point for the plane-strain material used by the last
 * assemble_elasticity call: sum_pq (-w (B lam_e)(B u_e)^T)_pq dD_pq/dE. */
ADFEM_API int adfem_system_grad_E_d(adfem_system *sys, const double *u_d, const double *lam_d, const double *E_d,
                                    const double *nu_d, double *grad_E_d, void *stream);
/* y = K x with the system's FP64 operator (unscaled), for checks. */
ADFEM_API int adfem_system_apply_d(adfem_system *sys, const double *x_d, double *y_d, void *stream);
/* copy out the assembled right-hand side (reference DOF ordering) */
ADFEM_API int adfem_system_rhs_d(adfem_system *sys, double *rhs_d, void *stream);
/* Same solve as adfem_system_solve_d with CUDA event pairs on the solver's stream, for
 * measurement: launched kernel by kernel with an event pair around every launch, except
 * that on the banded mixed path each run of iterations between two replacement checks
 * (16) is one captured graph (as in the solve) with an event pair around the run, whose
 * time is shared by its launches.  kernel_ms[j]
 * and launches[j] receive the summed duration and launch count of: 0 SpMV+dot (the whole
 * iteration on the banded mixed path), 1 vector update+dot, 2 p update (FP64) / fold
 * (mixed), 3 FP64 residual. */
ADFEM_API int adfem_system_solve_profiled_d(adfem_system *sys, double *u_d, const adfem_solver_opts *opts,
                                            adfem_solver_stats *stats, double *kernel_ms, long long *launches,
                                            void *stream);

/* Layout of a system's solver operator and the mixed-precision iteration it uses (no
 * counterpart in the reference; for traffic models and tests). */
typedef struct adfem_solver_info {
  long long rows;             /* solver DOFs */
  long long stored;           /* sliced-ELL entries, padding included */
  long long uniform_entries;  /* entries in slices whose column pattern is stored once */
  long long slices;           /* 32-row slices */
  long long band;             /* max |col - row| */
  int banded;                 /* 1: one-kernel banded mixed iteration, 0: scaled two-kernel iteration */
  int blocks;                 /* blocks of the banded iteration kernel (0 if not banded) */
  long long rows_per_block;   /* contiguous rows per block (0 if not banded) */
  int ring;                   /* shared-memory positions per super-tile: rows + 2 band (0 if not banded) */
  int renumbered;             /* 1: nodes renumbered for the solver (reverse Cuthill-McKee; inputs and
                                 outputs stay in the reference order) */
  int banded_fp64;            /* 1: FP64 solves use the one-kernel banded FP64 iteration (same layout and
                                 fusion as the mixed one), 0: the three-kernel FP64 iteration */
  int fp64_tile_rows;         /* rows per super-tile of the banded FP64 iteration (0 if not used) */
  int ring_stages;            /* stages of the shared-memory matrix ring of the banded mixed iteration
                                 (bulk copies of 1024 rows each; 0: values loaded by the threads) */
  int assembly_pairs;         /* 1: the Poisson assembly runs in FP32-pair arithmetic in one pass */
} adfem_solver_info;
ADFEM_API int adfem_system_solver_info(const adfem_system *sys, adfem_solver_info *info);
/* Packed solves of small systems: the systems (each assembled, at most 65536 DOFs,
 * distinct) are solved by one graph-captured launch, one thread block per system up to
 * 16384 DOFs and one cluster of eight thread blocks per larger system, with
 * FP32 inner CG iterations inside FP64 iterative refinement (the mixed method; opts
 * precision is ignored).  Forward: u_d[i] as adfem_system_solve_d.  Adjoint: lam_d[i]
 * for right-hand sides g_d[i], as adfem_system_adjoint_d.  stats[i] (may be NULL):
 * iterations = inner CG iterations, updates = FP64 refinement passes.  Each system's
 * result is independent of the others in the pack.  Synchronises the stream. */
ADFEM_API int adfem_system_solve_packed_d(adfem_system **sys, int count, double **u_d, const adfem_solver_opts *opts,
                                          adfem_solver_stats *stats, void *stream);
ADFEM_API int adfem_system_adjoint_packed_d(adfem_system **sys, int count, const double *const *g_d, double **lam_d,
                                            const adfem_solver_opts *opts, adfem_solver_stats *stats, void *stream);

/* No counterpart in the reference.  Allocation-free FP64 Jacobi-CG on a caller-owned
 * device CSR matrix (0-based rowptr[n+1], colind[nnz], vals[nnz], symmetric positive
 * definite), for callers that cannot call cudaMalloc -- e.g. code running inside a
 * TensorFlow/ADCME custom op or a CUDA.jl task, where the framework's pool owns the
 * device memory and an allocation could fail or synchronise the device.  All scratch
 * lives in a fixed static device array: n must not exceed 131072 rows (larger n
 * returns ADFEM_ERR_INVALID).  No cudaMalloc/cudaFree or allocating library call is
 * made.  The first call on a device looks up the array's device address, so it should
 * come before any stream capture.  Calls share the array: calls that overlap on the
 * GPU race and must be serialised by the caller.  The call is synchronous: it reads
 * the CG state back every 16 iterations and returns when the solve has ended; on a
 * stream that is being captured it returns ADFEM_ERR_UNSUPPORTED without enqueueing
 * work.  u_d receives the solution (the iteration starts from zero); iterations/relres
 * (optional) receive the CG count and the final recursive ||r||/||b||. */
ADFEM_API int adfem_csr_pcg_noalloc_d(int n, const int *rowptr_d, const int *colind_d, const double *vals_d,
                                      const double *rhs_d, double *u_d, double rtol, int max_iter, int *iterations,
                                      double *relres, void *stream);

/* ---- serving loop (no counterpart in the reference, which holds one global mesh,
 * deps/MFEM/API.cpp:6-10) ----
 * A request = one forward solve on a caller-owned mesh (Poisson or plane-strain
 * elasticity, the fields at the Gauss points, Dirichlet DOFs), optionally with a
 * misfit L = sum (u[obs] - uobs)^2 whose gradient with respect to the field
 * (kappa or E) is returned through the adjoint.  Worker threads, each with its own
 * CUDA stream, take requests in arrival order and run them on resident systems kept
 * per (mesh, kind) and reused (operator pattern, solver buffers and captured CUDA
 * graphs stay on the device); a new request starts as soon as a worker frees, so
 * requests of any size run concurrently.  Every request runs its own fixed-grid,
 * fixed-order kernels: its results do not depend on what else is in flight.
 * Admission: resident systems and worker buffers are counted against an HBM budget;
 * idle systems are evicted least-recently-used; a request that cannot fit even in an
 * empty server is rejected with ADFEM_ERR_BUSY, as is a submit to a full queue. */
typedef struct adfem_server adfem_server;
typedef struct adfem_server_config {
  long long hbm_budget_bytes; /* device bytes for resident systems and worker buffers; 0: 80% of free memory */
  int workers;                /* concurrent requests (one CUDA stream each); 0: 8 */
  int max_queue;              /* pending requests accepted; 0: 65536 */
  adfem_solver_opts opts;     /* solver options of every request (precision per request may override) */
  int pack_max_dof;           /* mixed-precision requests with at most this many DOFs are solved in
                                 packs (one launch, one thread block or cluster each); 0: 16384;
                                 < 0: never; at most 65536 */
  int pack_max;               /* systems per packed launch; 0: 64 (at most 128) */
} adfem_server_config;
ADFEM_API void adfem_server_config_default(adfem_server_config *cfg);

typedef struct adfem_request {
  adfem_mesh *mesh;          /* caller-owned, must outlive the request */
  int kind;                  /* ADFEM_SYS_POISSON or ADFEM_SYS_ELASTICITY */
  const double *in[4];       /* host, ngauss each: Poisson {kappa, f}; elasticity {E, nu, fx, fy} */
  const long long *bd;       /* Dirichlet DOF ids, 1-based (elasticity: [x; y] ordering) */
  long long nbd;
  const double *bdval;       /* NULL: all zero */
  const long long *obs;      /* optional observation DOF ids (1-based): misfit + gradient */
  long long nobs;
  const double *uobs;        /* observed values at obs */
  double *u;                 /* host out, ndof */
  double *grad;              /* host out, ngauss: dL/dkappa or dL/dE (required with obs) */
  double deadline_ms;        /* from submission; a request not started by then gets ADFEM_ERR_TIMEOUT; 0: none */
  int warm_start;            /* start from the last solution computed on the same resident system */
  int precision;             /* ADFEM_PREC_FP64 / ADFEM_PREC_MIXED, or -1 for the server's */
} adfem_request;

typedef struct adfem_response {
  int status;                /* ADFEM_OK or the failure status */
  int iterations;            /* forward CG iterations */
  int adjoint_iterations;    /* 0 without observations */
  double relres;             /* forward FP64 relative residual */
  double loss;               /* misfit, 0 without observations */
  double queue_ms;           /* submission to start */
  double run_ms;             /* start to completion */
  double total_ms;           /* submission to completion */
  char message[160];         /* failure message ("" on success) */
  int packed;                /* 1: the solves ran in a packed launch */
} adfem_response;

typedef struct adfem_server_stats {
  long long submitted, completed, rejected, timeouts, failed;
  long long cache_hits, cache_misses, evictions;
  long long resident_systems, device_bytes;
  double p50_ms, p99_ms, mean_ms, max_ms;  /* total latency of completed requests */
  double p50_queue_ms, p99_queue_ms;
  long long packs, packed_requests;        /* packed launches; requests solved in them */
} adfem_server_stats;

ADFEM_API int adfem_server_create(const adfem_server_config *cfg, adfem_server **out);
/* Stops accepting requests, finishes the queued ones, releases all resident systems. */
ADFEM_API int adfem_server_destroy(adfem_server *srv);
/* Queue a request (the request struct is copied; the arrays it points to must stay
 * valid until the request completes).  ticket receives its id. */
ADFEM_API int adfem_server_submit(adfem_server *srv, const adfem_request *req, long long *ticket);
/* Wait up to timeout_ms (< 0: forever) for a request; ADFEM_OK with the response once
 * it completed (the ticket is then released), ADFEM_ERR_TIMEOUT if still running. */
ADFEM_API int adfem_server_wait(adfem_server *srv, long long ticket, double timeout_ms, adfem_response *resp);
ADFEM_API int adfem_server_get_stats(adfem_server *srv, adfem_server_stats *stats);
ADFEM_API int adfem_server_reset_stats(adfem_server *srv);

/* One host-buffer call for the whole Poisson forward path: upload kappa and f,
 * assemble, impose u = bdval on bd, solve, download u.  The end-to-end entry a Julia
 * caller uses for `K\F` after compute_fem_laplace_matrix1 / compute_fem_source_term1 /
 * impose_Dirichlet_boundary_conditions. */
ADFEM_API int adfem_poisson_solve(adfem_system *sys, const double *kappa, const double *f, double *u,
                                  const adfem_solver_opts *opts, adfem_solver_stats *stats);

#ifdef __cplusplus
}
#endif
#endif /* ADFEM_GPU_H */
