// extern "C" entry points of libadfem_gpu.so (declared in include/adfem_gpu.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "adfem_internal.h"
#include "dirichlet.cuh"
#include <nvtx3/nvToolsExt.h>
#include "elastic.cuh"
#include "solver.cuh"

using namespace adfem;

namespace adfem {

NvtxRange::NvtxRange(const char* name) { nvtxRangePushA(name); }
NvtxRange::~NvtxRange() { nvtxRangePop(); }
const char* last_error_cstr();
}

struct adfem_mesh {
  Mesh* m;
};

struct adfem_system {
  adfem_mesh* mesh = nullptr;
  int kind = ADFEM_SYS_POISSON;
  int64_t ndof = 0;  // nv (Poisson) or 2 nv (elasticity)
  Sell A;            // operator in solver DOF order (interleaved for elasticity)
  DevBuf diagpos;    // int32 [ndof]
  DevBuf isbd;       // uint8 [ndof] 0 free, 1 Dirichlet, 2 free next to a Dirichlet DOF (solver order)
  DevBuf bdval;      // double [ndof] dense Dirichlet values (solver order)
  DevBuf isbd_ref;   // uint8 [ndof] the same tags in node order (interleaved for elasticity)
  // Solver DOF order: elasticity interleaves the [x; y] blocks (2i + c); either kind may
  // renumber its nodes (reverse Cuthill-McKee) when that at least halves the bandwidth,
  // so that the banded mixed iteration applies to arbitrarily numbered meshes.
  bool renumbered = false;
  std::vector<int32_t> hperm;  // node -> solver node (identity unless renumbered)
  DevBuf nperm;      // int32 [nv] (renumbered only)
  DevBuf kperm;      // uint8 [nnz] rank of each mesh pattern slot in its renumbered row
  DevBuf dofmap;     // int32 [ndof] reference DOF -> solver DOF (elasticity or renumbered)
  DevBuf rhs;        // double [ndof]
  DevBuf sigma, src3, srcy3, Dbar;  // per-element scratch
  DevBuf ke;                        // P2 Poisson: element matrices (36 per element)
  DevBuf sdiag;                     // P2 Poisson: diagonal slot of each space pattern row
  DevBuf t0, t1, t2;                // ndof scratch (interleaving, host staging)
  DevBuf in0, in1;                  // host-staging of per-Gauss-point inputs
  Solver solver;
  bool assembled = false;
  // P1 Poisson assembly in FP32-pair arithmetic (opt-in with ADFEM_ASM_PAIRS=1 at creation;
  // rows of up to 16 entries).  Not the default: its ~1e-14 relative differences in the
  // matrix entries moved the 4M-DOF mixed solution from 1.7e-11 to 6.7e-11 relative error
  // against the refined FP64 reference, for an assembly 0.05 ms faster.
  bool pairs = false;
  std::mutex mu;
};

namespace {

std::mutex g_cur_mu;
adfem_mesh* g_current = nullptr;
bool g_current_owned = false;

cudaStream_t S(void* p) { return reinterpret_cast<cudaStream_t>(p); }

Mesh* current_mesh() {
  std::lock_guard<std::mutex> lk(g_cur_mu);
  return g_current ? g_current->m : nullptr;
}

template <class T>
int to_dev(DevBuf& b, const T* h, size_t n) {
  ADFEM_TRY(b.alloc(sizeof(T) * std::max<size_t>(n, 1)));
  if (n) ADFEM_CUDA(cudaMemcpy(b.p, h, sizeof(T) * n, cudaMemcpyHostToDevice));
  return ADFEM_OK;
}
template <class T>
int to_host(T* h, const DevBuf& b, size_t n) {
  if (n) ADFEM_CUDA(cudaMemcpy(h, b.p, sizeof(T) * n, cudaMemcpyDeviceToHost));
  return ADFEM_OK;
}
int kerr(cudaError_t e, const char* what) {
  if (e != cudaSuccess) return cuda_fail(e, what);
  return ADFEM_OK;
}

// The space of the given degree on m (built on first use under m.mu).
int get_space(Mesh& m, int degree, Space** sp) {
  std::lock_guard<std::mutex> lk(m.mu);
  return mesh_space(&m, degree, sp);
}

void legacy_report(int st, const char* fn) {
  if (st != ADFEM_OK) std::fprintf(stderr, "libadfem_gpu: %s failed: %s\n", fn, last_error_cstr());
}

// Dirichlet data for a system: tags over the solver DOF order
int system_set_bd(adfem_system* s, const long long* bd, long long nbd, const double* bdval) {
  Mesh& m = *s->mesh->m;
  const int64_t nd = s->ndof;
  const bool el = s->kind == ADFEM_SYS_ELASTICITY;
  std::vector<uint8_t> tag(nd, 0), tref(nd, 0);
  std::vector<double> val(nd, 0.0);
  // node (and component) -> solver DOF; -> node-order DOF of the reference tags
  auto sdof = [&](int64_t i, int c) -> int64_t { return el ? 2 * (int64_t)s->hperm[i] + c : s->hperm[i]; };
  auto rdof = [&](int64_t i, int c) -> int64_t { return el ? 2 * i + c : i; };
  for (long long k = 0; k < nbd; k++) {
    const long long d = bd[k] - 1;
    if (d < 0 || d >= nd) return fail(ADFEM_ERR_INVALID, "Dirichlet DOF " + std::to_string(bd[k]) + " out of range");
    const int64_t i = el ? (d < m.nv ? d : d - m.nv) : d;
    const int c = el && d >= m.nv ? 1 : 0;
    const int64_t q = sdof(i, c);
    if (tag[q]) return fail(ADFEM_ERR_INVALID, "duplicate Dirichlet DOF " + std::to_string(bd[k]));
    tag[q] = 1;
    tref[rdof(i, c)] = 1;
    val[q] = bdval ? bdval[k] : 0.0;
  }
  const int nc = el ? 2 : 1;
  // the scalar pattern of the operator: the mesh's, or the P2 space's (built at creation)
  const Space* sp = m.degree == 2 ? m.space[2].get() : nullptr;
  const int64_t nn = sp ? sp->ndof : m.nv;
  const std::vector<int32_t>& RP = sp ? sp->rowptr : m.rowptr;
  const std::vector<int32_t>& CI = sp ? sp->colind : m.colind;
  for (int64_t i = 0; i < nn; i++) {
    bool near = false;
    for (int32_t k = RP[i]; k < RP[i + 1]; k++)
      for (int c = 0; c < nc; c++) near |= tag[sdof(CI[k], c)] == 1;
    if (!near) continue;
    for (int c = 0; c < nc; c++)
      if (tag[sdof(i, c)] == 0) {
        tag[sdof(i, c)] = 2;
        tref[rdof(i, c)] = 2;
      }
  }
  ADFEM_TRY(to_dev(s->isbd, tag.data(), tag.size()));
  ADFEM_TRY(to_dev(s->isbd_ref, tref.data(), tref.size()));
  ADFEM_TRY(to_dev(s->bdval, val.data(), val.size()));
  s->assembled = false;
  return ADFEM_OK;
}

// vectors between the reference DOF order and the solver's
bool mapped(const adfem_system* s) { return s->kind == ADFEM_SYS_ELASTICITY || s->renumbered; }
int to_solver(adfem_system* s, const double* ref, double* sol, cudaStream_t st) {
  return kerr(launch_to_solver(s->ndof, s->dofmap.as<int32_t>(), ref, sol, st), "to solver order");
}
int from_solver(adfem_system* s, const double* sol, double* ref, cudaStream_t st) {
  return kerr(launch_from_solver(s->ndof, s->dofmap.as<int32_t>(), sol, ref, st), "from solver order");
}

}  // namespace

namespace adfem {

size_t system_device_bytes(const adfem_system* s) {
  size_t b = 0;
  const Sell& A = s->A;
  for (const DevBuf* d : {&A.sptr, &A.col, &A.spat, &A.pat, &A.val64, &A.valD64, &A.val32, &s->diagpos, &s->isbd,
                          &s->bdval, &s->rhs, &s->sigma, &s->src3, &s->srcy3, &s->Dbar, &s->t0, &s->t1, &s->t2,
                          &s->in0, &s->in1, &s->isbd_ref, &s->nperm, &s->kperm, &s->dofmap})
    b += d->bytes;
  const Solver& v = s->solver;
  for (const DevBuf* d : {&v.s32, &v.state, &v.partials, &v.b, &v.y64, &v.r64, &v.p64, &v.q64, &v.z64, &v.r32, &v.pa32,
                          &v.pb32, &v.q32, &v.yh32, &v.yl32, &v.z1, &v.zq1, &v.dz32, &v.valz64, &v.valz32,
                          &v.colz16, &v.zpid32, &v.zpool32, &v.bz32})
    b += d->bytes;
  return b;
}

const Mesh* mesh_of(const adfem_mesh* h) { return h ? h->m : nullptr; }

}  // namespace adfem

extern "C" {

const char* adfem_status_string(int st) {
  switch (st) {
    case ADFEM_OK: return "ok";
    case ADFEM_ERR_INVALID: return "invalid argument";
    case ADFEM_ERR_CUDA: return "CUDA error";
    case ADFEM_ERR_NOMEM: return "out of memory";
    case ADFEM_ERR_NOT_CONVERGED: return "not converged";
    case ADFEM_ERR_BREAKDOWN: return "CG breakdown";
    case ADFEM_ERR_NO_MESH: return "no current mesh";
    case ADFEM_ERR_NONFINITE: return "non-finite input";
    case ADFEM_ERR_UNSUPPORTED: return "unsupported";
    case ADFEM_ERR_BUSY: return "busy";
    case ADFEM_ERR_TIMEOUT: return "timeout";
    default: return "unknown status";
  }
}
const char* adfem_last_error(void) { return last_error_cstr(); }
const char* adfem_version(void) { return "adfem_gpu 0.1 (sm_103a)"; }

// ------------------------------------------------------------------ meshes
int adfem_mesh_create(const double* xyz, long long nv, const int* elems0, long long ne, int degree,
                      adfem_mesh** out) {
  ADFEM_RANGE("adfem_mesh_create");
  if (!out) return fail(ADFEM_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (degree != 1 && degree != 2) return fail(ADFEM_ERR_UNSUPPORTED, "element degree must be 1 (P1) or 2 (P2)");
  Mesh* m = nullptr;
  ADFEM_TRY(mesh_build(xyz, nv, reinterpret_cast<const int32_t*>(elems0), ne, &m));
  std::unique_ptr<Mesh> own(m);
  m->degree = degree;
  if (degree == 2) {
    Space* sp = nullptr;
    ADFEM_TRY(get_space(*m, 2, &sp));
  }
  *out = new adfem_mesh{own.release()};
  return ADFEM_OK;
}

int adfem_mesh_destroy(adfem_mesh* mesh) {
  ADFEM_RANGE("adfem_mesh_destroy");
  if (!mesh) return ADFEM_OK;
  {
    std::lock_guard<std::mutex> lk(g_cur_mu);
    if (g_current == mesh) {
      g_current = nullptr;
      g_current_owned = false;
    }
  }
  delete mesh->m;
  delete mesh;
  return ADFEM_OK;
}

int adfem_mesh_sizes(const adfem_mesh* mesh, long long* nv, long long* ne, long long* ngauss, long long* nnz) {
  ADFEM_RANGE("adfem_mesh_sizes");
  if (!mesh) return fail(ADFEM_ERR_INVALID, "null mesh");
  if (nv) *nv = mesh->m->nv;
  if (ne) *ne = mesh->m->ne;
  if (ngauss) *ngauss = mesh_ngauss(*mesh->m);
  if (nnz) *nnz = mesh->m->degree == 2 ? mesh->m->space[2]->nnz : mesh->m->nnz;
  return ADFEM_OK;
}

int adfem_mesh_space(const adfem_mesh* mesh, int* degree, int* elem_ndof, int* ngauss_elem, long long* ndof,
                     long long* nnz) {
  ADFEM_RANGE("adfem_mesh_space");
  if (!mesh) return fail(ADFEM_ERR_INVALID, "null mesh");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  if (degree) *degree = m.degree;
  if (elem_ndof) *elem_ndof = sp->nd;
  if (ngauss_elem) *ngauss_elem = sp->ng;
  if (ndof) *ndof = sp->ndof;
  if (nnz) *nnz = sp->nnz;
  return ADFEM_OK;
}

int adfem_mesh_connectivity(const adfem_mesh* mesh, long long* conn1) {
  ADFEM_RANGE("adfem_mesh_connectivity");
  if (!mesh || !conn1) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  for (size_t k = 0; k < sp->dof.size(); k++) conn1[k] = (long long)sp->dof[k] + 1;
  return ADFEM_OK;
}

int adfem_mesh_gauss_weights(const adfem_mesh* mesh, double* w) {
  ADFEM_RANGE("adfem_mesh_gauss_weights");
  if (!mesh || !w) return fail(ADFEM_ERR_INVALID, "null argument");
  mesh_gauss_weights(mesh->m, w);
  return ADFEM_OK;
}

int adfem_set_current_mesh(adfem_mesh* mesh) {
  ADFEM_RANGE("adfem_set_current_mesh");
  std::lock_guard<std::mutex> lk(g_cur_mu);
  if (g_current && g_current_owned && g_current != mesh) {
    delete g_current->m;
    delete g_current;
  }
  g_current = mesh;
  g_current_owned = false;
  return ADFEM_OK;
}
adfem_mesh* adfem_current_mesh(void) {
  std::lock_guard<std::mutex> lk(g_cur_mu);
  return g_current;
}

int adfem_mesh_pattern(const adfem_mesh* mesh, long long* colptr1, long long* rowval1) {
  ADFEM_RANGE("adfem_mesh_pattern");
  if (!mesh || !colptr1 || !rowval1) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  for (int64_t i = 0; i <= sp->ndof; i++) colptr1[i] = (long long)sp->rowptr[i] + 1;
  for (int64_t k = 0; k < sp->nnz; k++) rowval1[k] = (long long)sp->colind[k] + 1;
  return ADFEM_OK;
}

int adfem_mesh_pattern_elasticity(const adfem_mesh* mesh, long long* colptr1, long long* rowval1) {
  ADFEM_RANGE("adfem_mesh_pattern_elasticity");
  if (!mesh || !colptr1 || !rowval1) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  const int64_t n = sp->ndof;
  long long z = 0;
  for (int c = 0; c < 2; c++)
    for (int64_t i = 0; i < n; i++) {
      colptr1[c * n + i] = z + 1;
      for (int cc = 0; cc < 2; cc++)
        for (int32_t k = sp->rowptr[i]; k < sp->rowptr[i + 1]; k++) rowval1[z++] = (long long)sp->colind[k] + cc * n + 1;
    }
  colptr1[2 * n] = z + 1;
  return ADFEM_OK;
}

int adfem_mesh_bcnode(const adfem_mesh* mesh, long long* out, long long* count) {
  ADFEM_RANGE("adfem_mesh_bcnode");
  if (!mesh || !count) return fail(ADFEM_ERR_INVALID, "null argument");
  *count = mesh_bcnode(mesh->m, reinterpret_cast<int64_t*>(out));
  return ADFEM_OK;
}

int adfem_mesh_gauss_nodes(const adfem_mesh* mesh, double* x, double* y) {
  ADFEM_RANGE("adfem_mesh_gauss_nodes");
  if (!mesh || !x || !y) return fail(ADFEM_ERR_INVALID, "null argument");
  mesh_gauss(mesh->m, x, y);
  return ADFEM_OK;
}

// ------------------------------------------------------------------ generic (P2) ops
namespace {
Space* p2_space(Mesh& m) { return m.degree == 2 ? m.space[2].get() : nullptr; }

int gen_matrix_d(Mesh& m, Space& sp, GenOp op, const double* coef_d, double* vals_d, bool transpose,
                 cudaStream_t st) {
  std::lock_guard<std::mutex> lk(m.mu);
  ADFEM_TRY(sp.d_ke.alloc(sizeof(double) * (size_t)sp.nd * sp.nd * m.ne));
  ADFEM_TRY(kerr(launch_gen_matrix(m, sp, op, coef_d, sp.d_ke.as<double>(), vals_d, transpose, st), "matrix"));
  ADFEM_CUDA(cudaStreamSynchronize(st));
  return ADFEM_OK;
}

int gen_stiffness_d(Mesh& m, Space& sp, const double* D_d, double* vals_d, bool transpose, cudaStream_t st) {
  std::lock_guard<std::mutex> lk(m.mu);
  ADFEM_TRY(sp.d_ke.alloc(sizeof(double) * 4 * (size_t)sp.nd * sp.nd * m.ne));
  ADFEM_TRY(kerr(launch_gen_stiffness_matrix(m, sp, D_d, sp.d_ke.as<double>(), vals_d, transpose, st), "stiffness"));
  ADFEM_CUDA(cudaStreamSynchronize(st));
  return ADFEM_OK;
}

// host-pointer summed operator: per-point input of len values -> nnz_mult * nnz values
int gen_matrix_host(adfem_mesh* mesh, int which, const double* in, long long nin, double* nzval) {
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  const int64_t ng = mesh_ngauss(m);
  const int64_t want = which == 2 ? 9 * ng : ng;
  if (nin != want)
    return fail(ADFEM_ERR_INVALID, which == 2 ? "D must hold a 3x3 matrix per Gauss point"
                                              : "the coefficient must have one value per Gauss point");
  const size_t nv = (which == 2 ? 4 : 1) * (size_t)sp->nnz;
  DevBuf k, v;
  ADFEM_TRY(to_dev(k, in, (size_t)nin));
  ADFEM_TRY(v.alloc(sizeof(double) * nv));
  if (which == 2) ADFEM_TRY(gen_stiffness_d(m, *sp, k.as<double>(), v.as<double>(), true, nullptr));
  else ADFEM_TRY(gen_matrix_d(m, *sp, which == 0 ? GenOp::LAPLACE : GenOp::MASS, k.as<double>(), v.as<double>(), true,
                              nullptr));
  return to_host(nzval, v, nv);
}
}  // namespace

int adfem_mass_csr_d(adfem_mesh* mesh, const double* rho_d, double* vals_d, void* stream) {
  ADFEM_RANGE("adfem_mass_csr_d");
  if (!mesh || !rho_d || !vals_d) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  return gen_matrix_d(m, *sp, GenOp::MASS, rho_d, vals_d, false, S(stream));
}

int adfem_mass_csc(adfem_mesh* mesh, const double* rho, long long nrho, double* nzval) {
  ADFEM_RANGE("adfem_mass_csc");
  if (!mesh || !rho || !nzval) return fail(ADFEM_ERR_INVALID, "null argument");
  return gen_matrix_host(mesh, 1, rho, nrho, nzval);
}

int adfem_mass_coo_d(adfem_mesh* mesh, const double* rho_d, long long* indices_d, double* vv_d, void* stream) {
  ADFEM_RANGE("adfem_mass_coo_d");
  if (!mesh || !rho_d || !indices_d || !vv_d) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  return kerr(launch_gen_coo(m, *sp, GenOp::MASS, rho_d, indices_d, vv_d, S(stream)), "mass coo");
}

int adfem_mass_coo_backward_d(adfem_mesh* mesh, const double* grad_vv_d, double* grad_rho_d, void* stream) {
  ADFEM_RANGE("adfem_mass_coo_backward_d");
  if (!mesh || !grad_vv_d || !grad_rho_d) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  return kerr(launch_gen_coo_backward(m, *sp, GenOp::MASS, grad_vv_d, grad_rho_d, S(stream)), "mass coo backward");
}

static int to_gauss_d(adfem_mesh* mesh, bool vertex_only, const double* u_d, double* out_d, void* stream) {
  if (!mesh || !u_d || !out_d) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  return kerr(launch_gen_to_gauss(m, *sp, vertex_only, u_d, out_d, S(stream)), "to gauss");
}

static int to_gauss_backward_d(adfem_mesh* mesh, bool vertex_only, const double* g_d, double* gu_d, long long nu,
                               int accumulate, void* stream) {
  if (!mesh || !g_d || !gu_d) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  const int64_t rows = vertex_only ? m.nv : sp->ndof;
  if (nu < rows) return fail(ADFEM_ERR_INVALID, "grad_u is shorter than the values it interpolates");
  ADFEM_TRY(kerr(launch_gen_to_gauss_backward(m, *sp, vertex_only, g_d, gu_d, accumulate != 0, S(stream)),
                 "to gauss backward"));
  if (!accumulate && nu > rows)
    ADFEM_CUDA(cudaMemsetAsync(gu_d + rows, 0, sizeof(double) * (size_t)(nu - rows), S(stream)));
  return ADFEM_OK;
}

int adfem_fem_to_gauss_d(adfem_mesh* mesh, const double* u_d, double* out_d, void* stream) {
  ADFEM_RANGE("adfem_fem_to_gauss_d");
  return to_gauss_d(mesh, true, u_d, out_d, stream);
}
int adfem_fem_to_gauss_backward_d(adfem_mesh* mesh, const double* grad_out_d, double* grad_u_d, long long nu,
                                  int accumulate, void* stream) {
  ADFEM_RANGE("adfem_fem_to_gauss_backward_d");
  return to_gauss_backward_d(mesh, true, grad_out_d, grad_u_d, nu, accumulate, stream);
}
int adfem_dof_to_gauss_d(adfem_mesh* mesh, const double* u_d, double* out_d, void* stream) {
  ADFEM_RANGE("adfem_dof_to_gauss_d");
  return to_gauss_d(mesh, false, u_d, out_d, stream);
}
int adfem_dof_to_gauss_backward_d(adfem_mesh* mesh, const double* grad_out_d, double* grad_u_d, long long nu,
                                  int accumulate, void* stream) {
  ADFEM_RANGE("adfem_dof_to_gauss_backward_d");
  return to_gauss_backward_d(mesh, false, grad_out_d, grad_u_d, nu, accumulate, stream);
}

static int to_gauss_host(adfem_mesh* mesh, bool vertex_only, const double* u, long long nu, double* out) {
  if (!mesh || !u || !out) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  if (nu < (vertex_only ? m.nv : sp->ndof)) return fail(ADFEM_ERR_INVALID, "u is shorter than the mesh's values");
  DevBuf du, dout;
  ADFEM_TRY(to_dev(du, u, (size_t)nu));
  ADFEM_TRY(dout.alloc(sizeof(double) * (size_t)mesh_ngauss(m)));
  ADFEM_TRY(to_gauss_d(mesh, vertex_only, du.as<double>(), dout.as<double>(), nullptr));
  return to_host(out, dout, (size_t)mesh_ngauss(m));
}

int adfem_fem_to_gauss(adfem_mesh* mesh, const double* u, long long nu, double* out) {
  ADFEM_RANGE("adfem_fem_to_gauss");
  return to_gauss_host(mesh, true, u, nu, out);
}
int adfem_dof_to_gauss(adfem_mesh* mesh, const double* u, long long nu, double* out) {
  ADFEM_RANGE("adfem_dof_to_gauss");
  return to_gauss_host(mesh, false, u, nu, out);
}

// ------------------------------------------------------------------ PCL Jacobians
// Values of the Laplace COO at kappa = 1 (nd^2 per Gauss point) in vv; the dense
// Jacobian holds them at (gp, nz) (FemLaplaceScalar.h:63-91).
static int pcl_laplace_values(Mesh& m, Space& sp, DevBuf& vv, int64_t* N, cudaStream_t st) {
  const int64_t ng = mesh_ngauss(m);
  *N = (int64_t)sp.nd * sp.nd * ng;
  DevBuf ones, idx;
  ADFEM_TRY(ones.alloc(sizeof(double) * (size_t)std::max<int64_t>(ng, 1)));
  ADFEM_TRY(idx.alloc(sizeof(long long) * 2 * (size_t)std::max<int64_t>(*N, 1)));
  ADFEM_TRY(vv.alloc(sizeof(double) * (size_t)std::max<int64_t>(*N, 1)));
  ADFEM_TRY(kerr(launch_fill(ng, 1.0, ones.as<double>(), st), "fill"));
  ADFEM_TRY(kerr(launch_gen_coo(m, sp, GenOp::LAPLACE, ones.as<double>(), idx.as<long long>(), vv.as<double>(), st),
                 "laplace coo"));
  ADFEM_CUDA(cudaStreamSynchronize(st));
  return ADFEM_OK;
}

int adfem_pcl_laplace_jacobian_d(adfem_mesh* mesh, double* H_d, void* stream) {
  ADFEM_RANGE("adfem_pcl_laplace_jacobian_d");
  if (!mesh || !H_d) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  DevBuf vv;
  int64_t N = 0;
  ADFEM_TRY(pcl_laplace_values(m, *sp, vv, &N, S(stream)));
  ADFEM_TRY(kerr(launch_pcl_scatter(N, sp->nd * sp->nd, mesh_ngauss(m), vv.as<double>(), H_d, S(stream)), "scatter"));
  ADFEM_CUDA(cudaStreamSynchronize(S(stream)));
  return ADFEM_OK;
}

int adfem_pcl_laplace_jacobian(adfem_mesh* mesh, double* H) {
  ADFEM_RANGE("adfem_pcl_laplace_jacobian");
  if (!mesh || !H) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  Space* sp = nullptr;
  ADFEM_TRY(get_space(m, m.degree, &sp));
  DevBuf vv;
  int64_t N = 0;
  ADFEM_TRY(pcl_laplace_values(m, *sp, vv, &N, nullptr));
  std::vector<double> v((size_t)N);
  ADFEM_TRY(to_host(v.data(), vv, (size_t)N));
  const int64_t ng = mesh_ngauss(m), nd2 = (int64_t)sp->nd * sp->nd;
  for (int64_t nz = 0; nz < N; nz++) H[nz / nd2 + nz * ng] = v[nz];  // only the nonzeros are written
  return ADFEM_OK;
}

int adfem_pcl_dirichlet(const long long* indices, long long sN, const long long* bd, long long nbd, long long N,
                        long long* pos, long long* nkeep) {
  ADFEM_RANGE("adfem_pcl_dirichlet");
  if (sN < 0 || N < 0 || !nkeep || (sN > 0 && (!indices || !pos)) || (nbd > 0 && !bd))
    return fail(ADFEM_ERR_INVALID, "bad arguments");
  std::vector<uint8_t> tag(std::max<long long>(N, 1), 0);
  for (long long q = 0; q < nbd; q++) {
    if (bd[q] < 1 || bd[q] > N) return fail(ADFEM_ERR_INVALID, "bd index out of range");
    tag[bd[q] - 1] = 1;
  }
  DevBuf di, isbd, dpos;
  ADFEM_TRY(to_dev(di, indices, 2 * (size_t)sN));
  ADFEM_TRY(to_dev(isbd, tag.data(), (size_t)std::max<long long>(N, 1)));
  ADFEM_TRY(dpos.alloc(sizeof(int64_t) * (size_t)std::max<long long>(sN, 1)));
  int64_t nk = 0;
  ADFEM_TRY(pcl_dirichlet_device(sN, di.as<long long>(), isbd.as<uint8_t>(), N, dpos.as<int64_t>(), &nk, nullptr));
  *nkeep = nk;
  return to_host(pos, dpos, (size_t)sN);
}

int adfem_mesh_elements(const adfem_mesh* mesh, long long* elems1) {
  ADFEM_RANGE("adfem_mesh_elements");
  if (!mesh || !elems1) return fail(ADFEM_ERR_INVALID, "null argument");
  for (int64_t k = 0; k < 3 * mesh->m->ne; k++) elems1[k] = (long long)mesh->m->elem[k] + 1;
  return ADFEM_OK;
}

int adfem_mesh_area(const adfem_mesh* mesh, double* area) {
  ADFEM_RANGE("adfem_mesh_area");
  if (!mesh || !area) return fail(ADFEM_ERR_INVALID, "null argument");
  std::memcpy(area, mesh->m->area.data(), sizeof(double) * mesh->m->ne);
  return ADFEM_OK;
}

int adfem_mesh_edges(const adfem_mesh* mesh, long long* out, long long* nedges) {
  ADFEM_RANGE("adfem_mesh_edges");
  if (!mesh || !nedges) return fail(ADFEM_ERR_INVALID, "null argument");
  ADFEM_TRY(mesh_edges(mesh->m));
  *nedges = mesh->m->nedges;
  if (out) std::memcpy(out, mesh->m->edges.data(), sizeof(long long) * 2 * mesh->m->nedges);
  return ADFEM_OK;
}

// ------------------------------------------------------------------ Laplace
int adfem_laplace_csr_d(adfem_mesh* mesh, const double* kappa_d, double* vals_d, void* stream) {
  ADFEM_RANGE("adfem_laplace_csr_d");
  if (!mesh || !kappa_d || !vals_d) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  if (Space* sp = p2_space(m)) return gen_matrix_d(m, *sp, GenOp::LAPLACE, kappa_d, vals_d, false, S(stream));
  std::lock_guard<std::mutex> lk(m.mu);
  ADFEM_TRY(m.s_el0.alloc(sizeof(double) * m.ne));
  ADFEM_TRY(kerr(launch_element_prepass(m, kappa_d, nullptr, m.s_el0.as<double>(), nullptr, S(stream)), "prepass"));
  ADFEM_TRY(kerr(launch_laplace_rows(m, m.s_el0.as<double>(), vals_d, Layout::CSR, S(stream)), "laplace rows"));
  ADFEM_CUDA(cudaStreamSynchronize(S(stream)));
  return ADFEM_OK;
}

int adfem_laplace_csc(adfem_mesh* mesh, const double* kappa, long long nkappa, double* nzval) {
  ADFEM_RANGE("adfem_laplace_csc");
  if (!mesh || !kappa || !nzval) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  if (m.degree == 2) return gen_matrix_host(mesh, 0, kappa, nkappa, nzval);
  if (nkappa != 3 * m.ne) return fail(ADFEM_ERR_INVALID, "kappa must have one value per Gauss point (3 per element)");
  DevBuf k, v;
  ADFEM_TRY(to_dev(k, kappa, (size_t)nkappa));
  ADFEM_TRY(v.alloc(sizeof(double) * (size_t)m.nnz));
  ADFEM_TRY(adfem_laplace_csr_d(mesh, k.as<double>(), v.as<double>(), nullptr));
  return to_host(nzval, v, (size_t)m.nnz);
}

int adfem_laplace_coo_d(adfem_mesh* mesh, const double* kappa_d, long long* indices_d, double* vv_d, void* stream) {
  ADFEM_RANGE("adfem_laplace_coo_d");
  if (!mesh || !kappa_d || !indices_d || !vv_d) return fail(ADFEM_ERR_INVALID, "null argument");
  if (Space* sp = p2_space(*mesh->m))
    return kerr(launch_gen_coo(*mesh->m, *sp, GenOp::LAPLACE, kappa_d, indices_d, vv_d, S(stream)), "laplace coo");
  ADFEM_TRY(kerr(launch_laplace_coo(*mesh->m, kappa_d, indices_d, vv_d, S(stream)), "laplace coo"));
  return ADFEM_OK;
}

int adfem_laplace_coo_backward_d(adfem_mesh* mesh, const double* grad_vv_d, double* grad_kappa_d, void* stream) {
  ADFEM_RANGE("adfem_laplace_coo_backward_d");
  if (!mesh || !grad_vv_d || !grad_kappa_d) return fail(ADFEM_ERR_INVALID, "null argument");
  if (Space* sp = p2_space(*mesh->m))
    return kerr(launch_gen_coo_backward(*mesh->m, *sp, GenOp::LAPLACE, grad_vv_d, grad_kappa_d, S(stream)),
                "laplace coo backward");
  ADFEM_TRY(kerr(launch_laplace_coo_backward(*mesh->m, grad_vv_d, grad_kappa_d, S(stream)), "laplace coo backward"));
  return ADFEM_OK;
}

// ------------------------------------------------------------------ source
int adfem_source_d(adfem_mesh* mesh, const double* f_d, double* rhs_d, int accumulate, void* stream) {
  ADFEM_RANGE("adfem_source_d");
  if (!mesh || !f_d || !rhs_d) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  if (Space* sp = p2_space(m)) {
    ADFEM_TRY(kerr(launch_gen_source(m, *sp, f_d, rhs_d, accumulate != 0, S(stream)), "source"));
    ADFEM_CUDA(cudaStreamSynchronize(S(stream)));
    return ADFEM_OK;
  }
  std::lock_guard<std::mutex> lk(m.mu);
  ADFEM_TRY(m.s_el1.alloc(sizeof(double) * 3 * m.ne));
  ADFEM_TRY(kerr(launch_element_prepass(m, nullptr, f_d, nullptr, m.s_el1.as<double>(), S(stream)), "prepass"));
  ADFEM_TRY(kerr(launch_source_rows(m, m.s_el1.as<double>(), rhs_d, accumulate != 0, S(stream)), "source rows"));
  ADFEM_CUDA(cudaStreamSynchronize(S(stream)));
  return ADFEM_OK;
}

int adfem_source(adfem_mesh* mesh, const double* f, long long nf, double* rhs, int accumulate) {
  ADFEM_RANGE("adfem_source");
  if (!mesh || !f || !rhs) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  if (nf != mesh_ngauss(m)) return fail(ADFEM_ERR_INVALID, "f must have one value per Gauss point");
  const size_t n = (size_t)mesh_ndof(&m);
  DevBuf fd, r;
  ADFEM_TRY(to_dev(fd, f, (size_t)nf));
  if (accumulate) ADFEM_TRY(to_dev(r, rhs, n));
  else ADFEM_TRY(r.alloc(sizeof(double) * n));
  ADFEM_TRY(adfem_source_d(mesh, fd.as<double>(), r.as<double>(), accumulate, nullptr));
  return to_host(rhs, r, n);
}

int adfem_source_backward_d(adfem_mesh* mesh, const double* grad_rhs_d, double* grad_f_d, void* stream) {
  ADFEM_RANGE("adfem_source_backward_d");
  if (!mesh || !grad_rhs_d || !grad_f_d) return fail(ADFEM_ERR_INVALID, "null argument");
  if (Space* sp = p2_space(*mesh->m))
    return kerr(launch_gen_source_backward(*mesh->m, *sp, grad_rhs_d, grad_f_d, S(stream)), "source backward");
  ADFEM_TRY(kerr(launch_source_backward(*mesh->m, grad_rhs_d, grad_f_d, S(stream)), "source backward"));
  return ADFEM_OK;
}

// ------------------------------------------------------------------ stiffness
int adfem_stiffness_csr_d(adfem_mesh* mesh, const double* D_d, double* vals_d, void* stream) {
  ADFEM_RANGE("adfem_stiffness_csr_d");
  if (!mesh || !D_d || !vals_d) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  if (Space* sp = p2_space(m)) return gen_stiffness_d(m, *sp, D_d, vals_d, false, S(stream));
  std::lock_guard<std::mutex> lk(m.mu);
  ADFEM_TRY(m.s_el0.alloc(sizeof(double) * 9 * m.ne));
  ADFEM_TRY(kerr(launch_stiffness_prepass(m, D_d, m.s_el0.as<double>(), S(stream)), "stiffness prepass"));
  ADFEM_TRY(kerr(launch_stiffness_rows(m, m.s_el0.as<double>(), vals_d, false, S(stream)), "stiffness rows"));
  ADFEM_CUDA(cudaStreamSynchronize(S(stream)));
  return ADFEM_OK;
}

int adfem_stiffness_csc(adfem_mesh* mesh, const double* D, long long nD, double* nzval) {
  ADFEM_RANGE("adfem_stiffness_csc");
  if (!mesh || !D || !nzval) return fail(ADFEM_ERR_INVALID, "null argument");
  Mesh& m = *mesh->m;
  if (m.degree == 2) return gen_matrix_host(mesh, 2, D, nD, nzval);
  if (nD != 27 * m.ne) return fail(ADFEM_ERR_INVALID, "D must hold a 3x3 matrix per Gauss point (27 per element)");
  DevBuf dd, v;
  ADFEM_TRY(to_dev(dd, D, (size_t)nD));
  ADFEM_TRY(v.alloc(sizeof(double) * 4 * (size_t)m.nnz));
  {
    std::lock_guard<std::mutex> lk(m.mu);
    ADFEM_TRY(m.s_el0.alloc(sizeof(double) * 9 * m.ne));
    ADFEM_TRY(kerr(launch_stiffness_prepass(m, dd.as<double>(), m.s_el0.as<double>(), nullptr), "stiffness prepass"));
    ADFEM_TRY(kerr(launch_stiffness_rows(m, m.s_el0.as<double>(), v.as<double>(), true, nullptr), "stiffness rows"));
  }
  return to_host(nzval, v, 4 * (size_t)m.nnz);
}

int adfem_stiffness_coo_d(adfem_mesh* mesh, const double* D_d, long long* indices_d, double* vv_d, void* stream) {
  ADFEM_RANGE("adfem_stiffness_coo_d");
  if (!mesh || !D_d || !indices_d || !vv_d) return fail(ADFEM_ERR_INVALID, "null argument");
  if (Space* sp = p2_space(*mesh->m))
    return kerr(launch_gen_stiffness_coo(*mesh->m, *sp, D_d, indices_d, vv_d, S(stream)), "stiffness coo");
  ADFEM_TRY(kerr(launch_stiffness_coo(*mesh->m, D_d, indices_d, vv_d, S(stream)), "stiffness coo"));
  return ADFEM_OK;
}

int adfem_stiffness_coo_backward_d(adfem_mesh* mesh, const double* grad_vv_d, double* grad_D_d, void* stream) {
  ADFEM_RANGE("adfem_stiffness_coo_backward_d");
  if (!mesh || !grad_vv_d || !grad_D_d) return fail(ADFEM_ERR_INVALID, "null argument");
  if (Space* sp = p2_space(*mesh->m))
    return kerr(launch_gen_stiffness_coo_backward(*mesh->m, *sp, grad_vv_d, grad_D_d, S(stream)),
                "stiffness coo backward");
  ADFEM_TRY(kerr(launch_stiffness_coo_backward(*mesh->m, grad_vv_d, grad_D_d, S(stream)), "stiffness coo backward"));
  return ADFEM_OK;
}

int adfem_plane_strain_d(int mode, long long n, const double* E_d, const double* nu_d, double* D_d, void* stream) {
  ADFEM_RANGE("adfem_plane_strain_d");
  if (mode != 0 && mode != 1) return fail(ADFEM_ERR_INVALID, "mode must be 0 (plane strain) or 1 (plane stress)");
  if (n < 0 || (n > 0 && (!E_d || !nu_d || !D_d))) return fail(ADFEM_ERR_INVALID, "bad arguments");
  if (n == 0) return ADFEM_OK;
  ADFEM_TRY(kerr(launch_plane_strain(mode, n, E_d, nu_d, D_d, S(stream)), "plane strain"));
  return ADFEM_OK;
}

int adfem_plane_strain_backward_d(int mode, long long n, const double* g_d, const double* E_d, const double* nu_d,
                                  double* gE_d, double* gnu_d, void* stream) {
  ADFEM_RANGE("adfem_plane_strain_backward_d");
  if (mode != 0 && mode != 1) return fail(ADFEM_ERR_INVALID, "mode must be 0 (plane strain) or 1 (plane stress)");
  if (n < 0 || (n > 0 && (!g_d || !E_d || !nu_d || !gE_d || !gnu_d))) return fail(ADFEM_ERR_INVALID, "bad arguments");
  if (n == 0) return ADFEM_OK;
  ADFEM_TRY(kerr(launch_plane_strain_backward(mode, n, g_d, E_d, nu_d, gE_d, gnu_d, S(stream)), "plane strain bwd"));
  return ADFEM_OK;
}

// ------------------------------------------------------------------ Dirichlet
// Validate a 1-based CSC matrix from the caller (monotone colptr, row ids in range) so
// that no kernel ever sees an index outside its arrays.
static int check_csc1(long long n, const long long* colptr1, const long long* rowval1) {
  if (colptr1[0] != 1) return fail(ADFEM_ERR_INVALID, "colptr[1] must be 1");
  for (long long j = 0; j < n; j++)
    if (colptr1[j + 1] < colptr1[j]) return fail(ADFEM_ERR_INVALID, "colptr is not monotone");
  const long long nnz = colptr1[n] - 1;
  for (long long k = 0; k < nnz; k++)
    if (rowval1[k] < 1 || rowval1[k] > n) return fail(ADFEM_ERR_INVALID, "row index out of range");
  return ADFEM_OK;
}

int adfem_dirichlet_csc(long long n, const long long* colptr1, const long long* rowval1, const double* nzval,
                        const double* rhs, const long long* bd, long long nbd, const double* bdval, int keep_zeros,
                        long long* out_colptr1, long long* out_rowval1, double* out_nzval, long long* out_nnz,
                        double* out_rhs) {
  ADFEM_RANGE("adfem_dirichlet_csc");
  if (n < 0 || !colptr1 || !out_nnz || (nbd > 0 && (!bd || !bdval))) return fail(ADFEM_ERR_INVALID, "bad arguments");
  const int64_t nnz = colptr1[n] - 1;
  if (nnz < 0 || (nnz > 0 && (!rowval1 || !nzval))) return fail(ADFEM_ERR_INVALID, "bad CSC arrays");
  ADFEM_TRY(check_csc1(n, colptr1, rowval1));
  std::vector<uint8_t> tag(std::max<long long>(n, 1), 0);
  for (long long k = 0; k < nbd; k++) {
    if (bd[k] < 1 || bd[k] > n) return fail(ADFEM_ERR_INVALID, "bd index " + std::to_string(bd[k]) + " out of range");
    if (tag[bd[k] - 1]) return fail(ADFEM_ERR_INVALID, "duplicate bd index " + std::to_string(bd[k]));
    tag[bd[k] - 1] = 1;
  }
  DevBuf cp1, cp0, rv1, rv0, nz, isbd, ocp, orv, onz;
  ADFEM_TRY(to_dev(cp1, colptr1, (size_t)n + 1));
  ADFEM_TRY(to_dev(rv1, rowval1, (size_t)nnz));
  ADFEM_TRY(to_dev(nz, nzval, (size_t)nnz));
  ADFEM_TRY(to_dev(isbd, tag.data(), (size_t)n));
  ADFEM_TRY(cp0.alloc(sizeof(int64_t) * (n + 1)));
  ADFEM_TRY(rv0.alloc(sizeof(int64_t) * std::max<int64_t>(nnz, 1)));
  ADFEM_TRY(kerr(launch_to0(n + 1, cp1.as<int64_t>(), cp0.as<int64_t>(), nullptr), "to0"));
  ADFEM_TRY(kerr(launch_to0(nnz, rv1.as<int64_t>(), rv0.as<int64_t>(), nullptr), "to0"));
  int64_t onn = 0;
  const bool count_only = (out_colptr1 == nullptr);
  ADFEM_TRY(dirichlet_csc_device(n, nnz, cp0.as<int64_t>(), rv0.as<int64_t>(), nz.as<double>(), isbd.as<uint8_t>(),
                                 keep_zeros, ocp, &onn, orv, onz, count_only, nullptr));
  *out_nnz = onn;
  if (count_only) return ADFEM_OK;
  if (!out_rowval1 || !out_nzval) return fail(ADFEM_ERR_INVALID, "null output arrays");
  ADFEM_TRY(kerr(launch_to1(n + 1, ocp.as<int64_t>(), ocp.as<int64_t>(), 1, nullptr), "to1"));
  ADFEM_TRY(to_host(out_colptr1, ocp, (size_t)n + 1));
  ADFEM_TRY(to_host(out_rowval1, orv, (size_t)onn));
  ADFEM_TRY(to_host(out_nzval, onz, (size_t)onn));
  if (out_rhs) {
    // r_I = rhs_I - A_IB bdval, the product accumulated column by column in bd order
    // (SparseMatrixCSC * Vector), r_B = bdval
    std::vector<double> acc(n, 0.0);
    for (long long k = 0; k < nbd; k++) {
      const int64_t j = bd[k] - 1;
      for (long long p = colptr1[j] - 1; p < colptr1[j + 1] - 1; p++) {
        const int64_t i = rowval1[p] - 1;
        if (!tag[i]) acc[i] += nzval[p] * bdval[k];
      }
    }
    for (long long i = 0; i < n; i++) out_rhs[i] = tag[i] ? 0.0 : rhs[i] - acc[i];
    for (long long k = 0; k < nbd; k++) out_rhs[bd[k] - 1] = bdval[k];
  }
  return ADFEM_OK;
}

// bd map with std::map semantics (sorted unique, last assignment wins)
static void bd_unique(const long long* bd, long long nbd, std::vector<std::pair<int64_t, int64_t>>& u) {
  u.clear();
  for (long long k = 0; k < nbd; k++) u.push_back({bd[k] - 1, k});
  std::stable_sort(u.begin(), u.end(), [](auto& a, auto& b) { return a.first < b.first; });
  std::vector<std::pair<int64_t, int64_t>> out;
  for (auto& p : u) {
    if (!out.empty() && out.back().first == p.first) out.back() = p;
    else out.push_back(p);
  }
  u.swap(out);
}

int adfem_dirichlet_coo(const long long* indices, const double* vv, long long sN, const long long* bd, long long nbd,
                        const double* rhs, const double* bdval, long long N, long long* oindices, double* ov,
                        double* orhs, long long* out_n) {
  ADFEM_RANGE("adfem_dirichlet_coo");
  if (sN < 0 || N < 0 || !out_n || (sN > 0 && (!indices || !vv)) || (nbd > 0 && (!bd || !bdval)))
    return fail(ADFEM_ERR_INVALID, "bad arguments");
  std::vector<std::pair<int64_t, int64_t>> u;
  bd_unique(bd, nbd, u);
  std::vector<uint8_t> tag(std::max<long long>(N, 1), 0);
  for (auto& p : u) {
    if (p.first < 0 || p.first >= N) return fail(ADFEM_ERR_INVALID, "bd index out of range");
    tag[p.first] = 1;
  }
  DevBuf di, dv, isbd, oidx, oval, liftk;
  ADFEM_TRY(to_dev(di, indices, 2 * (size_t)sN));
  ADFEM_TRY(to_dev(dv, vv, (size_t)sN));
  ADFEM_TRY(to_dev(isbd, tag.data(), (size_t)N));
  int64_t nkeep = 0, nlift = 0;
  const bool count_only = (oindices == nullptr);
  ADFEM_TRY(dirichlet_coo_device(sN, di.as<long long>(), dv.as<double>(), isbd.as<uint8_t>(), N, &nkeep, oidx, oval,
                                 &nlift, liftk, count_only, nullptr));
  *out_n = nkeep + (long long)u.size();
  if (count_only) return ADFEM_OK;
  if (!ov) return fail(ADFEM_ERR_INVALID, "null output values");
  ADFEM_TRY(to_host(oindices, oidx, 2 * (size_t)nkeep));
  ADFEM_TRY(to_host(ov, oval, (size_t)nkeep));
  for (size_t q = 0; q < u.size(); q++) {
    oindices[2 * (nkeep + q)] = u[q].first;
    oindices[2 * (nkeep + q) + 1] = u[q].first;
    ov[nkeep + q] = 1.0;
  }
  if (orhs) {
    std::vector<int64_t> lk(nlift);
    ADFEM_TRY(to_host(lk.data(), liftk, (size_t)nlift));
    std::vector<int64_t> pos(N, -1);
    for (auto& p : u) pos[p.first] = p.second;
    for (long long i = 0; i < N; i++) orhs[i] = rhs[i];
    for (int64_t k : lk) {  // ascending entry order, as ImposeDirichlet.h:41-43
      const int64_t i = indices[2 * k], j = indices[2 * k + 1];
      orhs[i] = orhs[i] - vv[k] * bdval[pos[j]];
    }
    for (auto& p : u) orhs[p.first] = bdval[p.second];
  }
  return ADFEM_OK;
}

int adfem_dirichlet_coo_backward(const double* grad_vv, const double* grad_rhs, const long long* indices,
                                 const double* vv, long long sN, const long long* bd, long long nbd,
                                 const double* bdval, long long N, double* grad_vv_in, double* grad_rhs_in,
                                 double* grad_bdval) {
  ADFEM_RANGE("adfem_dirichlet_coo_backward");
  if (sN < 0 || N < 0 || (sN > 0 && (!indices || !vv || !grad_vv_in)) || !grad_rhs || !grad_rhs_in ||
      (nbd > 0 && (!bd || !bdval || !grad_bdval)))
    return fail(ADFEM_ERR_INVALID, "bad arguments");
  std::vector<std::pair<int64_t, int64_t>> u;
  bd_unique(bd, nbd, u);
  std::vector<uint8_t> tag(std::max<long long>(N, 1), 0);
  std::vector<double> bdd(std::max<long long>(N, 1), 0.0);
  std::vector<int64_t> pos(std::max<long long>(N, 1), -1);
  for (auto& p : u) {
    if (p.first < 0 || p.first >= N) return fail(ADFEM_ERR_INVALID, "bd index out of range");
    tag[p.first] = 1;
    bdd[p.first] = bdval[p.second];
    pos[p.first] = p.second;
  }
  // number of kept entries = length of grad_vv
  DevBuf di, dv, isbd, gv, gr, bdv, gin, oidx, oval, liftk;
  ADFEM_TRY(to_dev(di, indices, 2 * (size_t)sN));
  ADFEM_TRY(to_dev(dv, vv, (size_t)sN));
  ADFEM_TRY(to_dev(isbd, tag.data(), (size_t)N));
  int64_t nkeep = 0, nlift = 0;
  ADFEM_TRY(dirichlet_coo_device(sN, di.as<long long>(), dv.as<double>(), isbd.as<uint8_t>(), N, &nkeep, oidx, oval,
                                 &nlift, liftk, false, nullptr));
  ADFEM_TRY(to_dev(gv, grad_vv, (size_t)nkeep));
  ADFEM_TRY(to_dev(gr, grad_rhs, (size_t)N));
  ADFEM_TRY(to_dev(bdv, bdd.data(), (size_t)N));
  ADFEM_TRY(gin.alloc(sizeof(double) * std::max<int64_t>(sN, 1)));
  ADFEM_TRY(dirichlet_coo_backward_device(sN, di.as<long long>(), isbd.as<uint8_t>(), N, gv.as<double>(),
                                          bdv.as<double>(), gr.as<double>(), gin.as<double>(), nullptr));
  ADFEM_TRY(to_host(grad_vv_in, gin, (size_t)sN));
  std::vector<int64_t> lk(nlift);
  ADFEM_TRY(to_host(lk.data(), liftk, (size_t)nlift));
  for (long long b = 0; b < nbd; b++) grad_bdval[b] = 0.0;
  for (int64_t k : lk) {  // ImposeDirichlet.h:79-83, entry order
    const int64_t i = indices[2 * k], j = indices[2 * k + 1];
    grad_bdval[pos[j]] -= vv[k] * grad_rhs[i];
  }
  for (long long i = 0; i < N; i++) grad_rhs_in[i] = tag[i] ? 0.0 : grad_rhs[i];
  for (auto& p : u) grad_bdval[p.second] += grad_rhs[p.first];
  return ADFEM_OK;
}

// ------------------------------------------------------------------ solves
void adfem_solver_opts_default(adfem_solver_opts* o) {
  if (!o) return;
  o->rtol = 1e-12;
  o->max_iter = 200000;
  o->precision = ADFEM_PREC_FP64;
  o->ru_delta = 0.1;
  o->chunk = 32;
  o->warm_start = 0;
}

// K\F by CG is only right for a symmetric K: the CSC arrays are read as CSR (which is
// the transpose), and CG on a non-symmetric operator has no meaning.  The reference's
// direct solve accepts any nonsingular K, so a non-symmetric one is refused here rather
// than solved wrongly.  Entries present on one side only must be (numerically) zero;
// matched pairs must agree to 1e-12 relative (or 1e-15 of the larger diagonal).
// rp/ci: 0-based CSR of K^T (the CSC arrays of K); returns ADFEM_OK or a refusal.
static int check_symmetric(int64_t n, const std::vector<int32_t>& rp, const std::vector<int32_t>& ci,
                           const double* val) {
  const int64_t nnz = rp[n];
  // transpose by counting sort: rows of K (sorted columns, since rows are visited in order)
  std::vector<int32_t> tp(n + 2, 0), tc(std::max<int64_t>(nnz, 1));
  std::vector<double> tv(std::max<int64_t>(nnz, 1));
  for (int64_t k = 0; k < nnz; k++) tp[ci[k] + 2]++;
  for (int64_t i = 0; i < n; i++) tp[i + 2] += tp[i + 1];
  for (int64_t r = 0; r < n; r++)
    for (int32_t k = rp[r]; k < rp[r + 1]; k++) {
      const int32_t t = tp[ci[k] + 1]++;
      tc[t] = (int32_t)r;
      tv[t] = val[k];
    }
  std::vector<double> diag(n, 0.0);
  for (int64_t r = 0; r < n; r++)
    for (int32_t k = rp[r]; k < rp[r + 1]; k++)
      if (ci[k] == r) diag[r] += std::fabs(val[k]);
  std::vector<std::pair<int32_t, double>> row;
  for (int64_t r = 0; r < n; r++) {
    row.clear();
    for (int32_t k = rp[r]; k < rp[r + 1]; k++) row.emplace_back(ci[k], val[k]);
    std::stable_sort(row.begin(), row.end(),
                     [](const std::pair<int32_t, double>& a, const std::pair<int32_t, double>& b) {
                       return a.first < b.first;
                     });
    // duplicates within a row (unsorted, repeated row indices in a column) are summed
    size_t m = 0;
    for (size_t q = 0; q < row.size(); q++) {
      if (m > 0 && row[m - 1].first == row[q].first) row[m - 1].second += row[q].second;
      else row[m++] = row[q];
    }
    row.resize(m);
    size_t a = 0;
    int32_t b = tp[r];
    const int32_t be = tp[r + 1];
    while (a < row.size() || b < be) {
      const int32_t ca = a < row.size() ? row[a].first : INT32_MAX;
      const int32_t cb = b < be ? tc[b] : INT32_MAX;
      const int32_t c = std::min(ca, cb);
      double x = 0.0, y = 0.0;
      if (ca == c) x = row[a++].second;
      while (b < be && tc[b] == c) y += tv[b++];
      const double d = std::fabs(x - y);
      const double scale = std::max(std::fabs(x), std::fabs(y));
      if (d > 1e-12 * scale && d > 1e-15 * std::max(diag[r], diag[c]))
        return fail(ADFEM_ERR_UNSUPPORTED,
                    "K\\F by CG needs a symmetric K: entries (" + std::to_string(r + 1) + ", " +
                        std::to_string(c + 1) + ") and (" + std::to_string(c + 1) + ", " + std::to_string(r + 1) +
                        ") differ");
    }
  }
  return ADFEM_OK;
}

int adfem_csc_solve(long long n, const long long* colptr1, const long long* rowval1, const double* nzval,
                    const double* rhs, double* u, const adfem_solver_opts* opts, adfem_solver_stats* stats) {
  ADFEM_RANGE("adfem_csc_solve");
  if (n <= 0 || !colptr1 || !rowval1 || !nzval || !rhs || !u) return fail(ADFEM_ERR_INVALID, "bad arguments");
  if (n > INT32_MAX) return fail(ADFEM_ERR_UNSUPPORTED, "n > 2^31");
  adfem_solver_opts o;
  adfem_solver_opts_default(&o);
  if (opts) o = *opts;
  ADFEM_TRY(check_csc1(n, colptr1, rowval1));
  const int64_t nnz = colptr1[n] - 1;
  if (nnz > INT32_MAX) return fail(ADFEM_ERR_UNSUPPORTED, "nnz > 2^31");
  // a symmetric matrix's CSC arrays are its CSR arrays
  std::vector<int32_t> rp(n + 1), ci(std::max<int64_t>(nnz, 1)), dp(n, 0);
  for (long long i = 0; i <= n; i++) rp[i] = (int32_t)(colptr1[i] - 1);
  for (int64_t k = 0; k < nnz; k++) {
    const long long c = rowval1[k] - 1;
    if (c < 0 || c >= n) return fail(ADFEM_ERR_INVALID, "row index out of range");
    ci[k] = (int32_t)c;
  }
  ADFEM_TRY(check_symmetric(n, rp, ci, nzval));
  for (long long i = 0; i < n; i++) {
    int found = -1;
    for (int32_t k = rp[i]; k < rp[i + 1]; k++)
      if (ci[k] == i) found = k - rp[i];
    if (found < 0) return fail(ADFEM_ERR_INVALID, "column " + std::to_string(i + 1) + " has no stored diagonal");
    dp[i] = found;
  }
  Sell A;
  ADFEM_TRY(sell_build_pattern(n, rp.data(), ci.data(), A, 1));
  ADFEM_TRY(A.val64.alloc(sizeof(double) * std::max<int64_t>(A.nent, 1)));
  ADFEM_TRY(A.val32.alloc(sizeof(float) * std::max<int64_t>(A.nent, 1)));
  ADFEM_TRY(A.valD64.alloc(sizeof(double) * std::max<int64_t>(A.nent, 1)));
  ADFEM_CUDA(cudaMemset(A.val64.p, 0, sizeof(double) * std::max<int64_t>(A.nent, 1)));
  DevBuf drp, dvals, ddp, db, du;
  ADFEM_TRY(to_dev(drp, rp.data(), rp.size()));
  ADFEM_TRY(to_dev(dvals, nzval, (size_t)nnz));
  ADFEM_TRY(to_dev(ddp, dp.data(), dp.size()));
  ADFEM_TRY(to_dev(db, rhs, (size_t)n));
  if (o.warm_start) ADFEM_TRY(to_dev(du, u, (size_t)n));
  else ADFEM_TRY(du.alloc(sizeof(double) * n));
  ADFEM_TRY(kerr(launch_csr_to_sell(A, n, drp.as<int32_t>(), dvals.as<double>(), A.val64.as<double>(), nullptr),
                 "csr to sell"));
  Solver sv;
  ADFEM_TRY(sv.init(&A, n));
  ADFEM_TRY(solver_prepare(sv, ddp.as<int32_t>(), nullptr));
  const int st = solver_solve(sv, db.as<double>(), du.as<double>(), nullptr, nullptr, nullptr, o, stats, nullptr);
  if (st != ADFEM_OK && st != ADFEM_ERR_NOT_CONVERGED) return st;
  ADFEM_TRY(to_host(u, du, (size_t)n));
  return st;
}

// ------------------------------------------------------------------ systems
int adfem_system_create(adfem_mesh* mesh, int kind, adfem_system** out) {
  ADFEM_RANGE("adfem_system_create");
  if (!mesh || !out) return fail(ADFEM_ERR_INVALID, "null argument");
  if (kind != ADFEM_SYS_POISSON && kind != ADFEM_SYS_ELASTICITY) return fail(ADFEM_ERR_INVALID, "unknown kind");
  *out = nullptr;
  std::unique_ptr<adfem_system> s(new adfem_system());
  s->mesh = mesh;
  s->kind = kind;
  Mesh& m = *mesh->m;
  const bool p2 = m.degree == 2;
  if (p2 && kind != ADFEM_SYS_POISSON)
    return fail(ADFEM_ERR_UNSUPPORTED, "resident elasticity systems are built on P1 meshes (assemble P2 "
                                       "stiffness operators and use adfem_csc_solve)");
  if (kind == ADFEM_SYS_ELASTICITY && m.maxrow > 16)
    return fail(ADFEM_ERR_UNSUPPORTED, "elasticity systems support at most 15 neighbours per node");
  // the scalar pattern the operator lives on: the mesh's (P1, one DOF per node) or that of
  // the P2 space (vertex DOFs, then one per edge)
  Space* sp = nullptr;
  if (p2) {
    std::lock_guard<std::mutex> lk(m.mu);
    ADFEM_TRY(mesh_space(&m, 2, &sp));
    // (rows of up to 24 entries take the banded mixed iteration, longer ones the scaled one)
    if (sp->maxrow > 32) return fail(ADFEM_ERR_UNSUPPORTED, "P2 systems support at most 32 entries per row");
  }
  const int64_t nn = p2 ? sp->ndof : m.nv;
  const std::vector<int32_t>& RP = p2 ? sp->rowptr : m.rowptr;
  const std::vector<int32_t>& CI = p2 ? sp->colind : m.colind;
  int64_t band0 = m.sell.band;
  if (p2) {
    band0 = 0;
    for (int64_t i = 0; i < nn; i++)
      for (int32_t k = RP[i]; k < RP[i + 1]; k++) band0 = std::max<int64_t>(band0, std::llabs((long long)CI[k] - i));
  }
  // DOF numbering of the solver: reverse Cuthill-McKee when it at least halves the band
  // (not tried when the band is already within 4 sqrt(n), about what RCM reaches on a
  // planar mesh; the P2 numbering -- vertices, then edges -- always has a wide band)
  {
    std::vector<int32_t> pi;
    const bool try_rcm = (double)band0 > 4.0 * std::sqrt((double)nn);
    const int64_t rb = try_rcm ? graph_rcm(nn, RP, CI, pi) : band0;
    s->renumbered = try_rcm && 2 * rb < band0;
    if (s->renumbered) s->hperm = std::move(pi);
    else {
      s->hperm.resize(nn);
      for (int64_t i = 0; i < nn; i++) s->hperm[i] = (int32_t)i;
    }
    if (p2) {
      // P2 rows come in two lengths (19 entries for a vertex DOF of valence 6, 9 for an edge
      // DOF): within each window of kGroup consecutive solver rows, rows are reordered by
      // decreasing length (stable), so that most 32-row slices hold rows of one length and
      // the sliced layout stores ~12 instead of 19 entries per row; the band grows by at most
      // the window
      constexpr int64_t kGroup = 256;
      std::vector<int32_t> ord(nn);  // solver row -> DOF
      for (int64_t i = 0; i < nn; i++) ord[s->hperm[i]] = (int32_t)i;
      auto len = [&](int32_t d) { return RP[d + 1] - RP[d]; };
      for (int64_t q0 = 0; q0 < nn; q0 += kGroup) {
        const int64_t q1 = std::min(nn, q0 + kGroup);
        std::stable_sort(ord.begin() + q0, ord.begin() + q1, [&](int32_t a, int32_t b) { return len(a) > len(b); });
      }
      bool ident = true;
      for (int64_t q = 0; q < nn; q++) {
        s->hperm[ord[q]] = (int32_t)q;
        ident &= ord[q] == q;
      }
      s->renumbered = !ident;
    }
  }
  const std::vector<int32_t>& pi = s->hperm;
  // scalar pattern in solver order: row pi(i) holds the sorted pi(j); kp = rank of each
  // pattern slot in its renumbered row
  const int64_t nnzS = (int64_t)CI.size();
  std::vector<int32_t> rpS(nn + 1, 0), ciS(nnzS), dpS(nn), dpRef(nn, 0);
  std::vector<uint8_t> kp(nnzS);
  {
    std::vector<int32_t> inv(nn);
    for (int64_t i = 0; i < nn; i++) inv[pi[i]] = (int32_t)i;
    for (int64_t r = 0; r < nn; r++) rpS[r + 1] = rpS[r] + (RP[inv[r] + 1] - RP[inv[r]]);
    std::vector<std::pair<int32_t, int32_t>> tmp;
    for (int64_t i = 0; i < nn; i++) {
      tmp.clear();
      for (int32_t k = RP[i]; k < RP[i + 1]; k++) {
        tmp.emplace_back(pi[CI[k]], k - RP[i]);
        if (CI[k] == i) dpRef[i] = k - RP[i];
      }
      std::sort(tmp.begin(), tmp.end());
      const int64_t r = pi[i];
      for (size_t q = 0; q < tmp.size(); q++) {
        ciS[rpS[r] + q] = tmp[q].first;
        kp[RP[i] + tmp[q].second] = (uint8_t)q;
        if (tmp[q].first == r) dpS[r] = (int32_t)q;
      }
    }
  }
  if (kind == ADFEM_SYS_POISSON) {
    s->ndof = nn;
    const char* penv = std::getenv("ADFEM_ASM_PAIRS");
    s->pairs = !p2 && m.maxrow <= 16 && penv && penv[0] == '1';
    ADFEM_TRY(sell_build_pattern(nn, rpS.data(), ciS.data(), s->A, 1));
    ADFEM_TRY(to_dev(s->diagpos, dpS.data(), dpS.size()));
    if (s->renumbered) ADFEM_TRY(to_dev(s->dofmap, pi.data(), pi.size()));
    if (p2) ADFEM_TRY(to_dev(s->sdiag, dpRef.data(), dpRef.size()));
  } else {
    s->ndof = 2 * m.nv;
    std::vector<int32_t> rp2(2 * m.nv + 1, 0), dp2(2 * m.nv);
    for (int64_t r = 0; r < 2 * m.nv; r++) {
      const int64_t i = r >> 1;
      rp2[r + 1] = rp2[r] + 2 * (rpS[i + 1] - rpS[i]);
      dp2[r] = 2 * dpS[i] + (int32_t)(r & 1);
    }
    std::vector<int32_t> ci2(rp2[2 * m.nv]);
    for (int64_t r = 0; r < 2 * m.nv; r++) {
      const int64_t i = r >> 1;
      int32_t z = rp2[r];
      for (int32_t k = rpS[i]; k < rpS[i + 1]; k++) {
        ci2[z++] = 2 * ciS[k];
        ci2[z++] = 2 * ciS[k] + 1;
      }
    }
    ADFEM_TRY(sell_build_pattern(2 * m.nv, rp2.data(), ci2.data(), s->A, 2));
    ADFEM_TRY(to_dev(s->diagpos, dp2.data(), dp2.size()));
    std::vector<int32_t> map(2 * m.nv);
    for (int64_t i = 0; i < m.nv; i++) {
      map[i] = 2 * pi[i];
      map[m.nv + i] = 2 * pi[i] + 1;
    }
    ADFEM_TRY(to_dev(s->dofmap, map.data(), map.size()));
  }
  if (s->renumbered) {
    ADFEM_TRY(to_dev(s->nperm, pi.data(), pi.size()));
    ADFEM_TRY(to_dev(s->kperm, kp.data(), kp.size()));
  }
  const size_t ne = std::max<int64_t>(s->A.nent, 1);
  ADFEM_TRY(s->A.val64.alloc(sizeof(double) * ne));
  ADFEM_TRY(s->A.val32.alloc(sizeof(float) * ne));
  ADFEM_TRY(s->A.valD64.alloc(sizeof(double) * ne));
  ADFEM_CUDA(cudaMemset(s->A.val64.p, 0, sizeof(double) * ne));
  ADFEM_CUDA(cudaMemset(s->A.val32.p, 0, sizeof(float) * ne));
  ADFEM_TRY(s->rhs.alloc(sizeof(double) * s->ndof));
  ADFEM_TRY(s->t0.alloc(sizeof(double) * s->ndof));
  ADFEM_TRY(s->t1.alloc(sizeof(double) * s->ndof));
  ADFEM_TRY(s->t2.alloc(sizeof(double) * s->ndof));
  ADFEM_TRY(s->solver.init(&s->A, s->ndof));
  ADFEM_TRY(system_set_bd(s.get(), nullptr, 0, nullptr));
  *out = s.release();
  return ADFEM_OK;
}

int adfem_system_destroy(adfem_system* sys) {
  ADFEM_RANGE("adfem_system_destroy");
  delete sys;
  return ADFEM_OK;
}

int adfem_system_set_dirichlet(adfem_system* sys, const long long* bd, long long nbd, const double* bdval) {
  ADFEM_RANGE("adfem_system_set_dirichlet");
  if (!sys || nbd < 0 || (nbd > 0 && !bd)) return fail(ADFEM_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(sys->mu);
  return system_set_bd(sys, bd, nbd, bdval);
}

// Poisson assembly: element pass (sigma, element loads), fused Laplace + load + Dirichlet
// rows into the sliced-ELL operator, operator conversion for the solver.  ev: optional
// four events recorded around the three phases.
static int assemble_poisson(adfem_system* sys, const double* kappa_d, const double* f_d, cudaStream_t st,
                            cudaEvent_t* ev) {
  Mesh& m = *sys->mesh->m;
  sys->assembled = false;
  if (m.degree == 2) {
    // P2: element matrices of the order-4 rule, then one pass over the DOF rows (Laplace
    // row + load + Dirichlet into the sliced-ELL operator)
    const Space& sp = *m.space[2];
    ADFEM_TRY(sys->ke.alloc(sizeof(double) * 36 * (size_t)m.ne));
    if (ev) ADFEM_CUDA(cudaEventRecord(ev[0], st));
    if (ev) ADFEM_CUDA(cudaEventRecord(ev[1], st));
    ADFEM_TRY(kerr(launch_gen_poisson_system(m, sp, kappa_d, f_d, sys->ke.as<double>(), sys->isbd.as<uint8_t>(),
                                             sys->bdval.as<double>(), sys->A.val64.as<double>(),
                                             sys->rhs.as<double>(), sys->A.sptr.as<int32_t>(),
                                             sys->sdiag.as<int32_t>(),
                                             sys->renumbered ? sys->nperm.as<int32_t>() : nullptr,
                                             sys->renumbered ? sys->kperm.as<uint8_t>() : nullptr, st),
                   "P2 poisson system"));
    if (ev) ADFEM_CUDA(cudaEventRecord(ev[2], st));
    ADFEM_TRY(solver_prepare(sys->solver, sys->diagpos.as<int32_t>(), st));
    if (ev) ADFEM_CUDA(cudaEventRecord(ev[3], st));
    sys->assembled = true;
    return ADFEM_OK;
  }
  if (sys->pairs) {
    // FP32-pair arithmetic: element pass (sigma and load terms as pairs, 32 B per element),
    // then the rows
    ADFEM_TRY(mesh_geo_pairs(m));
    ADFEM_TRY(sys->sigma.alloc(sizeof(float2) * m.ne));
    ADFEM_TRY(sys->src3.alloc(sizeof(float2) * 3 * m.ne));
    if (ev) ADFEM_CUDA(cudaEventRecord(ev[0], st));
    ADFEM_TRY(kerr(launch_element_prepass_pairs(m, kappa_d, f_d, sys->sigma.as<float2>(), sys->src3.as<float2>(), st),
                   "element prepass (pairs)"));
    if (ev) ADFEM_CUDA(cudaEventRecord(ev[1], st));
    ADFEM_TRY(kerr(launch_poisson_system_pairs(m, sys->sigma.as<float2>(), sys->src3.as<float2>(),
                                               sys->isbd.as<uint8_t>(), sys->bdval.as<double>(),
                                               sys->A.val64.as<double>(), sys->rhs.as<double>(),
                                               sys->A.sptr.as<int32_t>(), m.d_diagpos.as<int32_t>(),
                                               sys->renumbered ? sys->nperm.as<int32_t>() : nullptr,
                                               sys->renumbered ? sys->kperm.as<uint8_t>() : nullptr, st),
                   "poisson system (pairs)"));
  } else {
    ADFEM_TRY(sys->sigma.alloc(sizeof(double) * m.ne));
    ADFEM_TRY(sys->src3.alloc(sizeof(double) * 3 * m.ne));
    if (ev) ADFEM_CUDA(cudaEventRecord(ev[0], st));
    ADFEM_TRY(kerr(launch_element_prepass_unweighted(m, kappa_d, f_d, sys->sigma.as<double>(),
                                                     sys->src3.as<double>(), st),
                   "element prepass"));
    if (ev) ADFEM_CUDA(cudaEventRecord(ev[1], st));
    ADFEM_TRY(kerr(launch_poisson_system(m, sys->sigma.as<double>(), sys->src3.as<double>(),
                                         sys->isbd.as<uint8_t>(), sys->bdval.as<double>(), sys->A.val64.as<double>(),
                                         sys->rhs.as<double>(), sys->A.sptr.as<int32_t>(), m.d_diagpos.as<int32_t>(),
                                         sys->renumbered ? sys->nperm.as<int32_t>() : nullptr,
                                         sys->renumbered ? sys->kperm.as<uint8_t>() : nullptr, st),
                   "poisson system"));
  }
  if (ev) ADFEM_CUDA(cudaEventRecord(ev[2], st));
  ADFEM_TRY(solver_prepare(sys->solver, sys->diagpos.as<int32_t>(), st));
  if (ev) ADFEM_CUDA(cudaEventRecord(ev[3], st));
  sys->assembled = true;
  return ADFEM_OK;
}

int adfem_system_assemble_poisson_d(adfem_system* sys, const double* kappa_d, const double* f_d, void* stream) {
  ADFEM_RANGE("adfem_system_assemble_poisson_d");
  if (!sys || !kappa_d || !f_d) return fail(ADFEM_ERR_INVALID, "null argument");
  if (sys->kind != ADFEM_SYS_POISSON) return fail(ADFEM_ERR_INVALID, "not a Poisson system");
  std::lock_guard<std::mutex> lk(sys->mu);
  return assemble_poisson(sys, kappa_d, f_d, S(stream), nullptr);
}

int adfem_system_assemble_poisson_profiled_d(adfem_system* sys, const double* kappa_d, const double* f_d, double* ms,
                                             void* stream) {
  ADFEM_RANGE("adfem_system_assemble_poisson_profiled_d");
  if (!sys || !kappa_d || !f_d || !ms) return fail(ADFEM_ERR_INVALID, "null argument");
  if (sys->kind != ADFEM_SYS_POISSON) return fail(ADFEM_ERR_INVALID, "not a Poisson system");
  std::lock_guard<std::mutex> lk(sys->mu);
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  for (auto& e : ev) ADFEM_CUDA(cudaEventCreate(&e));
  const int r = assemble_poisson(sys, kappa_d, f_d, S(stream), ev);
  if (r == ADFEM_OK) {
    cudaEventSynchronize(ev[3]);
    for (int k = 0; k < 3; k++) {
      float t = 0.0f;
      cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      ms[k] = t;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return r;
}

int adfem_system_assemble_elasticity_d(adfem_system* sys, const double* E_d, const double* nu_d, const double* fx_d,
                                       const double* fy_d, void* stream) {
  ADFEM_RANGE("adfem_system_assemble_elasticity_d");
  if (!sys || !E_d || !nu_d || !fx_d || !fy_d) return fail(ADFEM_ERR_INVALID, "null argument");
  if (sys->kind != ADFEM_SYS_ELASTICITY) return fail(ADFEM_ERR_INVALID, "not an elasticity system");
  std::lock_guard<std::mutex> lk(sys->mu);
  Mesh& m = *sys->mesh->m;
  cudaStream_t st = S(stream);
  sys->assembled = false;
  ADFEM_TRY(sys->Dbar.alloc(sizeof(double) * 9 * m.ne));
  ADFEM_TRY(sys->src3.alloc(sizeof(double) * 3 * m.ne));
  ADFEM_TRY(sys->srcy3.alloc(sizeof(double) * 3 * m.ne));
  ADFEM_TRY(kerr(launch_stiffness_prepass_E(m, E_d, nu_d, sys->Dbar.as<double>(), st), "stiffness prepass"));
  ADFEM_TRY(kerr(launch_element_prepass(m, nullptr, fx_d, nullptr, sys->src3.as<double>(), st), "prepass fx"));
  ADFEM_TRY(kerr(launch_element_prepass(m, nullptr, fy_d, nullptr, sys->srcy3.as<double>(), st), "prepass fy"));
  ADFEM_TRY(kerr(launch_elastic_system(m, sys->Dbar.as<double>(), sys->src3.as<double>(), sys->srcy3.as<double>(),
                                       sys->A.sptr.as<int32_t>(), sys->isbd.as<uint8_t>(), sys->bdval.as<double>(),
                                       sys->A.val64.as<double>(), sys->rhs.as<double>(),
                                       sys->renumbered ? sys->nperm.as<int32_t>() : nullptr,
                                       sys->renumbered ? sys->kperm.as<uint8_t>() : nullptr, st),
                 "elastic system"));
  ADFEM_TRY(solver_prepare(sys->solver, sys->diagpos.as<int32_t>(), st));
  sys->assembled = true;
  return ADFEM_OK;
}

int adfem_system_solve_d(adfem_system* sys, double* u_d, const adfem_solver_opts* opts, adfem_solver_stats* stats,
                         void* stream) {
  ADFEM_RANGE("adfem_system_solve_d");
  if (!sys || !u_d) return fail(ADFEM_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(sys->mu);
  if (!sys->assembled) return fail(ADFEM_ERR_INVALID, "system not assembled");
  adfem_solver_opts o;
  adfem_solver_opts_default(&o);
  if (opts) o = *opts;
  cudaStream_t st = S(stream);
  if (!mapped(sys))
    return solver_solve(sys->solver, sys->rhs.as<double>(), u_d, nullptr, sys->isbd.as<uint8_t>(),
                        sys->bdval.as<double>(), o, stats, st);
  if (o.warm_start) ADFEM_TRY(to_solver(sys, u_d, sys->t0.as<double>(), st));
  const int r = solver_solve(sys->solver, sys->rhs.as<double>(), sys->t0.as<double>(), nullptr,
                             sys->isbd.as<uint8_t>(), sys->bdval.as<double>(), o, stats, st);
  if (r != ADFEM_OK && r != ADFEM_ERR_NOT_CONVERGED) return r;
  ADFEM_TRY(from_solver(sys, sys->t0.as<double>(), u_d, st));
  return r;
}

int adfem_system_solve_profiled_d(adfem_system* sys, double* u_d, const adfem_solver_opts* opts,
                                  adfem_solver_stats* stats, double* kernel_ms, long long* launches, void* stream) {
  ADFEM_RANGE("adfem_system_solve_profiled_d");
  if (!sys || !u_d || !kernel_ms || !launches) return fail(ADFEM_ERR_INVALID, "null argument");
  if (sys->kind != ADFEM_SYS_POISSON) return fail(ADFEM_ERR_UNSUPPORTED, "profiled solves are for Poisson systems");
  std::lock_guard<std::mutex> lk(sys->mu);
  if (!sys->assembled) return fail(ADFEM_ERR_INVALID, "system not assembled");
  adfem_solver_opts o;
  adfem_solver_opts_default(&o);
  if (opts) o = *opts;
  SolveProfile prof;
  const int r = solver_solve(sys->solver, sys->rhs.as<double>(), u_d, nullptr, sys->isbd.as<uint8_t>(),
                             sys->bdval.as<double>(), o, stats, S(stream), &prof);
  for (int j = 0; j < 4; j++) {
    kernel_ms[j] = prof.ms[j];
    launches[j] = prof.n[j];
  }
  return r;
}

int adfem_system_solver_info(const adfem_system* sys, adfem_solver_info* info) {
  ADFEM_RANGE("adfem_system_solver_info");
  if (!sys || !info) return fail(ADFEM_ERR_INVALID, "null argument");
  const Sell& A = sys->A;
  const Solver& sv = sys->solver;
  info->rows = A.n;
  info->stored = A.nent;
  info->uniform_entries = A.uniform_entries;
  info->slices = A.nslices;
  info->band = A.band;
  info->banded = sv.zcg ? 1 : 0;
  info->blocks = sv.zcg ? sv.zgrid : 0;
  info->rows_per_block = sv.zcg ? sv.zL : 0;
  info->ring = sv.zcg ? sv.zW : 0;
  info->renumbered = sys->renumbered ? 1 : 0;
  info->banded_fp64 = sv.dcg ? 1 : 0;
  info->fp64_tile_rows = sv.dcg ? sv.dS : 0;
  info->ring_stages = sv.zcg ? sv.zns : 0;
  info->assembly_pairs = sys->pairs ? 1 : 0;
  return ADFEM_OK;
}

// Packed solves (pack.cu): every system of the list solved by one launch, one thread
// block per system; forward (rhs of the system, Dirichlet rows fixed to their values) or
// adjoint (rhs g with Dirichlet rows zeroed, lambda zero there).
}  // extern "C"

namespace adfem {
int system_solve_packed(adfem_system** sys, int count, double** out, const double* const* g,
                        const adfem_solver_opts* opts, adfem_solver_stats* stats, void* stream, bool adjoint,
                        PackSlot* slot) {
  if (!sys || !out || count < 1 || (adjoint && !g)) return fail(ADFEM_ERR_INVALID, "packed solve: bad arguments");
  std::vector<adfem_system*> order(sys, sys + count);
  for (int i = 0; i < count; i++)
    if (!sys[i] || !out[i] || (adjoint && !g[i])) return fail(ADFEM_ERR_INVALID, "packed solve: null system or vector");
  std::sort(order.begin(), order.end());
  if (std::adjacent_find(order.begin(), order.end()) != order.end())
    return fail(ADFEM_ERR_INVALID, "packed solve: a system appears twice");
  std::vector<std::unique_lock<std::mutex>> locks;
  for (adfem_system* s : order) locks.emplace_back(s->mu);
  adfem_solver_opts o;
  adfem_solver_opts_default(&o);
  if (opts) o = *opts;
  cudaStream_t st = S(stream);
  std::vector<PackItem> items(count);
  for (int i = 0; i < count; i++) {
    adfem_system* s = sys[i];
    if (!s->assembled) return fail(ADFEM_ERR_INVALID, "packed solve: system not assembled");
    if (s->ndof > pack_rows_limit())
      return fail(ADFEM_ERR_INVALID,
                  "packed solve: a system has more than " + std::to_string(pack_rows_limit()) + " DOFs");
    PackItem& it = items[i];
    it.S = &s->solver;
    it.rtol = o.rtol;
    it.max_iter = o.max_iter;
    it.warm = o.warm_start != 0;
    it.zero_rows = adjoint ? s->isbd.as<uint8_t>() : nullptr;
    it.fix_rows = s->isbd.as<uint8_t>();
    it.fix_vals = adjoint ? nullptr : s->bdval.as<double>();
    if (!mapped(s)) {
      it.rhs = adjoint ? g[i] : s->rhs.as<double>();
      it.u = out[i];
    } else {
      if (adjoint) ADFEM_TRY(to_solver(s, g[i], s->t1.as<double>(), st));
      if (it.warm) ADFEM_TRY(to_solver(s, out[i], s->t0.as<double>(), st));
      it.rhs = adjoint ? s->t1.as<double>() : s->rhs.as<double>();
      it.u = s->t0.as<double>();
    }
  }
  ADFEM_TRY(solve_packed(items.data(), count, st, slot));
  int status = ADFEM_OK;
  for (int i = 0; i < count; i++) {
    adfem_system* s = sys[i];
    if (mapped(s)) ADFEM_TRY(from_solver(s, s->t0.as<double>(), out[i], st));
    if (stats) {
      stats[i].iterations = items[i].iters;
      stats[i].updates = items[i].passes;
      stats[i].relres = items[i].relres;
      stats[i].ms = 0.0;
      stats[i].status = items[i].status;
      stats[i].launches = 1;
    }
    if (status == ADFEM_OK && items[i].status != ADFEM_OK) status = items[i].status;
  }
  ADFEM_CUDA(cudaStreamSynchronize(st));
  if (status != ADFEM_OK) return fail(status, "packed solve: a system did not converge (see its stats)");
  return ADFEM_OK;
}
}  // namespace adfem

extern "C" {

int adfem_system_solve_packed_d(adfem_system** sys, int count, double** u_d, const adfem_solver_opts* opts,
                                adfem_solver_stats* stats, void* stream) {
  ADFEM_RANGE("adfem_system_solve_packed_d");
  return system_solve_packed(sys, count, u_d, nullptr, opts, stats, stream, false, nullptr);
}

int adfem_system_adjoint_packed_d(adfem_system** sys, int count, const double* const* g_d, double** lam_d,
                                  const adfem_solver_opts* opts, adfem_solver_stats* stats, void* stream) {
  ADFEM_RANGE("adfem_system_adjoint_packed_d");
  return system_solve_packed(sys, count, lam_d, g_d, opts, stats, stream, true, nullptr);
}

int adfem_system_adjoint_d(adfem_system* sys, const double* g_d, double* lam_d, const adfem_solver_opts* opts,
                           adfem_solver_stats* stats, void* stream) {
  ADFEM_RANGE("adfem_system_adjoint_d");
  if (!sys || !g_d || !lam_d) return fail(ADFEM_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(sys->mu);
  if (!sys->assembled) return fail(ADFEM_ERR_INVALID, "system not assembled");
  adfem_solver_opts o;
  adfem_solver_opts_default(&o);
  if (opts) o = *opts;
  cudaStream_t st = S(stream);
  if (!mapped(sys))
    return solver_solve(sys->solver, g_d, lam_d, sys->isbd.as<uint8_t>(), sys->isbd.as<uint8_t>(), nullptr, o, stats,
                        st);
  ADFEM_TRY(to_solver(sys, g_d, sys->t1.as<double>(), st));
  if (o.warm_start) ADFEM_TRY(to_solver(sys, lam_d, sys->t0.as<double>(), st));
  const int r = solver_solve(sys->solver, sys->t1.as<double>(), sys->t0.as<double>(), sys->isbd.as<uint8_t>(),
                             sys->isbd.as<uint8_t>(), nullptr, o, stats, st);
  if (r != ADFEM_OK && r != ADFEM_ERR_NOT_CONVERGED) return r;
  ADFEM_TRY(from_solver(sys, sys->t0.as<double>(), lam_d, st));
  return r;
}

int adfem_system_grad_kappa_d(adfem_system* sys, const double* u_d, const double* lam_d, double* grad_kappa_d,
                              void* stream) {
  ADFEM_RANGE("adfem_system_grad_kappa_d");
  if (!sys || !u_d || !lam_d || !grad_kappa_d) return fail(ADFEM_ERR_INVALID, "null argument");
  if (sys->kind != ADFEM_SYS_POISSON) return fail(ADFEM_ERR_INVALID, "not a Poisson system");
  const Mesh& m = *sys->mesh->m;
  if (m.degree == 2) {
    ADFEM_TRY(kerr(launch_gen_kappa_grad(m, *m.space[2], u_d, lam_d, sys->isbd_ref.as<uint8_t>(), grad_kappa_d,
                                         S(stream)),
                   "P2 kappa grad"));
    return ADFEM_OK;
  }
  ADFEM_TRY(kerr(launch_poisson_kappa_grad(m, u_d, lam_d, sys->isbd_ref.as<uint8_t>(), grad_kappa_d, S(stream)),
                 "kappa grad"));
  return ADFEM_OK;
}

int adfem_system_grad_E_d(adfem_system* sys, const double* u_d, const double* lam_d, const double* E_d,
                          const double* nu_d, double* grad_E_d, void* stream) {
  (void)E_d;
  if (!sys || !u_d || !lam_d || !nu_d || !grad_E_d) return fail(ADFEM_ERR_INVALID, "null argument");
  if (sys->kind != ADFEM_SYS_ELASTICITY) return fail(ADFEM_ERR_INVALID, "not an elasticity system");
  std::lock_guard<std::mutex> lk(sys->mu);
  const int64_t nv = sys->mesh->m->nv;
  cudaStream_t st = S(stream);
  ADFEM_TRY(kerr(launch_to_interleaved(nv, u_d, sys->t1.as<double>(), st), "interleave"));
  ADFEM_TRY(kerr(launch_to_interleaved(nv, lam_d, sys->t2.as<double>(), st), "interleave"));
  ADFEM_TRY(kerr(launch_elastic_grad_E(*sys->mesh->m, sys->t1.as<double>(), sys->t2.as<double>(),
                                       sys->isbd_ref.as<uint8_t>(), nu_d, grad_E_d, st),
                 "grad E"));
  return ADFEM_OK;
}

int adfem_system_apply_d(adfem_system* sys, const double* x_d, double* y_d, void* stream) {
  ADFEM_RANGE("adfem_system_apply_d");
  if (!sys || !x_d || !y_d) return fail(ADFEM_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(sys->mu);
  if (!sys->assembled) return fail(ADFEM_ERR_INVALID, "system not assembled");
  cudaStream_t st = S(stream);
  if (!mapped(sys)) return solver_apply(sys->solver, x_d, y_d, st);
  ADFEM_TRY(to_solver(sys, x_d, sys->t1.as<double>(), st));
  ADFEM_TRY(solver_apply(sys->solver, sys->t1.as<double>(), sys->t2.as<double>(), st));
  ADFEM_TRY(from_solver(sys, sys->t2.as<double>(), y_d, st));
  return ADFEM_OK;
}

int adfem_system_rhs_d(adfem_system* sys, double* rhs_d, void* stream) {
  ADFEM_RANGE("adfem_system_rhs_d");
  if (!sys || !rhs_d) return fail(ADFEM_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(sys->mu);
  if (!sys->assembled) return fail(ADFEM_ERR_INVALID, "system not assembled");
  cudaStream_t st = S(stream);
  if (!mapped(sys)) {
    ADFEM_CUDA(cudaMemcpyAsync(rhs_d, sys->rhs.p, sizeof(double) * sys->ndof, cudaMemcpyDeviceToDevice, st));
    return ADFEM_OK;
  }
  return from_solver(sys, sys->rhs.as<double>(), rhs_d, st);
}

int adfem_poisson_solve(adfem_system* sys, const double* kappa, const double* f, double* u,
                        const adfem_solver_opts* opts, adfem_solver_stats* stats) {
  ADFEM_RANGE("adfem_poisson_solve");
  if (!sys || !kappa || !f || !u) return fail(ADFEM_ERR_INVALID, "null argument");
  if (sys->kind != ADFEM_SYS_POISSON) return fail(ADFEM_ERR_INVALID, "not a Poisson system");
  Mesh& m = *sys->mesh->m;
  const size_t ng = (size_t)mesh_ngauss(m);
  ADFEM_TRY(sys->in0.alloc(sizeof(double) * ng));
  ADFEM_TRY(sys->in1.alloc(sizeof(double) * ng));
  ADFEM_CUDA(cudaMemcpy(sys->in0.p, kappa, sizeof(double) * ng, cudaMemcpyHostToDevice));
  ADFEM_CUDA(cudaMemcpy(sys->in1.p, f, sizeof(double) * ng, cudaMemcpyHostToDevice));
  ADFEM_TRY(adfem_system_assemble_poisson_d(sys, sys->in0.as<double>(), sys->in1.as<double>(), nullptr));
  const size_t nd = (size_t)sys->ndof;
  if (opts && opts->warm_start) ADFEM_CUDA(cudaMemcpy(sys->t2.p, u, sizeof(double) * nd, cudaMemcpyHostToDevice));
  const int r = adfem_system_solve_d(sys, sys->t2.as<double>(), opts, stats, nullptr);
  if (r != ADFEM_OK && r != ADFEM_ERR_NOT_CONVERGED) return r;
  ADFEM_CUDA(cudaMemcpy(u, sys->t2.p, sizeof(double) * nd, cudaMemcpyDeviceToHost));
  return r;
}

// ================================================================== legacy layer
long long* init_nnfem_mesh(double* vertices, int num_vertices, int* element_indices, int num_elements, int order,
                           int lorder, int degree, long long* nedges) {
  ADFEM_RANGE("init_nnfem_mesh");
  (void)lorder;
  const bool ok = (degree == 1 && (order == 2 || order == -1)) || (degree == 2 && (order == 4 || order == -1));
  if (!ok) {
    fail(ADFEM_ERR_UNSUPPORTED, "implemented: P1 elements with the order-2 triangle rule, P2 with the order-4 rule");
    legacy_report(ADFEM_ERR_UNSUPPORTED, "init_nnfem_mesh");
    return nullptr;
  }
  adfem_mesh* h = nullptr;
  int st = adfem_mesh_create(vertices, num_vertices, element_indices, num_elements, degree, &h);
  if (st != ADFEM_OK) {
    legacy_report(st, "init_nnfem_mesh");
    return nullptr;
  }
  {
    std::lock_guard<std::mutex> lk(g_cur_mu);
    if (g_current) {
      std::printf("WARNING: Internal mesh is being overwritten!\n");
      if (g_current_owned) {
        delete g_current->m;
        delete g_current;
      }
    }
    g_current = h;
    g_current_owned = true;
  }
  mesh_edges(h->m);
  if (nedges) *nedges = h->m->nedges;
  long long* out = static_cast<long long*>(std::malloc(sizeof(long long) * std::max<int64_t>(2 * h->m->nedges, 1)));
  if (out) std::memcpy(out, h->m->edges.data(), sizeof(long long) * 2 * h->m->nedges);
  return out;
}

#define LEGACY_MESH(fn, ret)                                 \
  Mesh* m = current_mesh();                                  \
  if (!m) {                                                  \
    fail(ADFEM_ERR_NO_MESH, "no current mesh");              \
    legacy_report(ADFEM_ERR_NO_MESH, fn);                    \
    return ret;                                              \
  }

int mfem_get_ngauss(void) {
  ADFEM_RANGE("mfem_get_ngauss");
  LEGACY_MESH("mfem_get_ngauss", 0);
  return (int)mesh_ngauss(*m);
}
void mfem_get_gauss(double* x, double* y) {
  ADFEM_RANGE("mfem_get_gauss");
  LEGACY_MESH("mfem_get_gauss", );
  mesh_gauss(m, x, y);
}
void mfem_get_gauss_weights(double* w) {
  ADFEM_RANGE("mfem_get_gauss_weights");
  LEGACY_MESH("mfem_get_gauss_weights", );
  mesh_gauss_weights(m, w);
}
void mfem_get_area(double* a) {
  ADFEM_RANGE("mfem_get_area");
  LEGACY_MESH("mfem_get_area", );
  for (int64_t e = 0; e < m->ne; e++) a[e] = m->area[e];
}
int mfem_get_elem_ndof(void) {
  ADFEM_RANGE("mfem_get_elem_ndof");
  LEGACY_MESH("mfem_get_elem_ndof", 0);
  return m->degree == 2 ? 6 : 3;
}
int mfem_get_ndof(void) {
  ADFEM_RANGE("mfem_get_ndof");
  LEGACY_MESH("mfem_get_ndof", 0);
  return (int)mesh_ndof(m);
}
void mfem_get_connectivity(long long* conn) {
  ADFEM_RANGE("mfem_get_connectivity");
  LEGACY_MESH("mfem_get_connectivity", );
  adfem_mesh h{m};
  legacy_report(adfem_mesh_connectivity(&h, conn), "mfem_get_connectivity");
}
void mfem_get_element_to_vertices(long long* elems) {
  ADFEM_RANGE("mfem_get_element_to_vertices");
  LEGACY_MESH("mfem_get_element_to_vertices", );
  for (int64_t e = 0; e < m->ne; e++)
    for (int k = 0; k < 3; k++) elems[k * m->ne + e] = (long long)m->elem[3 * e + k] + 1;
}

// DOFs per element of the current mesh
static size_t elem_nd(const Mesh* m) { return m->degree == 2 ? 6 : 3; }

static int legacy_laplace_coo(Mesh* m, long long* indices, double* vv, const double* kappa) {
  const size_t ng = (size_t)mesh_ngauss(*m), N = elem_nd(m) * elem_nd(m) * ng;
  DevBuf k, idx, v;
  ADFEM_TRY(to_dev(k, kappa, ng));
  ADFEM_TRY(idx.alloc(sizeof(long long) * 2 * N));
  ADFEM_TRY(v.alloc(sizeof(double) * N));
  adfem_mesh h{m};
  ADFEM_TRY(adfem_laplace_coo_d(&h, k.as<double>(), idx.as<long long>(), v.as<double>(), nullptr));
  ADFEM_TRY(to_host(indices, idx, 2 * N));
  return to_host(vv, v, N);
}

void FemLaplaceScalar_forward_Julia(long long* indices, double* vv, const double* kappa) {
  ADFEM_RANGE("FemLaplaceScalar_forward_Julia");
  LEGACY_MESH("FemLaplaceScalar_forward_Julia", );
  legacy_report(legacy_laplace_coo(m, indices, vv, kappa), "FemLaplaceScalar_forward_Julia");
}

void FemSourceScalar_forward_Julia(double* rhs, const double* f) {
  ADFEM_RANGE("FemSourceScalar_forward_Julia");
  LEGACY_MESH("FemSourceScalar_forward_Julia", );
  adfem_mesh h{m};
  legacy_report(adfem_source(&h, f, mesh_ngauss(*m), rhs, 1), "FemSourceScalar_forward_Julia");
}

static int legacy_stiffness_coo(Mesh* m, long long* indices, double* vv, const double* hmat) {
  const size_t ng = (size_t)mesh_ngauss(*m), N = 4 * elem_nd(m) * elem_nd(m) * ng;
  DevBuf d, idx, v;
  ADFEM_TRY(to_dev(d, hmat, 9 * ng));
  ADFEM_TRY(idx.alloc(sizeof(long long) * 2 * N));
  ADFEM_TRY(v.alloc(sizeof(double) * N));
  adfem_mesh h{m};
  ADFEM_TRY(adfem_stiffness_coo_d(&h, d.as<double>(), idx.as<long long>(), v.as<double>(), nullptr));
  ADFEM_TRY(to_host(indices, idx, 2 * N));
  return to_host(vv, v, N);
}

void ComputeFemStiffnessMatrixMfem_forward_Julia(long long* indices, double* vv, const double* hmat) {
  ADFEM_RANGE("ComputeFemStiffnessMatrixMfem_forward_Julia");
  LEGACY_MESH("ComputeFemStiffnessMatrixMfem_forward_Julia", );
  legacy_report(legacy_stiffness_coo(m, indices, vv, hmat), "ComputeFemStiffnessMatrixMfem_forward_Julia");
}

static int legacy_laplace_backward(Mesh* m, double* grad_kappa, const double* grad_vv) {
  const size_t ng = (size_t)mesh_ngauss(*m);
  DevBuf g, o;
  ADFEM_TRY(to_dev(g, grad_vv, elem_nd(m) * elem_nd(m) * ng));
  ADFEM_TRY(o.alloc(sizeof(double) * ng));
  adfem_mesh h{m};
  ADFEM_TRY(adfem_laplace_coo_backward_d(&h, g.as<double>(), o.as<double>(), nullptr));
  return to_host(grad_kappa, o, ng);
}

void FemLaplaceScalar_backward(double* grad_kappa, const double* grad_vv, const long long* indices, const double* vv,
                               const double* kappa) {
  ADFEM_RANGE("FemLaplaceScalar_backward");
  (void)indices;
  (void)vv;
  (void)kappa;
  LEGACY_MESH("FemLaplaceScalar_backward", );
  legacy_report(legacy_laplace_backward(m, grad_kappa, grad_vv), "FemLaplaceScalar_backward");
}

static int legacy_source_backward(Mesh* m, double* grad_f, const double* grad_rhs) {
  const size_t ng = (size_t)mesh_ngauss(*m);
  DevBuf g, o;
  ADFEM_TRY(to_dev(g, grad_rhs, (size_t)mesh_ndof(m)));
  ADFEM_TRY(o.alloc(sizeof(double) * ng));
  adfem_mesh h{m};
  ADFEM_TRY(adfem_source_backward_d(&h, g.as<double>(), o.as<double>(), nullptr));
  return to_host(grad_f, o, ng);
}

void FemSourceScalar_backward(double* grad_f, const double* grad_rhs, const double* rhs, const double* f) {
  ADFEM_RANGE("FemSourceScalar_backward");
  (void)rhs;
  (void)f;
  LEGACY_MESH("FemSourceScalar_backward", );
  legacy_report(legacy_source_backward(m, grad_f, grad_rhs), "FemSourceScalar_backward");
}

static int legacy_stiffness_backward(Mesh* m, double* grad_hmat, const double* grad_vv) {
  const size_t ng = (size_t)mesh_ngauss(*m);
  DevBuf g, o;
  ADFEM_TRY(to_dev(g, grad_vv, 4 * elem_nd(m) * elem_nd(m) * ng));
  ADFEM_TRY(o.alloc(sizeof(double) * 9 * ng));
  adfem_mesh h{m};
  ADFEM_TRY(adfem_stiffness_coo_backward_d(&h, g.as<double>(), o.as<double>(), nullptr));
  return to_host(grad_hmat, o, 9 * ng);
}

void ComputeFemStiffnessMatrixMfem_backward(double* grad_hmat, const double* grad_vv) {
  ADFEM_RANGE("ComputeFemStiffnessMatrixMfem_backward");
  LEGACY_MESH("ComputeFemStiffnessMatrixMfem_backward", );
  legacy_report(legacy_stiffness_backward(m, grad_hmat, grad_vv), "ComputeFemStiffnessMatrixMfem_backward");
}

// ComputeFemMassMatrix1 (deps/MFEM/ComputeFemMassMatrix1/ComputeFemMassMatrixMfem.h:4-55)
static int legacy_mass_coo(Mesh* m, long long* indices, double* vv, const double* rho) {
  const size_t ng = (size_t)mesh_ngauss(*m), N = elem_nd(m) * elem_nd(m) * ng;
  DevBuf k, idx, v;
  ADFEM_TRY(to_dev(k, rho, ng));
  ADFEM_TRY(idx.alloc(sizeof(long long) * 2 * N));
  ADFEM_TRY(v.alloc(sizeof(double) * N));
  adfem_mesh h{m};
  ADFEM_TRY(adfem_mass_coo_d(&h, k.as<double>(), idx.as<long long>(), v.as<double>(), nullptr));
  ADFEM_TRY(to_host(indices, idx, 2 * N));
  return to_host(vv, v, N);
}

void ComputeFemMassMatrix1_forward(long long* indices, double* vv, const double* rho) {
  ADFEM_RANGE("ComputeFemMassMatrix1_forward");
  LEGACY_MESH("ComputeFemMassMatrix1_forward", );
  legacy_report(legacy_mass_coo(m, indices, vv, rho), "ComputeFemMassMatrix1_forward");
}

static int legacy_mass_backward(Mesh* m, double* grad_rho, const double* grad_vv) {
  const size_t ng = (size_t)mesh_ngauss(*m);
  DevBuf g, o;
  ADFEM_TRY(to_dev(g, grad_vv, elem_nd(m) * elem_nd(m) * ng));
  ADFEM_TRY(o.alloc(sizeof(double) * ng));
  adfem_mesh h{m};
  ADFEM_TRY(adfem_mass_coo_backward_d(&h, g.as<double>(), o.as<double>(), nullptr));
  return to_host(grad_rho, o, ng);
}

void ComputeFemMassMatrix1_backward(double* grad_rho, const double* grad_vv, const double* vv, const double* rho) {
  ADFEM_RANGE("ComputeFemMassMatrix1_backward");
  (void)vv;
  (void)rho;
  LEGACY_MESH("ComputeFemMassMatrix1_backward", );
  legacy_report(legacy_mass_backward(m, grad_rho, grad_vv), "ComputeFemMassMatrix1_backward");
}

// FemToGaussPoints / DofToGaussPoints (host pointers, current mesh).  The forward
// functions read nv (vertex values) or ndof values of u; the backward functions add
// into grad_u like the reference loops (the TF ops zero grad_u first).
static int legacy_to_gauss(Mesh* m, bool vertex_only, double* out, const double* u) {
  adfem_mesh h{m};
  Space* sp = nullptr;
  ADFEM_TRY(get_space(*m, m->degree, &sp));
  return to_gauss_host(&h, vertex_only, u, vertex_only ? m->nv : sp->ndof, out);
}

static int legacy_to_gauss_backward(Mesh* m, bool vertex_only, double* grad_u, const double* grad_out) {
  adfem_mesh h{m};
  Space* sp = nullptr;
  ADFEM_TRY(get_space(*m, m->degree, &sp));
  const size_t n = vertex_only ? (size_t)m->nv : (size_t)sp->ndof, ng = (size_t)mesh_ngauss(*m);
  DevBuf g, gu;
  ADFEM_TRY(to_dev(g, grad_out, ng));
  ADFEM_TRY(to_dev(gu, grad_u, n));
  ADFEM_TRY(to_gauss_backward_d(&h, vertex_only, g.as<double>(), gu.as<double>(), (long long)n, 1, nullptr));
  ADFEM_CUDA(cudaStreamSynchronize(nullptr));
  return to_host(grad_u, gu, n);
}

void FemToGaussPointsMfem_Julia(double* out, const double* u) {
  ADFEM_RANGE("FemToGaussPointsMfem_Julia");
  LEGACY_MESH("FemToGaussPointsMfem_Julia", );
  legacy_report(legacy_to_gauss(m, true, out, u), "FemToGaussPointsMfem_Julia");
}
void FemToGaussPointsMfem_forward(double* out, const double* u) {
  ADFEM_RANGE("FemToGaussPointsMfem_forward");
  LEGACY_MESH("FemToGaussPointsMfem_forward", );
  legacy_report(legacy_to_gauss(m, true, out, u), "FemToGaussPointsMfem_forward");
}
void FemToGaussPointsMfem_backward(double* grad_u, const double* grad_out, const double* out, const double* u) {
  ADFEM_RANGE("FemToGaussPointsMfem_backward");
  (void)out;
  (void)u;
  LEGACY_MESH("FemToGaussPointsMfem_backward", );
  legacy_report(legacy_to_gauss_backward(m, true, grad_u, grad_out), "FemToGaussPointsMfem_backward");
}
void DofToGaussPointsMfem_forward_Julia(double* out, const double* u) {
  ADFEM_RANGE("DofToGaussPointsMfem_forward_Julia");
  LEGACY_MESH("DofToGaussPointsMfem_forward_Julia", );
  legacy_report(legacy_to_gauss(m, false, out, u), "DofToGaussPointsMfem_forward_Julia");
}
void DofToGaussPointsMfem_forward(double* out, const double* u) {
  ADFEM_RANGE("DofToGaussPointsMfem_forward");
  LEGACY_MESH("DofToGaussPointsMfem_forward", );
  legacy_report(legacy_to_gauss(m, false, out, u), "DofToGaussPointsMfem_forward");
}
void DofToGaussPointsMfem_backward(double* grad_u, const double* grad_out, const double* out, const double* u) {
  ADFEM_RANGE("DofToGaussPointsMfem_backward");
  (void)out;
  (void)u;
  LEGACY_MESH("DofToGaussPointsMfem_backward", );
  legacy_report(legacy_to_gauss_backward(m, false, grad_u, grad_out), "DofToGaussPointsMfem_backward");
}

// pcl_FemLaplaceScalar_Jacobian (FemLaplaceScalar.h:63-91, caller src/pcl.jl:34-38): H is
// the caller's zeroed ngauss x elem_ndof^2 ngauss column-major matrix
void pcl_FemLaplaceScalar_Jacobian(double* H) {
  ADFEM_RANGE("pcl_FemLaplaceScalar_Jacobian");
  LEGACY_MESH("pcl_FemLaplaceScalar_Jacobian", );
  adfem_mesh h{m};
  legacy_report(adfem_pcl_laplace_jacobian(&h, H), "pcl_FemLaplaceScalar_Jacobian");
}

// pcl_ImposeDirichlet (ImposeDirichlet.h:97-111, caller src/pcl.jl:14-21): indices is the
// 1-based sN x 2 column-major index array of A, J the caller's zeroed sN x outdof
// column-major matrix; J[k, s] = 1 for the s-th entry the Dirichlet op keeps.
static int legacy_pcl_dirichlet(double* J, const long long* indices, const long long* bd, int bdN, int sN) {
  if (sN < 0 || bdN < 0 || (sN > 0 && (!J || !indices)) || (bdN > 0 && !bd))
    return fail(ADFEM_ERR_INVALID, "bad arguments");
  std::vector<long long> idx0(2 * (size_t)sN);
  long long N = 0;
  for (int k = 0; k < sN; k++) {
    idx0[2 * (size_t)k] = indices[k] - 1;
    idx0[2 * (size_t)k + 1] = indices[k + (int64_t)sN] - 1;
    N = std::max(N, std::max(indices[k], indices[k + (int64_t)sN]));
  }
  for (int q = 0; q < bdN; q++) N = std::max(N, bd[q]);
  std::vector<long long> pos(std::max(sN, 1));
  long long nkeep = 0;
  ADFEM_TRY(adfem_pcl_dirichlet(idx0.data(), sN, bd, bdN, N, pos.data(), &nkeep));
  for (int k = 0; k < sN; k++)
    if (pos[k] >= 0) J[k + pos[k] * (int64_t)sN] = 1.0;
  return ADFEM_OK;
}

void pcl_ImposeDirichlet(double* J, const long long* indices, const long long* bd, int bdN, int sN) {
  ADFEM_RANGE("pcl_ImposeDirichlet");
  legacy_report(legacy_pcl_dirichlet(J, indices, bd, bdN, sN), "pcl_ImposeDirichlet");
}

static int host_plane(int mode, const double* E, const double* nu, int N, double* out) {
  if (N <= 0) return ADFEM_OK;
  DevBuf e, v, o;
  ADFEM_TRY(to_dev(e, E, (size_t)N));
  ADFEM_TRY(to_dev(v, nu, (size_t)N));
  ADFEM_TRY(o.alloc(sizeof(double) * 9 * (size_t)N));
  ADFEM_TRY(kerr(launch_plane_strain(mode, N, e.as<double>(), v.as<double>(), o.as<double>(), nullptr), "plane"));
  return to_host(out, o, 9 * (size_t)N);
}
static int host_plane_bwd(int mode, const double* g, const double* E, const double* nu, int N, double* gE,
                          double* gnu) {
  if (N <= 0) return ADFEM_OK;
  DevBuf dg, e, v, oe, on;
  ADFEM_TRY(to_dev(dg, g, 9 * (size_t)N));
  ADFEM_TRY(to_dev(e, E, (size_t)N));
  ADFEM_TRY(to_dev(v, nu, (size_t)N));
  ADFEM_TRY(oe.alloc(sizeof(double) * (size_t)N));
  ADFEM_TRY(on.alloc(sizeof(double) * (size_t)N));
  ADFEM_TRY(kerr(launch_plane_strain_backward(mode, N, dg.as<double>(), e.as<double>(), v.as<double>(),
                                              oe.as<double>(), on.as<double>(), nullptr),
                 "plane backward"));
  ADFEM_TRY(to_host(gE, oe, (size_t)N));
  return to_host(gnu, on, (size_t)N);
}

void PlaneStrainMatrix_forward(double* out, const double* E, const double* nu, int N) {
  ADFEM_RANGE("PlaneStrainMatrix_forward");
  legacy_report(host_plane(0, E, nu, N, out), "PlaneStrainMatrix_forward");
}
void PlaneStrainMatrix_backward(double* grad_nu, double* grad_E, const double* grad_out, const double* E,
                                const double* nu, int N) {
  ADFEM_RANGE("PlaneStrainMatrix_backward");
  legacy_report(host_plane_bwd(0, grad_out, E, nu, N, grad_E, grad_nu), "PlaneStrainMatrix_backward");
}
void PlaneStressMatrix_forward(double* out, const double* E, const double* nu, int N) {
  ADFEM_RANGE("PlaneStressMatrix_forward");
  legacy_report(host_plane(1, E, nu, N, out), "PlaneStressMatrix_forward");
}
void PlaneStressMatrix_backward(double* grad_nu, double* grad_E, const double* grad_out, const double* E,
                                const double* nu, int N) {
  ADFEM_RANGE("PlaneStressMatrix_backward");
  legacy_report(host_plane_bwd(1, grad_out, E, nu, N, grad_E, grad_nu), "PlaneStressMatrix_backward");
}

}  // extern "C"
