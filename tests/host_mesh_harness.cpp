// CPU harness for the library's host mesh code (adfem.jl_gb300/csrc/mesh.cpp), built with
// AddressSanitizer and UndefinedBehaviorSanitizer by tests/test_host_mesh_sanitized.py.
//
// mesh.cpp uploads what it builds through four CUDA runtime calls; here they are stood in
// for by host memory (cudaMalloc -> malloc, cudaMemcpy -> memcpy), so the whole host path
// -- orientation fix, geometry, incidence, CSR pattern, sliced-ELL layout with its
// slice-uniform column patterns, edges, boundary nodes, the P2 space -- runs without a
// GPU, and what it "uploaded" can be read back.  The extern "C" functions below are what
// the test calls through ctypes.  Test infrastructure only: nothing in the library uses it.
#include <cstdlib>
#include <cstring>

#include "adfem_internal.h"

extern "C" {
cudaError_t cudaMalloc(void** p, size_t n) {
  *p = std::malloc(n ? n : 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void* p) {
  std::free(p);
  return cudaSuccess;
}
cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind) {
  std::memcpy(dst, src, n);
  return cudaSuccess;
}
const char* cudaGetErrorString(cudaError_t) { return "host stand-in"; }
}

namespace adfem {
const char* last_error_cstr();  // mesh.cpp: message of the calling thread's last failure
int sell_build_pattern(int64_t n, const int32_t* rowptr, const int32_t* colind, Sell& s, int period);
// the debug-build index-check readers live with the kernels; nothing was checked here
int check_line_solver() { return 0; }
int check_line_zcg() { return 0; }
int check_line_assemble() { return 0; }
int check_line_generic() { return 0; }
}  // namespace adfem

using adfem::Mesh;

extern "C" {
int hm_build(const double* xyz, long long nv, const int* elems0, long long ne, void** out) {
  Mesh* m = nullptr;
  const int st = adfem::mesh_build(xyz, nv, elems0, ne, &m);
  *out = m;
  return st;
}
const char* hm_error() { return adfem::last_error_cstr(); }
void hm_destroy(void* h) { delete static_cast<Mesh*>(h); }
// what adfem_mesh_create does for a degree-2 mesh after mesh_build: the degree, then its space
int hm_make_p2(void* h) {
  Mesh* m = static_cast<Mesh*>(h);
  m->degree = 2;
  adfem::Space* sp = nullptr;
  return adfem::mesh_space(m, 2, &sp);
}
void hm_gauss_weights(void* h, double* w) { adfem::mesh_gauss_weights(static_cast<Mesh*>(h), w); }
void hm_sizes(void* h, long long* nnz, int* maxrow, int* flipped) {
  const Mesh* m = static_cast<Mesh*>(h);
  *nnz = m->nnz;
  *maxrow = m->maxrow;
  *flipped = m->flipped;
}
void hm_pattern(void* h, int* rowptr, int* colind) {
  const Mesh* m = static_cast<Mesh*>(h);
  std::memcpy(rowptr, m->rowptr.data(), sizeof(int) * m->rowptr.size());
  std::memcpy(colind, m->colind.data(), sizeof(int) * m->colind.size());
}
long long hm_bcnode(void* h, long long* out) {
  return adfem::mesh_bcnode(static_cast<Mesh*>(h), reinterpret_cast<int64_t*>(out));
}
long long hm_edges(void* h, long long* out) {
  Mesh* m = static_cast<Mesh*>(h);
  if (adfem::mesh_edges(m) != ADFEM_OK) return -1;
  if (out) std::memcpy(out, m->edges.data(), sizeof(long long) * m->edges.size());
  return m->nedges;
}
void hm_area(void* h, double* a) {
  const Mesh* m = static_cast<Mesh*>(h);
  std::memcpy(a, m->area.data(), sizeof(double) * m->area.size());
}
void hm_gauss(void* h, double* x, double* y) { adfem::mesh_gauss(static_cast<Mesh*>(h), x, y); }
// the sliced-ELL layout s: nslices, stored entries, widest slice; with non-null arrays, slice
// pointers [nslices + 1] and the column of every stored entry [nent] (decoded from the int16
// deltas or int32 columns, through the slice-uniform patterns where a slice has one)
static void sell_decode(const adfem::Sell& s, long long* nslices, long long* nent, int* maxw, int* sptr, int* col) {
  *nslices = s.nslices;
  *nent = s.nent;
  *maxw = s.maxw;
  if (!sptr) return;
  const int32_t* sp = s.sptr.as<int32_t>();
  std::memcpy(sptr, sp, sizeof(int) * (s.nslices + 1));
  const int32_t* spat = s.spat.as<int32_t>();
  const int16_t* pat = s.pat.as<int16_t>();
  for (int64_t sl = 0; sl < s.nslices; sl++) {
    const int w = (sp[sl + 1] - sp[sl]) / 32;
    for (int k = 0; k < w; k++)
      for (int l = 0; l < 32; l++) {
        const int64_t r = 32 * sl + l, q = sp[sl] + 32 * k + l;
        int64_t c;
        if (spat && spat[sl] >= 0) c = r + pat[spat[sl] + (r % s.pat_period) * w + k];
        else if (s.delta16) c = r + s.col.as<int16_t>()[q];
        else c = s.col.as<int32_t>()[q];
        col[q] = (int)c;
      }
  }
}
// the mesh's sliced-ELL copy of its pattern, as uploaded
void hm_sell(void* h, long long* nslices, long long* nent, int* maxw, int* sptr, int* col) {
  sell_decode(static_cast<Mesh*>(h)->sell, nslices, nent, maxw, sptr, col);
}
// sell_build_pattern on any CSR pattern (period 2: slice-uniform patterns per row parity, as
// for interleaved 2-DOF operators); info = {delta16, uniform slices, band}.  Two calls: sizes
// with null arrays, then the decoded layout.
int hm_sell_build(long long n, const int* rowptr, const int* colind, int period, long long* nslices, long long* nent,
                  int* maxw, long long* info, int* sptr, int* col) {
  adfem::Sell s;
  const int st = adfem::sell_build_pattern(n, rowptr, colind, s, period);
  if (st != ADFEM_OK) return st;
  info[0] = s.delta16 ? 1 : 0;
  info[1] = s.uniform_slices;
  info[2] = s.band;
  sell_decode(s, nslices, nent, maxw, sptr, col);
  return ADFEM_OK;
}
// reverse Cuthill-McKee order of the mesh's node graph (pi[node] = new index) and the band it
// reports
long long hm_rcm(void* h, int* pi) {
  std::vector<int32_t> p;
  const int64_t band = adfem::mesh_rcm(*static_cast<Mesh*>(h), p);
  std::memcpy(pi, p.data(), sizeof(int) * p.size());
  return band;
}
// the P2 (or P1) space: DOFs, pattern entries and widest row; with non-null arrays, its
// CSR pattern
int hm_space(void* h, int degree, long long* ndof, long long* nnz, int* maxrow, int* rowptr, int* colind) {
  Mesh* m = static_cast<Mesh*>(h);
  adfem::Space* sp = nullptr;
  const int st = adfem::mesh_space(m, degree, &sp);
  if (st != ADFEM_OK) return st;
  *ndof = sp->ndof;
  *nnz = sp->nnz;
  *maxrow = sp->maxrow;
  if (rowptr) std::memcpy(rowptr, sp->rowptr.data(), sizeof(int) * sp->rowptr.size());
  if (colind) std::memcpy(colind, sp->colind.data(), sizeof(int) * sp->colind.size());
  return ADFEM_OK;
}
}
