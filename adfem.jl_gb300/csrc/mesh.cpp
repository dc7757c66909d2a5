// Host side of the mesh runtime: the work AdFem's NNFEM_Mesh::init does once per
// mesh (deps/MFEM/Common.cpp:20-142), plus the data the GPU kernels need:
// node->element incidence, the scalar CSR pattern, per-incidence slot offsets
// and the sliced-ELL copy of the pattern.  Everything here runs once per mesh on
// the host (threaded), then is uploaded; the per-call work is on the device.
#include <atomic>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <thread>

#include "adfem_internal.h"

namespace adfem {

static thread_local std::string g_err;
void set_error(const std::string& m) { g_err = m; }
const char* last_error_cstr() { return g_err.c_str(); }
int fail(int st, const std::string& m) {
  set_error(m);
  return st;
}
int cuda_fail(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? ADFEM_ERR_NOMEM : ADFEM_ERR_CUDA;
}

std::mutex& device_alloc_mutex() {
  static std::mutex mu;
  return mu;
}

void DevBuf::release() {
  if (p) {
    std::lock_guard<std::mutex> lk(device_alloc_mutex());
    cudaFree(p);
  }
  p = nullptr;
  bytes = 0;
}

static std::atomic<long long> g_alloc_fail_countdown{-1};

bool injected_alloc_failure() {
  long long c = g_alloc_fail_countdown.load();
  while (c >= 0) {
    if (g_alloc_fail_countdown.compare_exchange_weak(c, c - 1)) return c == 0;
  }
  return false;
}

void arm_alloc_failure(long long k) { g_alloc_fail_countdown.store(k < 0 ? -1 : k); }

int DevBuf::alloc(size_t nb) {
  if (p && nb <= bytes) return ADFEM_OK;
  release();
  if (nb == 0) return ADFEM_OK;
  if (injected_alloc_failure()) return cuda_fail(cudaErrorMemoryAllocation, "cudaMalloc (injected failure)");
  std::lock_guard<std::mutex> lk(device_alloc_mutex());
  cudaError_t e = cudaMalloc(&p, nb);
  if (e != cudaSuccess) {
    p = nullptr;
    return cuda_fail(e, "cudaMalloc");
  }
  bytes = nb;
  return ADFEM_OK;
}

// run f(lo, hi) over [0, n) on up to 32 host threads
template <class F>
static void parallel_for(int64_t n, F f) {
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min(nt, 32u));
  if (n < 50000) nt = 1;
  if (nt == 1) {
    f((int64_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++) {
    int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
    th.emplace_back([=] { f(lo, hi); });
  }
  for (auto& x : th) x.join();
}

// barycentric coordinates of the three points of the degree-2 triangle rule
// (points (xi, eta) = (1/6,1/6), (1/6,2/3), (2/3,1/6), weight 1/6 each)
static const double QX[3] = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
static const double QY[3] = {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0};
static const double QW = 1.0 / 6.0;
// degree-4 rule (the order P2 meshes default to, src/MFEM/MFEM.jl:71-77): the published
// 6-point Strang-Fix/Dunavant rule, orbits (a,a), (a,1-2a), (1-2a,a)
static const double Q4X[6] = {0.091576213509770743460, 0.091576213509770743460, 0.81684757298045851308,
                              0.44594849091596488632, 0.44594849091596488632, 0.10810301816807022736};
static const double Q4Y[6] = {0.091576213509770743460, 0.81684757298045851308, 0.091576213509770743460,
                              0.44594849091596488632, 0.10810301816807022736, 0.44594849091596488632};
static const double Q4W[6] = {0.054975871827660933819, 0.054975871827660933819, 0.054975871827660933819,
                              0.11169079483900573285, 0.11169079483900573285, 0.11169079483900573285};

void rule_point(int degree, int k, double* xi, double* eta, double* w) {
  if (degree == 2) {
    *xi = Q4X[k];
    *eta = Q4Y[k];
    *w = Q4W[k];
  } else {
    *xi = QX[k];
    *eta = QY[k];
    *w = QW;
  }
}

static double heron(double x0, double y0, double x1, double y1, double x2, double y2) {
  // deps/MFEM/Common.cpp:9-15
  double a = std::sqrt((x0 - x1) * (x0 - x1) + (y0 - y1) * (y0 - y1));
  double b = std::sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1));
  double c = std::sqrt((x0 - x2) * (x0 - x2) + (y0 - y2) * (y0 - y2));
  double s = (a + b + c) / 2.0;
  return std::sqrt(s * (s - a) * (s - b) * (s - c));
}

template <class T>
static int upload(DevBuf& b, const T* src, size_t n) {
  ADFEM_TRY(b.alloc(sizeof(T) * std::max<size_t>(n, 1)));
  if (n) ADFEM_CUDA(cudaMemcpy(b.p, src, sizeof(T) * n, cudaMemcpyHostToDevice));
  return ADFEM_OK;
}

// Sliced-ELL pattern of a CSR matrix (rows n, 0-based rowptr/colind).  Columns are
// stored as int16 deltas when every |col-row| fits, else as int32.  Slices whose rows
// share their column offsets (with the given period in the row index) also get a
// slice-level pattern (see Sell::spat).
int sell_build_pattern(int64_t n, const int32_t* rowptr, const int32_t* colind, Sell& s, int period) {
  s.n = n;
  s.nslices = (n + 31) / 32;
  std::vector<int32_t> sptr(s.nslices + 1, 0);
  int64_t maxd = 0;
  int maxw = 0;
  for (int64_t sl = 0; sl < s.nslices; sl++) {
    int w = 0;
    for (int64_t r = sl * 32; r < std::min<int64_t>(n, sl * 32 + 32); r++) {
      int len = rowptr[r + 1] - rowptr[r];
      w = std::max(w, len);
      for (int32_t k = rowptr[r]; k < rowptr[r + 1]; k++) maxd = std::max<int64_t>(maxd, std::llabs((int64_t)colind[k] - r));
    }
    maxw = std::max(maxw, w);
    int64_t next = (int64_t)sptr[sl] + 32 * (int64_t)w;
    if (next > INT32_MAX) return fail(ADFEM_ERR_UNSUPPORTED, "sliced-ELL matrix exceeds 2^31 entries");
    sptr[sl + 1] = (int32_t)next;
  }
  s.nent = sptr[s.nslices];
  s.maxw = maxw;
  s.band = maxd;
  s.delta16 = maxd <= 32767;
  ADFEM_TRY(upload(s.sptr, sptr.data(), sptr.size()));
  if (s.delta16) {
    std::vector<int16_t> col(std::max<int64_t>(s.nent, 1), 0);
    parallel_for(s.nslices, [&](int64_t lo, int64_t hi) {
      for (int64_t sl = lo; sl < hi; sl++)
        for (int64_t r = sl * 32; r < std::min<int64_t>(n, sl * 32 + 32); r++)
          for (int32_t k = rowptr[r]; k < rowptr[r + 1]; k++)
            col[sptr[sl] + 32 * (int64_t)(k - rowptr[r]) + (r & 31)] = (int16_t)(colind[k] - r);
    });
    ADFEM_TRY(upload(s.col, col.data(), (size_t)s.nent));
  } else {
    std::vector<int32_t> col(std::max<int64_t>(s.nent, 1), 0);
    parallel_for(s.nslices, [&](int64_t lo, int64_t hi) {
      for (int64_t sl = lo; sl < hi; sl++) {
        for (int64_t r = sl * 32; r < std::min<int64_t>(n, sl * 32 + 32); r++) {
          int w = (sptr[sl + 1] - sptr[sl]) / 32;
          for (int k = 0; k < w; k++) col[sptr[sl] + 32 * (int64_t)k + (r & 31)] = (int32_t)r;  // padding -> diagonal
          for (int32_t k = rowptr[r]; k < rowptr[r + 1]; k++)
            col[sptr[sl] + 32 * (int64_t)(k - rowptr[r]) + (r & 31)] = colind[k];
        }
        // rows beyond n in the last slice point at row n-1 (a valid index)
        for (int64_t r = n; r < sl * 32 + 32 && sl == s.nslices - 1; r++) {
          int w = (sptr[sl + 1] - sptr[sl]) / 32;
          for (int k = 0; k < w; k++) col[sptr[sl] + 32 * (int64_t)k + (r & 31)] = (int32_t)(n - 1);
        }
      }
    });
    ADFEM_TRY(upload(s.col, col.data(), (size_t)s.nent));
  }
  // slice-uniform patterns
  s.pat_period = period;
  s.uniform_slices = 0;
  s.uniform_entries = 0;
  std::vector<int32_t> spat(std::max<int64_t>(s.nslices, 1), -1);
  std::vector<int16_t> pool;
  if (s.delta16 && (period == 1 || period == 2)) {
    std::map<std::vector<int16_t>, int32_t> dedupe;
    std::vector<int16_t> pt;
    for (int64_t sl = 0; sl < s.nslices; sl++) {
      const int w = (sptr[sl + 1] - sptr[sl]) / 32;
      if (sl * 32 + 32 > n || w == 0) continue;
      pt.assign((size_t)period * w, 0);
      bool ok = true;
      for (int64_t r = sl * 32; r < sl * 32 + 32 && ok; r++) {
        if (rowptr[r + 1] - rowptr[r] != w) {
          ok = false;
          break;
        }
        const int q = (int)(r % period);
        for (int k = 0; k < w; k++) {
          const int16_t d = (int16_t)(colind[rowptr[r] + k] - r);
          if (r - sl * 32 < period) pt[(size_t)q * w + k] = d;
          else if (pt[(size_t)q * w + k] != d) {
            ok = false;
            break;
          }
        }
      }
      if (!ok) continue;
      auto it = dedupe.find(pt);
      int32_t off;
      if (it == dedupe.end()) {
        off = (int32_t)pool.size();
        pool.insert(pool.end(), pt.begin(), pt.end());
        dedupe.emplace(pt, off);
      } else {
        off = it->second;
      }
      spat[sl] = off;
      s.uniform_slices++;
      s.uniform_entries += 32 * (int64_t)w;
    }
  }
  if (pool.empty()) pool.push_back(0);
  ADFEM_TRY(upload(s.spat, spat.data(), spat.size()));
  ADFEM_TRY(upload(s.pat, pool.data(), pool.size()));
  return ADFEM_OK;
}

int mesh_build(const double* xyz, int64_t nv, const int32_t* elems0, int64_t ne, Mesh** out) {
  if (!xyz || !elems0 || !out) return fail(ADFEM_ERR_INVALID, "mesh: null pointer");
  if (nv < 3 || ne < 1) return fail(ADFEM_ERR_INVALID, "mesh: need at least 3 vertices and 1 element");
  if (nv > INT32_MAX / 2 || 3 * ne > INT32_MAX) return fail(ADFEM_ERR_UNSUPPORTED, "mesh: too many vertices/elements");
  for (int64_t k = 0; k < 3 * ne; k++)
    if (elems0[k] < 0 || elems0[k] >= nv)
      return fail(ADFEM_ERR_INVALID, "mesh: element " + std::to_string(k / 3) + " has a vertex index out of range");
  std::unique_ptr<Mesh> m(new Mesh());
  m->nv = nv;
  m->ne = ne;
  m->xy.resize(2 * nv);
  for (int64_t i = 0; i < nv; i++) {
    m->xy[2 * i] = xyz[3 * i];
    m->xy[2 * i + 1] = xyz[3 * i + 1];
  }
  m->elem.resize(3 * ne);
  m->area.resize(ne);
  m->grad.resize(6 * ne);
  std::vector<double> geo(4 * ne);
  std::vector<int> flips(64, 0);
  std::vector<int64_t> bad(64, -1);
  // orientation fix (MFEM Mesh::CheckElementOrientation: swap the first two vertices
  // of a triangle with negative Jacobian determinant) and per-element geometry
  // (Common.cpp:76-126): Heron area, w = ip.weight * area / 0.5, physical gradients.
  {
    const int nt = 64;
    auto body = [&](int t) {
      int64_t lo = ne * t / nt, hi = ne * (t + 1) / nt;
      for (int64_t e = lo; e < hi; e++) {
        int32_t v0 = elems0[3 * e], v1 = elems0[3 * e + 1], v2 = elems0[3 * e + 2];
        const double* X = m->xy.data();
        double det = (X[2 * v1] - X[2 * v0]) * (X[2 * v2 + 1] - X[2 * v0 + 1]) -
                     (X[2 * v1 + 1] - X[2 * v0 + 1]) * (X[2 * v2] - X[2 * v0]);
        if (det < 0.0) {
          std::swap(v0, v1);
          flips[t]++;
        }
        if (det == 0.0 || !std::isfinite(det)) {
          if (bad[t] < 0) bad[t] = e;
          continue;
        }
        m->elem[3 * e] = v0;
        m->elem[3 * e + 1] = v1;
        m->elem[3 * e + 2] = v2;
        double x1 = X[2 * v0], y1 = X[2 * v0 + 1], x2 = X[2 * v1], y2 = X[2 * v1 + 1], x3 = X[2 * v2],
               y3 = X[2 * v2 + 1];
        double A = heron(x1, y1, x2, y2, x3, y3);
        m->area[e] = A;
        double j00 = x2 - x1, j01 = x3 - x1, j10 = y2 - y1, j11 = y3 - y1;
        double dj = j00 * j11 - j01 * j10;
        double it = 1.0 / dj;
        double i00 = j11 * it, i01 = -j01 * it, i10 = -j10 * it, i11 = j00 * it;
        double hx[3] = {-i00 - i10, i00, i10}, hy[3] = {-i01 - i11, i01, i11};
        for (int a = 0; a < 3; a++) {
          m->grad[6 * e + 2 * a] = hx[a];
          m->grad[6 * e + 2 * a + 1] = hy[a];
        }
        double w = QW * A / 0.5;
        geo[4 * e + 0] = w * (hx[0] * hx[1] + hy[0] * hy[1]);
        geo[4 * e + 1] = w * (hx[0] * hx[2] + hy[0] * hy[2]);
        geo[4 * e + 2] = w * (hx[1] * hx[2] + hy[1] * hy[2]);
        geo[4 * e + 3] = w;
      }
    };
    std::vector<std::thread> th;
    unsigned hc = std::max(1u, std::min(std::thread::hardware_concurrency(), 32u));
    if (ne < 50000) hc = 1;
    for (unsigned c = 0; c < hc; c++)
      th.emplace_back([&, c] {
        for (int t = (int)c; t < nt; t += (int)hc) body(t);
      });
    for (auto& x : th) x.join();
  }
  for (int t = 0; t < 64; t++) {
    if (bad[t] >= 0) return fail(ADFEM_ERR_INVALID, "mesh: element " + std::to_string(bad[t]) + " is degenerate");
    m->flipped += flips[t];
  }

  // node -> element incidence, ascending element order per node
  m->inc_ptr.assign(nv + 1, 0);
  for (int64_t k = 0; k < 3 * ne; k++) m->inc_ptr[m->elem[k] + 1]++;
  for (int64_t i = 0; i < nv; i++) {
    m->maxinc = std::max(m->maxinc, m->inc_ptr[i + 1]);
    m->inc_ptr[i + 1] += m->inc_ptr[i];
  }
  for (int64_t i = 0; i < nv; i++)
    if (m->inc_ptr[i + 1] == m->inc_ptr[i])
      return fail(ADFEM_ERR_INVALID, "mesh: vertex " + std::to_string(i) + " belongs to no element");
  m->inc.resize(2 * 3 * ne);
  {
    std::vector<int32_t> fill(m->inc_ptr.begin(), m->inc_ptr.end() - 1);
    for (int64_t e = 0; e < ne; e++)
      for (int a = 0; a < 3; a++) {
        int32_t v = m->elem[3 * e + a];
        int32_t s = fill[v]++;
        m->inc[2 * s] = (uint32_t)e;
        m->inc[2 * s + 1] = (uint32_t)a;
      }
  }
  // scalar CSR pattern: row i = sorted unique vertices of the elements around i
  std::vector<int32_t> rowlen(nv);
  parallel_for(nv, [&](int64_t lo, int64_t hi) {
    std::vector<int32_t> cand;
    for (int64_t i = lo; i < hi; i++) {
      cand.clear();
      for (int32_t s = m->inc_ptr[i]; s < m->inc_ptr[i + 1]; s++) {
        int64_t e = m->inc[2 * s];
        for (int b = 0; b < 3; b++) cand.push_back(m->elem[3 * e + b]);
      }
      std::sort(cand.begin(), cand.end());
      rowlen[i] = (int32_t)(std::unique(cand.begin(), cand.end()) - cand.begin());
    }
  });
  m->rowptr.assign(nv + 1, 0);
  for (int64_t i = 0; i < nv; i++) {
    m->maxrow = std::max(m->maxrow, rowlen[i]);
    m->rowptr[i + 1] = m->rowptr[i] + rowlen[i];
  }
  if (m->maxrow > 64)
    return fail(ADFEM_ERR_UNSUPPORTED, "mesh: a vertex has " + std::to_string(m->maxrow - 1) +
                                           " neighbours; at most 63 are supported");
  m->nnz = m->rowptr[nv];
  m->colind.resize(m->nnz);
  std::vector<int32_t> diagpos(nv);
  parallel_for(nv, [&](int64_t lo, int64_t hi) {
    std::vector<int32_t> cand;
    for (int64_t i = lo; i < hi; i++) {
      cand.clear();
      for (int32_t s = m->inc_ptr[i]; s < m->inc_ptr[i + 1]; s++) {
        int64_t e = m->inc[2 * s];
        for (int b = 0; b < 3; b++) cand.push_back(m->elem[3 * e + b]);
      }
      std::sort(cand.begin(), cand.end());
      cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
      std::copy(cand.begin(), cand.end(), m->colind.begin() + m->rowptr[i]);
      diagpos[i] = (int32_t)(std::lower_bound(cand.begin(), cand.end(), (int32_t)i) - cand.begin());
      for (int32_t s = m->inc_ptr[i]; s < m->inc_ptr[i + 1]; s++) {
        int64_t e = m->inc[2 * s];
        uint32_t a = m->inc[2 * s + 1];
        uint32_t y = a;
        for (int b = 0; b < 3; b++) {
          uint32_t off = (uint32_t)(std::lower_bound(cand.begin(), cand.end(), m->elem[3 * e + b]) - cand.begin());
          y |= off << (2 + 10 * b);
        }
        m->inc[2 * s + 1] = y;
      }
    }
  });

  // upload
  std::vector<int32_t> conn4(4 * ne);
  for (int64_t e = 0; e < ne; e++) {
    conn4[4 * e] = m->elem[3 * e];
    conn4[4 * e + 1] = m->elem[3 * e + 1];
    conn4[4 * e + 2] = m->elem[3 * e + 2];
    conn4[4 * e + 3] = 0;
  }
  ADFEM_TRY(upload(m->d_xy, m->xy.data(), m->xy.size()));
  ADFEM_TRY(upload(m->d_conn, conn4.data(), conn4.size()));
  ADFEM_TRY(upload(m->d_geo, geo.data(), geo.size()));
  ADFEM_TRY(upload(m->d_grad, m->grad.data(), m->grad.size()));
  ADFEM_TRY(upload(m->d_inc_ptr, m->inc_ptr.data(), m->inc_ptr.size()));
  ADFEM_TRY(upload(m->d_inc, m->inc.data(), m->inc.size()));
  ADFEM_TRY(upload(m->d_rowptr, m->rowptr.data(), m->rowptr.size()));
  ADFEM_TRY(upload(m->d_colind, m->colind.data(), m->colind.size()));
  ADFEM_TRY(upload(m->d_diagpos, diagpos.data(), diagpos.size()));
  ADFEM_TRY(sell_build_pattern(nv, m->rowptr.data(), m->colind.data(), m->sell, 1));
  *out = m.release();
  return ADFEM_OK;
}

// Edge numbering: first appearance while walking elements in order and each
// triangle's local edges (0,1), (1,2), (2,0); endpoints reported 1-based as
// (min, max) blocks like Common.cpp:133-139.
int mesh_edges(Mesh* m) {
  if (m->nedges >= 0) return ADFEM_OK;
  std::vector<int64_t> id(m->nnz, -1);
  std::vector<int64_t> emin, emax;
  emin.reserve(m->nnz / 2 + 1);
  emax.reserve(m->nnz / 2 + 1);
  for (int64_t e = 0; e < m->ne; e++)
    for (int l = 0; l < 3; l++) {
      int32_t a = m->elem[3 * e + l], b = m->elem[3 * e + (l + 1) % 3];
      int32_t lo = std::min(a, b), hi = std::max(a, b);
      const int32_t* row = m->colind.data() + m->rowptr[lo];
      int32_t len = m->rowptr[lo + 1] - m->rowptr[lo];
      int64_t slot = m->rowptr[lo] + (std::lower_bound(row, row + len, hi) - row);
      if (id[slot] < 0) {
        id[slot] = (int64_t)emin.size();
        emin.push_back(lo + 1);
        emax.push_back(hi + 1);
      }
    }
  m->eedge.resize(3 * m->ne);
  for (int64_t e = 0; e < m->ne; e++)
    for (int l = 0; l < 3; l++) {
      int32_t a = m->elem[3 * e + l], b = m->elem[3 * e + (l + 1) % 3];
      int32_t lo = std::min(a, b), hi = std::max(a, b);
      const int32_t* row = m->colind.data() + m->rowptr[lo];
      int32_t len = m->rowptr[lo + 1] - m->rowptr[lo];
      m->eedge[3 * e + l] = (int32_t)id[m->rowptr[lo] + (std::lower_bound(row, row + len, hi) - row)];
    }
  m->nedges = (int64_t)emin.size();
  m->edges.resize(2 * m->nedges);
  std::copy(emin.begin(), emin.end(), m->edges.begin());
  std::copy(emax.begin(), emax.end(), m->edges.begin() + m->nedges);
  return ADFEM_OK;
}

// Boundary nodes: endpoints of edges shared by an odd number of elements
// (the Set toggle of src/MFEM/MCore.jl:385-406), ascending, 1-based.  For P2 meshes
// the DOFs of those edges follow (nv + edge, ascending), as bcnode(mesh) appends the
// boundary edge DOFs for P2 elements (MCore.jl:439-450).
int64_t mesh_bcnode(Mesh* m, int64_t* out1) {
  std::vector<int32_t> cnt(m->nnz, 0);
  for (int64_t i = 0; i < m->nv; i++)
    for (int32_t s = m->inc_ptr[i]; s < m->inc_ptr[i + 1]; s++) {
      uint32_t y = m->inc[2 * s + 1];
      uint32_t a = inc_a(y);
      for (uint32_t b = 0; b < 3; b++)
        if (b != a) cnt[m->rowptr[i] + inc_off(y, b)]++;
    }
  int64_t c = 0;
  for (int64_t i = 0; i < m->nv; i++) {
    bool bd = false;
    for (int32_t k = m->rowptr[i]; k < m->rowptr[i + 1]; k++)
      if (m->colind[k] != i && (cnt[k] & 1)) bd = true;
    if (bd) {
      if (out1) out1[c] = i + 1;
      c++;
    }
  }
  if (m->degree == 2 && mesh_edges(m) == ADFEM_OK) {
    std::vector<int32_t> ecnt(m->nedges, 0);
    for (int32_t j : m->eedge) ecnt[j]++;
    for (int64_t j = 0; j < m->nedges; j++)
      if (ecnt[j] & 1) {
        if (out1) out1[c] = m->nv + j + 1;
        c++;
      }
  }
  return c;
}

// Reverse Cuthill-McKee order of the node graph: per connected component a BFS from a
// pseudo-peripheral node (two BFS sweeps from a minimum-degree node, each restarting at
// the last node reached), neighbours visited in ascending degree, the whole order then
// reversed.  pi[node] = new index.  Returns the bandwidth max |pi(i) - pi(j)| over the
// pattern.
int64_t mesh_rcm(const Mesh& m, std::vector<int32_t>& pi) { return graph_rcm(m.nv, m.rowptr, m.colind, pi); }

// The same order for any symmetric graph in CSR form (a degree-2 DOF graph, for instance).
int64_t graph_rcm(int64_t n, const std::vector<int32_t>& rowptr, const std::vector<int32_t>& colind,
                  std::vector<int32_t>& pi) {
  struct G {
    const std::vector<int32_t>& rowptr;
    const std::vector<int32_t>& colind;
  } m{rowptr, colind};
  auto deg = [&](int64_t i) { return m.rowptr[i + 1] - m.rowptr[i]; };
  std::vector<int32_t> order;
  order.reserve(n);
  std::vector<uint8_t> seen(n, 0), mark(n, 0);
  std::vector<int32_t> q, nb;
  q.reserve(n);
  // BFS from s over the unseen part of the graph (marks in `mark` reset afterwards);
  // returns the last node reached
  auto sweep = [&](int32_t s) {
    q.clear();
    q.push_back(s);
    mark[s] = 1;
    for (size_t h = 0; h < q.size(); h++) {
      const int32_t v = q[h];
      for (int32_t k = m.rowptr[v]; k < m.rowptr[v + 1]; k++) {
        const int32_t j = m.colind[k];
        if (!seen[j] && !mark[j]) {
          mark[j] = 1;
          q.push_back(j);
        }
      }
    }
    for (int32_t v : q) mark[v] = 0;
    return q.back();
  };
  for (int64_t start = 0; start < n; start++) {
    if (seen[start]) continue;
    // minimum-degree node of this component
    sweep((int32_t)start);
    int32_t s = (int32_t)start;
    for (int32_t v : q)
      if (deg(v) < deg(s)) s = v;
    for (int r = 0; r < 2; r++) s = sweep(s);
    // Cuthill-McKee BFS from s
    const size_t c0 = order.size();
    order.push_back(s);
    seen[s] = 1;
    for (size_t h = c0; h < order.size(); h++) {
      const int32_t v = order[h];
      nb.clear();
      for (int32_t k = m.rowptr[v]; k < m.rowptr[v + 1]; k++) {
        const int32_t j = m.colind[k];
        if (!seen[j]) {
          seen[j] = 1;
          nb.push_back(j);
        }
      }
      std::stable_sort(nb.begin(), nb.end(), [&](int32_t a, int32_t b) { return deg(a) < deg(b); });
      order.insert(order.end(), nb.begin(), nb.end());
    }
  }
  pi.assign(n, 0);
  for (int64_t k = 0; k < n; k++) pi[order[k]] = (int32_t)(n - 1 - k);
  int64_t band = 0;
  for (int64_t i = 0; i < n; i++)
    for (int32_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++)
      band = std::max<int64_t>(band, std::llabs((int64_t)pi[i] - pi[m.colind[k]]));
  return band;
}

int64_t mesh_ndof(Mesh* m) {
  if (m->degree != 2) return m->nv;
  mesh_edges(m);
  return m->nv + m->nedges;
}

void mesh_gauss(const Mesh* m, double* x, double* y) {
  const int ng = mesh_ng(*m);
  for (int64_t e = 0; e < m->ne; e++) {
    const double* X = m->xy.data();
    int32_t v0 = m->elem[3 * e], v1 = m->elem[3 * e + 1], v2 = m->elem[3 * e + 2];
    for (int k = 0; k < ng; k++) {
      double xi, eta, w;
      rule_point(m->degree, k, &xi, &eta, &w);
      double l0 = 1.0 - xi - eta, l1 = xi, l2 = eta;
      x[ng * e + k] = X[2 * v0] * l0 + X[2 * v1] * l1 + X[2 * v2] * l2;
      y[ng * e + k] = X[2 * v0 + 1] * l0 + X[2 * v1 + 1] * l1 + X[2 * v2 + 1] * l2;
    }
  }
}

void mesh_gauss_weights(const Mesh* m, double* wout) {
  const int ng = mesh_ng(*m);
  for (int64_t e = 0; e < m->ne; e++)
    for (int k = 0; k < ng; k++) {
      double xi, eta, w;
      rule_point(m->degree, k, &xi, &eta, &w);
      wout[ng * e + k] = w * m->area[e] / 0.5;  // Common.cpp:116
    }
}

// Space of degree 1 or 2 (see Space in adfem_internal.h): element DOFs as
// NNFEM_Mesh::init numbers them (Common.cpp:62-71), the DOF graph (full pattern of
// sparse() on the unsummed COO) and the DOF->element incidence with slot offsets.
int mesh_space(Mesh* m, int degree, Space** out) {
  if (degree != 1 && degree != 2) return fail(ADFEM_ERR_UNSUPPORTED, "element degree must be 1 or 2");
  if (m->space[degree]) {
    *out = m->space[degree].get();
    return ADFEM_OK;
  }
  if (degree == 2) ADFEM_TRY(mesh_edges(m));
  std::unique_ptr<Space> sp(new Space());
  const int nd = degree == 2 ? 6 : 3;
  const int64_t ne = m->ne;
  sp->degree = degree;
  sp->nd = nd;
  sp->ng = degree == 2 ? 6 : 3;
  sp->ndof = degree == 2 ? m->nv + m->nedges : m->nv;
  if (sp->ndof > INT32_MAX / 2 || nd * ne > INT32_MAX) return fail(ADFEM_ERR_UNSUPPORTED, "space: too many DOFs");
  const int64_t ndof = sp->ndof;
  sp->dof.resize(nd * ne);
  for (int64_t e = 0; e < ne; e++) {
    for (int a = 0; a < 3; a++) sp->dof[nd * e + a] = m->elem[3 * e + a];
    if (degree == 2)
      for (int j = 0; j < 3; j++) sp->dof[nd * e + 3 + j] = (int32_t)(m->nv + m->eedge[3 * e + j]);
  }
  std::vector<int32_t> inc_ptr(ndof + 1, 0);
  for (int32_t d : sp->dof) inc_ptr[d + 1]++;
  for (int64_t i = 0; i < ndof; i++) inc_ptr[i + 1] += inc_ptr[i];
  std::vector<uint32_t> inc(4 * (size_t)nd * ne, 0u);
  {
    std::vector<int32_t> fill(inc_ptr.begin(), inc_ptr.end() - 1);
    for (int64_t e = 0; e < ne; e++)
      for (int a = 0; a < nd; a++) {
        int32_t s = fill[sp->dof[nd * e + a]]++;
        inc[4 * (size_t)s] = (uint32_t)e;
        inc[4 * (size_t)s + 1] = (uint32_t)a;
      }
  }
  std::vector<int32_t> rowlen(ndof);
  parallel_for(ndof, [&](int64_t lo, int64_t hi) {
    std::vector<int32_t> cand;
    for (int64_t i = lo; i < hi; i++) {
      cand.clear();
      for (int32_t s = inc_ptr[i]; s < inc_ptr[i + 1]; s++) {
        int64_t e = inc[4 * (size_t)s];
        for (int b = 0; b < nd; b++) cand.push_back(sp->dof[nd * e + b]);
      }
      std::sort(cand.begin(), cand.end());
      rowlen[i] = (int32_t)(std::unique(cand.begin(), cand.end()) - cand.begin());
    }
  });
  sp->rowptr.assign(ndof + 1, 0);
  for (int64_t i = 0; i < ndof; i++) {
    sp->maxrow = std::max(sp->maxrow, rowlen[i]);
    if ((int64_t)sp->rowptr[i] + rowlen[i] > INT32_MAX) return fail(ADFEM_ERR_UNSUPPORTED, "space: pattern too large");
    sp->rowptr[i + 1] = sp->rowptr[i] + rowlen[i];
  }
  if (sp->maxrow > 1024) return fail(ADFEM_ERR_UNSUPPORTED, "space: a DOF row has more than 1024 entries");
  sp->nnz = sp->rowptr[ndof];
  sp->colind.resize(sp->nnz);
  parallel_for(ndof, [&](int64_t lo, int64_t hi) {
    std::vector<int32_t> cand;
    for (int64_t i = lo; i < hi; i++) {
      cand.clear();
      for (int32_t s = inc_ptr[i]; s < inc_ptr[i + 1]; s++) {
        int64_t e = inc[4 * (size_t)s];
        for (int b = 0; b < nd; b++) cand.push_back(sp->dof[nd * e + b]);
      }
      std::sort(cand.begin(), cand.end());
      cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
      std::copy(cand.begin(), cand.end(), sp->colind.begin() + sp->rowptr[i]);
      for (int32_t s = inc_ptr[i]; s < inc_ptr[i + 1]; s++) {
        int64_t e = inc[4 * (size_t)s];
        uint32_t z = 0, w = 0;
        for (int b = 0; b < nd; b++) {
          uint32_t off = (uint32_t)(std::lower_bound(cand.begin(), cand.end(), sp->dof[nd * e + b]) - cand.begin());
          if (b < 3) z |= off << (10 * b);
          else w |= off << (10 * (b - 3));
        }
        inc[4 * (size_t)s + 2] = z;
        inc[4 * (size_t)s + 3] = w;
      }
    }
  });
  ADFEM_TRY(upload(sp->d_dof, sp->dof.data(), sp->dof.size()));
  ADFEM_TRY(upload(sp->d_area, m->area.data(), m->area.size()));
  ADFEM_TRY(upload(sp->d_rowptr, sp->rowptr.data(), sp->rowptr.size()));
  ADFEM_TRY(upload(sp->d_colind, sp->colind.data(), sp->colind.size()));
  ADFEM_TRY(upload(sp->d_inc_ptr, inc_ptr.data(), inc_ptr.size()));
  ADFEM_TRY(upload(sp->d_inc, inc.data(), inc.size()));
  m->space[degree] = std::move(sp);
  *out = m->space[degree].get();
  return ADFEM_OK;
}

}  // namespace adfem

int adfem_debug_fail_alloc(long long k) {
  adfem::arm_alloc_failure(k);
  return ADFEM_OK;
}

int adfem_debug_check_code(void) {
  const int parts[4] = {adfem::check_line_solver(), adfem::check_line_zcg(), adfem::check_line_assemble(),
                        adfem::check_line_generic()};
  for (int k = 0; k < 4; k++)
    if (parts[k] != 0) return parts[k] < 0 ? -1 : 100000 * (k + 1) + parts[k];
  return 0;
}
