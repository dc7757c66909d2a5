// Plane-strain material and 2-D linear-elasticity assembly for P1 triangles (sm_103a).
//
// Element matrix (ComputeFemStiffnessMatrixMfem.h:4-48): K_e = sum_k w B^T D_k B with
// B = [hx 0; 0 hy; hy hx] (3 x 6) and DOFs [u_x of the 3 vertices; u_y of the 3].
// For P1 B is constant over the element, so K_e = B^T Dbar_e B with
// Dbar_e = w sum_k D_k, formed once per element by a prepass.  Rows are then
// assembled like the scalar operator: one thread per matrix row walks the
// elements around its node in ascending element order, so each value is summed
// by one thread in a fixed order (bit-reproducible, no atomics).
#include "adfem_internal.h"
#include "elastic.cuh"

namespace adfem {

static constexpr int kB = 128;
__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
static inline unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

// ---------------------------------------------------------------------------
// PlaneStrainAndStress.h:5-78
__global__ void k_plane_strain(int mode, int64_t n, const double* __restrict__ E, const double* __restrict__ nu,
                               double* __restrict__ D) {
  const int64_t i = gtid();
  if (i >= n) return;
  const double e = E[i], v = nu[i];
  double* o = D + 9 * i;
  if (mode == 0) {
    const double s = e * (1 - v) / (1 + v) / (1 - 2 * v);
    const double a = s * v / (1 - v);
    o[0] = s; o[1] = a; o[2] = a;
    o[3] = a; o[4] = s; o[5] = a;
    o[6] = a; o[7] = a; o[8] = s;
  } else {
    const double s = e / (1 + v) / (1 - 2 * v);
    o[0] = s * (1 - v); o[1] = s * v; o[2] = 0.0;
    o[3] = s * v; o[4] = s * (1 - v); o[5] = 0.0;
    o[6] = 0.0; o[7] = 0.0; o[8] = s * (1 - 2 * v) / 2.0;
  }
}

// derivative of the entries above (the reference obtains it with an AD tape)
__global__ void k_plane_strain_backward(int mode, int64_t n, const double* __restrict__ g,
                                        const double* __restrict__ E, const double* __restrict__ nu,
                                        double* __restrict__ gE, double* __restrict__ gnu) {
  const int64_t i = gtid();
  if (i >= n) return;
  const double* q = g + 9 * i;
  const double v = nu[i], D = (1 + v) * (1 - 2 * v);
  if (mode == 0) {
    const double gd = q[0] + q[4] + q[8];
    const double go = q[1] + q[2] + q[3] + q[5] + q[6] + q[7];
    gE[i] = gd * (1 - v) / D + go * v / D;
    gnu[i] = E[i] * (gd * 2 * v * (2 - v) + go * (1 + 2 * v * v)) / (D * D);
  } else {
    const double a = q[0] + q[4], b = q[1] + q[3], c = q[8];
    gE[i] = (a * (1 - v) + b * v + c * (1 - 2 * v) / 2.0) / D;
    gnu[i] = E[i] * (a * 2 * v * (2 - v) / (D * D) + b * (1 + 2 * v * v) / (D * D) + c * -0.5 / ((1 + v) * (1 + v)));
  }
}

cudaError_t launch_plane_strain(int mode, int64_t n, const double* E, const double* nu, double* D, cudaStream_t st) {
  k_plane_strain<<<nblk(n, 256), 256, 0, st>>>(mode, n, E, nu, D);
  return cudaGetLastError();
}
cudaError_t launch_plane_strain_backward(int mode, int64_t n, const double* g, const double* E, const double* nu,
                                         double* gE, double* gnu, cudaStream_t st) {
  k_plane_strain_backward<<<nblk(n, 256), 256, 0, st>>>(mode, n, g, E, nu, gE, gnu);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Dbar_e = w * (D_0 + D_1 + D_2), 9 values per element
__global__ void k_stiffness_prepass(int64_t ne, const double* __restrict__ D, const double4* __restrict__ geo,
                                    double* __restrict__ Dbar) {
  const int64_t t = gtid();
  if (t >= 9 * ne) return;
  const int64_t e = t / 9;
  const int j = (int)(t - 9 * e);
  const double* d = D + 27 * e + j;
  Dbar[t] = geo[e].w * (d[0] + d[9] + d[18]);
}

// fused material: D_k = plane_strain(E_k, nu_k) (mode 0), Dbar as above
__global__ void k_stiffness_prepass_E(int64_t ne, const double* __restrict__ E, const double* __restrict__ nu,
                                      const double4* __restrict__ geo, double* __restrict__ Dbar) {
  const int64_t e = gtid();
  if (e >= ne) return;
  double sd = 0.0, so = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double ev = E[3 * e + k], v = nu[3 * e + k];
    const double s = ev * (1 - v) / (1 + v) / (1 - 2 * v);
    sd += s;
    so += s * v / (1 - v);
  }
  const double w = geo[e].w;
  sd *= w;
  so *= w;
  double* o = Dbar + 9 * e;
  o[0] = sd; o[1] = so; o[2] = so;
  o[3] = so; o[4] = sd; o[5] = so;
  o[6] = so; o[7] = so; o[8] = sd;
}

cudaError_t launch_stiffness_prepass(const Mesh& m, const double* D, double* Dbar, cudaStream_t st) {
  k_stiffness_prepass<<<nblk(9 * m.ne, 256), 256, 0, st>>>(m.ne, D, m.d_geo.as<double4>(), Dbar);
  return cudaGetLastError();
}
cudaError_t launch_stiffness_prepass_E(const Mesh& m, const double* E, const double* nu, double* Dbar,
                                       cudaStream_t st) {
  k_stiffness_prepass_E<<<nblk(m.ne, 256), 256, 0, st>>>(m.ne, E, nu, m.d_geo.as<double4>(), Dbar);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// One element's contribution to matrix row (c, a): local DOF l = a + 3c of element e,
// added to acc at slot offsets: x-column of vertex b -> ox(b), y-column -> oy(b).
// v = B(:,l)^T Dbar (or Dbar B(:,l) for the transpose), then entry(col) = v . B(:,col).
struct RowSlots {
  int x[3], y[3];
};

template <bool TRANSPOSE, int BT = kB>
__device__ __forceinline__ void elastic_row_add(const double* __restrict__ Db, const double2* __restrict__ gr, int a,
                                                int c, const RowSlots& sl, double (*acc)[BT], int t) {
  double d[9];
#pragma unroll
  for (int j = 0; j < 9; j++) d[j] = TRANSPOSE ? Db[(j % 3) * 3 + (j / 3)] : Db[j];
  const double2 ga = gr[a];
  double v0, v1, v2;
  if (c == 0) {  // B(:,a) = (hx_a, 0, hy_a)
    v0 = fma(ga.x, d[0], ga.y * d[6]);
    v1 = fma(ga.x, d[1], ga.y * d[7]);
    v2 = fma(ga.x, d[2], ga.y * d[8]);
  } else {  // B(:,a+3) = (0, hy_a, hx_a)
    v0 = fma(ga.y, d[3], ga.x * d[6]);
    v1 = fma(ga.y, d[4], ga.x * d[7]);
    v2 = fma(ga.y, d[5], ga.x * d[8]);
  }
#pragma unroll
  for (int b = 0; b < 3; b++) {
    const double2 gb = gr[b];
    acc[sl.x[b]][t] = fma(v0, gb.x, fma(v2, gb.y, acc[sl.x[b]][t]));
    acc[sl.y[b]][t] = fma(v1, gb.y, fma(v2, gb.x, acc[sl.y[b]][t]));
  }
}

// Reference [x-block; y-block] ordering, CSR rows r in [0, 2nv): node i = r mod nv,
// component c = r / nv.  Row r holds the scalar row of i twice: x columns then
// y columns.  Row pointer: x-rows at 2 rowptr[i], y-rows at 2 nnz + 2 rowptr[i].
// BT threads per block: kB for rows of up to 16 scalar entries; meshes with vertices of up
// to 63 neighbours (the most mesh_build accepts) take MAXW = 64 in blocks of 32 threads, so
// the accumulator stays at 32 KB of static shared memory.
template <int MAXW, bool TRANSPOSE, int BT = kB>
__global__ void __launch_bounds__(BT) k_stiffness_rows(int64_t nv, int64_t nnz, const int32_t* __restrict__ inc_ptr,
                                                       const uint2* __restrict__ inc,
                                                       const double2* __restrict__ grad,
                                                       const double* __restrict__ Dbar,
                                                       const int32_t* __restrict__ rowptr,
                                                       double* __restrict__ vals) {
  __shared__ double acc[2 * MAXW][BT];
  const int t = threadIdx.x;
  const int64_t r = gtid();
  if (r >= 2 * nv) return;
  const int c = r >= nv ? 1 : 0;
  const int64_t i = r - c * nv;
  const int w = rowptr[i + 1] - rowptr[i];
  for (int k = 0; k < 2 * w; k++) acc[k][t] = 0.0;
  for (int32_t s = inc_ptr[i]; s < inc_ptr[i + 1]; s++) {
    const uint2 rec = inc[s];
    const unsigned e = rec.x, y = rec.y, a = inc_a(y);
    RowSlots sl;
#pragma unroll
    for (int b = 0; b < 3; b++) {
      sl.x[b] = (int)inc_off(y, b);
      sl.y[b] = w + (int)inc_off(y, b);
    }
    elastic_row_add<TRANSPOSE, BT>(Dbar + 9 * (int64_t)e, grad + 3 * (int64_t)e, (int)a, c, sl, acc, t);
  }
  const int64_t base = c ? 2 * nnz + 2 * (int64_t)rowptr[i] : 2 * (int64_t)rowptr[i];
  for (int k = 0; k < 2 * w; k++) vals[base + k] = acc[k][t];
}

cudaError_t launch_stiffness_rows(const Mesh& m, const double* Dbar, double* vals, bool transpose, cudaStream_t st) {
  const auto* ip = m.d_inc_ptr.as<int32_t>();
  const auto* inc = m.d_inc.as<uint2>();
  const auto* gr = m.d_grad.as<double2>();
  const auto* rp = m.d_rowptr.as<int32_t>();
  const unsigned nb = nblk(2 * m.nv, kB);
  if (m.maxrow <= 8) {
    if (transpose) k_stiffness_rows<8, true><<<nb, kB, 0, st>>>(m.nv, m.nnz, ip, inc, gr, Dbar, rp, vals);
    else k_stiffness_rows<8, false><<<nb, kB, 0, st>>>(m.nv, m.nnz, ip, inc, gr, Dbar, rp, vals);
  } else if (m.maxrow <= 16) {
    if (transpose) k_stiffness_rows<16, true><<<nb, kB, 0, st>>>(m.nv, m.nnz, ip, inc, gr, Dbar, rp, vals);
    else k_stiffness_rows<16, false><<<nb, kB, 0, st>>>(m.nv, m.nnz, ip, inc, gr, Dbar, rp, vals);
  } else if (m.maxrow <= 64) {
    const unsigned nbw = nblk(2 * m.nv, 32);
    if (transpose) k_stiffness_rows<64, true, 32><<<nbw, 32, 0, st>>>(m.nv, m.nnz, ip, inc, gr, Dbar, rp, vals);
    else k_stiffness_rows<64, false, 32><<<nbw, 32, 0, st>>>(m.nv, m.nnz, ip, inc, gr, Dbar, rp, vals);
  } else {
    return cudaErrorNotSupported;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Fused elasticity system in the interleaved DOF order (2i = x, 2i+1 = y of node i),
// sliced-ELL.  Row 2i+c holds columns (2j, 2j+1) for each j of the scalar row of i:
// slot 2k is the x-column of the k-th neighbour, slot 2k+1 its y-column.
// isbd: 0 free, 1 Dirichlet DOF, 2 free with a Dirichlet neighbour (interleaved ids).
// rhs: body force [src(fx); src(fy)] interleaved, minus the Dirichlet lift.
// PERM: nodes renumbered (nperm[node]); row 2i+c goes to solver row 2 nperm[i] + c and
// slot 2k+cc to 2 kperm[rowptr[i] + k] + cc; isbd, bdval and rhs in solver order.
template <int MAXW, bool PERM>
__global__ void __launch_bounds__(kB) k_elastic_system(int64_t nv, const int32_t* __restrict__ inc_ptr,
                                                       const uint2* __restrict__ inc,
                                                       const double2* __restrict__ grad,
                                                       const double* __restrict__ Dbar,
                                                       const double* __restrict__ srcx,
                                                       const double* __restrict__ srcy,
                                                       const int32_t* __restrict__ rowptr,
                                                       const int32_t* __restrict__ colind,
                                                       const int32_t* __restrict__ sptr,
                                                       const uint8_t* __restrict__ isbd,
                                                       const double* __restrict__ bdval,
                                                       double* __restrict__ vals, double* __restrict__ rhs,
                                                       const int32_t* __restrict__ nperm,
                                                       const uint8_t* __restrict__ kperm) {
  __shared__ double acc[2 * MAXW][kB];
  const int t = threadIdx.x;
  const int64_t r = gtid();
  if (r >= 2 * nv) return;
  const int64_t i = r >> 1;
  const int c = (int)(r & 1);
  const int w = rowptr[i + 1] - rowptr[i];
  const int32_t r0 = rowptr[i];
  const int64_t rs = PERM ? 2 * (int64_t)nperm[i] + c : r;
  const int64_t base = (int64_t)sptr[rs >> 5] + (rs & 31);
  auto slot = [&](int k) { return PERM ? (int)kperm[r0 + k] : k; };
  const uint8_t tag = isbd[rs];
  if (tag == 1) {
    // diagonal: slot 2*diagpos + c
    const int32_t* row = colind + r0;
    int dk = 0;
    for (int k = 0; k < w; k++)
      if (row[k] == i) dk = k;
    const int ds = 2 * slot(dk) + c;
    for (int k = 0; k < 2 * w; k++) vals[base + 32 * k] = (k == ds) ? 1.0 : 0.0;
    rhs[rs] = bdval[rs];
    return;
  }
  for (int k = 0; k < 2 * w; k++) acc[k][t] = 0.0;
  double rr = 0.0;
  const double* src = c ? srcy : srcx;
  for (int32_t s = inc_ptr[i]; s < inc_ptr[i + 1]; s++) {
    const uint2 rec = inc[s];
    const unsigned e = rec.x, y = rec.y, a = inc_a(y);
    RowSlots sl;
#pragma unroll
    for (int b = 0; b < 3; b++) {
      sl.x[b] = 2 * (int)inc_off(y, b);
      sl.y[b] = 2 * (int)inc_off(y, b) + 1;
    }
    elastic_row_add<false>(Dbar + 9 * (int64_t)e, grad + 3 * (int64_t)e, (int)a, c, sl, acc, t);
    rr += src[3 * (int64_t)e + a];
  }
  if (tag == 2) {
    const int32_t* row = colind + r0;
    for (int k = 0; k < w; k++) {
      const int64_t j = PERM ? (int64_t)nperm[row[k]] : (int64_t)row[k];
#pragma unroll
      for (int cc = 0; cc < 2; cc++) {
        const int64_t dj = 2 * j + cc;
        if (isbd[dj] == 1) {
          rr = fma(-acc[2 * k + cc][t], bdval[dj], rr);
          acc[2 * k + cc][t] = 0.0;
        }
      }
    }
  }
  rhs[rs] = rr;
  for (int k = 0; k < w; k++) {
    const int sk = 2 * slot(k);
    vals[base + 32 * sk] = acc[2 * k][t];
    vals[base + 32 * (sk + 1)] = acc[2 * k + 1][t];
  }
}

cudaError_t launch_elastic_system(const Mesh& m, const double* Dbar, const double* srcx, const double* srcy,
                                  const int32_t* sptr2, const uint8_t* isbd2, const double* bdval2, double* vals,
                                  double* rhs, const int32_t* nperm, const uint8_t* kperm, cudaStream_t st) {
  const auto* ip = m.d_inc_ptr.as<int32_t>();
  const auto* inc = m.d_inc.as<uint2>();
  const auto* gr = m.d_grad.as<double2>();
  const auto* rp = m.d_rowptr.as<int32_t>();
  const auto* ci = m.d_colind.as<int32_t>();
  const unsigned nb = nblk(2 * m.nv, kB);
#define ADFEM_ES(W)                                                                                              \
  do {                                                                                                           \
    if (nperm)                                                                                                   \
      k_elastic_system<W, true><<<nb, kB, 0, st>>>(m.nv, ip, inc, gr, Dbar, srcx, srcy, rp, ci, sptr2, isbd2,    \
                                                   bdval2, vals, rhs, nperm, kperm);                            \
    else                                                                                                         \
      k_elastic_system<W, false><<<nb, kB, 0, st>>>(m.nv, ip, inc, gr, Dbar, srcx, srcy, rp, ci, sptr2, isbd2,   \
                                                    bdval2, vals, rhs, nullptr, nullptr);                       \
  } while (0)
  if (m.maxrow <= 8) ADFEM_ES(8);
  else if (m.maxrow <= 16) ADFEM_ES(16);
  else return cudaErrorNotSupported;
#undef ADFEM_ES
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Unsummed COO of ComputeFemStiffnessMatrixMfem_forward: thread per (e, k, l) writes
// the 6 entries of row l of NN_k = B^T D_k B w.  Entry index 108 e + 36 k + 6 l + s.
__global__ void k_stiffness_coo(int64_t ne, int64_t ndof, const int4* __restrict__ conn,
                                const double2* __restrict__ grad, const double4* __restrict__ geo,
                                const double* __restrict__ D, longlong2* __restrict__ idx, double* __restrict__ vv) {
  const int64_t t = gtid();
  if (t >= 18 * ne) return;
  const int64_t e = t / 18;
  const int rem = (int)(t - 18 * e);
  const int k = rem / 6, l = rem % 6;
  const int4 cn = conn[e];
  const int vtx[3] = {cn.x, cn.y, cn.z};
  const double2* gr = grad + 3 * e;
  const double* d = D + 27 * e + 9 * k;
  const double w = geo[e].w;
  const int a = l % 3;
  const double2 ga = gr[a];
  double v0, v1, v2;
  if (l < 3) {
    v0 = fma(ga.x, d[0], ga.y * d[6]);
    v1 = fma(ga.x, d[1], ga.y * d[7]);
    v2 = fma(ga.x, d[2], ga.y * d[8]);
  } else {
    v0 = fma(ga.y, d[3], ga.x * d[6]);
    v1 = fma(ga.y, d[4], ga.x * d[7]);
    v2 = fma(ga.y, d[5], ga.x * d[8]);
  }
  const long long row = vtx[a] + (l < 3 ? 0 : ndof);
  const int64_t z0 = 108 * e + 36 * k + 6 * l;
#pragma unroll
  for (int s = 0; s < 6; s++) {
    const int b = s % 3;
    const double2 gb = gr[b];
    const double val = s < 3 ? fma(v0, gb.x, v2 * gb.y) : fma(v1, gb.y, v2 * gb.x);
    idx[z0 + s] = make_longlong2(row, (long long)vtx[b] + (s < 3 ? 0 : ndof));
    vv[z0 + s] = val * w;
  }
}

cudaError_t launch_stiffness_coo(const Mesh& m, const double* D, long long* indices, double* vv, cudaStream_t st) {
  k_stiffness_coo<<<nblk(18 * m.ne, 256), 256, 0, st>>>(m.ne, m.nv, m.d_conn.as<int4>(), m.d_grad.as<double2>(),
                                                        m.d_geo.as<double4>(), D,
                                                        reinterpret_cast<longlong2*>(indices), vv);
  return cudaGetLastError();
}

// ComputeFemStiffnessMatrixMfem_backward: grad_D_k = w B G B^T, G = grad_vv block (6x6)
__global__ void k_stiffness_coo_backward(int64_t ne, const double2* __restrict__ grad,
                                         const double4* __restrict__ geo, const double* __restrict__ gvv,
                                         double* __restrict__ gD) {
  const int64_t t = gtid();
  if (t >= 3 * ne) return;
  const int64_t e = t / 3;
  const double2* gr = grad + 3 * e;
  const double* G = gvv + 36 * t;
  double B[3][6];
#pragma unroll
  for (int b = 0; b < 3; b++) {
    B[0][b] = gr[b].x; B[0][b + 3] = 0.0;
    B[1][b] = 0.0;     B[1][b + 3] = gr[b].y;
    B[2][b] = gr[b].y; B[2][b + 3] = gr[b].x;
  }
  double T[3][6];
#pragma unroll
  for (int p = 0; p < 3; p++)
#pragma unroll
    for (int s = 0; s < 6; s++) {
      double acc = 0.0;
#pragma unroll
      for (int l = 0; l < 6; l++)
        if (B[p][l] != 0.0) acc = fma(B[p][l], G[6 * l + s], acc);
      T[p][s] = acc;
    }
  const double w = geo[e].w;
#pragma unroll
  for (int p = 0; p < 3; p++)
#pragma unroll
    for (int q = 0; q < 3; q++) {
      double acc = 0.0;
#pragma unroll
      for (int s = 0; s < 6; s++) acc = fma(T[p][s], B[q][s], acc);
      gD[9 * t + 3 * p + q] = acc * w;
    }
}

cudaError_t launch_stiffness_coo_backward(const Mesh& m, const double* grad_vv, double* grad_D, cudaStream_t st) {
  k_stiffness_coo_backward<<<nblk(3 * m.ne, 256), 256, 0, st>>>(m.ne, m.d_grad.as<double2>(), m.d_geo.as<double4>(),
                                                                grad_vv, grad_D);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// dL/dE at each Gauss point: -w (B lam_e)^T (dD/dE) (B u_e), plane strain with the
// reference formula, lam zero on Dirichlet DOFs.  u, lam interleaved.
__global__ void k_elastic_grad_E(int64_t ne, const int4* __restrict__ conn, const double2* __restrict__ grad,
                                 const double4* __restrict__ geo, const double* __restrict__ u,
                                 const double* __restrict__ lam, const uint8_t* __restrict__ isbd2,
                                 const double* __restrict__ nu, double* __restrict__ gE) {
  const int64_t e = gtid();
  if (e >= ne) return;
  const int4 cn = conn[e];
  const int vtx[3] = {cn.x, cn.y, cn.z};
  const double2* gr = grad + 3 * e;
  double eu[3] = {0, 0, 0}, el[3] = {0, 0, 0};
#pragma unroll
  for (int b = 0; b < 3; b++) {
    const int64_t dx = 2 * (int64_t)vtx[b], dy = dx + 1;
    const double ux = u[dx], uy = u[dy];
    const double lx = isbd2[dx] == 1 ? 0.0 : lam[dx], ly = isbd2[dy] == 1 ? 0.0 : lam[dy];
    const double2 g = gr[b];
    eu[0] = fma(g.x, ux, eu[0]);
    eu[1] = fma(g.y, uy, eu[1]);
    eu[2] = fma(g.y, ux, fma(g.x, uy, eu[2]));
    el[0] = fma(g.x, lx, el[0]);
    el[1] = fma(g.y, ly, el[1]);
    el[2] = fma(g.y, lx, fma(g.x, ly, el[2]));
  }
  const double dd = el[0] * eu[0] + el[1] * eu[1] + el[2] * eu[2];
  const double all = (el[0] + el[1] + el[2]) * (eu[0] + eu[1] + eu[2]);
  const double off = all - dd;  // sum over p != q of el_p eu_q
  const double w = geo[e].w;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double v = nu[3 * e + k];
    const double den = (1 + v) * (1 - 2 * v);
    const double sp = (1 - v) / den, ap = v / den;  // dD/dE entries
    gE[3 * e + k] = -w * (sp * dd + ap * off);
  }
}

cudaError_t launch_elastic_grad_E(const Mesh& m, const double* u2, const double* lam2, const uint8_t* isbd2,
                                  const double* nu, double* gE, cudaStream_t st) {
  k_elastic_grad_E<<<nblk(m.ne, 256), 256, 0, st>>>(m.ne, m.d_conn.as<int4>(), m.d_grad.as<double2>(),
                                                    m.d_geo.as<double4>(), u2, lam2, isbd2, nu, gE);
  return cudaGetLastError();
}

// reference order <-> solver order through a DOF map: sol[map[d]] = ref[d]
__global__ void k_to_solver(int64_t n, const int32_t* __restrict__ map, const double* __restrict__ ref,
                            double* __restrict__ sol) {
  const int64_t d = gtid();
  if (d >= n) return;
  sol[map[d]] = ref[d];
}
__global__ void k_from_solver(int64_t n, const int32_t* __restrict__ map, const double* __restrict__ sol,
                              double* __restrict__ ref) {
  const int64_t d = gtid();
  if (d >= n) return;
  ref[d] = sol[map[d]];
}
cudaError_t launch_to_solver(int64_t n, const int32_t* map, const double* ref, double* sol, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_to_solver<<<nblk(n, 256), 256, 0, st>>>(n, map, ref, sol);
  return cudaGetLastError();
}
cudaError_t launch_from_solver(int64_t n, const int32_t* map, const double* sol, double* ref, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_from_solver<<<nblk(n, 256), 256, 0, st>>>(n, map, sol, ref);
  return cudaGetLastError();
}

// reference [x; y] <-> interleaved
__global__ void k_to_interleaved(int64_t nv, const double* __restrict__ ref, double* __restrict__ il) {
  const int64_t r = gtid();
  if (r >= 2 * nv) return;
  il[r] = ref[(r & 1) * nv + (r >> 1)];
}
__global__ void k_from_interleaved(int64_t nv, const double* __restrict__ il, double* __restrict__ ref) {
  const int64_t r = gtid();
  if (r >= 2 * nv) return;
  ref[(r & 1) * nv + (r >> 1)] = il[r];
}
cudaError_t launch_to_interleaved(int64_t nv, const double* ref, double* il, cudaStream_t st) {
  k_to_interleaved<<<nblk(2 * nv, 256), 256, 0, st>>>(nv, ref, il);
  return cudaGetLastError();
}
cudaError_t launch_from_interleaved(int64_t nv, const double* il, double* ref, cudaStream_t st) {
  k_from_interleaved<<<nblk(2 * nv, 256), 256, 0, st>>>(nv, il, ref);
  return cudaGetLastError();
}

}  // namespace adfem
