// Degree-generic element kernels for P1 and P2 Lagrange triangles: the reference's
// element loops written over elem_ndof and the per-point tables h, hx, hy, w
// (deps/MFEM/Common.cpp:46-126), for
//   FemLaplaceScalar forward/backward   deps/MFEM/FemLaplace1/FemLaplaceScalar.h:3-54
//   ComputeFemMassMatrix1 fwd/bwd       deps/MFEM/ComputeFemMassMatrix1/ComputeFemMassMatrixMfem.h:4-55
//   FemSourceScalar forward/backward    deps/MFEM/FemSource1/FemSourceScalar.h:4-32
//   ComputeFemStiffnessMatrixMfem       deps/MFEM/ComputeFemStiffnessMatrixMfem/ComputeFemStiffnessMatrixMfem.h:4-81
//   FemToGaussPoints / DofToGaussPoints deps/MFEM/FemToGaussPoints/FemToGaussPointsMfem.h:5-34,
//                                       deps/MFEM/DofToGaussPoints/DofToGaussPointsMfem.h:5-35
// and the summed (SparseMatrixCSC) operators of the Laplace, mass and elasticity
// matrices.  The P1 Laplace/source/stiffness path of P1 meshes has its own fused
// kernels (assemble.cu, elastic.cu); these serve P2 meshes and the mass and
// interpolation ops of both degrees.
//
// Layout: one thread per (Gauss point, local row) for the unsummed COO outputs, so a
// warp writes one contiguous stretch of entries; one thread per DOF row for every
// scatter (load vector, summed operators, interpolation transposes), walking the
// DOF->element incidence in ascending element order, so results are deterministic
// and no atomics are needed.  The per-point basis tables of the degree are built in
// shared memory by every block from the rule (a few hundred flops).
#include <mutex>

#include "adfem_internal.h"
#include "cg_common.cuh"
#include "checks.cuh"

namespace adfem {
namespace {

constexpr int kGT = 256;
constexpr int kRowBTs = 128;  // rows per block of the resident-system row kernel

// rule points (xi, eta, weight) on the reference triangle: order 2 (3 points, P1) and
// order 4 (6 points, P2: the published Strang-Fix/Dunavant rule); same constants as
// the host tables of mesh.cpp
__constant__ double c_rule[2][6][3] = {
    {{1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0},
     {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0},
     {2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0},
     {0.0, 0.0, 0.0},
     {0.0, 0.0, 0.0},
     {0.0, 0.0, 0.0}},
    {{0.091576213509770743460, 0.091576213509770743460, 0.054975871827660933819},
     {0.091576213509770743460, 0.81684757298045851308, 0.054975871827660933819},
     {0.81684757298045851308, 0.091576213509770743460, 0.054975871827660933819},
     {0.44594849091596488632, 0.44594849091596488632, 0.11169079483900573285},
     {0.44594849091596488632, 0.10810301816807022736, 0.11169079483900573285},
     {0.10810301816807022736, 0.44594849091596488632, 0.11169079483900573285}}};

template <int DEG>
struct Tab {
  static constexpr int ND = DEG == 2 ? 6 : 3;  // DOFs per element
  static constexpr int NG = DEG == 2 ? 6 : 3;  // Gauss points per element
  double h[NG][ND];     // phi_r at point k
  double t[NG][ND][3];  // d phi_r / d l_c at point k
  double l[NG][3];      // barycentric coordinates of point k
  double w[NG];         // rule weight of point k
};

// Lagrange basis in barycentric coordinates.  P1: phi_r = l_r.  P2 (nodes at the
// vertices and edge midpoints, vertex functions first, then edges (0,1), (1,2),
// (2,0)): phi_a = l_a (2 l_a - 1), phi_ab = 4 l_a l_b.
template <int DEG>
__device__ void tab_init(Tab<DEG>& T) {
  constexpr int ND = Tab<DEG>::ND, NG = Tab<DEG>::NG;
  for (int k = threadIdx.x; k < NG; k += blockDim.x) {
    const double xi = c_rule[DEG - 1][k][0], eta = c_rule[DEG - 1][k][1];
    const double l[3] = {1.0 - xi - eta, xi, eta};
    T.w[k] = c_rule[DEG - 1][k][2];
    for (int c = 0; c < 3; c++) T.l[k][c] = l[c];
    for (int r = 0; r < ND; r++) T.t[k][r][0] = T.t[k][r][1] = T.t[k][r][2] = 0.0;
    if (DEG == 1) {
      for (int r = 0; r < 3; r++) {
        T.h[k][r] = l[r];
        T.t[k][r][r] = 1.0;
      }
    } else {
      for (int a = 0; a < 3; a++) {
        T.h[k][a] = l[a] * (2.0 * l[a] - 1.0);
        T.t[k][a][a] = 4.0 * l[a] - 1.0;
      }
      for (int j = 0; j < 3; j++) {
        const int a = j, b = (j + 1) % 3;
        T.h[k][3 + j] = 4.0 * l[a] * l[b];
        T.t[k][3 + j][a] = 4.0 * l[b];
        T.t[k][3 + j][b] = 4.0 * l[a];
      }
    }
  }
  __syncthreads();
}

// physical gradient of basis r at point k: sum_c (d phi_r / d l_c) grad l_c
template <int DEG>
__device__ __forceinline__ void grad_at(const Tab<DEG>& T, int k, int r, const double2 (&g)[3], double& hx,
                                        double& hy) {
  const double t0 = T.t[k][r][0], t1 = T.t[k][r][1], t2 = T.t[k][r][2];
  hx = t0 * g[0].x + t1 * g[1].x + t2 * g[2].x;
  hy = t0 * g[0].y + t1 * g[1].y + t2 * g[2].y;
}

__device__ __forceinline__ void load_grad(const double2* __restrict__ grad, int64_t e, double2 (&g)[3]) {
  g[0] = grad[3 * e];
  g[1] = grad[3 * e + 1];
  g[2] = grad[3 * e + 2];
}

// w_k = ip.weight * area / 0.5 (Common.cpp:116)
template <int DEG>
__device__ __forceinline__ double weight_at(const Tab<DEG>& T, int k, double area) {
  return T.w[k] * area / 0.5;
}

int grid_for(int64_t n, int bt = kGT) {
  int64_t b = (n + bt - 1) / bt;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 32));
}

// ---------------------------------------------------------------- unsummed COO
template <int DEG, int OP>
__global__ void __launch_bounds__(kGT) k_gen_coo(int64_t ne, const int32_t* __restrict__ dof,
                                                 const double* __restrict__ area, const double2* __restrict__ grad,
                                                 const double* __restrict__ coef, long long* __restrict__ idx,
                                                 double* __restrict__ vv) {
  constexpr int ND = Tab<DEG>::ND, NG = Tab<DEG>::NG;
  __shared__ Tab<DEG> T;
  tab_init(T);
  const int64_t n = ne * NG * ND;
  for (int64_t t = gtid(); t < n; t += gstride()) {
    const int64_t gp = t / ND;
    const int p = (int)(t - gp * ND);
    const int64_t e = gp / NG;
    const int k = (int)(gp - e * NG);
    const double w = weight_at(T, k, area[e]);
    const double c = coef[gp];
    int32_t d[ND];
#pragma unroll
    for (int q = 0; q < ND; q++) d[q] = dof[ND * e + q];
    const int32_t dp = dof[ND * e + p];
    double2 g[3];
    double px = 0.0, py = 0.0;
    if (OP == (int)GenOp::LAPLACE) {
      load_grad(grad, e, g);
      grad_at(T, k, p, g, px, py);
    }
    const int64_t base = t * ND;
#pragma unroll
    for (int q = 0; q < ND; q++) {
      double v;
      if (OP == (int)GenOp::LAPLACE) {
        double qx, qy;
        grad_at(T, k, q, g, qx, qy);
        v = (px * qx + py * qy) * c * w;
      } else {
        v = T.h[k][p] * T.h[k][q] * c * w;
      }
      reinterpret_cast<longlong2*>(idx)[base + q] = make_longlong2(dp, d[q]);
      vv[base + q] = v;
    }
  }
}

// grad_coef[gp] = sum_pq grad_vv[gp, p, q] * (d N_pq / d coef): threads (gp, p) form
// the row sums, the gp's first thread adds the rows in order
template <int DEG, int OP>
__global__ void __launch_bounds__(64 * Tab<DEG>::ND) k_gen_coo_backward(int64_t ne, const double* __restrict__ area,
                                                                      const double2* __restrict__ grad,
                                                                      const double* __restrict__ gv,
                                                                      double* __restrict__ out) {
  constexpr int ND = Tab<DEG>::ND, NG = Tab<DEG>::NG;
  __shared__ Tab<DEG> T;
  __shared__ double part[64 * ND];
  tab_init(T);
  const int64_t ngp = ne * NG;
  const int64_t gp = (int64_t)blockIdx.x * 64 + threadIdx.x / ND;
  const int p = threadIdx.x % ND;
  double s = 0.0;
  if (gp < ngp) {
    const int64_t e = gp / NG;
    const int k = (int)(gp - e * NG);
    const double w = weight_at(T, k, area[e]);
    const double* row = gv + (gp * ND + p) * ND;
    if (OP == (int)GenOp::LAPLACE) {
      double2 g[3];
      load_grad(grad, e, g);
      double px, py;
      grad_at(T, k, p, g, px, py);
#pragma unroll
      for (int q = 0; q < ND; q++) {
        double qx, qy;
        grad_at(T, k, q, g, qx, qy);
        s += row[q] * ((px * qx + py * qy) * w);
      }
    } else {
#pragma unroll
      for (int q = 0; q < ND; q++) s += T.h[k][p] * T.h[k][q] * w * row[q];
    }
  }
  part[threadIdx.x] = s;
  __syncthreads();
  if (p == 0 && gp < ngp) {
    double v = 0.0;
#pragma unroll
    for (int r = 0; r < ND; r++) v += part[threadIdx.x + r];
    out[gp] = v;
  }
}

// B = [hx 0; 0 hy; hy hx] (3 x 2 nd), ComputeFemStiffnessMatrixMfem.h:18-23: column l
template <int ND>
__device__ __forceinline__ void bcol(const double (&hx)[ND], const double (&hy)[ND], int l, double& b0, double& b1,
                                     double& b2) {
  if (l < ND) {
    b0 = hx[l];
    b1 = 0.0;
    b2 = hy[l];
  } else {
    b0 = 0.0;
    b1 = hy[l - ND];
    b2 = hx[l - ND];
  }
}

// elasticity COO: thread (gp, l) writes row l of B^T K B w (2 nd entries)
template <int DEG>
__global__ void __launch_bounds__(kGT) k_gen_stiffness_coo(int64_t ne, int64_t ndof, const int32_t* __restrict__ dof,
                                                           const double* __restrict__ area,
                                                           const double2* __restrict__ grad,
                                                           const double* __restrict__ D, long long* __restrict__ idx,
                                                           double* __restrict__ vv) {
  constexpr int ND = Tab<DEG>::ND, NG = Tab<DEG>::NG, N2 = 2 * ND;
  __shared__ Tab<DEG> T;
  tab_init(T);
  const int64_t n = ne * NG * N2;
  for (int64_t t = gtid(); t < n; t += gstride()) {
    const int64_t gp = t / N2;
    const int l = (int)(t - gp * N2);
    const int64_t e = gp / NG;
    const int k = (int)(gp - e * NG);
    const double w = weight_at(T, k, area[e]);
    double2 g[3];
    load_grad(grad, e, g);
    double hx[ND], hy[ND];
#pragma unroll
    for (int r = 0; r < ND; r++) grad_at(T, k, r, g, hx[r], hy[r]);
    const double* K = D + 9 * gp;
    double b0, b1, b2;
    bcol<ND>(hx, hy, l, b0, b1, b2);
    double tq[3];
#pragma unroll
    for (int q = 0; q < 3; q++) tq[q] = b0 * K[q] + b1 * K[3 + q] + b2 * K[6 + q];
    const long long dl = (long long)dof[ND * e + (l % ND)] + (l >= ND ? ndof : 0);
    const int64_t base = t * N2;
#pragma unroll
    for (int c = 0; c < N2; c++) {
      double c0, c1, c2;
      bcol<ND>(hx, hy, c, c0, c1, c2);
      const long long dc = (long long)dof[ND * e + (c % ND)] + (c >= ND ? ndof : 0);
      reinterpret_cast<longlong2*>(idx)[base + c] = make_longlong2(dl, dc);
      vv[base + c] = (tq[0] * c0 + tq[1] * c1 + tq[2] * c2) * w;
    }
  }
}

// grad_D[gp] = w B G B^T: thread (gp, l) reads row l of G and contributes
// B[:, l] (G[l, :] B^T); the gp's threads then add the 2 nd rows, in order, for each of the nine entries
template <int DEG>
__global__ void __launch_bounds__(32 * 2 * Tab<DEG>::ND) k_gen_stiffness_coo_backward(
    int64_t ne, const double* __restrict__ area, const double2* __restrict__ grad, const double* __restrict__ gv,
    double* __restrict__ out) {
  constexpr int ND = Tab<DEG>::ND, NG = Tab<DEG>::NG, N2 = 2 * ND;
  __shared__ Tab<DEG> T;
  __shared__ double part[32 * N2][9];
  tab_init(T);
  const int64_t ngp = ne * NG;
  const int slot = threadIdx.x / N2;
  const int64_t gp = (int64_t)blockIdx.x * 32 + slot;
  const int l = threadIdx.x % N2;
  double acc[9];
#pragma unroll
  for (int j = 0; j < 9; j++) acc[j] = 0.0;
  double w = 0.0;
  if (gp < ngp) {
    const int64_t e = gp / NG;
    const int k = (int)(gp - e * NG);
    w = weight_at(T, k, area[e]);
    double2 g[3];
    load_grad(grad, e, g);
    double hx[ND], hy[ND];
#pragma unroll
    for (int r = 0; r < ND; r++) grad_at(T, k, r, g, hx[r], hy[r]);
    const double* row = gv + (gp * N2 + l) * N2;
    double u[3] = {0.0, 0.0, 0.0};  // G[l, :] B^T
#pragma unroll
    for (int c = 0; c < N2; c++) {
      double c0, c1, c2;
      bcol<ND>(hx, hy, c, c0, c1, c2);
      const double gl = row[c];
      u[0] += gl * c0;
      u[1] += gl * c1;
      u[2] += gl * c2;
    }
    double b[3];
    bcol<ND>(hx, hy, l, b[0], b[1], b[2]);
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int q = 0; q < 3; q++) acc[3 * a + q] = b[a] * u[q];
  }
#pragma unroll
  for (int j = 0; j < 9; j++) part[threadIdx.x][j] = acc[j];
  __syncthreads();
  if (gp < ngp)
    for (int j = l; j < 9; j += N2) {  // 2 nd threads per point write its 9 entries
      double v = 0.0;
      for (int r = 0; r < N2; r++) v += part[slot * N2 + r][j];
      out[9 * gp + j] = v * w;
    }
}

// ---------------------------------------------------------------- summed operators
// Gradients of every basis function at point k with compile-time indices (the P2
// vertex functions depend on one barycentric gradient, the edge functions on two).
template <int DEG>
__device__ __forceinline__ void grads_all(const Tab<DEG>& T, int k, const double2 (&g)[3],
                                          double (&hx)[Tab<DEG>::ND], double (&hy)[Tab<DEG>::ND]) {
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double t = T.t[k][a][a];
    hx[a] = t * g[a].x;
    hy[a] = t * g[a].y;
  }
  if constexpr (DEG == 2) {
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int a = j, b = (j + 1) % 3;
      const double ta = T.t[k][3 + j][a], tb = T.t[k][3 + j][b];
      hx[3 + j] = ta * g[a].x + tb * g[b].x;
      hy[3 + j] = ta * g[a].y + tb * g[b].y;
    }
  }
}

// packed index of (a, b), a <= b, in the upper triangle of an nd x nd matrix
__host__ __device__ constexpr int sym_idx(int nd, int a, int b) { return a * nd - a * (a - 1) / 2 + (b - a); }

// Laplace / mass element matrices, one thread per element: the nd (nd + 1) / 2 distinct
// entries of sum_k coef_k w_k N_k, stored as the full nd x nd matrix of the element
// (row-major, ke[(e * nd + a) * nd + b]) so that a row gather reads one contiguous row.
template <int DEG, int OP>
__global__ void __launch_bounds__(kGT) k_gen_ke(int64_t ne, const double* __restrict__ area,
                                                const double2* __restrict__ grad, const double* __restrict__ coef,
                                                double* __restrict__ ke) {
  constexpr int ND = Tab<DEG>::ND, NG = Tab<DEG>::NG, NS = ND * (ND + 1) / 2;
  __shared__ Tab<DEG> T;
  tab_init(T);
  for (int64_t e = gtid(); e < ne; e += gstride()) {
    const double ar = area[e];
    double2 g[3];
    if (OP == (int)GenOp::LAPLACE) load_grad(grad, e, g);
    double acc[NS];
#pragma unroll
    for (int j = 0; j < NS; j++) acc[j] = 0.0;
#pragma unroll 1
    for (int k = 0; k < NG; k++) {
      const double cw = coef[NG * e + k] * weight_at(T, k, ar);
      if (OP == (int)GenOp::LAPLACE) {
        double hx[ND], hy[ND];
        grads_all(T, k, g, hx, hy);
#pragma unroll
        for (int a = 0; a < ND; a++)
#pragma unroll
          for (int b = a; b < ND; b++) acc[sym_idx(ND, a, b)] += (hx[a] * hx[b] + hy[a] * hy[b]) * cw;
      } else {
#pragma unroll
        for (int a = 0; a < ND; a++)
#pragma unroll
          for (int b = a; b < ND; b++) acc[sym_idx(ND, a, b)] += T.h[k][a] * T.h[k][b] * cw;
      }
    }
    double* out = ke + e * ND * ND;
#pragma unroll
    for (int a = 0; a < ND; a++)
#pragma unroll
      for (int b = 0; b < ND; b++) out[a * ND + b] = acc[a <= b ? sym_idx(ND, a, b) : sym_idx(ND, b, a)];
  }
}

// elasticity element matrices (2 nd x 2 nd, not symmetric for a general D): thread
// (l, e) forms row l of sum_k w_k B_k^T D_k B_k, elements fastest so that a warp shares
// l; stored row-major per element, ke[(e * 2nd + l) * 2nd + c]
template <int DEG>
__global__ void __launch_bounds__(kGT) k_gen_ke_stiffness(int64_t ne, const double* __restrict__ area,
                                                          const double2* __restrict__ grad,
                                                          const double* __restrict__ D, double* __restrict__ ke) {
  constexpr int ND = Tab<DEG>::ND, NG = Tab<DEG>::NG, N2 = 2 * ND;
  __shared__ Tab<DEG> T;
  tab_init(T);
  const int64_t n = ne * N2;
  for (int64_t t = gtid(); t < n; t += gstride()) {
    const int l = (int)(t / ne);
    const int64_t e = t - (int64_t)l * ne;
    const int r = l < ND ? l : l - ND;
    const double ar = area[e];
    double2 g[3];
    load_grad(grad, e, g);
    double row[N2];
#pragma unroll
    for (int c = 0; c < N2; c++) row[c] = 0.0;
#pragma unroll 1
    for (int k = 0; k < NG; k++) {
      const double w = weight_at(T, k, ar);
      double hx[ND], hy[ND];
      grads_all(T, k, g, hx, hy);
      double rx, ry;  // gradient of the row's own basis function
      grad_at(T, k, r, g, rx, ry);
      const double* K = D + 9 * (NG * e + k);
      // column l of B: (rx, 0, ry) for an x row, (0, ry, rx) for a y row
      const double b0 = l < ND ? rx : 0.0, b1 = l < ND ? 0.0 : ry, b2 = l < ND ? ry : rx;
      double tq[3];
#pragma unroll
      for (int q = 0; q < 3; q++) tq[q] = (b0 * K[q] + b1 * K[3 + q] + b2 * K[6 + q]) * w;
#pragma unroll
      for (int c = 0; c < ND; c++) {
        row[c] += tq[0] * hx[c] + tq[2] * hy[c];       // column (c, x): B[:, c] = (hx, 0, hy)
        row[ND + c] += tq[1] * hy[c] + tq[2] * hx[c];  // column (c, y): B[:, c + nd] = (0, hy, hx)
      }
    }
    double* out = ke + (e * N2 + l) * N2;
#pragma unroll
    for (int c = 0; c < N2; c++) out[c] = row[c];
  }
}

// Summed rows, one thread per scalar DOF row (every FP64 add of a warp does 32 rows'
// work): the row is accumulated in a per-thread shared-memory buffer of CAP entries in
// ascending element order, then written out.  The block's rows occupy one contiguous
// range of vals, written by the whole block in order.  NB = 1: scalar operator (row of
// len entries).  NB = 2: [x; y] elasticity blocks; the thread owns the x row at
// 2 rowptr[i] and the y row at 2 nnz + 2 rowptr[i], each with the x columns, then the y
// columns, of the scalar row; transpose gives the CSC values.  Rows longer than the
// buffer are summed in place in global memory.
template <int DEG, int NB, int BT, int CAP>
__global__ void __launch_bounds__(BT) k_gen_rows(int64_t ndof, int64_t nnz, const int32_t* __restrict__ rowptr,
                                                 const int32_t* __restrict__ inc_ptr, const uint4* __restrict__ inc,
                                                 const double* __restrict__ ke, double* __restrict__ vals,
                                                 bool transpose) {
  constexpr int ND = Tab<DEG>::ND, KN = NB * ND;  // element matrix is KN x KN
  extern __shared__ double buf[];                 // [NB][CAP][BT]
  __shared__ int32_t srp[BT + 1];
  const int tid = threadIdx.x;
  for (int64_t i0 = (int64_t)blockIdx.x * BT; i0 < ndof; i0 += (int64_t)gridDim.x * BT) {
    const int nrow = (int)std::min<int64_t>(BT, ndof - i0);
    __syncthreads();  // previous tile's write-out done with buf / srp
    if (tid < nrow) srp[tid] = rowptr[i0 + tid];
    if (tid == 0) srp[nrow] = rowptr[i0 + nrow];
    const int64_t i = i0 + tid;
    int len = 0;
    if (tid < nrow) {
      len = rowptr[i + 1] - rowptr[i];
      const int rl = NB * len;  // entries of each of the thread's NB rows
      const bool fits = rl <= CAP;
      const int64_t gb[2] = {NB * (int64_t)rowptr[i], 2 * nnz + 2 * (int64_t)rowptr[i]};
#pragma unroll
      for (int rc = 0; rc < NB; rc++)
        for (int j = 0; j < rl; j++) {
          if (fits) buf[(rc * CAP + j) * BT + tid] = 0.0;
          else vals[gb[rc] + j] = 0.0;
        }
      for (int32_t s = inc_ptr[i]; s < inc_ptr[i + 1]; s++) {
        const uint4 r = inc[s];
        const double* K = ke + (int64_t)r.x * KN * KN;
#pragma unroll
        for (int rc = 0; rc < NB; rc++) {
          const int li = (int)r.y + rc * ND;
#pragma unroll
          for (int cb = 0; cb < NB; cb++)
#pragma unroll
            for (int b = 0; b < ND; b++) {
              const int lj = b + cb * ND;
              const double v = transpose ? K[lj * KN + li] : K[li * KN + lj];
              const int j = (int)space_off(r, b) + cb * len;
              if (fits) buf[(rc * CAP + j) * BT + tid] += v;
              else vals[gb[rc] + j] += v;
            }
        }
      }
      if (!fits) len = -1;  // written in place
    }
    __syncthreads();
    // write-out: the tile's rows of each block are contiguous in vals
    const int64_t b0 = srp[0], b1 = srp[nrow];
    for (int rc = 0; rc < NB; rc++) {
      const int64_t out0 = rc == 0 ? NB * b0 : 2 * nnz + 2 * b0;
      const int64_t total = NB * (b1 - b0);
      for (int64_t q = tid; q < total; q += BT) {
        // row of entry q: the last row whose start (in this block's entries) is <= q
        int lo = 0, hi = nrow - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if ((int64_t)NB * (srp[mid] - b0) <= q) lo = mid;
          else hi = mid - 1;
        }
        const int rlen = NB * (srp[lo + 1] - srp[lo]);
        if (rlen > CAP) continue;  // that row was summed in place
        const int j = (int)(q - (int64_t)NB * (srp[lo] - b0));
        vals[out0 + q] = buf[(rc * CAP + j) * BT + lo];
      }
    }
  }
}

// ---------------------------------------------------------------- load vector
template <int DEG>
__global__ void __launch_bounds__(kGT) k_gen_source(int64_t ndof, const int32_t* __restrict__ inc_ptr,
                                                    const uint4* __restrict__ inc, const double* __restrict__ area,
                                                    const double* __restrict__ f, double* __restrict__ rhs,
                                                    bool accumulate) {
  constexpr int NG = Tab<DEG>::NG;
  __shared__ Tab<DEG> T;
  tab_init(T);
  for (int64_t i = gtid(); i < ndof; i += gstride()) {
    double acc = accumulate ? rhs[i] : 0.0;
    for (int32_t s = inc_ptr[i]; s < inc_ptr[i + 1]; s++) {
      const uint4 r = inc[s];
      const double ar = area[r.x];
#pragma unroll
      for (int k = 0; k < NG; k++) acc += f[(int64_t)r.x * NG + k] * T.h[k][r.y] * weight_at(T, k, ar);
    }
    rhs[i] = acc;
  }
}

template <int DEG>
__global__ void __launch_bounds__(kGT) k_gen_source_backward(int64_t ne, const int32_t* __restrict__ dof,
                                                             const double* __restrict__ area,
                                                             const double* __restrict__ grhs,
                                                             double* __restrict__ gf) {
  constexpr int ND = Tab<DEG>::ND, NG = Tab<DEG>::NG;
  __shared__ Tab<DEG> T;
  tab_init(T);
  for (int64_t gp = gtid(); gp < ne * NG; gp += gstride()) {
    const int64_t e = gp / NG;
    const int k = (int)(gp - e * NG);
    const double w = weight_at(T, k, area[e]);
    double v = 0.0;
#pragma unroll
    for (int r = 0; r < ND; r++) v += T.h[k][r] * w * grhs[dof[ND * e + r]];
    gf[gp] = v;
  }
}

// ---------------------------------------------------------------- interpolation
template <int DEG, bool VERT>
__global__ void __launch_bounds__(kGT) k_gen_to_gauss(int64_t ne, const int4* __restrict__ conn,
                                                      const int32_t* __restrict__ dof, const double* __restrict__ u,
                                                      double* __restrict__ out) {
  constexpr int ND = Tab<DEG>::ND, NG = Tab<DEG>::NG;
  __shared__ Tab<DEG> T;
  tab_init(T);
  for (int64_t gp = gtid(); gp < ne * NG; gp += gstride()) {
    const int64_t e = gp / NG;
    const int k = (int)(gp - e * NG);
    double v;
    if (VERT) {
      const int4 c = conn[e];
      v = u[c.x] * T.l[k][0] + u[c.y] * T.l[k][1] + u[c.z] * T.l[k][2];
    } else {
      v = 0.0;
#pragma unroll
      for (int r = 0; r < ND; r++) v += u[dof[ND * e + r]] * T.h[k][r];
    }
    out[gp] = v;
  }
}

// transposes: VERT walks the vertex->element incidence of the mesh (local vertex in
// the low bits of the record), else the space's DOF->element incidence
template <int DEG, bool VERT>
__global__ void __launch_bounds__(kGT) k_gen_to_gauss_backward(int64_t nrow, const int32_t* __restrict__ inc_ptr,
                                                               const void* __restrict__ incp,
                                                               const double* __restrict__ gout,
                                                               double* __restrict__ gu, bool accumulate) {
  constexpr int NG = Tab<DEG>::NG;
  __shared__ Tab<DEG> T;
  tab_init(T);
  for (int64_t i = gtid(); i < nrow; i += gstride()) {
    double acc = accumulate ? gu[i] : 0.0;
    for (int32_t s = inc_ptr[i]; s < inc_ptr[i + 1]; s++) {
      int64_t e;
      int a;
      if (VERT) {
        const uint2 r = reinterpret_cast<const uint2*>(incp)[s];
        e = r.x;
        a = (int)inc_a(r.y);
      } else {
        const uint4 r = reinterpret_cast<const uint4*>(incp)[s];
        e = r.x;
        a = (int)r.y;
      }
#pragma unroll
      for (int k = 0; k < NG; k++) acc += gout[e * NG + k] * (VERT ? T.l[k][a] : T.h[k][a]);
    }
    gu[i] = acc;
  }
}

// ---------------------------------------------------------------- resident P2 systems
// Poisson system rows of a degree-DEG space: one thread per DOF row i (space order), the
// row summed from the element matrices ke in ascending element order, the load
// sum_e sum_k f_k phi_a(x_k) w_k over the same incidence, and the Dirichlet condition
// applied as by the P1 system kernel: a Dirichlet row (tag 1) becomes the identity row
// with rhs = bdval; a row next to Dirichlet DOFs (tag 2) moves those columns into the
// right-hand side lift.  Values go to the system's sliced-ELL operator: row nperm[i],
// slot kperm[rowptr[i] + k] (identity without renumbering); isbd, bdval, rhs in solver
// order.  Deterministic: every value is summed by one thread in a fixed order.
template <int DEG, int MAXW>
__global__ void __launch_bounds__(kRowBTs) k_gen_poisson_rows(
    int64_t ndof, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
    const int32_t* __restrict__ inc_ptr, const uint4* __restrict__ inc, const double* __restrict__ area,
    const double* __restrict__ ke, const double* __restrict__ f, const int32_t* __restrict__ sptr,
    const uint8_t* __restrict__ isbd, const double* __restrict__ bdval, double* __restrict__ vals,
    double* __restrict__ rhs, const int32_t* __restrict__ nperm, const uint8_t* __restrict__ kperm,
    const int32_t* __restrict__ diagpos) {
  constexpr int ND = Tab<DEG>::ND, NG = Tab<DEG>::NG;
  __shared__ Tab<DEG> T;
  __shared__ double acc[MAXW][kRowBTs];
  tab_init(T);
  const int t = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * kRowBTs + t;
  if (i >= ndof) return;
  const int32_t r0 = rowptr[i];
  const int w = rowptr[i + 1] - r0;
  const int64_t ri = nperm ? (int64_t)nperm[i] : i;
  const int64_t base = (int64_t)sptr[ri >> 5] + (ri & 31);
  const uint8_t tag = isbd[ri];
  auto slot = [&](int k) -> int64_t { return base + 32 * (int64_t)(kperm ? (int)kperm[r0 + k] : k); };
  if (tag == 1) {
    const int dp = diagpos[i];
    for (int k = 0; k < w; k++) vals[slot(k)] = (k == dp) ? 1.0 : 0.0;
    rhs[ri] = bdval[ri];
    return;
  }
  for (int k = 0; k < w; k++) acc[k][t] = 0.0;
  double r = 0.0;
  for (int32_t s = inc_ptr[i]; s < inc_ptr[i + 1]; s++) {
    const uint4 rec = inc[s];
    const int a = (int)rec.y;
    const double* K = ke + ((int64_t)rec.x * ND + a) * ND;
#pragma unroll
    for (int b = 0; b < ND; b++) {
      const unsigned o = space_off(rec, b);
      if (!ADFEM_DCHECK(o < (unsigned)w && o < (unsigned)MAXW)) continue;
      acc[o][t] += K[b];
    }
    const double ar = area[rec.x];
#pragma unroll
    for (int k = 0; k < NG; k++) r += f[(int64_t)rec.x * NG + k] * T.h[k][a] * weight_at(T, k, ar);
  }
  if (tag == 2) {
    for (int k = 0; k < w; k++) {
      const int64_t j = nperm ? (int64_t)nperm[colind[r0 + k]] : (int64_t)colind[r0 + k];
      if (isbd[j] == 1) {
        r = fma(-acc[k][t], bdval[j], r);
        acc[k][t] = 0.0;
      }
    }
  }
  rhs[ri] = r;
  for (int k = 0; k < w; k++) vals[slot(k)] = acc[k][t];
}

// dL/dkappa at Gauss point k of element e for the resident system: -w_k grad(lam).grad(u)
// at x_k, lam zero on the Dirichlet DOFs (isbd_ref in space order) -- the composition of
// the sparse-solve gradient (-lam_i u_j per entry), the Dirichlet backward and the
// FemLaplaceScalar backward, with the element matrix's rank-one structure per point.
template <int DEG>
__global__ void __launch_bounds__(kGT) k_gen_kappa_grad(int64_t ne, const int32_t* __restrict__ dof,
                                                        const double* __restrict__ area,
                                                        const double2* __restrict__ grad,
                                                        const double* __restrict__ u, const double* __restrict__ lam,
                                                        const uint8_t* __restrict__ isbd, double* __restrict__ gk) {
  constexpr int ND = Tab<DEG>::ND, NG = Tab<DEG>::NG;
  __shared__ Tab<DEG> T;
  tab_init(T);
  for (int64_t gp = gtid(); gp < ne * NG; gp += gstride()) {
    const int64_t e = gp / NG;
    const int k = (int)(gp - e * NG);
    double2 g[3];
    load_grad(grad, e, g);
    double hx[ND], hy[ND];
    grads_all(T, k, g, hx, hy);
    double ux = 0.0, uy = 0.0, lx = 0.0, ly = 0.0;
#pragma unroll
    for (int b = 0; b < ND; b++) {
      const int32_t d = dof[ND * e + b];
      const double ub = u[d];
      const double lb = isbd[d] == 1 ? 0.0 : lam[d];
      ux = fma(hx[b], ub, ux);
      uy = fma(hy[b], ub, uy);
      lx = fma(hx[b], lb, lx);
      ly = fma(hy[b], lb, ly);
    }
    gk[gp] = -weight_at(T, k, area[e]) * fma(lx, ux, ly * uy);
  }
}

// ---------------------------------------------------------------- PCL
__global__ void __launch_bounds__(kGT) k_fill(int64_t n, double v, double* __restrict__ out) {
  for (int64_t i = gtid(); i < n; i += gstride()) out[i] = v;
}

// H[gp + nz * ng] = vv[nz] for the nd^2 entries nz of Gauss point gp (column-major
// ngauss x nd^2 ngauss, pcl_FemLaplaceScalar_Jacobian, FemLaplaceScalar.h:63-91)
__global__ void __launch_bounds__(kGT) k_pcl_scatter(int64_t N, int nd2, int64_t ng, const double* __restrict__ vv,
                                                     double* __restrict__ H) {
  for (int64_t nz = gtid(); nz < N; nz += gstride()) H[nz / nd2 + nz * ng] = vv[nz];
}

}  // namespace

cudaError_t launch_fill(int64_t n, double v, double* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_fill<<<grid_for(n), kGT, 0, st>>>(n, v, out);
  return cudaGetLastError();
}

cudaError_t launch_pcl_scatter(int64_t N, int nd2, int64_t ng, const double* vv, double* H, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  k_pcl_scatter<<<grid_for(N), kGT, 0, st>>>(N, nd2, ng, vv, H);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- launchers
#define GEN_DISPATCH(sp, KERNEL_CALL1, KERNEL_CALL2) \
  do {                                               \
    if ((sp).degree == 2) {                          \
      KERNEL_CALL2;                                  \
    } else {                                         \
      KERNEL_CALL1;                                  \
    }                                                \
  } while (0)

cudaError_t launch_gen_coo(const Mesh& m, const Space& sp, GenOp op, const double* coef, long long* indices,
                           double* vv, cudaStream_t st) {
  const int64_t n = m.ne * sp.ng * sp.nd;
  const int g = grid_for(n);
  const int32_t* dof = sp.d_dof.as<int32_t>();
  const double* area = sp.d_area.as<double>();
  const double2* grad = m.d_grad.as<double2>();
  if (op == GenOp::LAPLACE)
    GEN_DISPATCH(sp, (k_gen_coo<1, 0><<<g, kGT, 0, st>>>(m.ne, dof, area, grad, coef, indices, vv)),
                 (k_gen_coo<2, 0><<<g, kGT, 0, st>>>(m.ne, dof, area, grad, coef, indices, vv)));
  else
    GEN_DISPATCH(sp, (k_gen_coo<1, 1><<<g, kGT, 0, st>>>(m.ne, dof, area, grad, coef, indices, vv)),
                 (k_gen_coo<2, 1><<<g, kGT, 0, st>>>(m.ne, dof, area, grad, coef, indices, vv)));
  return cudaGetLastError();
}

cudaError_t launch_gen_coo_backward(const Mesh& m, const Space& sp, GenOp op, const double* grad_vv, double* grad_coef,
                                    cudaStream_t st) {
  const int64_t ngp = m.ne * sp.ng;
  if (ngp == 0) return cudaSuccess;
  const int g = (int)((ngp + 63) / 64);
  const double* area = sp.d_area.as<double>();
  const double2* grad = m.d_grad.as<double2>();
  if (op == GenOp::LAPLACE)
    GEN_DISPATCH(sp, (k_gen_coo_backward<1, 0><<<g, 64 * 3, 0, st>>>(m.ne, area, grad, grad_vv, grad_coef)),
                 (k_gen_coo_backward<2, 0><<<g, 64 * 6, 0, st>>>(m.ne, area, grad, grad_vv, grad_coef)));
  else
    GEN_DISPATCH(sp, (k_gen_coo_backward<1, 1><<<g, 64 * 3, 0, st>>>(m.ne, area, grad, grad_vv, grad_coef)),
                 (k_gen_coo_backward<2, 1><<<g, 64 * 6, 0, st>>>(m.ne, area, grad, grad_vv, grad_coef)));
  return cudaGetLastError();
}

cudaError_t launch_gen_stiffness_coo(const Mesh& m, const Space& sp, const double* D, long long* indices, double* vv,
                                     cudaStream_t st) {
  const int g = grid_for(m.ne * sp.ng * 2 * sp.nd);
  const int32_t* dof = sp.d_dof.as<int32_t>();
  const double* area = sp.d_area.as<double>();
  const double2* grad = m.d_grad.as<double2>();
  GEN_DISPATCH(sp, (k_gen_stiffness_coo<1><<<g, kGT, 0, st>>>(m.ne, sp.ndof, dof, area, grad, D, indices, vv)),
               (k_gen_stiffness_coo<2><<<g, kGT, 0, st>>>(m.ne, sp.ndof, dof, area, grad, D, indices, vv)));
  return cudaGetLastError();
}

cudaError_t launch_gen_stiffness_coo_backward(const Mesh& m, const Space& sp, const double* grad_vv, double* grad_D,
                                              cudaStream_t st) {
  const int64_t ngp = m.ne * sp.ng;
  if (ngp == 0) return cudaSuccess;
  const int g = (int)((ngp + 31) / 32);
  const double* area = sp.d_area.as<double>();
  const double2* grad = m.d_grad.as<double2>();
  GEN_DISPATCH(sp, (k_gen_stiffness_coo_backward<1><<<g, 32 * 6, 0, st>>>(m.ne, area, grad, grad_vv, grad_D)),
               (k_gen_stiffness_coo_backward<2><<<g, 32 * 12, 0, st>>>(m.ne, area, grad, grad_vv, grad_D)));
  return cudaGetLastError();
}

constexpr int kRowBT = 128;     // rows per block of the row gathers
constexpr int kRowCap1 = 32;    // buffered entries per scalar row
constexpr int kRowCap2 = 48;    // buffered entries per elasticity row (x and y columns)

cudaError_t launch_gen_matrix(const Mesh& m, const Space& sp, GenOp op, const double* coef, double* ke, double* vals,
                              bool transpose, cudaStream_t st) {
  (void)transpose;  // Laplace and mass element matrices are symmetric: CSR and CSC values agree
  const int g = grid_for(m.ne);
  const double* area = sp.d_area.as<double>();
  const double2* grad = m.d_grad.as<double2>();
  if (op == GenOp::LAPLACE)
    GEN_DISPATCH(sp, (k_gen_ke<1, 0><<<g, kGT, 0, st>>>(m.ne, area, grad, coef, ke)),
                 (k_gen_ke<2, 0><<<g, kGT, 0, st>>>(m.ne, area, grad, coef, ke)));
  else
    GEN_DISPATCH(sp, (k_gen_ke<1, 1><<<g, kGT, 0, st>>>(m.ne, area, grad, coef, ke)),
                 (k_gen_ke<2, 1><<<g, kGT, 0, st>>>(m.ne, area, grad, coef, ke)));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int gr = grid_for(sp.ndof, kRowBT);
  const size_t smem = sizeof(double) * kRowCap1 * kRowBT;
  const int32_t* rp = sp.d_rowptr.as<int32_t>();
  const int32_t* ip = sp.d_inc_ptr.as<int32_t>();
  const uint4* inc = sp.d_inc.as<uint4>();
  GEN_DISPATCH(sp,
               (k_gen_rows<1, 1, kRowBT, kRowCap1><<<gr, kRowBT, smem, st>>>(sp.ndof, sp.nnz, rp, ip, inc, ke, vals,
                                                                              false)),
               (k_gen_rows<2, 1, kRowBT, kRowCap1><<<gr, kRowBT, smem, st>>>(sp.ndof, sp.nnz, rp, ip, inc, ke, vals,
                                                                              false)));
  return cudaGetLastError();
}

cudaError_t launch_gen_poisson_system(const Mesh& m, const Space& sp, const double* kappa, const double* f, double* ke,
                                      const uint8_t* isbd, const double* bdval, double* sell_vals, double* rhs,
                                      const int32_t* sptr, const int32_t* diagpos_space, const int32_t* nperm,
                                      const uint8_t* kperm, cudaStream_t st) {
  const int g = grid_for(m.ne);
  const double* area = sp.d_area.as<double>();
  const double2* grad = m.d_grad.as<double2>();
  GEN_DISPATCH(sp, (k_gen_ke<1, 0><<<g, kGT, 0, st>>>(m.ne, area, grad, kappa, ke)),
               (k_gen_ke<2, 0><<<g, kGT, 0, st>>>(m.ne, area, grad, kappa, ke)));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // (P2 rows of a triangle mesh: 19 entries for a vertex of valence 6, 25 for valence 8)
  if (sp.maxrow > 32) return cudaErrorNotSupported;
  const unsigned gr = (unsigned)((sp.ndof + kRowBTs - 1) / kRowBTs);
  const int32_t* rp = sp.d_rowptr.as<int32_t>();
  const int32_t* ci = sp.d_colind.as<int32_t>();
  const int32_t* ip = sp.d_inc_ptr.as<int32_t>();
  const uint4* inc = sp.d_inc.as<uint4>();
#define ADFEM_GPR(DEG, W)                                                                                        \
  k_gen_poisson_rows<DEG, W><<<gr, kRowBTs, 0, st>>>(sp.ndof, rp, ci, ip, inc, area, ke, f, sptr, isbd, bdval, \
                                                     sell_vals, rhs, nperm, kperm, diagpos_space)
  if (sp.maxrow <= 24) GEN_DISPATCH(sp, (ADFEM_GPR(1, 24)), (ADFEM_GPR(2, 24)));
  else GEN_DISPATCH(sp, (ADFEM_GPR(1, 32)), (ADFEM_GPR(2, 32)));
#undef ADFEM_GPR
  return cudaGetLastError();
}

cudaError_t launch_gen_kappa_grad(const Mesh& m, const Space& sp, const double* u, const double* lam,
                                  const uint8_t* isbd_space, double* grad_kappa, cudaStream_t st) {
  const int g = grid_for(m.ne * sp.ng);
  const int32_t* dof = sp.d_dof.as<int32_t>();
  const double* area = sp.d_area.as<double>();
  const double2* grad = m.d_grad.as<double2>();
  GEN_DISPATCH(sp, (k_gen_kappa_grad<1><<<g, kGT, 0, st>>>(m.ne, dof, area, grad, u, lam, isbd_space, grad_kappa)),
               (k_gen_kappa_grad<2><<<g, kGT, 0, st>>>(m.ne, dof, area, grad, u, lam, isbd_space, grad_kappa)));
  return cudaGetLastError();
}

cudaError_t launch_gen_stiffness_matrix(const Mesh& m, const Space& sp, const double* D, double* ke, double* vals,
                                        bool transpose, cudaStream_t st) {
  const int g = grid_for(m.ne * 2 * sp.nd);
  const double* area = sp.d_area.as<double>();
  const double2* grad = m.d_grad.as<double2>();
  GEN_DISPATCH(sp, (k_gen_ke_stiffness<1><<<g, kGT, 0, st>>>(m.ne, area, grad, D, ke)),
               (k_gen_ke_stiffness<2><<<g, kGT, 0, st>>>(m.ne, area, grad, D, ke)));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  static std::once_flag once;
  std::call_once(once, [] {
    const int bytes = (int)(sizeof(double) * 2 * kRowCap2 * kRowBT);
    cudaFuncSetAttribute(k_gen_rows<1, 2, kRowBT, kRowCap2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_gen_rows<2, 2, kRowBT, kRowCap2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  });
  const int gr = grid_for(sp.ndof, kRowBT);
  const size_t smem = sizeof(double) * 2 * kRowCap2 * kRowBT;
  const int32_t* rp = sp.d_rowptr.as<int32_t>();
  const int32_t* ip = sp.d_inc_ptr.as<int32_t>();
  const uint4* inc = sp.d_inc.as<uint4>();
  GEN_DISPATCH(sp,
               (k_gen_rows<1, 2, kRowBT, kRowCap2><<<gr, kRowBT, smem, st>>>(sp.ndof, sp.nnz, rp, ip, inc, ke, vals,
                                                                              transpose)),
               (k_gen_rows<2, 2, kRowBT, kRowCap2><<<gr, kRowBT, smem, st>>>(sp.ndof, sp.nnz, rp, ip, inc, ke, vals,
                                                                              transpose)));
  return cudaGetLastError();
}

cudaError_t launch_gen_source(const Mesh& m, const Space& sp, const double* f, double* rhs, bool accumulate,
                              cudaStream_t st) {
  const int g = grid_for(sp.ndof);
  const int32_t* ip = sp.d_inc_ptr.as<int32_t>();
  const uint4* inc = sp.d_inc.as<uint4>();
  const double* area = sp.d_area.as<double>();
  GEN_DISPATCH(sp, (k_gen_source<1><<<g, kGT, 0, st>>>(sp.ndof, ip, inc, area, f, rhs, accumulate)),
               (k_gen_source<2><<<g, kGT, 0, st>>>(sp.ndof, ip, inc, area, f, rhs, accumulate)));
  return cudaGetLastError();
}

cudaError_t launch_gen_source_backward(const Mesh& m, const Space& sp, const double* grad_rhs, double* grad_f,
                                       cudaStream_t st) {
  const int g = grid_for(m.ne * sp.ng);
  const int32_t* dof = sp.d_dof.as<int32_t>();
  const double* area = sp.d_area.as<double>();
  GEN_DISPATCH(sp, (k_gen_source_backward<1><<<g, kGT, 0, st>>>(m.ne, dof, area, grad_rhs, grad_f)),
               (k_gen_source_backward<2><<<g, kGT, 0, st>>>(m.ne, dof, area, grad_rhs, grad_f)));
  return cudaGetLastError();
}

cudaError_t launch_gen_to_gauss(const Mesh& m, const Space& sp, bool vertex_only, const double* u, double* out,
                                cudaStream_t st) {
  const int g = grid_for(m.ne * sp.ng);
  const int4* conn = m.d_conn.as<int4>();
  const int32_t* dof = sp.d_dof.as<int32_t>();
  if (vertex_only)
    GEN_DISPATCH(sp, (k_gen_to_gauss<1, true><<<g, kGT, 0, st>>>(m.ne, conn, dof, u, out)),
                 (k_gen_to_gauss<2, true><<<g, kGT, 0, st>>>(m.ne, conn, dof, u, out)));
  else
    GEN_DISPATCH(sp, (k_gen_to_gauss<1, false><<<g, kGT, 0, st>>>(m.ne, conn, dof, u, out)),
                 (k_gen_to_gauss<2, false><<<g, kGT, 0, st>>>(m.ne, conn, dof, u, out)));
  return cudaGetLastError();
}

cudaError_t launch_gen_to_gauss_backward(const Mesh& m, const Space& sp, bool vertex_only, const double* grad_out,
                                         double* grad_u, bool accumulate, cudaStream_t st) {
  if (vertex_only) {
    const int g = grid_for(m.nv);
    const int32_t* ip = m.d_inc_ptr.as<int32_t>();
    const void* inc = m.d_inc.p;
    GEN_DISPATCH(sp, (k_gen_to_gauss_backward<1, true><<<g, kGT, 0, st>>>(m.nv, ip, inc, grad_out, grad_u, accumulate)),
                 (k_gen_to_gauss_backward<2, true><<<g, kGT, 0, st>>>(m.nv, ip, inc, grad_out, grad_u, accumulate)));
  } else {
    const int g = grid_for(sp.ndof);
    const int32_t* ip = sp.d_inc_ptr.as<int32_t>();
    const void* inc = sp.d_inc.p;
    GEN_DISPATCH(sp,
                 (k_gen_to_gauss_backward<1, false><<<g, kGT, 0, st>>>(sp.ndof, ip, inc, grad_out, grad_u, accumulate)),
                 (k_gen_to_gauss_backward<2, false><<<g, kGT, 0, st>>>(sp.ndof, ip, inc, grad_out, grad_u, accumulate)));
  }
  return cudaGetLastError();
}

ADFEM_CHECK_READER(check_line_generic)

}  // namespace adfem
