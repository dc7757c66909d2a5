/*
 * fem_oracle.c -- CPU restatement of AdFem's triangle forward/backward path (P1, and
 * the P2 / mass-matrix / Gauss-point interpolation ops next to it).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: it is called by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline legs, and
 * never by the product library.  Every routine restates one reference routine
 * (AdFem.jl, paths relative to the project root) in plain serial C, in the same
 * loop order and arithmetic order, so that results can be compared with the
 * CUDA path.  Compile with -ffp-contract=off so no FMA contraction changes the
 * rounding of the restated expressions.
 *
 * Third-party arithmetic that the reference takes from MFEM (not vendored, not
 * pinned) is restated from MFEM's published algorithms:
 *   - IntegrationRules::Get(TRIANGLE, 2): three interior points
 *     (1/6,1/6), (1/6,2/3), (2/3,1/6) with weight 1/6 each (degree-2 rule);
 *   - Mesh::CheckElementOrientation(fix=true): a triangle whose Jacobian
 *     determinant is negative has its first two vertices swapped;
 *   - edge numbering: first appearance while walking elements in order and
 *     each triangle's local edges (0,1), (1,2), (2,0).
 * The point order and the edge numbering are not pinned by any reference test.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

typedef long long i64;

/* ---- quadrature: degree-2, 3 interior points on the reference triangle ---- */
static const double QX[3] = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
static const double QY[3] = {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0};
static const double QW = 1.0 / 6.0;

/* Heron's formula, deps/MFEM/Common.cpp:9-15 */
static double heron(double x0, double y0, double x1, double y1, double x2, double y2) {
  double a = sqrt((x0 - x1) * (x0 - x1) + (y0 - y1) * (y0 - y1));
  double b = sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1));
  double c = sqrt((x0 - x2) * (x0 - x2) + (y0 - y2) * (y0 - y2));
  double s = (a + b + c) / 2.0;
  return sqrt(s * (s - a) * (s - b) * (s - c));
}

/*
 * Mesh geometry, deps/MFEM/Common.cpp:20-142 (NNFEM_Mesh::init, P1 branch).
 *   xyz      : 3*nv vertex triples (z ignored), as packed by src/MFEM/MFEM.jl:92
 *   elems0   : 3*ne 0-based vertex ids
 * outputs (caller-allocated):
 *   elem     : 3*ne vertex ids after the orientation fix
 *   area     : ne   Heron area
 *   w        : 3*ne weights ip.weight*area/0.5 (Common.cpp:116)
 *   hx, hy   : 3*ne physical shape gradients per element and local vertex
 *              (constant over the element for P1; Common.cpp:119-126)
 *   h        : 9*ne shape values, h[9e + 3k + r] = phi_r at point k
 *   gx, gy   : 3*ne Gauss-point coordinates (Common.cpp:103-111)
 * returns the number of elements whose orientation was flipped.
 */
int orc_mesh_geometry(int nv, const double *xyz, int ne, const int *elems0, int *elem, double *area,
                      double *w, double *hx, double *hy, double *h, double *gx, double *gy) {
  (void)nv;
  int flipped = 0;
  for (int e = 0; e < ne; e++) {
    int v0 = elems0[3 * e], v1 = elems0[3 * e + 1], v2 = elems0[3 * e + 2];
    double ax = xyz[3 * v0], ay = xyz[3 * v0 + 1];
    double bx = xyz[3 * v1], by = xyz[3 * v1 + 1];
    double cx = xyz[3 * v2], cy = xyz[3 * v2 + 1];
    double det = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
    if (det < 0.0) {
      int t = v0; v0 = v1; v1 = t;
      flipped++;
    }
    elem[3 * e] = v0; elem[3 * e + 1] = v1; elem[3 * e + 2] = v2;
    double x1 = xyz[3 * v0], y1 = xyz[3 * v0 + 1];
    double x2 = xyz[3 * v1], y2 = xyz[3 * v1 + 1];
    double x3 = xyz[3 * v2], y3 = xyz[3 * v2 + 1];
    double A = heron(x1, y1, x2, y2, x3, y3);
    area[e] = A;
    /* affine map Jacobian J = [x2-x1 x3-x1; y2-y1 y3-y1]; inverse = adj(J) * (1/det) */
    double j00 = x2 - x1, j01 = x3 - x1, j10 = y2 - y1, j11 = y3 - y1;
    double dj = j00 * j11 - j01 * j10;
    double t = 1.0 / dj;
    double i00 = j11 * t, i01 = -j01 * t, i10 = -j10 * t, i11 = j00 * t;
    /* reference gradients (-1,-1), (1,0), (0,1) times J^{-1} */
    hx[3 * e + 0] = -i00 - i10; hy[3 * e + 0] = -i01 - i11;
    hx[3 * e + 1] = i00;        hy[3 * e + 1] = i01;
    hx[3 * e + 2] = i10;        hy[3 * e + 2] = i11;
    for (int k = 0; k < 3; k++) {
      double l0 = 1.0 - QX[k] - QY[k], l1 = QX[k], l2 = QY[k];
      gx[3 * e + k] = x1 * l0 + x2 * l1 + x3 * l2;
      gy[3 * e + k] = y1 * l0 + y2 * l1 + y3 * l2;
      w[3 * e + k] = QW * A / 0.5;
      h[9 * e + 3 * k + 0] = l0;
      h[9 * e + 3 * k + 1] = l1;
      h[9 * e + 3 * k + 2] = l2;
    }
  }
  return flipped;
}

/*
 * Edge list, Common.cpp:133-139 (edges[i] = min+1, edges[nedges+i] = max+1).
 * Numbering: first appearance over elements and local edges (0,1),(1,2),(2,0).
 * Returns nedges; writes edges when out != NULL.  O(ne log) via a per-vertex
 * adjacency scan (vertex valence is small).
 */
static i64 edges_impl(int nv, int ne, const int *elem, i64 *out, int *eedge) {
  /* adjacency lists keyed by the smaller vertex */
  int *cnt = (int *)calloc((size_t)nv + 1, sizeof(int));
  for (int e = 0; e < ne; e++)
    for (int l = 0; l < 3; l++) {
      int a = elem[3 * e + l], b = elem[3 * e + (l + 1) % 3];
      cnt[(a < b ? a : b) + 1]++;
    }
  for (int i = 0; i < nv; i++) cnt[i + 1] += cnt[i];
  int *nbr = (int *)malloc(sizeof(int) * (size_t)(cnt[nv] > 0 ? cnt[nv] : 1));
  i64 *id = (i64 *)malloc(sizeof(i64) * (size_t)(cnt[nv] > 0 ? cnt[nv] : 1));
  int *fill = (int *)calloc((size_t)nv, sizeof(int));
  i64 nedges = 0;
  i64 cap = cnt[nv];
  i64 *emin = (i64 *)malloc(sizeof(i64) * (size_t)(cap > 0 ? cap : 1));
  i64 *emax = (i64 *)malloc(sizeof(i64) * (size_t)(cap > 0 ? cap : 1));
  for (int e = 0; e < ne; e++)
    for (int l = 0; l < 3; l++) {
      int a = elem[3 * e + l], b = elem[3 * e + (l + 1) % 3];
      int lo = a < b ? a : b, hi = a < b ? b : a;
      i64 found = -1;
      for (int s = cnt[lo]; s < cnt[lo] + fill[lo]; s++)
        if (nbr[s] == hi) { found = id[s]; break; }
      if (found < 0) {
        int s = cnt[lo] + fill[lo]++;
        nbr[s] = hi;
        id[s] = nedges;
        emin[nedges] = lo; emax[nedges] = hi;
        found = nedges++;
      }
      if (eedge) eedge[3 * e + l] = (int)found;
    }
  if (out) {
    for (i64 i = 0; i < nedges; i++) {
      out[i] = emin[i] + 1;
      out[nedges + i] = emax[i] + 1;
    }
  }
  free(cnt); free(nbr); free(id); free(fill); free(emin); free(emax);
  return nedges;
}

i64 orc_mesh_edges(int nv, int ne, const int *elem, i64 *out) { return edges_impl(nv, ne, elem, out, NULL); }

/* Element-to-edge map in the same numbering: eedge[3e + l] is the edge of local edge l
 * ((0,1), (1,2), (2,0)), as mesh.GetElementEdges gives it in Common.cpp:68-71. */
i64 orc_element_edges(int nv, int ne, const int *elem, int *eedge) { return edges_impl(nv, ne, elem, NULL, eedge); }

/* FemLaplaceScalar_forward, deps/MFEM/FemLaplace1/FemLaplaceScalar.h:3-26 */
void orc_laplace_coo(int ne, const int *elem, const double *w, const double *hx, const double *hy,
                     const double *kappa, i64 *indices, double *vv) {
  i64 s = 0, nz = 0;
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < 3; k++) {
      double kw = kappa[s++];
      for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++) {
          double dd = hx[3 * e + p] * hx[3 * e + q] + hy[3 * e + p] * hy[3 * e + q];
          indices[2 * nz] = elem[3 * e + p];
          indices[2 * nz + 1] = elem[3 * e + q];
          vv[nz] = dd * kw * w[3 * e + k];
          nz++;
        }
    }
}

/* FemLaplaceScalar_backward, FemLaplaceScalar.h:28-54 */
void orc_laplace_coo_backward(int ne, const double *w, const double *hx, const double *hy,
                              const double *grad_vv, double *grad_kappa) {
  i64 s = 0, nz = 0;
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < 3; k++) {
      double v = 0.0;
      for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++) {
          double dd = hx[3 * e + p] * hx[3 * e + q] + hy[3 * e + p] * hy[3 * e + q];
          v += grad_vv[nz] * (dd * w[3 * e + k]);
          nz++;
        }
      grad_kappa[s++] = v;
    }
}

/* FemSourceScalar_forward, deps/MFEM/FemSource1/FemSourceScalar.h:4-15 (accumulates into rhs) */
void orc_source(int ne, const int *elem, const double *w, const double *h, const double *f, double *rhs) {
  i64 k = 0;
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < 3; j++) {
      for (int r = 0; r < 3; r++)
        rhs[elem[3 * e + r]] += f[k] * h[9 * e + 3 * j + r] * w[3 * e + j];
      k++;
    }
}

/* FemSourceScalar_backward, FemSourceScalar.h:17-32 */
void orc_source_backward(int ne, const int *elem, const double *w, const double *h, const double *grad_rhs,
                         double *grad_f) {
  i64 k = 0;
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < 3; j++) {
      grad_f[k] = 0.0;
      for (int r = 0; r < 3; r++)
        grad_f[k] += h[9 * e + 3 * j + r] * w[3 * e + j] * grad_rhs[elem[3 * e + r]];
      k++;
    }
}

/* B = [hx 0; 0 hy; hy hx] (3 x 6), ComputeFemStiffnessMatrixMfem.h:18-23 */
static void build_B(const double *hx, const double *hy, int e, double B[3][6]) {
  for (int p = 0; p < 3; p++)
    for (int c = 0; c < 6; c++) B[p][c] = 0.0;
  for (int r = 0; r < 3; r++) {
    B[0][r] = hx[3 * e + r];
    B[1][r + 3] = hy[3 * e + r];
    B[2][r] = hy[3 * e + r];
    B[2][r + 3] = hx[3 * e + r];
  }
}

/* ComputeFemStiffnessMatrixMfem_forward, ComputeFemStiffnessMatrixMfem.h:4-48 */
void orc_stiffness_coo(int ne, int ndof, const int *elem, const double *w, const double *hx, const double *hy,
                       const double *hmat, i64 *indices, double *vv) {
  i64 k = 0, k0 = 0;
  double B[3][6];
  for (int e = 0; e < ne; e++) {
    build_B(hx, hy, e, B);
    for (int j = 0; j < 3; j++) {
      double K[3][3];
      for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++) K[p][q] = hmat[k0++];
      double T[6][3];
      for (int l = 0; l < 6; l++)
        for (int q = 0; q < 3; q++) {
          double s = 0.0;
          for (int p = 0; p < 3; p++) s += B[p][l] * K[p][q];
          T[l][q] = s;
        }
      int dofs[6];
      for (int p = 0; p < 3; p++) {
        dofs[p] = elem[3 * e + p];
        dofs[p + 3] = elem[3 * e + p] + ndof;
      }
      for (int l = 0; l < 6; l++)
        for (int s = 0; s < 6; s++) {
          double acc = 0.0;
          for (int q = 0; q < 3; q++) acc += T[l][q] * B[q][s];
          indices[2 * k] = dofs[l];
          indices[2 * k + 1] = dofs[s];
          vv[k] = acc * w[3 * e + j];
          k++;
        }
    }
  }
}

/* ComputeFemStiffnessMatrixMfem_backward, ComputeFemStiffnessMatrixMfem.h:50-81 */
void orc_stiffness_coo_backward(int ne, const double *w, const double *hx, const double *hy, const double *grad_vv,
                                double *grad_hmat) {
  i64 k = 0, k0 = 0;
  double B[3][6];
  for (int e = 0; e < ne; e++) {
    build_B(hx, hy, e, B);
    for (int j = 0; j < 3; j++) {
      double G[6][6];
      for (int l = 0; l < 6; l++)
        for (int s = 0; s < 6; s++) G[l][s] = grad_vv[k++];
      double T[3][6]; /* B * G */
      for (int p = 0; p < 3; p++)
        for (int s = 0; s < 6; s++) {
          double acc = 0.0;
          for (int l = 0; l < 6; l++) acc += B[p][l] * G[l][s];
          T[p][s] = acc;
        }
      for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++) {
          double acc = 0.0;
          for (int s = 0; s < 6; s++) acc += T[p][s] * B[q][s];
          grad_hmat[k0++] = acc * w[3 * e + j];
        }
    }
  }
}

/* ======================================================================
 * Degree-generic element loops (P1 and P2 Lagrange triangles).
 *
 * The reference kernels are written over elem_ndof and elem->ngauss with per-point
 * tables h, hx, hy, w and dof[] filled by NNFEM_Mesh::init (Common.cpp:46-126);
 * the loops below restate them over tables of the same meaning:
 *   nd = elem_ndof (3 or 6), ng = Gauss points per element (3 or 6),
 *   dof[nd*e + r], w[ng*e + k], h/hx/hy[(ng*e + k)*nd + r], hs[(ng*e + k)*3 + a].
 * ---------------------------------------------------------------------- */

/* Degree-4 triangle rule (IntegrationRules::Get(TRIANGLE, 4), the order P2 meshes
 * default to, src/MFEM/MFEM.jl:71-77): the published 6-point Strang-Fix/Dunavant rule,
 * two orbits (a,a), (a,1-2a), (1-2a,a) with a = 0.0915762... (weight 0.0549758...)
 * and a = 0.4459484... (weight 0.1116907...); weights sum to the reference area 1/2.
 * Point order within the rule is not pinned by any reference test. */
static const double Q4X[6] = {0.091576213509770743460, 0.091576213509770743460, 0.81684757298045851308,
                              0.44594849091596488632, 0.44594849091596488632, 0.10810301816807022736};
static const double Q4Y[6] = {0.091576213509770743460, 0.81684757298045851308, 0.091576213509770743460,
                              0.44594849091596488632, 0.10810301816807022736, 0.44594849091596488632};
static const double Q4W[6] = {0.054975871827660933819, 0.054975871827660933819, 0.054975871827660933819,
                              0.11169079483900573285, 0.11169079483900573285, 0.11169079483900573285};

/* Lagrange basis on the triangle in barycentric coordinates l[3] and its partial
 * derivatives t[r][c] = d phi_r / d l_c.  P1: phi_r = l_r.  P2 (H1_FECollection(2):
 * nodes at the vertices and edge midpoints, vertex functions first, then the edges
 * (0,1), (1,2), (2,0)): phi_a = l_a (2 l_a - 1), phi_ab = 4 l_a l_b. */
static void basis(int degree, const double l[3], double phi[6], double t[6][3]) {
  for (int r = 0; r < 6; r++) t[r][0] = t[r][1] = t[r][2] = 0.0;
  if (degree == 1) {
    for (int r = 0; r < 3; r++) {
      phi[r] = l[r];
      t[r][r] = 1.0;
    }
    return;
  }
  for (int a = 0; a < 3; a++) {
    phi[a] = l[a] * (2.0 * l[a] - 1.0);
    t[a][a] = 4.0 * l[a] - 1.0;
  }
  static const int E0[3] = {0, 1, 2}, E1[3] = {1, 2, 0};
  for (int j = 0; j < 3; j++) {
    int a = E0[j], b = E1[j];
    phi[3 + j] = 4.0 * l[a] * l[b];
    t[3 + j][a] = 4.0 * l[b];
    t[3 + j][b] = 4.0 * l[a];
  }
}

/*
 * Per-point tables of NNFEM_Mesh::init (Common.cpp:46-126) for degree 1 or 2:
 *   elem, area, hx1, hy1 : outputs of orc_mesh_geometry (P1 gradients = grad l_a)
 *   eedge                : orc_element_edges (needed for degree 2, else NULL)
 * outputs: dof (nd per element: vertices, then nv + edge of each local edge,
 * Common.cpp:62-71), w, h, hx, hy, hs (P1 shape at the point, Common.cpp:103-105) and
 * the Gauss-point coordinates gx, gy.  Physical gradients follow the chain rule
 * grad phi_r = sum_c (d phi_r / d l_c) grad l_c, which is what CalcPhysDShape
 * evaluates through the inverse Jacobian.
 */
void orc_space_tables(int degree, int nv, const double *xyz, int ne, const int *elem, const int *eedge,
                      const double *area, const double *hx1, const double *hy1, int *dof, double *w, double *h,
                      double *hx, double *hy, double *hs, double *gx, double *gy) {
  const int nd = degree == 2 ? 6 : 3, ng = degree == 2 ? 6 : 3;
  for (int e = 0; e < ne; e++) {
    for (int a = 0; a < 3; a++) dof[nd * e + a] = elem[3 * e + a];
    if (degree == 2)
      for (int j = 0; j < 3; j++) dof[nd * e + 3 + j] = nv + eedge[3 * e + j];
    const int v0 = elem[3 * e], v1 = elem[3 * e + 1], v2 = elem[3 * e + 2];
    for (int k = 0; k < ng; k++) {
      const double xi = degree == 2 ? Q4X[k] : QX[k], eta = degree == 2 ? Q4Y[k] : QY[k];
      const double qw = degree == 2 ? Q4W[k] : QW;
      double l[3] = {1.0 - xi - eta, xi, eta};
      double phi[6], t[6][3];
      basis(degree, l, phi, t);
      const i64 p = (i64)ng * e + k;
      w[p] = qw * area[e] / 0.5;
      gx[p] = xyz[3 * v0] * l[0] + xyz[3 * v1] * l[1] + xyz[3 * v2] * l[2];
      gy[p] = xyz[3 * v0 + 1] * l[0] + xyz[3 * v1 + 1] * l[1] + xyz[3 * v2 + 1] * l[2];
      for (int a = 0; a < 3; a++) hs[3 * p + a] = l[a];
      for (int r = 0; r < nd; r++) {
        h[nd * p + r] = phi[r];
        hx[nd * p + r] = t[r][0] * hx1[3 * e] + t[r][1] * hx1[3 * e + 1] + t[r][2] * hx1[3 * e + 2];
        hy[nd * p + r] = t[r][0] * hy1[3 * e] + t[r][1] * hy1[3 * e + 1] + t[r][2] * hy1[3 * e + 2];
      }
    }
  }
}

/* FemLaplaceScalar_forward, FemLaplaceScalar.h:3-26, over elem_ndof */
void orc_gen_laplace_coo(int ne, int nd, int ng, const int *dof, const double *w, const double *hx,
                         const double *hy, const double *kappa, i64 *indices, double *vv) {
  i64 nz = 0;
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      for (int a = 0; a < nd; a++)
        for (int b = 0; b < nd; b++) {
          double dd = hx[nd * p + a] * hx[nd * p + b] + hy[nd * p + a] * hy[nd * p + b];
          indices[2 * nz] = dof[nd * e + a];
          indices[2 * nz + 1] = dof[nd * e + b];
          vv[nz] = dd * kappa[p] * w[p];
          nz++;
        }
    }
}

/* FemLaplaceScalar_backward, FemLaplaceScalar.h:28-54 */
void orc_gen_laplace_coo_backward(int ne, int nd, int ng, const double *w, const double *hx, const double *hy,
                                  const double *grad_vv, double *grad_kappa) {
  i64 nz = 0;
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      double v = 0.0;
      for (int a = 0; a < nd; a++)
        for (int b = 0; b < nd; b++) {
          double dd = hx[nd * p + a] * hx[nd * p + b] + hy[nd * p + a] * hy[nd * p + b];
          v += grad_vv[nz] * (dd * w[p]);
          nz++;
        }
      grad_kappa[p] = v;
    }
}

/* ComputeFemMassMatrix1_forward, deps/MFEM/ComputeFemMassMatrix1/ComputeFemMassMatrixMfem.h:4-29 */
void orc_gen_mass_coo(int ne, int nd, int ng, const int *dof, const double *w, const double *h, const double *rho,
                      i64 *indices, double *vv) {
  i64 nz = 0;
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      for (int a = 0; a < nd; a++)
        for (int b = 0; b < nd; b++) {
          indices[2 * nz] = dof[nd * e + a];
          indices[2 * nz + 1] = dof[nd * e + b];
          vv[nz] = h[nd * p + a] * h[nd * p + b] * rho[p] * w[p];
          nz++;
        }
    }
}

/* ComputeFemMassMatrix1_backward, ComputeFemMassMatrixMfem.h:31-55 (grad_rho zeroed first,
 * as the TF grad op does, ComputeFemMassMatrixMfem.cpp:139) */
void orc_gen_mass_coo_backward(int ne, int nd, int ng, const double *w, const double *h, const double *grad_vv,
                               double *grad_rho) {
  i64 nz = 0;
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      grad_rho[p] = 0.0;
      for (int a = 0; a < nd; a++)
        for (int b = 0; b < nd; b++) {
          grad_rho[p] += h[nd * p + a] * h[nd * p + b] * w[p] * grad_vv[nz];
          nz++;
        }
    }
}

/* FemSourceScalar_forward, FemSourceScalar.h:4-15, over elem_ndof (accumulates into rhs) */
void orc_gen_source(int ne, int nd, int ng, const int *dof, const double *w, const double *h, const double *f,
                    double *rhs) {
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      for (int r = 0; r < nd; r++) rhs[dof[nd * e + r]] += f[p] * h[nd * p + r] * w[p];
    }
}

/* FemSourceScalar_backward, FemSourceScalar.h:17-32 */
void orc_gen_source_backward(int ne, int nd, int ng, const int *dof, const double *w, const double *h,
                             const double *grad_rhs, double *grad_f) {
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      grad_f[p] = 0.0;
      for (int r = 0; r < nd; r++) grad_f[p] += h[nd * p + r] * w[p] * grad_rhs[dof[nd * e + r]];
    }
}

/* ComputeFemStiffnessMatrixMfem_forward, ComputeFemStiffnessMatrixMfem.h:4-48, over
 * elem_ndof: B = [hx 0; 0 hy; hy hx] (3 x 2nd), DOFs [dof; dof + ndof] */
void orc_gen_stiffness_coo(int ne, int nd, int ng, int ndof, const int *dof, const double *w, const double *hx,
                           const double *hy, const double *hmat, i64 *indices, double *vv) {
  i64 nz = 0;
  double B[3][12];
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      for (int a = 0; a < 3; a++)
        for (int c = 0; c < 2 * nd; c++) B[a][c] = 0.0;
      for (int r = 0; r < nd; r++) {
        B[0][r] = hx[nd * p + r];
        B[1][r + nd] = hy[nd * p + r];
        B[2][r] = hy[nd * p + r];
        B[2][r + nd] = hx[nd * p + r];
      }
      const double *K = hmat + 9 * p;
      double T[12][3];
      for (int l = 0; l < 2 * nd; l++)
        for (int q = 0; q < 3; q++) {
          double acc = 0.0;
          for (int a = 0; a < 3; a++) acc += B[a][l] * K[3 * a + q];
          T[l][q] = acc;
        }
      for (int l = 0; l < 2 * nd; l++)
        for (int c = 0; c < 2 * nd; c++) {
          double acc = 0.0;
          for (int q = 0; q < 3; q++) acc += T[l][q] * B[q][c];
          indices[2 * nz] = dof[nd * e + (l % nd)] + (l >= nd ? ndof : 0);
          indices[2 * nz + 1] = dof[nd * e + (c % nd)] + (c >= nd ? ndof : 0);
          vv[nz] = acc * w[p];
          nz++;
        }
    }
}

/* ComputeFemStiffnessMatrixMfem_backward, ComputeFemStiffnessMatrixMfem.h:50-81 */
void orc_gen_stiffness_coo_backward(int ne, int nd, int ng, const double *w, const double *hx, const double *hy,
                                    const double *grad_vv, double *grad_hmat) {
  i64 nz = 0;
  double B[3][12], T[3][12];
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      for (int a = 0; a < 3; a++)
        for (int c = 0; c < 2 * nd; c++) B[a][c] = 0.0;
      for (int r = 0; r < nd; r++) {
        B[0][r] = hx[nd * p + r];
        B[1][r + nd] = hy[nd * p + r];
        B[2][r] = hy[nd * p + r];
        B[2][r + nd] = hx[nd * p + r];
      }
      const double *G = grad_vv + nz;
      for (int a = 0; a < 3; a++)
        for (int c = 0; c < 2 * nd; c++) {
          double acc = 0.0;
          for (int l = 0; l < 2 * nd; l++) acc += B[a][l] * G[2 * nd * l + c];
          T[a][c] = acc;
        }
      for (int a = 0; a < 3; a++)
        for (int q = 0; q < 3; q++) {
          double acc = 0.0;
          for (int c = 0; c < 2 * nd; c++) acc += T[a][c] * B[q][c];
          grad_hmat[9 * p + 3 * a + q] = acc * w[p];
        }
      nz += 4 * nd * nd;
    }
}

/* FemToGaussPointsMfem_forward / _backward, deps/MFEM/FemToGaussPoints/FemToGaussPointsMfem.h:5-34:
 * nodal values through the P1 shape hs at each Gauss point.  The backward accumulates
 * into grad_u (the TF op zeroes it first, FemToGaussPointsMfem.cpp:128). */
void orc_fem_to_gauss(int ne, int ng, const int *elem, const double *hs, const double *u, double *out) {
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      out[p] = u[elem[3 * e]] * hs[3 * p] + u[elem[3 * e + 1]] * hs[3 * p + 1] + u[elem[3 * e + 2]] * hs[3 * p + 2];
    }
}

void orc_fem_to_gauss_backward(int ne, int ng, const int *elem, const double *hs, const double *grad_out,
                               double *grad_u) {
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      for (int a = 0; a < 3; a++) grad_u[elem[3 * e + a]] += grad_out[p] * hs[3 * p + a];
    }
}

/* DofToGaussPointsMfem_forward / _backward, deps/MFEM/DofToGaussPoints/DofToGaussPointsMfem.h:5-35 */
void orc_dof_to_gauss(int ne, int nd, int ng, const int *dof, const double *h, const double *u, double *out) {
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      out[p] = 0.0;
      for (int r = 0; r < nd; r++) out[p] += u[dof[nd * e + r]] * h[nd * p + r];
    }
}

void orc_dof_to_gauss_backward(int ne, int nd, int ng, const int *dof, const double *h, const double *grad_out,
                               double *grad_u) {
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      for (int r = 0; r < nd; r++) grad_u[dof[nd * e + r]] += grad_out[p] * h[nd * p + r];
    }
}

/* bcnode(mesh) for P2 (src/MFEM/MCore.jl:439-450): boundary vertices, then the DOFs of
 * boundary edges (nv + edge).  Boundary edges are those used by one element
 * (bcedge's toggle set, MCore.jl:385-406).  Both parts ascending, 1-based.
 * Returns the count; writes out when non-NULL. */
i64 orc_bcnode_p2(int nv, int ne, const int *elem, const int *eedge, i64 nedges, i64 *out) {
  int *cnt = (int *)calloc((size_t)(nedges > 0 ? nedges : 1), sizeof(int));
  char *bv = (char *)calloc((size_t)nv, 1);
  for (int e = 0; e < ne; e++)
    for (int l = 0; l < 3; l++) cnt[eedge[3 * e + l]]++;
  for (int e = 0; e < ne; e++)
    for (int l = 0; l < 3; l++)
      if (cnt[eedge[3 * e + l]] & 1) {
        bv[elem[3 * e + l]] = 1;
        bv[elem[3 * e + (l + 1) % 3]] = 1;
      }
  i64 c = 0;
  for (int i = 0; i < nv; i++)
    if (bv[i]) {
      if (out) out[c] = i + 1;
      c++;
    }
  for (i64 j = 0; j < nedges; j++)
    if (cnt[j] & 1) {
      if (out) out[c] = nv + j + 1;
      c++;
    }
  free(cnt); free(bv);
  return c;
}

/*
 * Plane strain / plane stress matrices, deps/MFEM/PlaneStrainAndStress/PlaneStrainAndStress.h:5-78.
 * mode 0 = plane strain (all nine entries filled, reference formula), mode 1 = plane stress.
 * The backward restates the derivative that the reference obtains with its AD tape.
 */
void orc_plane_strain_stress(int mode, i64 n, const double *E, const double *nu, double *out) {
  for (i64 i = 0; i < n; i++) {
    if (mode == 0) {
      double s = E[i] * (1 - nu[i]) / (1 + nu[i]) / (1 - 2 * nu[i]);
      double a = s * nu[i] / (1 - nu[i]);
      out[9 * i + 0] = s; out[9 * i + 1] = a; out[9 * i + 2] = a;
      out[9 * i + 3] = a; out[9 * i + 4] = s; out[9 * i + 5] = a;
      out[9 * i + 6] = a; out[9 * i + 7] = a; out[9 * i + 8] = s;
    } else {
      double s = E[i] / (1 + nu[i]) / (1 - 2 * nu[i]);
      out[9 * i + 0] = s * (1 - nu[i]); out[9 * i + 1] = s * nu[i]; out[9 * i + 2] = 0.0;
      out[9 * i + 3] = s * nu[i]; out[9 * i + 4] = s * (1 - nu[i]); out[9 * i + 5] = 0.0;
      out[9 * i + 6] = 0.0; out[9 * i + 7] = 0.0; out[9 * i + 8] = s * (1 - 2 * nu[i]) / 2.0;
    }
  }
}

void orc_plane_strain_stress_backward(int mode, i64 n, const double *grad_out, const double *E, const double *nu,
                                      double *grad_E, double *grad_nu) {
  for (i64 i = 0; i < n; i++) {
    const double *g = grad_out + 9 * i;
    double v = nu[i], D = (1 + v) * (1 - 2 * v);
    if (mode == 0) {
      double gd = g[0] + g[4] + g[8];
      double go = g[1] + g[2] + g[3] + g[5] + g[6] + g[7];
      /* s = E (1-v)/D, s*v/(1-v) = E v / D */
      grad_E[i] = gd * (1 - v) / D + go * v / D;
      grad_nu[i] = E[i] * (gd * 2 * v * (2 - v) + go * (1 + 2 * v * v)) / (D * D);
    } else {
      /* s = E/D; entries s(1-v), s v, s(1-2v)/2 */
      double a = g[0] + g[4], b = g[1] + g[3], c = g[8];
      grad_E[i] = (a * (1 - v) + b * v + c * (1 - 2 * v) / 2.0) / D;
      /* d/dv [ (1-v)/D ] = 2v(2-v)/D^2 ; d/dv [ v/D ] = (1+2v^2)/D^2 ; d/dv [ (1-2v)/(2D) ] = -1/(2 (1+v)^2) */
      grad_nu[i] = E[i] * (a * 2 * v * (2 - v) / (D * D) + b * (1 + 2 * v * v) / (D * D) + c * -0.5 / ((1 + v) * (1 + v)));
    }
  }
}

/* ---- ImposeDirichlet (COO / SparseTensor arm), deps/MFEM/ImposeDirichlet/ImposeDirichlet.h:27-93 ---- */
static int cmp_i64(const void *a, const void *b) {
  i64 x = *(const i64 *)a, y = *(const i64 *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* bd lookup: sorted unique 0-based ids with the bd position of the LAST occurrence
 * (std::map assignment keeps the last value written, ImposeDirichlet.h:32,70-71) */
typedef struct { i64 node; i64 pos; } bdent;
static int cmp_bdent(const void *a, const void *b) {
  const bdent *x = (const bdent *)a, *y = (const bdent *)b;
  if (x->node != y->node) return x->node < y->node ? -1 : 1;
  return x->pos < y->pos ? -1 : (x->pos > y->pos ? 1 : 0);
}
static i64 make_bdmap(const i64 *bd, int bdN, bdent **out) {
  bdent *t = (bdent *)malloc(sizeof(bdent) * (size_t)(bdN > 0 ? bdN : 1));
  for (int i = 0; i < bdN; i++) { t[i].node = bd[i] - 1; t[i].pos = i; }
  qsort(t, (size_t)bdN, sizeof(bdent), cmp_bdent);
  i64 u = 0;
  for (int i = 0; i < bdN; i++) {
    if (u > 0 && t[u - 1].node == t[i].node) t[u - 1] = t[i]; /* keep last */
    else t[u++] = t[i];
  }
  *out = t;
  return u;
}
static i64 bd_find(const bdent *t, i64 nu, i64 node) {
  i64 lo = 0, hi = nu - 1;
  while (lo <= hi) {
    i64 mid = (lo + hi) / 2;
    if (t[mid].node == node) return mid;
    if (t[mid].node < node) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

/* forward: returns output nnz; writes oindices/ov/orhs when non-NULL */
i64 orc_dirichlet_coo(const i64 *indices, const double *v, i64 sN, const i64 *bd, int bdN, const double *rhs,
                      const double *bdval, i64 N, i64 *oindices, double *ov, double *orhs) {
  bdent *t; i64 nu = make_bdmap(bd, bdN, &t);
  double *r = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
  for (i64 i = 0; i < N; i++) r[i] = rhs[i];
  i64 z = 0;
  for (i64 k = 0; k < sN; k++) {
    i64 i = indices[2 * k], j = indices[2 * k + 1];
    i64 bi = bd_find(t, nu, i), bj = bd_find(t, nu, j);
    if (bi < 0 && bj < 0) {
      if (oindices) { oindices[2 * z] = i; oindices[2 * z + 1] = j; ov[z] = v[k]; }
      z++;
    }
    if (bi < 0 && bj >= 0) r[i] = r[i] - v[k] * bdval[t[bj].pos];
  }
  for (i64 u = 0; u < nu; u++) {
    if (oindices) { oindices[2 * z] = t[u].node; oindices[2 * z + 1] = t[u].node; ov[z] = 1.0; }
    z++;
    r[t[u].node] = bdval[t[u].pos];
  }
  if (orhs) for (i64 i = 0; i < N; i++) orhs[i] = r[i];
  free(r); free(t);
  return z;
}

/* backward (ImposeDirichlet.h:63-93); outputs are zeroed first, as the TF grad op allocates them zeroed */
void orc_dirichlet_coo_backward(const double *grad_vv, const double *grad_rhs, const i64 *indices, const double *v,
                                i64 sN, const i64 *bd, int bdN, const double *bdval, i64 N, double *grad_vv_in,
                                double *grad_rhs_in, double *grad_bdval) {
  bdent *t; i64 nu = make_bdmap(bd, bdN, &t);
  for (i64 k = 0; k < sN; k++) grad_vv_in[k] = 0.0;
  for (i64 i = 0; i < N; i++) grad_rhs_in[i] = 0.0;
  for (int i = 0; i < bdN; i++) grad_bdval[i] = 0.0;
  i64 z = 0;
  for (i64 k = 0; k < sN; k++) {
    i64 i = indices[2 * k], j = indices[2 * k + 1];
    i64 bi = bd_find(t, nu, i), bj = bd_find(t, nu, j);
    if (bi < 0 && bj < 0) grad_vv_in[k] = grad_vv[z++];
    if (bi < 0 && bj >= 0) {
      grad_vv_in[k] -= bdval[t[bj].pos] * grad_rhs[i];
      grad_bdval[t[bj].pos] -= v[k] * grad_rhs[i];
    }
  }
  for (i64 i = 0; i < N; i++)
    if (bd_find(t, nu, i) < 0) grad_rhs_in[i] = grad_rhs[i];
  for (i64 u = 0; u < nu; u++) grad_bdval[t[u].pos] += grad_rhs[t[u].node];
  free(t);
}

/* pcl_FemLaplaceScalar_Jacobian, deps/MFEM/FemLaplace1/FemLaplaceScalar.h:63-91: H is
 * column-major ngauss x (nd^2 ngauss); H[s + nz*ngauss] = (D D^T w)_pq for entry nz of
 * Gauss point s.  Only these entries are written (the caller zeroes H). */
void orc_pcl_laplace_jacobian(int ne, int nd, int ng, const double *w, const double *hx, const double *hy,
                              double *H) {
  const i64 ngauss = (i64)ng * ne;
  i64 nz = 0;
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < ng; k++) {
      const i64 p = (i64)ng * e + k;
      for (int a = 0; a < nd; a++)
        for (int b = 0; b < nd; b++) {
          double dd = hx[nd * p + a] * hx[nd * p + b] + hy[nd * p + a] * hy[nd * p + b];
          H[p + nz * ngauss] = dd * w[p];
          nz++;
        }
    }
}

/* pcl_ImposeDirichlet, deps/MFEM/ImposeDirichlet/ImposeDirichlet.h:97-111: indices is the
 * 1-based sN x 2 column-major index array, J column-major sN x outdof (zeroed by the
 * caller); J[k + s*sN] = 1 for the s-th entry whose row and column are both off bd. */
void orc_pcl_dirichlet(double *J, const i64 *indices, const i64 *bd, int bdN, int sN) {
  i64 *b = (i64 *)malloc(sizeof(i64) * (size_t)(bdN > 0 ? bdN : 1));
  for (int q = 0; q < bdN; q++) b[q] = bd[q] - 1;
  qsort(b, (size_t)bdN, sizeof(i64), cmp_i64);
  i64 s = 0;
  for (int k = 0; k < sN; k++) {
    i64 i = indices[k] - 1, j = indices[k + sN] - 1;
    int ini = bdN > 0 && bsearch(&i, b, (size_t)bdN, sizeof(i64), cmp_i64) != NULL;
    int inj = bdN > 0 && bsearch(&j, b, (size_t)bdN, sizeof(i64), cmp_i64) != NULL;
    if (!ini && !inj) {
      J[k + s * sN] = 1.0;
      s++;
    }
  }
  free(b);
}

/*
 * COO -> CSC with Julia SparseArrays `sparse(I, J, V, m, n)` semantics
 * (src/MFEM/MCore.jl:118-119): duplicates summed in input order, row indices
 * sorted within each column, numerical zeros kept as stored entries.
 * indices are 0-based (row, col) pairs.  Two-call protocol: with colptr==NULL
 * returns nnz only.  colptr/rowval are written 0-based.
 */
typedef struct { i64 col, row, pos; } cooent;
static int cmp_cooent(const void *a, const void *b) {
  const cooent *x = (const cooent *)a, *y = (const cooent *)b;
  if (x->col != y->col) return x->col < y->col ? -1 : 1;
  if (x->row != y->row) return x->row < y->row ? -1 : 1;
  return x->pos < y->pos ? -1 : (x->pos > y->pos ? 1 : 0);
}
i64 orc_coo_to_csc_sorted(const i64 *indices, const double *v, i64 N, i64 n, i64 *colptr, i64 *rowval, double *nzval) {
  cooent *t = (cooent *)malloc(sizeof(cooent) * (size_t)(N > 0 ? N : 1));
  for (i64 k = 0; k < N; k++) { t[k].row = indices[2 * k]; t[k].col = indices[2 * k + 1]; t[k].pos = k; }
  qsort(t, (size_t)N, sizeof(cooent), cmp_cooent);
  i64 nnz = 0;
  if (colptr) for (i64 j = 0; j <= n; j++) colptr[j] = 0;
  for (i64 k = 0; k < N; k++) {
    if (k > 0 && t[k].col == t[k - 1].col && t[k].row == t[k - 1].row) {
      if (nzval) nzval[nnz - 1] = nzval[nnz - 1] + v[t[k].pos];
      continue;
    }
    if (rowval) { rowval[nnz] = t[k].row; nzval[nnz] = v[t[k].pos]; }
    if (colptr) colptr[t[k].col + 1]++;
    nnz++;
  }
  if (colptr) for (i64 j = 0; j < n; j++) colptr[j + 1] += colptr[j];
  free(t);
  return nnz;
}


/*
 * The same COO -> CSC in linear time, by counting sorts, the way Julia's SparseArrays
 * builds a CSC from triplets: the entries are bucketed by row in input order, the
 * duplicates of each row are combined in input order, and a counting transpose moves
 * the combined entries into their columns (rows ascending).  Every stored value is the
 * same sum, taken in the same (input) order, as in orc_coo_to_csc_sorted, so the two are
 * bit-identical.  Out-of-range indices are skipped.  Returns nnz, or -1 when out of memory;
 * the three arrays are malloc'ed (release with orc_free).
 */
i64 orc_coo_to_csc_alloc(const i64 *indices, const double *v, i64 N, i64 n, i64 **colptr_out, i64 **rowval_out,
                         double **nzval_out) {
  i64 *rcnt = (i64 *)calloc((size_t)n + 2, sizeof(i64));
  i64 *bcol = (i64 *)malloc(sizeof(i64) * (size_t)(N > 0 ? N : 1));
  i64 *bpos = (i64 *)malloc(sizeof(i64) * (size_t)(N > 0 ? N : 1));
  i64 *stamp = (i64 *)malloc(sizeof(i64) * (size_t)(n > 0 ? n : 1));
  i64 *slot = (i64 *)malloc(sizeof(i64) * (size_t)(n > 0 ? n : 1));
  if (!rcnt || !bcol || !bpos || !stamp || !slot) {
    free(rcnt); free(bcol); free(bpos); free(stamp); free(slot);
    return -1;
  }
  for (i64 k = 0; k < N; k++) {
    const i64 r = indices[2 * k], c = indices[2 * k + 1];
    if (r >= 0 && r < n && c >= 0 && c < n) rcnt[r + 2]++;
  }
  for (i64 r = 0; r < n; r++) rcnt[r + 2] += rcnt[r + 1];
  /* rcnt[r + 1] is the next free bucket slot of row r */
  for (i64 k = 0; k < N; k++) {
    const i64 r = indices[2 * k], c = indices[2 * k + 1];
    if (r < 0 || r >= n || c < 0 || c >= n) continue;
    const i64 q = rcnt[r + 1]++;
    bcol[q] = c;
    bpos[q] = k;
  }
  /* combine duplicates row by row (in place: the combined row is a prefix of its bucket) */
  for (i64 c = 0; c < n; c++) stamp[c] = -1;
  double *bval = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
  i64 *rlen = (i64 *)calloc((size_t)n + 1, sizeof(i64));
  if (!bval || !rlen) {
    free(rcnt); free(bcol); free(bpos); free(stamp); free(slot); free(bval); free(rlen);
    return -1;
  }
  i64 nnz = 0;
  for (i64 r = 0; r < n; r++) {
    const i64 b0 = rcnt[r], b1 = rcnt[r + 1];
    i64 z = b0;
    for (i64 q = b0; q < b1; q++) {
      const i64 c = bcol[q];
      const double x = v[bpos[q]];
      if (stamp[c] == r) {
        bval[slot[c]] = bval[slot[c]] + x;
      } else {
        stamp[c] = r;
        slot[c] = z;
        bcol[z] = c;
        bval[z] = x;
        z++;
      }
    }
    rlen[r] = z - b0;
    nnz += z - b0;
  }
  free(bpos); free(stamp); free(slot);
  i64 *colptr = (i64 *)calloc((size_t)n + 2, sizeof(i64));
  i64 *rowval = (i64 *)malloc(sizeof(i64) * (size_t)(nnz > 0 ? nnz : 1));
  double *nzval = (double *)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  if (!colptr || !rowval || !nzval) {
    free(rcnt); free(bcol); free(bval); free(rlen); free(colptr); free(rowval); free(nzval);
    return -1;
  }
  for (i64 r = 0; r < n; r++)
    for (i64 q = rcnt[r]; q < rcnt[r] + rlen[r]; q++) colptr[bcol[q] + 2]++;
  for (i64 c = 0; c < n; c++) colptr[c + 2] += colptr[c + 1];
  /* colptr[c + 1] is the next free slot of column c; rows visited in ascending order */
  for (i64 r = 0; r < n; r++)
    for (i64 q = rcnt[r]; q < rcnt[r] + rlen[r]; q++) {
      const i64 t = colptr[bcol[q] + 1]++;
      rowval[t] = r;
      nzval[t] = bval[q];
    }
  free(rcnt); free(bcol); free(bval); free(rlen);
  *colptr_out = colptr;
  *rowval_out = rowval;
  *nzval_out = nzval;
  return nnz;
}

void orc_free(void *p) { free(p); }

/*
 * impose_Dirichlet_boundary_conditions, Array/SparseMatrixCSC arm, src/MFEM/MUtils.jl:184-199.
 * Output pattern follows Julia's sparse setindex! into spzeros: entries of A[idx,idx]
 * that are exactly zero are not inserted; the bd diagonal holds 1.0.
 * r[idx] = r[idx] - A[idx,bd]*bdval, the product accumulated column by column in bd order.
 * bd is 1-based, assumed free of duplicates.  0-based CSC in and out.
 * Two-call protocol: with ocolptr==NULL only returns the output nnz.
 */
i64 orc_dirichlet_csc(i64 n, const i64 *colptr, const i64 *rowval, const double *nzval, const double *rhs,
                      const i64 *bd, int bdN, const double *bdval, int keep_zeros, i64 *ocolptr, i64 *orowval,
                      double *onzval, double *orhs) {
  unsigned char *isbd = (unsigned char *)calloc((size_t)(n > 0 ? n : 1), 1);
  for (int k = 0; k < bdN; k++) isbd[bd[k] - 1] = 1;
  i64 z = 0;
  if (ocolptr) ocolptr[0] = 0;
  for (i64 j = 0; j < n; j++) {
    for (i64 p = colptr[j]; p < colptr[j + 1]; p++) {
      i64 i = rowval[p];
      int keep = 0;
      double val = 0.0;
      if (isbd[j]) { if (i == j) { keep = 1; val = 1.0; } }
      else if (!isbd[i]) { val = nzval[p]; keep = keep_zeros || val != 0.0; }
      if (keep) {
        if (orowval) { orowval[z] = i; onzval[z] = val; }
        z++;
      }
    }
    /* a bd column with no stored diagonal still receives the 1.0 */
    if (isbd[j]) {
      int has = 0;
      for (i64 p = colptr[j]; p < colptr[j + 1]; p++) if (rowval[p] == j) has = 1;
      if (!has) {
        /* insert in sorted position: rebuild this column's tail */
        if (orowval) {
          i64 s = ocolptr[j];
          i64 q = z;
          while (q > s && orowval[q - 1] > j) { orowval[q] = orowval[q - 1]; onzval[q] = onzval[q - 1]; q--; }
          orowval[q] = j; onzval[q] = 1.0;
        }
        z++;
      }
    }
    if (ocolptr) ocolptr[j + 1] = z;
  }
  if (orhs) {
    double *acc = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    for (int k = 0; k < bdN; k++) {
      i64 j = bd[k] - 1;
      for (i64 p = colptr[j]; p < colptr[j + 1]; p++) {
        i64 i = rowval[p];
        if (!isbd[i]) acc[i] += nzval[p] * bdval[k];
      }
    }
    for (i64 i = 0; i < n; i++) orhs[i] = isbd[i] ? 0.0 : rhs[i] - acc[i];
    for (int k = 0; k < bdN; k++) orhs[bd[k] - 1] = bdval[k];
    free(acc);
  }
  free(isbd);
  return z;
}

/*
 * bcnode, src/MFEM/MCore.jl:385-406,439-450: an edge belongs to the boundary when it
 * occurs an odd number of times (Set toggle); the node set is the union of their
 * endpoints.  Julia returns Set iteration order; this returns ascending order.
 * Returns the count; writes 1-based ids when out != NULL.
 */
i64 orc_bcnode(int nv, int ne, const int *elem, i64 *out) {
  i64 cap = 3 * (i64)ne;
  i64 *keys = (i64 *)malloc(sizeof(i64) * (size_t)(cap > 0 ? cap : 1));
  for (int e = 0; e < ne; e++)
    for (int l = 0; l < 3; l++) {
      i64 a = elem[3 * e + l], b = elem[3 * e + (l + 1) % 3];
      i64 lo = a < b ? a : b, hi = a < b ? b : a;
      keys[3 * e + l] = lo * (i64)nv + hi;
    }
  qsort(keys, (size_t)cap, sizeof(i64), cmp_i64);
  unsigned char *mark = (unsigned char *)calloc((size_t)nv + 1, 1);
  for (i64 k = 0; k < cap;) {
    i64 k2 = k;
    while (k2 < cap && keys[k2] == keys[k]) k2++;
    if ((k2 - k) % 2 == 1) { mark[keys[k] / nv] = 1; mark[keys[k] % nv] = 1; }
    k = k2;
  }
  i64 c = 0;
  for (int i = 0; i < nv; i++)
    if (mark[i]) { if (out) out[c] = i + 1; c++; }
  free(keys); free(mark);
  return c;
}

/*
 * Residual r = b - A x of a 0-based CSC matrix in doubled precision (error-free
 * transformations: the product a*x split exactly with fma, each row's running sum kept
 * as an unevaluated pair hi + lo updated by a two-sum), rounded to double at the end.
 * The result is the residual of the stored FP64 vector x to about 2^-100 relative, so
 * residuals at the FP64 rounding floor of x are measured, not swamped by the rounding of
 * their own evaluation.  Used to check GPU solutions against the oracle's operator.
 */
void orc_residual_csc_dd(i64 n, const i64 *colptr, const i64 *rowval, const double *nzval, const double *x,
                         const double *b, double *r) {
  double *lo = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  for (i64 i = 0; i < n; i++) r[i] = b[i];
  for (i64 j = 0; j < n; j++) {
    const double xj = x[j];
    for (i64 p = colptr[j]; p < colptr[j + 1]; p++) {
      const i64 i = rowval[p];
      const double ph = -nzval[p] * xj;
      const double pl = fma(-nzval[p], xj, -ph); /* exact: -a*x = ph + pl */
      const double s = r[i] + ph;
      const double bb = s - r[i];
      const double e = (r[i] - (s - bb)) + (ph - bb); /* exact: r + ph = s + e */
      r[i] = s;
      lo[i] += e + pl;
    }
  }
  for (i64 i = 0; i < n; i++) r[i] = r[i] + lo[i];
  free(lo);
}

/* ---- CPU Jacobi-PCG on a 0-based CSR matrix (FP64), multithreaded with pthreads ----
 * Used as the timed CPU baseline where a direct solve does not fit the time bound.
 * Per-thread partial dot products are combined in thread order, so results are
 * deterministic for a fixed thread count. */
typedef struct {
  int tid, nth; i64 n;
  const i64 *rowptr; const int *col; const double *val;
  const double *dinv;
  double *x, *r, *z, *p, *q;
  double alpha, beta;
  double part, part2;
  int phase;
} pcg_arg;

static void *pcg_work(void *vp) {
  pcg_arg *a = (pcg_arg *)vp;
  i64 lo = a->n * a->tid / a->nth, hi = a->n * (a->tid + 1) / a->nth;
  double s = 0.0, s2 = 0.0;
  if (a->phase == 0) { /* q = A p; part = p.q */
    for (i64 i = lo; i < hi; i++) {
      double acc = 0.0;
      for (i64 k = a->rowptr[i]; k < a->rowptr[i + 1]; k++) acc += a->val[k] * a->p[a->col[k]];
      a->q[i] = acc;
      s += a->p[i] * acc;
    }
  } else if (a->phase == 1) { /* x += alpha p; r -= alpha q; z = dinv r; part = r.z */
    for (i64 i = lo; i < hi; i++) {
      a->x[i] += a->alpha * a->p[i];
      a->r[i] -= a->alpha * a->q[i];
      a->z[i] = a->dinv[i] * a->r[i];
      s += a->r[i] * a->z[i];
      s2 += a->r[i] * a->r[i];
    }
  } else { /* p = z + beta p */
    for (i64 i = lo; i < hi; i++) a->p[i] = a->z[i] + a->beta * a->p[i];
  }
  a->part = s;
  a->part2 = s2;
  return NULL;
}

static double pcg_phase(pcg_arg *args, int nth, int phase, double *second) {
  pthread_t th[256];
  for (int t = 0; t < nth; t++) { args[t].phase = phase; if (t > 0) pthread_create(&th[t], NULL, pcg_work, &args[t]); }
  pcg_work(&args[0]);
  for (int t = 1; t < nth; t++) pthread_join(th[t], NULL);
  double s = 0.0, s2 = 0.0;
  for (int t = 0; t < nth; t++) { s += args[t].part; s2 += args[t].part2; }
  if (second) *second = s2;
  return s;
}

/* Solves A x = b from x = 0.  Stops when ||r|| <= rtol ||b|| (recursive residual) or after
 * max_iter iterations.  Returns the iteration count. */
int orc_pcg(i64 n, const i64 *rowptr, const int *col, const double *val, const double *b, double *x, double rtol,
            int max_iter, int nth, double *final_relres) {
  if (nth < 1) nth = 1;
  if (nth > 256) nth = 256;
  double *r = (double *)malloc(sizeof(double) * (size_t)n), *z = (double *)malloc(sizeof(double) * (size_t)n);
  double *p = (double *)malloc(sizeof(double) * (size_t)n), *q = (double *)malloc(sizeof(double) * (size_t)n);
  double *dinv = (double *)malloc(sizeof(double) * (size_t)n);
  double bb = 0.0, rz = 0.0;
  for (i64 i = 0; i < n; i++) {
    double d = 0.0;
    for (i64 k = rowptr[i]; k < rowptr[i + 1]; k++) if (col[k] == i) d = val[k];
    dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
    x[i] = 0.0; r[i] = b[i]; z[i] = dinv[i] * r[i]; p[i] = z[i];
    bb += b[i] * b[i]; rz += r[i] * z[i];
  }
  pcg_arg args[256];
  for (int t = 0; t < nth; t++) {
    args[t].tid = t; args[t].nth = nth; args[t].n = n; args[t].rowptr = rowptr; args[t].col = col; args[t].val = val;
    args[t].dinv = dinv; args[t].x = x; args[t].r = r; args[t].z = z; args[t].p = p; args[t].q = q;
  }
  double bnorm = sqrt(bb);
  int it = 0;
  double relres = bnorm > 0 ? 1.0 : 0.0;
  while (it < max_iter && bnorm > 0) {
    double pq = pcg_phase(args, nth, 0, NULL);
    if (!(pq > 0.0)) break;
    double alpha = rz / pq;
    for (int t = 0; t < nth; t++) args[t].alpha = alpha;
    double rr = 0.0;
    double rz_new = pcg_phase(args, nth, 1, &rr);
    it++;
    relres = sqrt(rr) / bnorm;
    if (relres <= rtol) break;
    double beta = rz_new / rz;
    rz = rz_new;
    for (int t = 0; t < nth; t++) args[t].beta = beta;
    pcg_phase(args, nth, 2, NULL);
  }
  if (final_relres) *final_relres = relres;
  free(r); free(z); free(p); free(q); free(dinv);
  return it;
}

/* A few PCG iterations only (for bounded CPU timing samples): identical arithmetic to orc_pcg. */
int orc_pcg_iters(i64 n, const i64 *rowptr, const int *col, const double *val, const double *b, double *x, int iters,
                  int nth) {
  double rr;
  return orc_pcg(n, rowptr, col, val, b, x, 0.0, iters, nth, &rr);
}
