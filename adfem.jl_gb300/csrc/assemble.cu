// Assembly kernels for the P1 path (sm_103a).
//
// Design: GB300 executes FP64 at ~1.2 TFLOP/s (1/58 of FP32), so the kernels are
// built to spend as few FP64 instructions as possible per byte moved:
//  * per-mesh geometry is precomputed once: g_ab = w * grad phi_a . grad phi_b for
//    the three vertex pairs of each element, and w = ip.weight * area / 0.5;
//  * an element prepass reduces the per-Gauss-point inputs to per-element values
//    (sigma_e = sum_k kappa_k, src_e[r] = w sum_k f_k phi_r(x_k));
//  * the matrix is then assembled ROW BY ROW: the thread owning node i walks the
//    elements around i in ascending element order and accumulates its row in
//    shared memory.  Each CSR value is summed by exactly one thread in a fixed
//    order, so assembly is bit-reproducible, needs no atomics and writes each
//    output value once.  The diagonal is the negated sum of the off-diagonals
//    (P1 element matrices have zero row sums).
#include "adfem_internal.h"
#include "checks.cuh"
#include "pairs.cuh"

namespace adfem {

static constexpr int kBlock = 256;

__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
static inline unsigned nblocks(int64_t n, int b = kBlock) { return (unsigned)((n + b - 1) / b); }

// barycentric coordinate of vertex r at quadrature point k: points 0,1,2 are
// (xi,eta) = (1/6,1/6), (1/6,2/3), (2/3,1/6) so phi = (1-xi-eta, xi, eta)
__device__ __forceinline__ double lam(int k, int r) {
  const double qx = (k == 2) ? 2.0 / 3.0 : 1.0 / 6.0;
  const double qy = (k == 1) ? 2.0 / 3.0 : 1.0 / 6.0;
  return r == 0 ? 1.0 - qx - qy : (r == 1 ? qx : qy);
}

// g of the vertex pair (a, b), a != b, from {g01, g02, g12}
__device__ __forceinline__ double gpair(const double4& g, int a, int b) {
  int s = a + b;  // 1 -> (0,1), 2 -> (0,2), 3 -> (1,2)
  return s == 1 ? g.x : (s == 2 ? g.y : g.z);
}

// ---------------------------------------------------------------------------
// src_e[r] = w sum_k f_k phi_r(x_k).  With the degree-2 rule above, phi_r is 2/3 at one
// point k*(r) and 1/6 at the other two (k* = 0, 2, 1 for r = 0, 1, 2), so the sum is
// w (S/6 + f_{k*}/2) with S = f0 + f1 + f2: 11 FP64 operations per element instead of 14
// (the element pass is FP64-instruction bound on GB300).
// WEIGHTED = false leaves out the factor w (8 FP64 operations per element, and no read of
// the 32-byte geometry record, whose other three doubles came along with w in the same
// sector: 640 of the pass's 868 MB at 4M DOF were reads, 256 MB of them geometry); the
// fused Poisson row pass multiplies each term by w, which it reads with the geometry anyway.
template <bool WEIGHTED>
__global__ void k_element_prepass(int64_t ne, const double* __restrict__ kappa, const double* __restrict__ f,
                                  const double4* __restrict__ geo, double* __restrict__ sigma,
                                  double* __restrict__ src3) {
  int64_t e = gtid();
  if (e >= ne) return;
  if (kappa) sigma[e] = kappa[3 * e] + kappa[3 * e + 1] + kappa[3 * e + 2];
  if (f) {
    const double f0 = f[3 * e], f1 = f[3 * e + 1], f2 = f[3 * e + 2];
    const double s6 = (f0 + f1 + f2) * (1.0 / 6.0);
    if (WEIGHTED) {
      const double w = geo[e].w;
      src3[3 * e] = w * fma(f0, 0.5, s6);
      src3[3 * e + 1] = w * fma(f2, 0.5, s6);
      src3[3 * e + 2] = w * fma(f1, 0.5, s6);
    } else {
      src3[3 * e] = fma(f0, 0.5, s6);
      src3[3 * e + 1] = fma(f2, 0.5, s6);
      src3[3 * e + 2] = fma(f1, 0.5, s6);
    }
  }
}

cudaError_t launch_element_prepass(const Mesh& m, const double* kappa, const double* f, double* sigma, double* src3,
                                   cudaStream_t st) {
  k_element_prepass<true><<<nblocks(m.ne), kBlock, 0, st>>>(m.ne, kappa, f, m.d_geo.as<double4>(), sigma, src3);
  return cudaGetLastError();
}

cudaError_t launch_element_prepass_unweighted(const Mesh& m, const double* kappa, const double* f, double* sigma,
                                              double* src3, cudaStream_t st) {
  k_element_prepass<false><<<nblocks(m.ne), kBlock, 0, st>>>(m.ne, kappa, f, nullptr, sigma, src3);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// output addressing of entry k of row i
struct OutCSR {
  const int32_t* rowptr;
  __device__ __forceinline__ int64_t at(int64_t i, int k) const { return (int64_t)rowptr[i] + k; }
};
struct OutSELL {
  const int32_t* sptr;
  __device__ __forceinline__ int64_t at(int64_t i, int k) const { return (int64_t)sptr[i >> 5] + 32 * k + (i & 31); }
};

// Accumulate the Laplace row of node i into acc[.][t].  LOAD: in the same walk over the
// incident elements, return the node's load sum_e w_e src3[e][a] (src3 without the weight;
// the weight is the fourth double of the geometry record the row reads anyway).
template <int MAXW, bool LOAD = false, int BT = kBlock>
__device__ __forceinline__ double laplace_row_acc(int64_t i, const int32_t* __restrict__ inc_ptr,
                                                  const uint2* __restrict__ inc, const double4* __restrict__ geo,
                                                  const double* __restrict__ sigma, int w, int dp,
                                                  double (*acc)[BT], int t,
                                                  const double* __restrict__ src3 = nullptr) {
  for (int k = 0; k < w; k++) acc[k][t] = 0.0;
  double r = 0.0;
  const int32_t s1 = inc_ptr[i + 1];
  for (int32_t s = inc_ptr[i]; s < s1; s++) {
    const uint2 rec = inc[s];
    const unsigned e = rec.x, y = rec.y, a = inc_a(y);
    const double4 g = geo[e];
    const double sg = sigma[e];
    if (LOAD) r = fma(g.w, src3[3 * (int64_t)e + a], r);
    const unsigned b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
    const unsigned ob = inc_off(y, b), oc = inc_off(y, c);
    if (!ADFEM_DCHECK(ob < (unsigned)w && oc < (unsigned)w && ob < MAXW && oc < MAXW)) continue;
    acc[ob][t] = fma(gpair(g, a, b), sg, acc[ob][t]);
    acc[oc][t] = fma(gpair(g, a, c), sg, acc[oc][t]);
  }
  double d = 0.0;
  for (int k = 0; k < w; k++)
    if (k != dp) d -= acc[k][t];
  acc[dp][t] = d;
  return r;
}

template <int MAXW, class Out>
__global__ void __launch_bounds__(kBlock) k_laplace_rows(int64_t n, const int32_t* __restrict__ inc_ptr,
                                                         const uint2* __restrict__ inc,
                                                         const double4* __restrict__ geo,
                                                         const double* __restrict__ sigma,
                                                         const int32_t* __restrict__ rowptr,
                                                         const int32_t* __restrict__ diagpos, Out out,
                                                         double* __restrict__ vals) {
  __shared__ double acc[MAXW][kBlock];
  const int t = threadIdx.x;
  const int64_t i = gtid();
  if (i >= n) return;
  const int w = rowptr[i + 1] - rowptr[i];
  const int dp = diagpos[i];
  laplace_row_acc<MAXW>(i, inc_ptr, inc, geo, sigma, w, dp, acc, t);
  for (int k = 0; k < w; k++) vals[out.at(i, k)] = acc[k][t];
}

template <class Out>
static cudaError_t laplace_rows_dispatch(const Mesh& m, const double* sigma, double* vals, Out out, cudaStream_t st) {
  const auto* ip = m.d_inc_ptr.as<int32_t>();
  const auto* inc = m.d_inc.as<uint2>();
  const auto* geo = m.d_geo.as<double4>();
  const auto* rp = m.d_rowptr.as<int32_t>();
  const auto* dp = m.d_diagpos.as<int32_t>();
  if (m.maxrow <= 8)
    k_laplace_rows<8, Out><<<nblocks(m.nv), kBlock, 0, st>>>(m.nv, ip, inc, geo, sigma, rp, dp, out, vals);
  else if (m.maxrow <= 16)
    k_laplace_rows<16, Out><<<nblocks(m.nv), kBlock, 0, st>>>(m.nv, ip, inc, geo, sigma, rp, dp, out, vals);
  else if (m.maxrow <= 24)
    k_laplace_rows<24, Out><<<nblocks(m.nv), kBlock, 0, st>>>(m.nv, ip, inc, geo, sigma, rp, dp, out, vals);
  else
    return cudaErrorInvalidValue;  // mesh_build rejects rows > 64; wider rows take the generic path below
  return cudaGetLastError();
}

// generic (wide rows, up to 64): dynamic shared memory, smaller blocks
template <class Out>
__global__ void __launch_bounds__(64) k_laplace_rows_wide(int64_t n, const int32_t* __restrict__ inc_ptr,
                                                          const uint2* __restrict__ inc,
                                                          const double4* __restrict__ geo,
                                                          const double* __restrict__ sigma,
                                                          const int32_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ diagpos, Out out,
                                                          double* __restrict__ vals) {
  __shared__ double acc[64][64];
  const int t = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * 64 + t;
  if (i >= n) return;
  const int w = rowptr[i + 1] - rowptr[i];
  const int dp = diagpos[i];
  for (int k = 0; k < w; k++) acc[k][t] = 0.0;
  for (int32_t s = inc_ptr[i]; s < inc_ptr[i + 1]; s++) {
    const uint2 rec = inc[s];
    const unsigned e = rec.x, y = rec.y, a = inc_a(y);
    const double4 g = geo[e];
    const double sg = sigma[e];
    const unsigned b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
    acc[inc_off(y, b)][t] = fma(gpair(g, a, b), sg, acc[inc_off(y, b)][t]);
    acc[inc_off(y, c)][t] = fma(gpair(g, a, c), sg, acc[inc_off(y, c)][t]);
  }
  double d = 0.0;
  for (int k = 0; k < w; k++)
    if (k != dp) d -= acc[k][t];
  acc[dp][t] = d;
  for (int k = 0; k < w; k++) vals[out.at(i, k)] = acc[k][t];
}

cudaError_t launch_laplace_rows(const Mesh& m, const double* sigma, double* vals, Layout lay, cudaStream_t st) {
  if (m.maxrow > 24) {
    if (lay == Layout::SELL)
      k_laplace_rows_wide<OutSELL><<<nblocks(m.nv, 64), 64, 0, st>>>(
          m.nv, m.d_inc_ptr.as<int32_t>(), m.d_inc.as<uint2>(), m.d_geo.as<double4>(), sigma,
          m.d_rowptr.as<int32_t>(), m.d_diagpos.as<int32_t>(), OutSELL{m.sell.sptr.as<int32_t>()}, vals);
    else
      k_laplace_rows_wide<OutCSR><<<nblocks(m.nv, 64), 64, 0, st>>>(
          m.nv, m.d_inc_ptr.as<int32_t>(), m.d_inc.as<uint2>(), m.d_geo.as<double4>(), sigma,
          m.d_rowptr.as<int32_t>(), m.d_diagpos.as<int32_t>(), OutCSR{m.d_rowptr.as<int32_t>()}, vals);
    return cudaGetLastError();
  }
  if (lay == Layout::SELL) return laplace_rows_dispatch(m, sigma, vals, OutSELL{m.sell.sptr.as<int32_t>()}, st);
  return laplace_rows_dispatch(m, sigma, vals, OutCSR{m.d_rowptr.as<int32_t>()}, st);
}

// ---------------------------------------------------------------------------
__global__ void k_source_rows(int64_t n, const int32_t* __restrict__ inc_ptr, const uint2* __restrict__ inc,
                              const double* __restrict__ src3, double* __restrict__ rhs, int accumulate) {
  const int64_t i = gtid();
  if (i >= n) return;
  double s = accumulate ? rhs[i] : 0.0;
  for (int32_t j = inc_ptr[i]; j < inc_ptr[i + 1]; j++) {
    const uint2 rec = inc[j];
    s += src3[3 * (int64_t)rec.x + inc_a(rec.y)];
  }
  rhs[i] = s;
}

cudaError_t launch_source_rows(const Mesh& m, const double* src3, double* rhs, bool accumulate, cudaStream_t st) {
  k_source_rows<<<nblocks(m.nv), kBlock, 0, st>>>(m.nv, m.d_inc_ptr.as<int32_t>(), m.d_inc.as<uint2>(), src3, rhs,
                                                  accumulate ? 1 : 0);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Fused Poisson system: Laplace row + load + Dirichlet in one pass, into sliced-ELL.
// isbd[i]: 0 interior, 1 Dirichlet node, 2 interior with a Dirichlet neighbour.
// PERM: the system's DOFs are renumbered (nperm[node] = solver row); the row of mesh
// node i goes to solver row nperm[i], its slot k to the rank kperm[rowptr[i] + k] of the
// renumbered column in that row; isbd, bdval and rhs are in solver order.
// src3 holds the element load terms without the weight (k_element_prepass<false>): the
// row's one walk over its elements gathers them with the geometry and multiplies each by
// its element's w in an FMA, in place of a plain add, so the row costs the same FP64
// operations as with weighted terms (a second walk for the load, loading w once more,
// measured 271 us against 234 us at 4M DOF).
// BT threads per block: kBlock up to 24 entries per row; rows of up to 64 (vertices of up to
// 63 neighbours, the most mesh_build accepts) in blocks of 64, 32 KB of static shared memory.
template <int MAXW, bool PERM, int BT = kBlock>
__global__ void __launch_bounds__(BT) k_poisson_system(
    int64_t n, const int32_t* __restrict__ inc_ptr, const uint2* __restrict__ inc, const double4* __restrict__ geo,
    const double* __restrict__ sigma, const double* __restrict__ src3, const int32_t* __restrict__ rowptr,
    const int32_t* __restrict__ colind, const int32_t* __restrict__ diagpos, const int32_t* __restrict__ sptr,
    const uint8_t* __restrict__ isbd, const double* __restrict__ bdval, double* __restrict__ vals,
    double* __restrict__ rhs, const int32_t* __restrict__ nperm, const uint8_t* __restrict__ kperm) {
  __shared__ double acc[MAXW][BT];
  const int t = threadIdx.x;
  const int64_t i = gtid();
  if (i >= n) return;
  const int w = rowptr[i + 1] - rowptr[i];
  const int32_t r0 = rowptr[i];
  const int64_t ri = PERM ? (int64_t)nperm[i] : i;
  const int dp = diagpos[i];
  const int64_t base = (int64_t)sptr[ri >> 5] + (ri & 31);
  const uint8_t tag = isbd[ri];
  if (tag == 1) {
    const int dps = PERM ? (int)kperm[r0 + dp] : dp;
    for (int k = 0; k < w; k++) vals[base + 32 * k] = (k == dps) ? 1.0 : 0.0;
    rhs[ri] = bdval[ri];
    return;
  }
  double r = laplace_row_acc<MAXW, true, BT>(i, inc_ptr, inc, geo, sigma, w, dp, acc, t, src3);
  if (tag == 2) {
    for (int k = 0; k < w; k++) {
      const int64_t j = PERM ? (int64_t)nperm[colind[r0 + k]] : (int64_t)colind[r0 + k];
      if (isbd[j] == 1) {
        r = fma(-acc[k][t], bdval[j], r);
        acc[k][t] = 0.0;
      }
    }
  }
  rhs[ri] = r;
  for (int k = 0; k < w; k++) vals[base + 32 * (PERM ? (int)kperm[r0 + k] : k)] = acc[k][t];
}

// ---------------------------------------------------------------------------
// The same fused Poisson system in FP32-pair arithmetic.  GB300 retires FP64 instructions
// ~70x slower than FP32 / integer ones, and the FP64 kernels above are bound by them
// (0.41 ms at 4M DOF for 184M FP64 operations, 0.7 of the FP64 issue rate, when the element
// pass applied the weight; 0.36 ms for 160M since the row pass applies it); here every
// operation is a pair operation (~48 bits: each value lands within ~1e-14 relative of the
// FP64 one), the FP64 inputs are split into pairs with integer instructions (d2p, in the
// element pass k_element_prepass_p: once per input) and each output costs one FP64 add
// (p2d).  The thread owning node i walks its elements in ascending order as the FP64 kernel
// does: the two off-diagonal entries g_ab sigma_e, g_ac sigma_e and the element's load term
// for vertex a; the diagonal is the negated sum of the off-diagonals.  Geometry pairs per
// element (gpa: g01, g02; gpb: g12, w/6; gpc: w/2) are derived once per mesh
// (mesh_geo_pairs).  (Splitting kappa and f in this pass instead, once per vertex of each
// element, measured 0.39 ms at 4M DOF against 0.41 ms for the FP64 kernels.)
template <int MAXW, bool PERM>
__global__ void __launch_bounds__(kBlock) k_poisson_system_p(
    int64_t n, const int32_t* __restrict__ inc_ptr, const uint2* __restrict__ inc, const float4* __restrict__ gpa,
    const float4* __restrict__ gpb, const float2* __restrict__ sigma, const float2* __restrict__ src3,
    const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
    const int32_t* __restrict__ diagpos, const int32_t* __restrict__ sptr, const uint8_t* __restrict__ isbd,
    const double* __restrict__ bdval, double* __restrict__ vals, double* __restrict__ rhs,
    const int32_t* __restrict__ nperm, const uint8_t* __restrict__ kperm) {
  __shared__ float2 acc[MAXW][kBlock];
  const int t = threadIdx.x;
  const int64_t i = gtid();
  if (i >= n) return;
  const int w = rowptr[i + 1] - rowptr[i];
  const int32_t r0 = rowptr[i];
  const int64_t ri = PERM ? (int64_t)nperm[i] : i;
  const int dp = diagpos[i];
  const int64_t base = (int64_t)sptr[ri >> 5] + (ri & 31);
  const uint8_t tag = isbd[ri];
  if (tag == 1) {
    const int dps = PERM ? (int)kperm[r0 + dp] : dp;
    for (int k = 0; k < w; k++) vals[base + 32 * k] = (k == dps) ? 1.0 : 0.0;
    rhs[ri] = bdval[ri];
    return;
  }
  for (int k = 0; k < w; k++) acc[k][t] = make_float2(0.0f, 0.0f);
  float2 r = make_float2(0.0f, 0.0f);
  // incidences in batches of kIB: all record loads, then all element loads, then the sums
  // (two dependent load steps per batch instead of two per incidence), in element order
  constexpr int kIB = 4;
  const int32_t s1 = inc_ptr[i + 1];
  for (int32_t sb = inc_ptr[i]; sb < s1; sb += kIB) {
    uint2 rec[kIB];
#pragma unroll
    for (int u = 0; u < kIB; u++) rec[u] = sb + u < s1 ? inc[sb + u] : make_uint2(0u, 0u);
    float4 A[kIB];
    float2 G[kIB], SG[kIB], SR[kIB];
#pragma unroll
    for (int u = 0; u < kIB; u++) {
      const unsigned e = rec[u].x, a = inc_a(rec[u].y);
      A[u] = gpa[e];
      G[u] = reinterpret_cast<const float2*>(gpb)[2 * (int64_t)e];  // g12
      SG[u] = sigma[e];
      SR[u] = src3[3 * (int64_t)e + a];
    }
#pragma unroll
    for (int u = 0; u < kIB; u++) {
      if (sb + u >= s1) break;
      const unsigned y = rec[u].y, a = inc_a(y);
      const unsigned b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
      const unsigned ob = inc_off(y, b), oc = inc_off(y, c);
      if (!ADFEM_DCHECK(ob < (unsigned)w && oc < (unsigned)w && ob < MAXW && oc < MAXW)) continue;
      // g of the pairs (a, b) and (a, c): (0,1) (0,2) for a = 0, (0,1) (1,2) for a = 1, (0,2) (1,2) for a = 2
      const float2 g01 = make_float2(A[u].x, A[u].y), g02 = make_float2(A[u].z, A[u].w);
      const float2 gab = a == 2 ? g02 : g01;
      const float2 gac = a == 0 ? g02 : G[u];
      acc[ob][t] = df_add(acc[ob][t], df_mul(gab, SG[u]));
      acc[oc][t] = df_add(acc[oc][t], df_mul(gac, SG[u]));
      r = df_add(r, SR[u]);
    }
  }
  float2 d = make_float2(0.0f, 0.0f);
  for (int k = 0; k < w; k++)
    if (k != dp) d = df_add(d, acc[k][t]);
  acc[dp][t] = df_neg(d);
  if (tag == 2) {
    for (int k = 0; k < w; k++) {
      const int64_t j = PERM ? (int64_t)nperm[colind[r0 + k]] : (int64_t)colind[r0 + k];
      if (isbd[j] == 1) {
        r = df_add(r, df_neg(df_mul(acc[k][t], d2p(bdval[j]))));
        acc[k][t] = make_float2(0.0f, 0.0f);
      }
    }
  }
  rhs[ri] = p2d(r);
  for (int k = 0; k < w; k++) vals[base + 32 * (PERM ? (int)kperm[r0 + k] : k)] = p2d(acc[k][t]);
}

// Element pass of the pair-arithmetic system: sigma_e = kappa_0 + kappa_1 + kappa_2 and the
// three load terms src_e[r] = w (S/6 + f_k*(r)/2) as FP32 pairs (each FP64 input split once
// per element instead of once per vertex of the element)
__global__ void k_element_prepass_p(int64_t ne, const double* __restrict__ kappa, const double* __restrict__ f,
                                    const float4* __restrict__ gpb, const float2* __restrict__ gpc,
                                    float2* __restrict__ sigma, float2* __restrict__ src3) {
  const int64_t e = gtid();
  if (e >= ne) return;
  const double* kp = kappa + 3 * e;
  sigma[e] = df_add(df_add(d2p(kp[0]), d2p(kp[1])), d2p(kp[2]));
  const double* fp = f + 3 * e;
  const float2 f0 = d2p(fp[0]), f1 = d2p(fp[1]), f2 = d2p(fp[2]);
  const float4 B = gpb[e];
  const float2 w6 = make_float2(B.z, B.w), w2 = gpc[e];
  const float2 t = df_mul(df_add(df_add(f0, f1), f2), w6);
  src3[3 * e] = df_add(t, df_mul(f0, w2));
  src3[3 * e + 1] = df_add(t, df_mul(f2, w2));
  src3[3 * e + 2] = df_add(t, df_mul(f1, w2));
}

// geometry pairs of every element from the FP64 geometry (once per mesh)
__global__ void k_geo_pairs(int64_t ne, const double4* __restrict__ geo, float4* __restrict__ gpa,
                            float4* __restrict__ gpb, float2* __restrict__ gpc) {
  const int64_t e = gtid();
  if (e >= ne) return;
  const double4 g = geo[e];
  auto split = [](double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
  };
  const float2 a = split(g.x), b = split(g.y), c = split(g.z), w6 = split(g.w / 6.0), w2 = split(g.w * 0.5);
  gpa[e] = make_float4(a.x, a.y, b.x, b.y);
  gpb[e] = make_float4(c.x, c.y, w6.x, w6.y);
  gpc[e] = w2;
}

int mesh_geo_pairs(Mesh& m) {
  std::lock_guard<std::mutex> lk(m.mu);
  if (m.d_gpc.p) return ADFEM_OK;
  DevBuf a, b, c;
  ADFEM_TRY(a.alloc(sizeof(float4) * (size_t)std::max<int64_t>(m.ne, 1)));
  ADFEM_TRY(b.alloc(sizeof(float4) * (size_t)std::max<int64_t>(m.ne, 1)));
  ADFEM_TRY(c.alloc(sizeof(float2) * (size_t)std::max<int64_t>(m.ne, 1)));
  if (m.ne > 0) {
    k_geo_pairs<<<nblocks(m.ne), kBlock>>>(m.ne, m.d_geo.as<double4>(), a.as<float4>(), b.as<float4>(),
                                            c.as<float2>());
    ADFEM_CUDA(cudaGetLastError());
    // (legacy-stream sync, not a device-wide one: other threads may be capturing graphs)
    ADFEM_CUDA(cudaStreamSynchronize(0));
  }
  std::swap(m.d_gpa.p, a.p);
  std::swap(m.d_gpa.bytes, a.bytes);
  std::swap(m.d_gpb.p, b.p);
  std::swap(m.d_gpb.bytes, b.bytes);
  std::swap(m.d_gpc.p, c.p);
  std::swap(m.d_gpc.bytes, c.bytes);
  return ADFEM_OK;
}

cudaError_t launch_element_prepass_pairs(const Mesh& m, const double* kappa, const double* f, float2* sigma,
                                         float2* src3, cudaStream_t st) {
  k_element_prepass_p<<<nblocks(m.ne), kBlock, 0, st>>>(m.ne, kappa, f, m.d_gpb.as<float4>(), m.d_gpc.as<float2>(),
                                                         sigma, src3);
  return cudaGetLastError();
}

cudaError_t launch_poisson_system_pairs(const Mesh& m, const float2* sigma, const float2* src3, const uint8_t* isbd,
                                        const double* bdval_dense, double* sell_vals, double* rhs,
                                        const int32_t* sptr, const int32_t* diagpos_mesh, const int32_t* nperm,
                                        const uint8_t* kperm, cudaStream_t st) {
  const auto* ip = m.d_inc_ptr.as<int32_t>();
  const auto* inc = m.d_inc.as<uint2>();
  const auto* gpa = m.d_gpa.as<float4>();
  const auto* gpb = m.d_gpb.as<float4>();
  const auto* rp = m.d_rowptr.as<int32_t>();
  const auto* ci = m.d_colind.as<int32_t>();
  const unsigned nb = nblocks(m.nv);
#define ADFEM_PSP(W)                                                                                             \
  do {                                                                                                           \
    if (nperm)                                                                                                   \
      k_poisson_system_p<W, true><<<nb, kBlock, 0, st>>>(m.nv, ip, inc, gpa, gpb, sigma, src3, rp, ci,            \
                                                         diagpos_mesh, sptr, isbd, bdval_dense, sell_vals, rhs,  \
                                                         nperm, kperm);                                          \
    else                                                                                                         \
      k_poisson_system_p<W, false><<<nb, kBlock, 0, st>>>(m.nv, ip, inc, gpa, gpb, sigma, src3, rp, ci,           \
                                                          diagpos_mesh, sptr, isbd, bdval_dense, sell_vals, rhs, \
                                                          nullptr, nullptr);                                     \
  } while (0)
  if (m.maxrow <= 8) ADFEM_PSP(8);
  else if (m.maxrow <= 16) ADFEM_PSP(16);
  else return cudaErrorNotSupported;  // (the FP64 kernel serves wider rows)
#undef ADFEM_PSP
  return cudaGetLastError();
}

cudaError_t launch_poisson_system(const Mesh& m, const double* sigma, const double* src3, const uint8_t* isbd,
                                  const double* bdval_dense, double* sell_vals, double* rhs, const int32_t* sptr,
                                  const int32_t* diagpos_mesh, const int32_t* nperm, const uint8_t* kperm,
                                  cudaStream_t st) {
  const auto* ip = m.d_inc_ptr.as<int32_t>();
  const auto* inc = m.d_inc.as<uint2>();
  const auto* geo = m.d_geo.as<double4>();
  const auto* rp = m.d_rowptr.as<int32_t>();
  const auto* ci = m.d_colind.as<int32_t>();
  const auto* dp = diagpos_mesh;
  const unsigned nb = nblocks(m.nv);
#define ADFEM_PS(W)                                                                                            \
  do {                                                                                                         \
    if (nperm)                                                                                                 \
      k_poisson_system<W, true><<<nb, kBlock, 0, st>>>(m.nv, ip, inc, geo, sigma, src3, rp, ci, dp, sptr, isbd, \
                                                       bdval_dense, sell_vals, rhs, nperm, kperm);              \
    else                                                                                                       \
      k_poisson_system<W, false><<<nb, kBlock, 0, st>>>(m.nv, ip, inc, geo, sigma, src3, rp, ci, dp, sptr,      \
                                                        isbd, bdval_dense, sell_vals, rhs, nullptr, nullptr);  \
  } while (0)
  if (m.maxrow <= 8) ADFEM_PS(8);
  else if (m.maxrow <= 16) ADFEM_PS(16);
  else if (m.maxrow <= 24) ADFEM_PS(24);
  else if (m.maxrow <= 64) {
    const unsigned nbw = nblocks(m.nv, 64);
    if (nperm)
      k_poisson_system<64, true, 64><<<nbw, 64, 0, st>>>(m.nv, ip, inc, geo, sigma, src3, rp, ci, dp, sptr, isbd,
                                                           bdval_dense, sell_vals, rhs, nperm, kperm);
    else
      k_poisson_system<64, false, 64><<<nbw, 64, 0, st>>>(m.nv, ip, inc, geo, sigma, src3, rp, ci, dp, sptr, isbd,
                                                            bdval_dense, sell_vals, rhs, nullptr, nullptr);
  } else {
    return cudaErrorNotSupported;
  }
#undef ADFEM_PS
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Unsummed COO of FemLaplaceScalar_forward (FemLaplaceScalar.h:3-26): entry
// z = 27 e + 9 k + 3 p + q is (dof_p, dof_q, (w grad_p.grad_q) kappa_{3e+k}).
// One thread per entry keeps the 16-byte index and 8-byte value stores coalesced.
__global__ void k_laplace_coo(int64_t ne, const int4* __restrict__ conn, const double4* __restrict__ geo,
                              const double* __restrict__ kappa, longlong2* __restrict__ idx,
                              double* __restrict__ vv) {
  const int64_t z = gtid();
  if (z >= 27 * ne) return;
  const int64_t e = z / 27;
  const int rem = (int)(z - 27 * e);
  const int k = rem / 9, p = (rem / 3) % 3, q = rem % 3;
  const int4 c = conn[e];
  const double4 g = geo[e];
  double gpq;
  if (p != q) {
    gpq = gpair(g, p, q);
  } else {
    const int b = (p == 0) ? 1 : 0, cc = (p == 2) ? 1 : 2;
    gpq = -(gpair(g, p, b) + gpair(g, p, cc));
  }
  const int vp = p == 0 ? c.x : (p == 1 ? c.y : c.z);
  const int vq = q == 0 ? c.x : (q == 1 ? c.y : c.z);
  idx[z] = make_longlong2(vp, vq);
  vv[z] = gpq * kappa[3 * e + k];
}

cudaError_t launch_laplace_coo(const Mesh& m, const double* kappa, long long* indices, double* vv, cudaStream_t st) {
  k_laplace_coo<<<nblocks(27 * m.ne), kBlock, 0, st>>>(m.ne, m.d_conn.as<int4>(), m.d_geo.as<double4>(), kappa,
                                                       reinterpret_cast<longlong2*>(indices), vv);
  return cudaGetLastError();
}

// FemLaplaceScalar_backward (FemLaplaceScalar.h:28-54): grad_kappa[3e+k] = sum_pq grad_vv * (w grad_p.grad_q)
__global__ void k_laplace_coo_backward(int64_t ne, const double4* __restrict__ geo, const double* __restrict__ gvv,
                                       double* __restrict__ gk) {
  const int64_t s = gtid();
  if (s >= 3 * ne) return;
  const int64_t e = s / 3;
  const double4 g = geo[e];
  const double g00 = -(g.x + g.y), g11 = -(g.x + g.z), g22 = -(g.y + g.z);
  const double G[9] = {g00, g.x, g.y, g.x, g11, g.z, g.y, g.z, g22};
  const double* src = gvv + 9 * s;
  double v = 0.0;
#pragma unroll
  for (int j = 0; j < 9; j++) v = fma(src[j], G[j], v);
  gk[s] = v;
}

cudaError_t launch_laplace_coo_backward(const Mesh& m, const double* grad_vv, double* grad_kappa, cudaStream_t st) {
  k_laplace_coo_backward<<<nblocks(3 * m.ne), kBlock, 0, st>>>(m.ne, m.d_geo.as<double4>(), grad_vv, grad_kappa);
  return cudaGetLastError();
}

// FemSourceScalar_backward (FemSourceScalar.h:17-32)
__global__ void k_source_backward(int64_t ne, const int4* __restrict__ conn, const double4* __restrict__ geo,
                                  const double* __restrict__ grhs, double* __restrict__ gf) {
  const int64_t s = gtid();
  if (s >= 3 * ne) return;
  const int64_t e = s / 3;
  const int k = (int)(s - 3 * e);
  const int4 c = conn[e];
  const double w = geo[e].w;
  gf[s] = w * (lam(k, 0) * grhs[c.x] + lam(k, 1) * grhs[c.y] + lam(k, 2) * grhs[c.z]);
}

cudaError_t launch_source_backward(const Mesh& m, const double* grad_rhs, double* grad_f, cudaStream_t st) {
  k_source_backward<<<nblocks(3 * m.ne), kBlock, 0, st>>>(m.ne, m.d_conn.as<int4>(), m.d_geo.as<double4>(),
                                                          grad_rhs, grad_f);
  return cudaGetLastError();
}

// Adjoint element kernel: dL/dkappa_{3e+k} = -w (grad lam).(grad u)
//   = sum_{a<b} g_ab (lam_a - lam_b)(u_a - u_b)      (row sums of g vanish)
__global__ void k_poisson_kappa_grad(int64_t ne, const int4* __restrict__ conn, const double4* __restrict__ geo,
                                     const double* __restrict__ u, const double* __restrict__ lam,
                                     const uint8_t* __restrict__ isbd, double* __restrict__ gk) {
  const int64_t e = gtid();
  if (e >= ne) return;
  const int4 c = conn[e];
  const double4 g = geo[e];
  const double u0 = u[c.x], u1 = u[c.y], u2 = u[c.z];
  const double l0 = isbd[c.x] == 1 ? 0.0 : lam[c.x];
  const double l1 = isbd[c.y] == 1 ? 0.0 : lam[c.y];
  const double l2 = isbd[c.z] == 1 ? 0.0 : lam[c.z];
  double v = g.x * (l0 - l1) * (u0 - u1);
  v = fma(g.y * (l0 - l2), (u0 - u2), v);
  v = fma(g.z * (l1 - l2), (u1 - u2), v);
  gk[3 * e] = v;
  gk[3 * e + 1] = v;
  gk[3 * e + 2] = v;
}

cudaError_t launch_poisson_kappa_grad(const Mesh& m, const double* u, const double* lam, const uint8_t* isbd,
                                      double* grad_kappa, cudaStream_t st) {
  k_poisson_kappa_grad<<<nblocks(m.ne), kBlock, 0, st>>>(m.ne, m.d_conn.as<int4>(), m.d_geo.as<double4>(), u, lam,
                                                         isbd, grad_kappa);
  return cudaGetLastError();
}

ADFEM_CHECK_READER(check_line_assemble)

}  // namespace adfem
