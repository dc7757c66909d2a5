"""The CPU oracle pinned against the reference's own tests and against math known-answers.

The reference cannot be built here (it needs MFEM, Eigen, TensorFlow, ADCME and
Julia), so the oracle (oracle/fem_oracle.c) is pinned by:
  * the known answers in the reference's tests (tests/golden/kats.json):
    test/MFEM2.jl:7-27, test/mfem.jl:78-87, deps/MFEM/FemSource1/ftest.jl:5-14;
  * math known-answers the reference's FEniCS golden files would have pinned
    (5-point stencil, zero row sums, linear patch test, load sums to the area);
  * the Taylor test of deps/MFEM/*/gradtest.jl (seed 233) turned into assertions;
  * a committed regression fixture (tests/golden/c_small.npz).
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

from adfem_gpu import synth

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def kats():
    with open(os.path.join(GOLD, "kats.json")) as f:
        return json.load(f)


def test_mfem2_mesh_kat(oracle):
    k = kats()["mfem2_mesh_2_2_0.5"]
    coords, elems = synth.jittered_square(2, jitter=0.0)
    np.testing.assert_allclose(coords, np.array(k["nodes"]), rtol=0, atol=1e-15)
    M = oracle.OracleMesh(coords, elems)
    assert M.ngauss == k["ngauss"]
    np.testing.assert_allclose(M.area, k["area"], rtol=1e-14)


def test_dirichlet_dense_vs_sparse_kat(oracle):
    """test/mfem.jl:78-87: Array arm and SparseTensor arm agree."""
    k = kats()["dirichlet_dense_vs_sparse"]
    rng = np.random.default_rng(k["seed"])
    n = k["n"]
    A = rng.random((n, n))
    rhs = rng.random(n)
    bd = np.array(k["bd"])
    bv = np.array(k["bdval"])
    B1, r1 = oracle.dirichlet_csc(sp.csc_matrix(A), rhs, bd, bv)
    # constant(sparse(A)): COO of the stored entries in column-major order
    S = sp.csc_matrix(A)
    cols = np.repeat(np.arange(n), np.diff(S.indptr))
    idx = np.stack([S.indices, cols], axis=1)
    oi, ov, r2 = oracle.dirichlet_coo(idx, S.data, bd, rhs, bv, n)
    B2 = sp.coo_matrix((ov, (oi[:, 0], oi[:, 1])), shape=(n, n)).toarray()
    assert np.max(np.abs(B2 - B1.toarray())) < k["tol"] * 1e-9
    assert np.max(np.abs(r2 - r1)) < k["tol"] * 1e-9
    # structure: interior block copied, identity on bd, lifted rhs
    idx_i = np.setdiff1d(np.arange(n), bd - 1)
    np.testing.assert_array_equal(B1.toarray()[np.ix_(idx_i, idx_i)], A[np.ix_(idx_i, idx_i)])
    np.testing.assert_allclose(r1[idx_i], rhs[idx_i] - A[np.ix_(idx_i, bd - 1)] @ bv, rtol=1e-14)
    np.testing.assert_array_equal(r1[bd - 1], bv)


def test_source_equals_mass_times_constant(oracle):
    c = kats()["source_equals_mass_times_constant"]["c"]
    coords, elems = synth.jittered_square(6, seed=3)
    M = oracle.OracleMesh(coords, elems)
    ne = M.nelem
    Mm = np.zeros((M.ndof, M.ndof))
    for e in range(ne):
        for k in range(3):
            for a in range(3):
                for b in range(3):
                    Mm[M.elem[e, a], M.elem[e, b]] += M.w[e, k] * M.h[e, k, a] * M.h[e, k, b]
    src = M.source(np.full(M.ngauss, c))
    np.testing.assert_allclose(src, Mm @ np.full(M.ndof, c), rtol=1e-13, atol=1e-15)


def test_five_point_stencil(oracle):
    m = 8
    coords, elems = synth.jittered_square(m, jitter=0.0)
    M = oracle.OracleMesh(coords, elems)
    K = M.laplace_csc(np.ones(M.ngauss)).toarray()
    for i in range(1, m):
        for j in range(1, m):
            r = i * (m + 1) + j
            row = K[r]
            assert abs(row[r] - 4) < 1e-13
            for nb in (r - 1, r + 1, r - (m + 1), r + (m + 1)):
                assert abs(row[nb] + 1) < 1e-13
            mask = np.ones(row.size, bool)
            mask[[r, r - 1, r + 1, r - m - 1, r + m + 1]] = False
            assert np.max(np.abs(row[mask])) < 1e-13


def test_row_sums_patch_and_area(oracle):
    coords, elems = synth.jittered_square(12, seed=1)
    M = oracle.OracleMesh(coords, elems)
    rng = np.random.default_rng(5)
    K = M.laplace_csc(1 + rng.random(M.ngauss))
    rows = np.abs(K).sum(axis=1).A1
    assert np.max(np.abs(K.sum(axis=1).A1) / rows) < 1e-13
    Kc = M.laplace_csc(np.full(M.ngauss, 2.0))
    u = 3 * coords[:, 0] - 2 * coords[:, 1] + 1
    interior = np.setdiff1d(np.arange(M.ndof), M.bcnode() - 1)
    res = (Kc @ u)[interior]
    assert np.max(np.abs(res)) < 1e-12 * np.max(np.abs(Kc).sum(axis=1))
    assert abs(M.source(np.ones(M.ngauss)).sum() - 1.0) < 1e-13


def test_coo_to_csc_matches_scipy_sum(oracle):
    coords, elems = synth.jittered_square(5, seed=2)
    M = oracle.OracleMesh(coords, elems)
    rng = np.random.default_rng(0)
    idx, vv = M.laplace_coo(rng.random(M.ngauss))
    A = M.laplace_csc(rng.random(M.ngauss))
    assert A.nnz == M.ndof + 2 * M.edges().shape[0]
    K1 = oracle.coo_to_csc(idx, vv, M.ndof)
    K2 = sp.coo_matrix((vv, (idx[:, 0], idx[:, 1])), shape=(M.ndof, M.ndof)).tocsc()
    np.testing.assert_allclose(K1.toarray(), K2.toarray(), rtol=1e-14, atol=1e-14)


def test_linear_coo_to_csc_bit_identical_to_sorted(oracle):
    """The counting-sort conversion equals the comparison-sort statement bit for bit,
    including repeated (row, col) pairs in shuffled order, unsorted input and empty rows."""
    coords, elems = synth.jittered_square(9, seed=4)
    M = oracle.OracleMesh(coords, elems)
    rng = np.random.default_rng(1)
    idx, vv = M.laplace_coo(rng.random(M.ngauss))
    perm = rng.permutation(vv.size)
    n = M.ndof + 3  # three rows/columns without entries
    for i, v in ((idx, vv), (idx[perm], vv[perm] * 1e3)):
        a = oracle.coo_to_csc(i, v, n)
        b = oracle.coo_to_csc_sorted(i, v, n)
        assert np.array_equal(a.indptr, b.indptr) and np.array_equal(a.indices, b.indices)
        assert np.array_equal(a.data.view(np.int64), b.data.view(np.int64))
    e = oracle.coo_to_csc(np.zeros((0, 2), np.int64), np.zeros(0), 4)
    assert e.nnz == 0 and e.shape == (4, 4)


def test_doubled_precision_residual(oracle):
    """residual_dd is the exact residual of the stored vector within the doubled-precision
    bound (one rounding of the result plus ~(k eps)^2 of the row's |a||x| for k terms):
    checked with exact rational arithmetic on a small system whose residual is all rounding
    noise of the FP64 product (terms ~1e7 times larger than the residual)."""
    from fractions import Fraction

    rng = np.random.default_rng(2)
    n = 40
    A = sp.random(n, n, density=0.3, random_state=3, format="csc") + sp.eye(n, format="csc") * 4.0
    A = sp.csc_matrix(A)
    x = rng.standard_normal(n) * 1e6
    b = A @ x  # the FP64 product: its residual against x is pure rounding noise
    r = oracle.residual_dd(A, x, b)
    Ad = A.toarray()
    exact = [Fraction(float(b[i])) - sum(Fraction(float(Ad[i, j])) * Fraction(float(x[j])) for j in range(n))
             for i in range(n)]
    ax = np.abs(Ad) @ np.abs(x)
    eps = np.finfo(float).eps
    for i in range(n):
        ex = float(exact[i])
        k = np.count_nonzero(Ad[i]) + 1
        assert abs(r[i] - ex) <= 2 * np.spacing(abs(ex)) + (k * eps) ** 2 * ax[i], (i, r[i], ex)
        assert abs(r[i] - ex) <= 1e-12 * abs(ex)
    assert np.any(r != 0.0)
    plain = b - A @ x  # the FP64 evaluation sees nothing but its own rounding
    assert np.max(np.abs(plain - r)) > 10 * np.max(np.abs(r)) or np.max(np.abs(plain)) == 0.0


def test_orientation_and_edges(oracle):
    coords, elems = synth.jittered_square(4, seed=0)
    M = oracle.OracleMesh(coords, elems)
    assert M.flipped == M.nelem // 2  # the second triangle of each cell is clockwise
    x, y = coords[:, 0], coords[:, 1]
    e = M.elem
    det = (x[e[:, 1]] - x[e[:, 0]]) * (y[e[:, 2]] - y[e[:, 0]]) - (y[e[:, 1]] - y[e[:, 0]]) * (x[e[:, 2]] - x[e[:, 0]])
    assert np.all(det > 0)
    ed = M.edges()
    assert ed.shape[0] == 3 * 16 + 2 * 4
    assert np.all(ed[:, 0] < ed[:, 1])
    assert len({tuple(r) for r in ed}) == ed.shape[0]


def _taylor_linear(f, grad, m, v, gammas=(1e-1, 1e-2, 1e-3)):
    """For an operator linear in its input the first-order Taylor remainder is roundoff."""
    f0 = f(m)
    for g in gammas:
        s = f(m + g * v) - f0
        w = s - g * np.dot(v, grad)
        assert abs(w) <= 1e-9 * max(abs(s), 1e-30), (g, s, w)


def test_gradtest_laplace_source_stiffness(oracle):
    rng = np.random.default_rng(233)
    coords, elems = synth.jittered_square(4, seed=0)
    M = oracle.OracleMesh(coords, elems)
    ng = M.ngauss
    # laplace: L(kappa) = c . vv(kappa)
    idx, _ = M.laplace_coo(np.ones(ng))
    c = rng.standard_normal(idx.shape[0])
    _taylor_linear(lambda k: c @ M.laplace_coo(k)[1], M.laplace_coo_backward(c), 1 + rng.random(ng),
                   rng.standard_normal(ng))
    # source
    c2 = rng.standard_normal(M.ndof)
    _taylor_linear(lambda f: c2 @ M.source(f), M.source_backward(c2), rng.random(ng), rng.standard_normal(ng))
    # stiffness
    D0 = rng.random((ng, 3, 3))
    c3 = rng.standard_normal(36 * ng)
    _taylor_linear(lambda D: c3 @ M.stiffness_coo(D.reshape(ng, 3, 3))[1],
                   M.stiffness_coo_backward(c3).ravel(), D0.ravel(), rng.standard_normal(9 * ng))


@pytest.mark.parametrize("mode", [0, 1])
def test_gradtest_plane_strain(oracle, mode):
    rng = np.random.default_rng(233)
    n = 20
    E = 1 + rng.random(n)
    nu = 0.1 + 0.3 * rng.random(n)
    c = rng.standard_normal(9 * n)
    gE, gn = oracle.plane_strain_backward(c, E, nu, mode)
    vE, vn = rng.standard_normal(n), rng.standard_normal(n)
    f = lambda e, v: c @ oracle.plane_strain(e, v, mode).ravel()  # noqa: E731
    f0 = f(E, nu)
    ws = []
    for g in (1e-2, 1e-3, 1e-4):
        w = f(E + g * vE, nu + g * vn) - f0 - g * (vE @ gE + vn @ gn)
        ws.append(abs(w))
    assert ws[1] < ws[0] / 50 and ws[2] < ws[1] / 50  # second order


def test_plane_strain_reference_formula(oracle):
    D = oracle.plane_strain([2.0], [0.25], 0)[0]
    s = 2.0 * 0.75 / 1.25 / 0.5
    a = s * 0.25 / 0.75
    np.testing.assert_allclose(D, [[s, a, a], [a, s, a], [a, a, s]], rtol=1e-15)
    D = oracle.plane_strain([2.0], [0.25], 1)[0]
    s = 2.0 / 1.25 / 0.5
    np.testing.assert_allclose(D, [[s * 0.75, s * 0.25, 0], [s * 0.25, s * 0.75, 0], [0, 0, s * 0.25]], rtol=1e-15)


def test_gradtest_dirichlet(oracle):
    rng = np.random.default_rng(233)
    coords, elems = synth.jittered_square(4, seed=0)
    M = oracle.OracleMesh(coords, elems)
    idx, vv = M.laplace_coo(1 + rng.random(M.ngauss))
    bd = M.bcnode()[::2]
    n = M.ndof
    rhs = rng.random(n)
    bv = rng.random(bd.size)
    oi, ov, orhs = oracle.dirichlet_coo(idx, vv, bd, rhs, bv, n)
    cv, cr = rng.standard_normal(ov.size), rng.standard_normal(n)
    gvv, grhs, gbd = oracle.dirichlet_coo_backward(cv, cr, idx, vv, bd, bv, n)

    def L(v, r, b):
        _, o, orr = oracle.dirichlet_coo(idx, v, bd, r, b, n)
        return cv @ o + cr @ orr

    L0 = L(vv, rhs, bv)
    dv, dr, db = rng.standard_normal(vv.size), rng.standard_normal(n), rng.standard_normal(bd.size)
    for g in (1e-1, 1e-2):
        s = L(vv + g * dv, rhs, bv) - L0
        assert abs(s - g * dv @ gvv) < 1e-9 * max(abs(s), 1)
        s = L(vv, rhs + g * dr, bv) - L0
        assert abs(s - g * dr @ grhs) < 1e-9 * max(abs(s), 1)
    # bilinear in (vv, bdval): second-order remainder
    ws = []
    for g in (1e-2, 1e-3):
        s = L(vv, rhs, bv + g * db) - L0
        ws.append(abs(s - g * db @ gbd))
    assert ws[0] < 1e-9 * max(1.0, abs(L0))


def test_dirichlet_csc_drops_zeros(oracle):
    coords, elems = synth.jittered_square(4, jitter=0.0)
    M = oracle.OracleMesh(coords, elems)
    K = M.laplace_csc(np.ones(M.ngauss))
    assert np.sum(K.data == 0.0) > 0  # hypotenuse couplings vanish on right triangles
    bd = M.bcnode()
    B, _ = oracle.dirichlet_csc(K, np.zeros(M.ndof), bd, np.zeros(bd.size))
    assert np.sum(B.data == 0.0) == 0
    Bk, _ = oracle.dirichlet_csc(K, np.zeros(M.ndof), bd, np.zeros(bd.size), keep_zeros=True)
    assert np.sum(Bk.data == 0.0) > 0
    np.testing.assert_array_equal(Bk.toarray(), B.toarray())


def test_golden_fixture_regression(oracle):
    z = np.load(os.path.join(GOLD, "c_small.npz"))
    M = oracle.OracleMesh(z["coords"], z["elems"])
    K = M.laplace_csc(z["kappa"])
    np.testing.assert_array_equal(K.indptr, z["K_indptr"])
    np.testing.assert_array_equal(K.indices, z["K_indices"])
    np.testing.assert_allclose(K.data, z["K_data"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(M.source(z["f"]), z["F"], rtol=1e-15, atol=0)
    np.testing.assert_array_equal(M.bcnode(), z["bd"])


def test_cpu_pcg_matches_direct(oracle):
    z = np.load(os.path.join(GOLD, "c_small.npz"))
    B = sp.csc_matrix((z["B_data"], z["B_indices"], z["B_indptr"]))
    x, it, rr = oracle.pcg(B, z["r"], rtol=1e-14, threads=2)
    assert rr <= 1e-14
    np.testing.assert_allclose(x, z["u"], rtol=1e-10, atol=1e-10 * np.max(np.abs(z["u"])))


@pytest.mark.parametrize("k", [30, 63])
def test_high_valence_mesh_kats(oracle, k):
    """The oracle on a fan mesh whose centre vertex has k neighbours (the wide-row GPU
    tests' checker): the centre row has k + 1 entries; Laplace rows sum to zero; a linear
    field is annihilated at interior nodes for constant kappa (patch test); the load of
    f = 1 + x integrates f exactly (sum of areas times the centroid value); the stiffness
    operator annihilates the rigid-body modes and is symmetric for a symmetric D."""
    coords, elems = synth.fan_mesh(k)
    M = oracle.OracleMesh(coords, elems)
    rng = np.random.default_rng(k)
    K = M.laplace_csc(1 + rng.random(M.ngauss))
    assert np.diff(K.indptr).max() == k + 1
    rows = np.abs(K).sum(axis=1).A1
    assert np.max(np.abs(K.sum(axis=1).A1) / rows) < 1e-13
    Kc = M.laplace_csc(np.full(M.ngauss, 1.5))
    u = 1 + 2 * coords[:, 0] - 3 * coords[:, 1]
    interior = np.setdiff1d(np.arange(M.ndof), M.bcnode() - 1)
    assert interior.size == 1 + (3 - 1) * k  # the centre and the inner rings
    assert np.max(np.abs((Kc @ u)[interior])) < 1e-12 * np.max(rows)
    g = M.gauss_nodes()
    e0 = np.asarray(elems) - 1
    xc = coords[e0, 0].mean(axis=1)
    exact = float(np.sum(M.area * (1 + xc)))
    assert abs(M.source(1 + g[:, 0]).sum() - exact) < 1e-13 * abs(exact)
    D = np.tile(np.array([[2.0, 1.0, 0.0], [1.0, 2.0, 0.0], [0.0, 0.0, 0.5]]), (M.ngauss, 1, 1))
    Ks = M.stiffness_csc(D)
    n = M.ndof
    for v in (np.r_[np.ones(n), np.zeros(n)], np.r_[np.zeros(n), np.ones(n)], np.r_[-coords[:, 1], coords[:, 0]]):
        assert np.abs(Ks @ v).max() < 1e-12 * np.abs(Ks).max()
    assert abs(Ks - Ks.T).max() < 1e-15 * np.abs(Ks).max()
