"""The CPU oracle of the P2, mass-matrix and Gauss-point interpolation ops, pinned by
known answers.

The reference's own checks of these ops either print rather than assert or read FEniCS
matrices that are not in the reference (deps/MFEM/ComputeFemMassMatrix1/ftest.jl:5-33
reads fenics/A.txt, A2.txt).  What they check is restated here as assertions:
  * deps/MFEM/DofToGaussPoints/test.jl: dof_to_gauss_points is exact for 2x^2 + y on P2;
  * deps/MFEM/FemToGaussPoints/TestFemToGaussPoints.jl: fem_to_gauss_points against
    f at the Gauss points (exact for linear f);
  * the FEniCS P1/P2 mass matrices: the closed-form element matrices (area/12 [2 1 1; ...],
    area/180 [6 -1 -1 0 -4 0; ...]) and the total mass = area;
plus the closed-form P2 Laplace element matrix, the P2 patch test (K x^2 = -2 M 1 on
interior rows: quadratics are in the space), the rigid-body null space of the P2
elasticity operator, the Taylor test of deps/MFEM/*/gradtest.jl (seed 233) for every
backward, and the PCL Jacobians (src/pcl.jl) against the forward ops they differentiate.
"""
import numpy as np
import pytest

from adfem_gpu import synth


def space(oracle, m=4, degree=2, seed=0, jitter=0.2):
    coords, elems = synth.jittered_square(m, seed=seed, jitter=jitter)
    return oracle.OracleSpace(coords, elems, degree)


def test_p2_element_matrices_closed_form(oracle):
    coords = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])
    S = oracle.OracleSpace(coords, np.array([[1, 2, 3]]), 2)
    assert S.ndof == 6 and S.nd == 6 and S.ngauss == 6
    d = S.dof[0]
    M = S.mass_csc(np.ones(6)).toarray()[np.ix_(d, d)]
    Mref = np.array([[6, -1, -1, 0, -4, 0], [-1, 6, -1, 0, 0, -4], [-1, -1, 6, -4, 0, 0],
                     [0, 0, -4, 32, 16, 16], [-4, 0, 0, 16, 32, 16], [0, -4, 0, 16, 16, 32]]) * (0.5 / 180)
    np.testing.assert_allclose(M, Mref, rtol=0, atol=1e-16)
    K = S.laplace_csc(np.ones(6)).toarray()[np.ix_(d, d)]
    Kref = np.array([[6, 1, 1, -4, 0, -4], [1, 3, 0, -4, 0, 0], [1, 0, 3, 0, 0, -4],
                     [-4, -4, 0, 16, -8, 0], [0, 0, 0, -8, 16, -8], [-4, 0, -4, 0, -8, 16]]) / 6.0
    np.testing.assert_allclose(K, Kref, rtol=0, atol=1e-15)


def test_p1_mass_closed_form(oracle):
    S = space(oracle, 3, 1)
    M = S.mass_csc(np.ones(S.ngauss)).toarray()
    e, a = S.p1.elem, S.p1.area
    Mref = np.zeros_like(M)
    for k in range(S.nelem):
        for i in range(3):
            for j in range(3):
                Mref[e[k, i], e[k, j]] += a[k] / 12 * (2 if i == j else 1)
    np.testing.assert_allclose(M, Mref, rtol=0, atol=1e-16)


@pytest.mark.parametrize("degree", [1, 2])
def test_total_mass_and_load(oracle, degree):
    S = space(oracle, 5, degree)
    M = S.mass_csc(np.ones(S.ngauss))
    assert abs(M.sum() - 1.0) < 1e-14
    src = S.source(np.ones(S.ngauss))
    assert abs(src.sum() - 1.0) < 1e-14
    if degree == 2:
        # the integral of a P2 vertex function over its element is zero
        assert np.abs(src[:S.nnode]).max() < 1e-16


def test_p2_patch_test(oracle):
    """-div grad x^2 = -2: for interior DOFs (K u)_i = -2 (M 1)_i exactly."""
    S = space(oracle, 6, 2)
    X = S.dof_nodes()
    K = S.laplace_csc(np.ones(S.ngauss))
    M = S.mass_csc(np.ones(S.ngauss))
    inter = np.setdiff1d(np.arange(S.ndof), S.bcnode() - 1)
    for u, lap in ((X[:, 0] ** 2, 2.0), (X[:, 0] * X[:, 1], 0.0), (X[:, 1] ** 2 - X[:, 0], 2.0)):
        r = K @ u + lap * (M @ np.ones(S.ndof))
        assert np.abs(r[inter]).max() < 1e-12


def test_p2_stiffness_rigid_modes(oracle):
    S = space(oracle, 4, 2)
    ng = S.ngauss
    D = np.tile(np.array([[2.0, 1.0, 0.0], [1.0, 2.0, 0.0], [0.0, 0.0, 0.5]]), (ng, 1, 1))
    K = S.stiffness_csc(D)
    X = S.dof_nodes()
    n = S.ndof
    for u in (np.r_[np.ones(n), np.zeros(n)], np.r_[np.zeros(n), np.ones(n)], np.r_[-X[:, 1], X[:, 0]]):
        assert np.abs(K @ u).max() < 1e-13
    assert abs(K - K.T).max() < 1e-15


@pytest.mark.parametrize("degree", [1, 2])
def test_interpolation_kats(oracle, degree):
    S = space(oracle, 5, degree)
    g = S.gauss_nodes()
    X = S.dof_nodes()
    lin = lambda x, y: 3 * x - y + 0.5  # noqa: E731
    np.testing.assert_allclose(S.fem_to_gauss(lin(S.p1.coords[:, 0], S.p1.coords[:, 1])), lin(g[:, 0], g[:, 1]),
                               atol=1e-14)
    f = (lambda x, y: 2 * x ** 2 + y) if degree == 2 else lin
    np.testing.assert_allclose(S.dof_to_gauss(f(X[:, 0], X[:, 1])), f(g[:, 0], g[:, 1]), atol=1e-14)


def test_p2_bcnode_and_counts(oracle):
    m = 5
    S = space(oracle, m, 2)
    assert S.nedge == 3 * m * m + 2 * m
    assert S.ndof == (m + 1) ** 2 + S.nedge
    assert S.ngauss == 6 * 2 * m * m
    bd = S.bcnode()
    assert bd.size == 8 * m  # 4m boundary vertices + 4m boundary edges
    assert np.all(bd[:4 * m] <= S.nnode) and np.all(bd[4 * m:] > S.nnode)


def _taylor_linear(f, grad, m, v):
    f0 = f(m)
    for g in (1e-1, 1e-2, 1e-3, 1e-4, 1e-5):
        s = f(m + g * v) - f0
        w = s - g * np.dot(v, grad)
        assert abs(w) <= 1e-9 * max(abs(s), 1e-30), (g, s, w)


@pytest.mark.parametrize("degree", [1, 2])
def test_gradtest_generic_ops(oracle, degree):
    rng = np.random.default_rng(233)
    S = space(oracle, 3, degree)
    ng, nd = S.ngauss, S.nd
    c = rng.standard_normal(nd * nd * ng)
    _taylor_linear(lambda k: c @ S.laplace_coo(k)[1], S.laplace_coo_backward(c), 1 + rng.random(ng),
                   rng.standard_normal(ng))
    _taylor_linear(lambda r: c @ S.mass_coo(r)[1], S.mass_coo_backward(c), 1 + rng.random(ng),
                   rng.standard_normal(ng))
    c2 = rng.standard_normal(S.ndof)
    _taylor_linear(lambda f: c2 @ S.source(f), S.source_backward(c2), rng.random(ng), rng.standard_normal(ng))
    c3 = rng.standard_normal(4 * nd * nd * ng)
    D0 = rng.random(9 * ng)
    _taylor_linear(lambda D: c3 @ S.stiffness_coo(D)[1], S.stiffness_coo_backward(c3), D0,
                   rng.standard_normal(9 * ng))
    c4 = rng.standard_normal(ng)
    _taylor_linear(lambda u: c4 @ S.fem_to_gauss(u), S.fem_to_gauss_backward(c4), rng.random(S.nnode),
                   rng.standard_normal(S.nnode))
    _taylor_linear(lambda u: c4 @ S.dof_to_gauss(u), S.dof_to_gauss_backward(c4), rng.random(S.ndof),
                   rng.standard_normal(S.ndof))


def test_generic_degree1_equals_p1_oracle(oracle):
    """The degree-generic loops at degree 1 reproduce the P1 restatement bit for bit."""
    coords, elems = synth.jittered_square(6, seed=3)
    S = oracle.OracleSpace(coords, elems, 1)
    P = oracle.OracleMesh(coords, elems)
    rng = np.random.default_rng(1)
    k = 1 + rng.random(S.ngauss)
    i1, v1 = S.laplace_coo(k)
    i2, v2 = P.laplace_coo(k)
    np.testing.assert_array_equal(i1, i2)
    np.testing.assert_array_equal(v1, v2)
    np.testing.assert_array_equal(S.source(k), P.source(k))
    D = rng.random((S.ngauss, 3, 3))
    i1, v1 = S.stiffness_coo(D)
    i2, v2 = P.stiffness_coo(D)
    np.testing.assert_array_equal(i1, i2)
    np.testing.assert_allclose(v1, v2, rtol=1e-15, atol=1e-15 * np.abs(v2).max())


@pytest.mark.parametrize("degree", [1, 2])
def test_pcl_laplace_jacobian_kat(oracle, degree):
    """src/pcl.jl:24-39: J[i, j] = d v_j / d kappa_i, so v(kappa) = J^T kappa exactly."""
    S = space(oracle, 2, degree)
    J = S.pcl_laplace_jacobian()
    assert J.shape == (S.ngauss, S.nd * S.nd * S.ngauss)
    kappa = 1 + np.random.default_rng(2).random(S.ngauss)
    _, vv = S.laplace_coo(kappa)
    np.testing.assert_allclose(J.T @ kappa, vv, rtol=1e-14, atol=0)
    assert np.count_nonzero(J) <= vv.size


def test_pcl_dirichlet_kat(oracle):
    """src/pcl.jl:1-21: J[i, j] = d (v_B)_j / d (v_A)_i; J^T v_A gives the kept values of the
    COO Dirichlet op in its output order."""
    S = space(oracle, 3, 1)
    idx, vv = S.laplace_coo(1 + np.random.default_rng(4).random(S.ngauss))
    bd = S.bcnode()
    oi, ov, _ = oracle.dirichlet_coo(idx, vv, bd, np.zeros(S.ndof), np.zeros(bd.size), S.ndof)
    nkeep = ov.size - bd.size
    J = oracle.pcl_dirichlet(idx + 1, bd, ov.size)
    np.testing.assert_array_equal(J.T @ vv, np.r_[ov[:nkeep], np.zeros(bd.size)])
    assert J.sum() == nkeep
