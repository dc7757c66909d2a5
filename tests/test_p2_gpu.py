"""GPU parity of the degree-generic ops (P2 Laplace/source/stiffness, mass matrix,
Gauss-point interpolation) through the C ABI against the CPU oracle.

Same bar as the P1 parity tests: patterns and COO indices bit-exact; values within
1e-12 relative to their row maximum (matrices) or their max norm (vectors).
"""
import ctypes

import numpy as np
import pytest

from adfem_gpu import synth

pytestmark = pytest.mark.gpu
TOL = 1e-12


def row_scaled_err(A, B):
    import scipy.sparse as sp

    A = sp.csr_matrix(A)
    B = sp.csr_matrix(B)
    d = abs(A - B).max(axis=1).toarray().ravel()
    s = abs(B).max(axis=1).toarray().ravel()
    s[s == 0] = 1.0
    return float(np.max(d / s))


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def spaces(oracle, gpulib, m, degree, seed=0, jitter=0.2):
    coords, elems = synth.jittered_square(m, seed=seed, jitter=jitter)
    return oracle.OracleSpace(coords, elems, degree), gpulib.Mesh(coords, elems, degree=degree)


@pytest.mark.parametrize("degree", [1, 2])
@pytest.mark.parametrize("m,jitter", [(1, 0.0), (2, 0.0), (9, 0.2), (24, 0.2)])
def test_space_mesh_runtime(oracle, gpulib, degree, m, jitter):
    O, G = spaces(oracle, gpulib, m, degree, 0, jitter)
    assert (G.ndof, G.elem_ndof, gpulib.get_ngauss(G)) == (O.ndof, O.nd, O.ngauss)
    np.testing.assert_array_equal(G.conn, O.connectivity1())
    np.testing.assert_allclose(gpulib.gauss_nodes(G), O.gauss_nodes(), rtol=0, atol=1e-15)
    np.testing.assert_allclose(gpulib.gauss_weights(G), O.w.ravel(), rtol=1e-15)
    np.testing.assert_array_equal(gpulib.bcnode(G), O.bcnode())
    np.testing.assert_allclose(gpulib.dof_nodes(G), O.dof_nodes(), rtol=0, atol=1e-15)
    K = O.laplace_csc(np.ones(O.ngauss))
    cp, rv = G.pattern()
    np.testing.assert_array_equal(cp - 1, K.indptr)
    np.testing.assert_array_equal(rv - 1, K.indices)
    Ks = O.stiffness_csc(np.tile(np.eye(3), (O.ngauss, 1, 1)))
    cp2, rv2 = G.pattern_elasticity()
    np.testing.assert_array_equal(cp2 - 1, Ks.indptr)
    np.testing.assert_array_equal(rv2 - 1, Ks.indices)


@pytest.mark.parametrize("m,seed", [(7, 0), (20, 3)])
def test_p2_summed_operators(oracle, gpulib, m, seed):
    O, G = spaces(oracle, gpulib, m, 2, seed)
    g = O.gauss_nodes()
    rng = np.random.default_rng(seed)
    kappa = np.sin(g[:, 0]) * (1 + g[:, 1] ** 2) + 1
    A = gpulib.compute_fem_laplace_matrix1(kappa, G)
    B = O.laplace_csc(kappa)
    np.testing.assert_array_equal(A.indptr, B.indptr)
    np.testing.assert_array_equal(A.indices, B.indices)
    assert row_scaled_err(A, B) < TOL
    f = 1e5 * (g[:, 0] + g[:, 1])
    assert rel(gpulib.compute_fem_source_term1(f, G), O.source(f)) < TOL
    D = rng.random((O.ngauss, 3, 3)) + np.eye(3)  # not symmetric: checks the CSC transpose
    As = gpulib.compute_fem_stiffness_matrix(D, G)
    Bs = O.stiffness_csc(D)
    np.testing.assert_array_equal(As.indptr, Bs.indptr)
    np.testing.assert_array_equal(As.indices, Bs.indices)
    assert row_scaled_err(As, Bs) < TOL


@pytest.mark.parametrize("degree", [1, 2])
def test_mass_matrix(oracle, gpulib, degree):
    import torch

    from adfem_gpu import system as S

    O, G = spaces(oracle, gpulib, 13, degree, 2)
    rho = 1 + np.random.default_rng(5).random(O.ngauss)
    A = gpulib.compute_fem_mass_matrix1(rho, G)
    B = O.mass_csc(rho)
    np.testing.assert_array_equal(A.indptr, B.indptr)
    np.testing.assert_array_equal(A.indices, B.indices)
    assert row_scaled_err(A, B) < TOL
    A1 = gpulib.compute_fem_mass_matrix1(G)
    assert abs(A1.sum() - 1.0) < 1e-13
    assert gpulib.compute_fem_mass_matrix(G).shape == (2 * G.ndof, 2 * G.ndof)
    v = S.mass_csr(G, torch.tensor(rho, device="cuda")).cpu().numpy()
    np.testing.assert_array_equal(v, A.data)  # symmetric pattern and values: CSR == CSC
    idx, vv = S.mass_coo(G, torch.tensor(rho, device="cuda"))
    oi, ov = O.mass_coo(rho)
    np.testing.assert_array_equal(idx.cpu().numpy(), oi)
    assert rel(vv.cpu().numpy(), ov) < TOL
    gvv = np.random.default_rng(6).standard_normal(ov.size)
    gr = S.mass_coo_backward(G, torch.tensor(gvv, device="cuda")).cpu().numpy()
    assert rel(gr, O.mass_coo_backward(gvv)) < TOL


def test_p2_coo_and_backward(oracle, gpulib):
    import torch

    from adfem_gpu import system as S

    O, G = spaces(oracle, gpulib, 9, 2, 1)
    rng = np.random.default_rng(7)
    kappa = 1 + rng.random(O.ngauss)
    idx, vv = S.laplace_coo(G, torch.tensor(kappa, device="cuda"))
    oi, ov = O.laplace_coo(kappa)
    np.testing.assert_array_equal(idx.cpu().numpy(), oi)
    assert rel(vv.cpu().numpy(), ov) < TOL
    gvv = rng.standard_normal(ov.size)
    gk = S.laplace_coo_backward(G, torch.tensor(gvv, device="cuda")).cpu().numpy()
    assert rel(gk, O.laplace_coo_backward(gvv)) < TOL
    gr = rng.standard_normal(O.ndof)
    gf = S.source_backward(G, torch.tensor(gr, device="cuda")).cpu().numpy()
    assert rel(gf, O.source_backward(gr)) < TOL
    D = rng.random(9 * O.ngauss)
    idx2, vv2 = S.stiffness_coo(G, torch.tensor(D, device="cuda"))
    oi2, ov2 = O.stiffness_coo(D)
    np.testing.assert_array_equal(idx2.cpu().numpy(), oi2)
    assert rel(vv2.cpu().numpy(), ov2) < TOL
    gvv2 = rng.standard_normal(ov2.size)
    gD = S.stiffness_coo_backward(G, torch.tensor(gvv2, device="cuda")).cpu().numpy()
    assert rel(gD, O.stiffness_coo_backward(gvv2)) < TOL


@pytest.mark.parametrize("degree", [1, 2])
def test_interpolation(oracle, gpulib, degree):
    import torch

    from adfem_gpu import system as S

    O, G = spaces(oracle, gpulib, 11, degree, 4)
    rng = np.random.default_rng(9)
    un = rng.standard_normal(O.nnode)
    ud = rng.standard_normal(O.ndof)
    assert rel(gpulib.fem_to_gauss_points(un, G), O.fem_to_gauss(un)) < TOL
    assert rel(gpulib.dof_to_gauss_points(ud, G), O.dof_to_gauss(ud)) < TOL
    assert rel(S.fem_to_gauss(G, torch.tensor(un, device="cuda")).cpu().numpy(), O.fem_to_gauss(un)) < TOL
    assert rel(S.dof_to_gauss(G, torch.tensor(ud, device="cuda")).cpu().numpy(), O.dof_to_gauss(ud)) < TOL
    go = rng.standard_normal(O.ngauss)
    gt = torch.tensor(go, device="cuda")
    # transposes: overwrite (entries past the vertices zeroed), then accumulate
    gu = S.fem_to_gauss_backward(G, gt, nu=O.ndof).cpu().numpy()
    assert rel(gu, O.fem_to_gauss_backward(go, O.ndof)) < TOL
    base = torch.tensor(ud, device="cuda")
    acc = S.fem_to_gauss_backward(G, gt, grad_u=base.clone()).cpu().numpy()
    want = ud.copy()
    want[:O.nnode] += O.fem_to_gauss_backward(go)
    assert rel(acc, want) < TOL
    gd = S.dof_to_gauss_backward(G, gt).cpu().numpy()
    assert rel(gd, O.dof_to_gauss_backward(go)) < TOL
    acc2 = S.dof_to_gauss_backward(G, gt, grad_u=base.clone()).cpu().numpy()
    assert rel(acc2, ud + O.dof_to_gauss_backward(go)) < TOL
    # DofToGaussPoints/test.jl: exact for 2x^2 + y on P2 (linear f on P1)
    f = (lambda x, y: 2 * x ** 2 + y) if degree == 2 else (lambda x, y: 3 * x - y)
    fg = gpulib.dof_to_gauss_points(gpulib.eval_f_on_dof_pts(f, G), G)
    assert np.abs(fg - gpulib.eval_f_on_gauss_pts(f, G)).max() < 1e-13


def test_legacy_p2_layer(oracle, gpulib):
    """The libadmfem symbols on a P2 current mesh, driven like src/MFEM/MFEM.jl:92-106."""
    from adfem_gpu import _lib

    L = _lib.load()
    coords, elems = synth.jittered_square(5, seed=9)
    O = oracle.OracleSpace(coords, elems, 2)
    c = np.concatenate([coords, np.zeros((coords.shape[0], 1))], 1).ravel()
    e = np.ascontiguousarray((elems - 1).ravel(), np.int32)
    ned = np.zeros(1, np.int64)
    p = L.init_nnfem_mesh(_lib.ptr(c), coords.shape[0], _lib.ptr(e), elems.shape[0], -1, -1, 2, _lib.ptr(ned))
    assert p
    edges = np.ctypeslib.as_array(p, shape=(2 * ned[0],)).copy()
    ctypes.CDLL(None).free(ctypes.cast(p, ctypes.c_void_p))
    np.testing.assert_array_equal(edges.reshape(2, -1).T, O.p1.edges())
    assert L.mfem_get_ngauss() == O.ngauss and L.mfem_get_ndof() == O.ndof and L.mfem_get_elem_ndof() == 6
    x, y, w = np.empty(O.ngauss), np.empty(O.ngauss), np.empty(O.ngauss)
    L.mfem_get_gauss(_lib.ptr(x), _lib.ptr(y))
    L.mfem_get_gauss_weights(_lib.ptr(w))
    np.testing.assert_allclose(np.stack([x, y], 1), O.gauss_nodes(), atol=1e-15)
    np.testing.assert_allclose(w, O.w.ravel(), rtol=1e-15)
    conn = np.empty(6 * O.nelem, np.int64)
    L.mfem_get_connectivity(_lib.ptr(conn))
    np.testing.assert_array_equal(conn.reshape(-1, 6), O.connectivity1())
    rng = np.random.default_rng(0)
    kappa = 1 + rng.random(O.ngauss)
    N = 36 * O.ngauss
    idx, vv = np.zeros(2 * N, np.int64), np.zeros(N)
    L.FemLaplaceScalar_forward_Julia(_lib.ptr(idx), _lib.ptr(vv), _lib.ptr(kappa))
    oi, ov = O.laplace_coo(kappa)
    np.testing.assert_array_equal(idx.reshape(-1, 2), oi)
    assert rel(vv, ov) < TOL
    L.ComputeFemMassMatrix1_forward(_lib.ptr(idx), _lib.ptr(vv), _lib.ptr(kappa))
    oi, ov = O.mass_coo(kappa)
    np.testing.assert_array_equal(idx.reshape(-1, 2), oi)
    assert rel(vv, ov) < TOL
    gvv = rng.standard_normal(N)
    gr = np.empty(O.ngauss)
    L.ComputeFemMassMatrix1_backward(_lib.ptr(gr), _lib.ptr(gvv), None, None)
    assert rel(gr, O.mass_coo_backward(gvv)) < TOL
    L.FemLaplaceScalar_backward(_lib.ptr(gr), _lib.ptr(gvv), None, None, None)
    assert rel(gr, O.laplace_coo_backward(gvv)) < TOL
    rhs = np.ones(O.ndof)  # accumulates into the caller's array
    L.FemSourceScalar_forward_Julia(_lib.ptr(rhs), _lib.ptr(kappa))
    assert rel(rhs, O.source(kappa, np.ones(O.ndof))) < TOL
    D = rng.random(9 * O.ngauss)
    N2 = 144 * O.ngauss
    idx2, vv2 = np.zeros(2 * N2, np.int64), np.zeros(N2)
    L.ComputeFemStiffnessMatrixMfem_forward_Julia(_lib.ptr(idx2), _lib.ptr(vv2), _lib.ptr(D))
    oi2, ov2 = O.stiffness_coo(D)
    np.testing.assert_array_equal(idx2.reshape(-1, 2), oi2)
    assert rel(vv2, ov2) < TOL
    un, ud = rng.standard_normal(O.nnode), rng.standard_normal(O.ndof)
    out = np.empty(O.ngauss)
    L.FemToGaussPointsMfem_Julia(_lib.ptr(out), _lib.ptr(un))
    assert rel(out, O.fem_to_gauss(un)) < TOL
    L.DofToGaussPointsMfem_forward_Julia(_lib.ptr(out), _lib.ptr(ud))
    assert rel(out, O.dof_to_gauss(ud)) < TOL
    go = rng.standard_normal(O.ngauss)
    gu = np.ones(O.ndof)
    L.DofToGaussPointsMfem_backward(_lib.ptr(gu), _lib.ptr(go), None, None)
    assert rel(gu, 1 + O.dof_to_gauss_backward(go)) < TOL
    gn = np.ones(O.nnode)
    L.FemToGaussPointsMfem_backward(_lib.ptr(gn), _lib.ptr(go), None, None)
    assert rel(gn, 1 + O.fem_to_gauss_backward(go)) < TOL
    L.adfem_set_current_mesh(None)


def test_p2_poisson_exact_for_quadratics(oracle, gpulib):
    """-lap u = -6 with u = 1 + x^2 + 2 y^2 on the boundary: the P2 solution equals u at
    every DOF (quadratics are in the space), through assembly, Dirichlet and K\\F."""
    coords, elems = synth.jittered_square(16, seed=2)
    G = gpulib.Mesh(coords, elems, degree=2)
    O = oracle.OracleSpace(coords, elems, 2)
    ng = gpulib.get_ngauss(G)
    K = gpulib.compute_fem_laplace_matrix1(np.ones(ng), G)
    F = gpulib.compute_fem_source_term1(np.full(ng, -6.0), G)
    ue = gpulib.eval_f_on_dof_pts(lambda x, y: 1 + x ** 2 + 2 * y ** 2, G)
    bd = gpulib.bcnode(G)
    A, r = gpulib.impose_Dirichlet_boundary_conditions(K, F, bd, ue[bd - 1])
    u = gpulib.solve(A, r, rtol=1e-14)
    assert np.abs(u - ue).max() < 1e-10
    Ao, ro = oracle.dirichlet_csc(O.laplace_csc(np.ones(ng)), O.source(np.full(ng, -6.0)), bd, ue[bd - 1])
    uo = oracle.spsolve(Ao, ro)
    assert np.abs(u - uo).max() < 1e-10


def test_p2_input_checks(gpulib):
    coords, elems = synth.jittered_square(3, seed=0)
    G = gpulib.Mesh(coords, elems, degree=2)
    with pytest.raises(gpulib.AdFemError):
        gpulib.compute_fem_laplace_matrix1(np.ones(3 * G.nelem), G)  # P1 length on a P2 mesh
    with pytest.raises(gpulib.AdFemError):
        gpulib.ElasticitySystem(G)  # resident elasticity systems are P1
    with pytest.raises(gpulib.AdFemError):
        gpulib.Mesh(coords, elems, degree=2, order=2)


@pytest.mark.parametrize("degree", [1, 2])
def test_pcl_jacobians(oracle, gpulib, degree):
    import torch

    from adfem_gpu import _lib

    O, G = spaces(oracle, gpulib, 3, degree, 1)
    H = gpulib.pcl_compute_fem_laplace_matrix1(G)
    Ho = O.pcl_laplace_jacobian()
    assert H.shape == Ho.shape
    assert rel(H, Ho) < TOL
    Hd = torch.zeros(Ho.shape[1], Ho.shape[0], dtype=torch.float64, device="cuda")  # column-major ng x N
    _lib.check(_lib.load().adfem_pcl_laplace_jacobian_d(G.handle, _lib.ptr(Hd), None))
    assert rel(Hd.cpu().numpy().T, Ho) < TOL
    idx, vv = O.laplace_coo(np.ones(O.ngauss))
    bd = O.bcnode()
    nout = oracle.dirichlet_coo(idx, vv, bd, np.zeros(O.ndof), np.zeros(bd.size), O.ndof)[1].size
    J = gpulib.pcl_impose_Dirichlet_boundary_conditions(idx + 1, bd, nout)
    np.testing.assert_array_equal(J, oracle.pcl_dirichlet(idx + 1, bd, nout))


def test_pcl_legacy_symbols(oracle, gpulib):
    from adfem_gpu import _lib

    L = _lib.load()
    coords, elems = synth.jittered_square(3, seed=5)
    O = oracle.OracleSpace(coords, elems, 2)
    G = gpulib.Mesh(coords, elems, degree=2)
    L.adfem_set_current_mesh(G.handle)
    H = np.zeros((O.ngauss, 36 * O.ngauss), order="F")
    L.pcl_FemLaplaceScalar_Jacobian(_lib.ptr(H))
    assert rel(H, O.pcl_laplace_jacobian()) < TOL
    idx, _ = O.laplace_coo(np.ones(O.ngauss))
    idx1 = np.asfortranarray(idx + 1)
    bd = O.bcnode()
    J = np.zeros((idx.shape[0], idx.shape[0]), order="F")
    L.pcl_ImposeDirichlet(_lib.ptr(J), idx1.ctypes.data_as(ctypes.c_void_p), _lib.ptr(bd), bd.size, idx.shape[0])
    np.testing.assert_array_equal(J, oracle.pcl_dirichlet(idx + 1, bd, idx.shape[0]))
    L.adfem_set_current_mesh(None)


@pytest.mark.parametrize("degree", [1, 2])
def test_mesh_from_file(oracle, gpulib, tmp_path, degree):
    """Mesh(filename) (src/MFEM/MUtils.jl:33-50) from an ASCII STL written here."""
    from adfem_gpu.meshfile import read_mesh_file

    coords, elems = synth.jittered_square(6, seed=8)
    tri = np.concatenate([coords, np.zeros((coords.shape[0], 1))], 1)[elems - 1]
    p = tmp_path / "sq.stl"
    with open(p, "w") as f:
        f.write("solid sq\n")
        for t in tri:
            f.write("facet normal 0 0 1\nouter loop\n" + "".join("vertex %.17g %.17g %.17g\n" % tuple(v) for v in t)
                    + "endloop\nendfacet\n")
        f.write("endsolid sq\n")
    G = gpulib.Mesh(str(p), degree=degree)
    c, e = read_mesh_file(str(p))
    O = oracle.OracleSpace(c, e, degree)
    assert (G.nnode, G.nelem, G.ndof) == (coords.shape[0], elems.shape[0], O.ndof)
    kappa = 1 + np.random.default_rng(1).random(O.ngauss)
    assert row_scaled_err(gpulib.compute_fem_laplace_matrix1(kappa, G), O.laplace_csc(kappa)) < TOL
    np.testing.assert_array_equal(gpulib.bcnode(G), O.bcnode())


def _p2_case(oracle, gpulib, m, seed, bdval=False):
    coords, elems = synth.jittered_square(m, seed=seed)
    O = oracle.OracleSpace(coords, elems, 2)
    G = gpulib.Mesh(coords, elems, degree=2)
    g = O.gauss_nodes()
    G1 = synth.fourier_field(g[:, 0], g[:, 1], seed=1)
    kappa = 1 + np.exp(synth.contrast_sigma(G1, 1e2) * G1)
    f = 1e3 * (1 + g[:, 0] - 2 * g[:, 1])
    bd = O.bcnode()
    dn = O.dof_nodes()
    bv = (np.sin(3 * dn[bd - 1, 0]) + dn[bd - 1, 1]) if bdval else np.zeros(bd.size)
    B, r = oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(f), bd, bv)
    return O, G, kappa, f, bd, bv, B, r


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("m,seed,bdval", [(12, 0, False), (30, 4, True)])
def test_p2_resident_system_forward_adjoint_gradient(oracle, gpulib, precision, m, seed, bdval):
    """Resident P2 Poisson system (order-4 rule, vertex-then-edge DOFs, solver in reverse
    Cuthill-McKee order): right-hand side and operator against the oracle's Dirichlet-
    imposed P2 system, forward solve against the direct solve, adjoint solve, and
    dL/dkappa at the 6 Gauss points against the reference's backward chain (sparse-solve
    gradient -lam_i u_j per stored entry, ImposeDirichlet backward, FemLaplaceScalar
    backward over the P2 element matrices)."""
    import torch

    O, G, kappa, f, bd, bv, B, r = _p2_case(oracle, gpulib, m, seed, bdval)
    S = gpulib.PoissonSystem(G)
    assert S.ndof == O.ndof
    S.set_dirichlet(bd, bv)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    info = S.solver_info()
    assert info["rows"] == O.ndof and info["renumbered"] == 1
    assert info["banded"] == 1  # 19-entry P2 rows: the 24-wide banded mixed iteration
    assert rel(S.rhs().cpu().numpy(), r) < TOL
    x = np.random.default_rng(seed).standard_normal(O.ndof)
    assert rel(S.apply(torch.tensor(x, device="cuda")).cpu().numpy(), B @ x) < TOL
    rtol = 1e-13 if precision == "fp64" else 1e-11
    u = S.solve(precision=precision, rtol=rtol)
    assert S.last_stats.status == 0
    u0 = oracle.spsolve(B, r)
    assert rel(u.cpu().numpy(), u0) < 1e-9
    np.testing.assert_array_equal(u.cpu().numpy()[bd - 1], bv)
    # adjoint of a misfit on a tenth of the DOFs
    obs = synth.observation_nodes(O.ndof, seed=3, frac=0.1)
    gu = np.zeros(O.ndof)
    gu[obs] = 1.0  # (0-based ids)
    gu_t = torch.tensor(gu, device="cuda")
    lam = S.adjoint(gu_t, precision=precision, rtol=rtol)
    assert S.last_stats.status == 0
    gz = gu.copy()
    gz[bd - 1] = 0.0
    lam0 = oracle.spsolve(B.T.tocsc(), gz)
    assert rel(lam.cpu().numpy(), lam0) < 1e-9
    gk = S.grad_kappa(u, lam).cpu().numpy()
    uu, ll = u0, lam0.copy()
    ll[bd - 1] = 0.0
    idx, vv = O.laplace_coo(kappa)
    gref = O.laplace_coo_backward(-ll[idx[:, 0]] * uu[idx[:, 1]])
    assert gk.size == O.ngauss
    assert rel(gk, gref) < 1e-7


def test_p2_banded_and_scaled_mixed_paths_agree(oracle, gpulib, monkeypatch):
    """The P2 operator on the 24-wide banded mixed iteration and on the scaled two-kernel
    mixed iteration (forced with ADFEM_ZCG=0): both within the 1e-10 mixed-precision bar
    of the direct solve."""
    import torch

    O, G, kappa, f, bd, bv, B, r = _p2_case(oracle, gpulib, 40, 5, True)
    u0 = oracle.spsolve(B, r)
    for zcg, banded in (("1", 1), ("0", 0)):
        monkeypatch.setenv("ADFEM_ZCG", zcg)
        S = gpulib.PoissonSystem(G)
        S.set_dirichlet(bd, bv)
        S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
        assert S.solver_info()["banded"] == banded
        u = S.solve(precision="mixed", rtol=1e-12)
        assert S.last_stats.status == 0
        assert rel(u.cpu().numpy(), u0) < 1e-10


def test_p2_system_super_tiles_and_packed(oracle, gpulib, monkeypatch):
    """P2 systems on the 24-wide banded iteration with block ranges split into super-tiles,
    and a small P2 system through the packed solver (one thread block per system)."""
    import torch

    O, G, kappa, f, bd, bv, B, r = _p2_case(oracle, gpulib, 60, 2, True)
    u0 = oracle.spsolve(B, r)
    monkeypatch.setenv("ADFEM_ZCG_SMAX", "96")
    S = gpulib.PoissonSystem(G)
    S.set_dirichlet(bd, bv)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    info = S.solver_info()
    assert info["banded"] == 1 and info["rows_per_block"] > 96
    u = S.solve(precision="mixed", rtol=1e-12)
    assert S.last_stats.status == 0 and rel(u.cpu().numpy(), u0) < 1e-10
    monkeypatch.delenv("ADFEM_ZCG_SMAX", raising=False)
    Os, Gs, ks, fs, bds, bvs, Bs, rs = _p2_case(oracle, gpulib, 10, 3, True)
    P = gpulib.PoissonSystem(Gs)
    P.set_dirichlet(bds, bvs)
    P.assemble(torch.tensor(ks, device="cuda"), torch.tensor(fs, device="cuda"))
    (up,), (stp,) = gpulib.system.solve_packed([P], rtol=1e-12)
    assert stp.status == 0
    assert rel(up.cpu().numpy(), oracle.spsolve(Bs, rs)) < 1e-10


def _union_jack(m):
    """m x m unit-square grid whose cells are split along alternating diagonals: interior
    vertices alternate between valence 4 and 8 (P2 rows of 25 entries)."""
    x = np.linspace(0.0, 1.0, m + 1)
    X, Y = np.meshgrid(x, x, indexing="xy")
    coords = np.stack([X.ravel(), Y.ravel()], axis=1)
    el = []
    for j in range(m):
        for i in range(m):
            a, b = j * (m + 1) + i, j * (m + 1) + i + 1
            c, d = a + m + 1, b + m + 1
            if (i + j) % 2 == 0:
                el += [(a, b, d), (a, d, c)]
            else:
                el += [(a, b, c), (b, d, c)]
    return coords, np.array(el, dtype=np.int64) + 1


def test_p2_system_long_rows_take_the_scaled_path(oracle, gpulib):
    """P2 rows longer than the banded iteration's 24 (valence-8 vertices: 25 entries) are
    assembled by the 32-wide row kernel and solved on the scaled mixed path."""
    import torch

    coords, elems = _union_jack(24)
    O = oracle.OracleSpace(coords, elems, 2)
    G = gpulib.Mesh(coords, elems, degree=2)
    g = O.gauss_nodes()
    kappa = 1.0 + g[:, 0] ** 2 + np.sin(3 * g[:, 1])
    f = 1e3 * (1.0 + g[:, 0] - g[:, 1])
    bd = O.bcnode()
    B, r = oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(f), bd, np.zeros(bd.size))
    cp, _ = G.pattern()
    assert np.diff(cp).max() > 24  # the P2 pattern (exact zeros included) has 25-entry rows
    S = gpulib.PoissonSystem(G)
    S.set_dirichlet(bd)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    assert S.solver_info()["banded"] == 0
    assert rel(S.rhs().cpu().numpy(), r) < TOL
    u0 = oracle.spsolve(B, r)
    for prec, rtol in (("fp64", 1e-13), ("mixed", 1e-12)):
        u = S.solve(precision=prec, rtol=rtol)
        assert S.last_stats.status == 0
        assert rel(u.cpu().numpy(), u0) < 1e-10
