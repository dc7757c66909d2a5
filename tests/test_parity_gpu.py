"""GPU parity: every operator of the path through the C ABI against the CPU oracle.

Tolerances (the reference bar): CSR/CSC patterns and COO indices bit-exact;
matrix values within 1e-12 relative to the largest entry of their row; load
vectors and gradients within 1e-12 relative to their max norm; Dirichlet
outputs exact where they are copies.
"""
import ctypes
import os

import numpy as np
import pytest
import scipy.sparse as sp

from adfem_gpu import synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12


def row_scaled_err(A, B):
    """max_ij |A_ij - B_ij| / max_k |B_ik| over the rows of CSC/CSR matrices with equal patterns."""
    A = sp.csr_matrix(A)
    B = sp.csr_matrix(B)
    d = abs(A - B).max(axis=1).toarray().ravel()
    s = abs(B).max(axis=1).toarray().ravel()
    s[s == 0] = 1.0
    return float(np.max(d / s))


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def meshes(oracle, gpulib, m=16, seed=0, jitter=0.2):
    coords, elems = synth.jittered_square(m, seed=seed, jitter=jitter)
    return oracle.OracleMesh(coords, elems), gpulib.Mesh(coords, elems)


@pytest.mark.parametrize("m,jitter", [(1, 0.0), (2, 0.0), (16, 0.2), (33, 0.2)])
def test_mesh_runtime(oracle, gpulib, m, jitter):
    O, G = meshes(oracle, gpulib, m, 0, jitter)
    np.testing.assert_array_equal(G.elems, O.elems1())
    np.testing.assert_allclose(gpulib.get_area(G), O.area, rtol=1e-15, atol=0)
    np.testing.assert_allclose(gpulib.gauss_nodes(G), O.gauss_nodes(), rtol=0, atol=1e-15)
    np.testing.assert_array_equal(G.edges, O.edges())
    np.testing.assert_array_equal(gpulib.bcnode(G), O.bcnode())
    K = O.laplace_csc(np.ones(O.ngauss))
    cp, rv = G.pattern()
    np.testing.assert_array_equal(cp - 1, K.indptr)
    np.testing.assert_array_equal(rv - 1, K.indices)
    assert gpulib.get_ngauss(G) == O.ngauss


def test_reference_triangle_mesh(oracle, gpulib):
    """Mesh() (MFEM.jl:179-191): the single reference triangle."""
    coords = np.array([[1.0, 0.0], [0.0, 1.0], [0.0, 0.0]])
    elems = np.array([[1, 2, 3]])
    O = oracle.OracleMesh(coords, elems)
    G = gpulib.Mesh(coords, elems)
    np.testing.assert_array_equal(G.elems, O.elems1())
    k = np.array([1.0, 2.0, 3.0])
    A = gpulib.compute_fem_laplace_matrix1(k, G)
    assert row_scaled_err(A, O.laplace_csc(k)) < TOL
    np.testing.assert_allclose(gpulib.compute_fem_source_term1(k, G), O.source(k), rtol=TOL)


@pytest.mark.parametrize("m,seed", [(8, 0), (64, 0), (37, 4)])
def test_laplace_csc(oracle, gpulib, m, seed):
    O, G = meshes(oracle, gpulib, m, seed)
    g = O.gauss_nodes()
    kappa = np.sin(g[:, 0]) * (1 + g[:, 1] ** 2) + 1
    A = gpulib.compute_fem_laplace_matrix1(kappa, G)
    B = O.laplace_csc(kappa)
    np.testing.assert_array_equal(A.indptr, B.indptr)
    np.testing.assert_array_equal(A.indices, B.indices)
    assert row_scaled_err(A, B) < TOL
    # bit-reproducible: a second call gives the same bits
    A2 = gpulib.compute_fem_laplace_matrix1(kappa, G)
    assert np.array_equal(A.data.view(np.int64), A2.data.view(np.int64))


def test_laplace_coo_and_backward(oracle, gpulib):
    import torch

    from adfem_gpu import system as S

    O, G = meshes(oracle, gpulib, 12, 1)
    rng = np.random.default_rng(7)
    kappa = 1 + rng.random(O.ngauss)
    idx, vv = S.laplace_coo(G, torch.tensor(kappa, device="cuda"))
    oi, ov = O.laplace_coo(kappa)
    np.testing.assert_array_equal(idx.cpu().numpy(), oi)
    assert rel(vv.cpu().numpy(), ov) < TOL
    gvv = rng.standard_normal(ov.size)
    gk = S.laplace_coo_backward(G, torch.tensor(gvv, device="cuda")).cpu().numpy()
    assert rel(gk, O.laplace_coo_backward(gvv)) < TOL


def test_source_and_backward(oracle, gpulib):
    import torch

    from adfem_gpu import system as S

    O, G = meshes(oracle, gpulib, 20, 2)
    g = O.gauss_nodes()
    f = 1e5 * (g[:, 0] + g[:, 1])
    assert rel(gpulib.compute_fem_source_term1(f, G), O.source(f)) < TOL
    both = gpulib.compute_fem_source_term(f, 2 * f, G)
    assert rel(both, np.concatenate([O.source(f), O.source(2 * f)])) < TOL
    gr = np.random.default_rng(3).standard_normal(O.ndof)
    gf = S.source_backward(G, torch.tensor(gr, device="cuda")).cpu().numpy()
    assert rel(gf, O.source_backward(gr)) < TOL


def test_stiffness_csc_coo_backward(oracle, gpulib):
    import torch

    from adfem_gpu import system as S

    O, G = meshes(oracle, gpulib, 10, 5)
    rng = np.random.default_rng(11)
    D = rng.random((O.ngauss, 3, 3)) + np.eye(3)  # not symmetric: checks the CSC transpose
    A = gpulib.compute_fem_stiffness_matrix(D, G)
    B = O.stiffness_csc(D)
    np.testing.assert_array_equal(A.indptr, B.indptr)
    np.testing.assert_array_equal(A.indices, B.indices)
    assert row_scaled_err(A, B) < TOL
    # constant (3,3) D
    D1 = gpulib.compute_plane_strain_matrix(1.0, 0.3)
    A1 = gpulib.compute_fem_stiffness_matrix(D1, G)
    assert row_scaled_err(A1, O.stiffness_csc(np.broadcast_to(D1, (O.ngauss, 3, 3)))) < TOL
    idx, vv = S.stiffness_coo(G, torch.tensor(D.ravel(), device="cuda"))
    oi, ov = O.stiffness_coo(D)
    np.testing.assert_array_equal(idx.cpu().numpy(), oi)
    assert rel(vv.cpu().numpy(), ov) < TOL
    gvv = rng.standard_normal(ov.size)
    gD = S.stiffness_coo_backward(G, torch.tensor(gvv, device="cuda")).cpu().numpy()
    assert rel(gD, O.stiffness_coo_backward(gvv).ravel()) < TOL
    # CSR device values are the transpose of the CSC ones
    v = S.stiffness_csr(G, torch.tensor(D.ravel(), device="cuda")).cpu().numpy()
    cp, rv = G.pattern_elasticity()
    Acsr = sp.csr_matrix((v, rv - 1, cp - 1), shape=A.shape)
    assert row_scaled_err(Acsr, B) < TOL


@pytest.mark.parametrize("mode", [0, 1])
def test_plane_strain(oracle, gpulib, mode):
    import torch

    from adfem_gpu import system as S

    rng = np.random.default_rng(mode)
    E = 1e9 * (1 + rng.random(500))
    nu = 0.05 + 0.4 * rng.random(500)
    D = S.plane_strain(torch.tensor(E, device="cuda"), torch.tensor(nu, device="cuda"), mode).cpu().numpy()
    assert rel(D, oracle.plane_strain(E, nu, mode).ravel()) < 1e-14
    fn = gpulib.compute_plane_strain_matrix if mode == 0 else gpulib.compute_plane_stress_matrix
    assert rel(fn(E, nu), oracle.plane_strain(E, nu, mode)) < 1e-14
    g = rng.standard_normal(9 * 500)
    gE, gn = S.plane_strain_backward(torch.tensor(g, device="cuda"), torch.tensor(E, device="cuda"),
                                     torch.tensor(nu, device="cuda"), mode)
    oE, on = oracle.plane_strain_backward(g, E, nu, mode)
    assert rel(gE.cpu().numpy(), oE) < 1e-13
    assert rel(gn.cpu().numpy(), on) < 1e-13


@pytest.mark.parametrize("jitter,keep", [(0.2, False), (0.0, False), (0.0, True)])
def test_dirichlet_csc(oracle, gpulib, jitter, keep):
    O, G = meshes(oracle, gpulib, 16, 0, jitter)
    rng = np.random.default_rng(2)
    kappa = np.ones(O.ngauss) if jitter == 0.0 else 1 + rng.random(O.ngauss)
    K = O.laplace_csc(kappa)
    F = rng.standard_normal(O.ndof)
    bd = O.bcnode()
    bv = rng.standard_normal(bd.size)
    perm = rng.permutation(bd.size)  # the reference passes Julia Set order
    B1, r1 = gpulib.impose_Dirichlet_boundary_conditions(K, F, bd[perm], bv[perm], keep_zeros=keep)
    B2, r2 = oracle.dirichlet_csc(K, F, bd[perm], bv[perm], keep_zeros=keep)
    np.testing.assert_array_equal(B1.indptr, B2.indptr)
    np.testing.assert_array_equal(B1.indices, B2.indices)
    np.testing.assert_array_equal(B1.data, B2.data)
    assert rel(r1, r2) < TOL


def test_dirichlet_coo_and_backward(oracle, gpulib):
    O, G = meshes(oracle, gpulib, 9, 3)
    rng = np.random.default_rng(4)
    idx, vv = O.laplace_coo(1 + rng.random(O.ngauss))
    n = O.ndof
    bd = O.bcnode()
    bd = np.concatenate([bd[::-1], bd[:3]])  # unsorted, with repeats (last value wins)
    bv = rng.standard_normal(bd.size)
    rhs = rng.standard_normal(n)
    oi, ov, orhs = gpulib.impose_Dirichlet_coo(idx, vv, n, rhs, bd, bv)
    ei, ev, erhs = oracle.dirichlet_coo(idx, vv, bd, rhs, bv, n)
    np.testing.assert_array_equal(oi, ei)
    np.testing.assert_array_equal(ov, ev)
    np.testing.assert_array_equal(orhs, erhs)  # same sequential order of updates
    gvv = rng.standard_normal(ov.size)
    grhs = rng.standard_normal(n)
    a = gpulib.impose_Dirichlet_coo_backward(gvv, grhs, idx, vv, n, bd, bv)
    b = oracle.dirichlet_coo_backward(gvv, grhs, idx, vv, bd, bv, n)
    for x, y in zip(a, b):
        np.testing.assert_allclose(x, y, rtol=0, atol=1e-15 * max(1.0, np.max(np.abs(y))))


def test_legacy_ccall_layer(oracle, gpulib):
    """The libadmfem symbols AdFem ccalls, driven exactly like src/MFEM/MFEM.jl:92-106."""
    from adfem_gpu import _lib

    L = _lib.load()
    coords, elems = synth.jittered_square(6, seed=9)
    O = oracle.OracleMesh(coords, elems)
    c = np.concatenate([coords, np.zeros((coords.shape[0], 1))], 1).ravel()
    e = np.ascontiguousarray((elems - 1).ravel(), np.int32)
    ned = np.zeros(1, np.int64)
    p = L.init_nnfem_mesh(_lib.ptr(c), coords.shape[0], _lib.ptr(e), elems.shape[0], -1, -1, 1, _lib.ptr(ned))
    assert p
    edges = np.ctypeslib.as_array(p, shape=(2 * ned[0],)).copy()
    ctypes.CDLL(None).free(ctypes.cast(p, ctypes.c_void_p))
    np.testing.assert_array_equal(edges.reshape(2, -1).T, O.edges())
    assert L.mfem_get_ngauss() == O.ngauss and L.mfem_get_ndof() == O.ndof and L.mfem_get_elem_ndof() == 3
    x, y, w, a = np.empty(O.ngauss), np.empty(O.ngauss), np.empty(O.ngauss), np.empty(O.nelem)
    L.mfem_get_gauss(_lib.ptr(x), _lib.ptr(y))
    L.mfem_get_gauss_weights(_lib.ptr(w))
    L.mfem_get_area(_lib.ptr(a))
    np.testing.assert_allclose(np.stack([x, y], 1), O.gauss_nodes(), atol=1e-15)
    np.testing.assert_allclose(w, O.w.ravel(), rtol=1e-15)
    np.testing.assert_allclose(a, O.area, rtol=1e-15)
    conn = np.empty(3 * O.nelem, np.int64)
    L.mfem_get_connectivity(_lib.ptr(conn))
    np.testing.assert_array_equal(conn.reshape(-1, 3), O.elems1())
    ev = np.empty(3 * O.nelem, np.int64)
    L.mfem_get_element_to_vertices(_lib.ptr(ev))
    np.testing.assert_array_equal(ev.reshape(3, -1).T, O.elems1())
    kappa = 1 + np.random.default_rng(0).random(O.ngauss)
    N = 9 * O.ngauss
    idx = np.zeros(2 * N, np.int64)
    vv = np.zeros(N)
    L.FemLaplaceScalar_forward_Julia(_lib.ptr(idx), _lib.ptr(vv), _lib.ptr(kappa))
    oi, ov = O.laplace_coo(kappa)
    np.testing.assert_array_equal(idx.reshape(-1, 2), oi)
    assert rel(vv, ov) < TOL
    rhs = np.ones(O.ndof)  # accumulates into the caller's array
    L.FemSourceScalar_forward_Julia(_lib.ptr(rhs), _lib.ptr(kappa))
    assert rel(rhs, O.source(kappa, np.ones(O.ndof))) < TOL
    D = np.random.default_rng(1).random(9 * O.ngauss)
    N2 = 36 * O.ngauss
    idx2 = np.zeros(2 * N2, np.int64)
    vv2 = np.zeros(N2)
    L.ComputeFemStiffnessMatrixMfem_forward_Julia(_lib.ptr(idx2), _lib.ptr(vv2), _lib.ptr(D))
    oi2, ov2 = O.stiffness_coo(D)
    np.testing.assert_array_equal(idx2.reshape(-1, 2), oi2)
    assert rel(vv2, ov2) < TOL
    gk = np.empty(O.ngauss)
    gv = np.random.default_rng(2).standard_normal(N)
    L.FemLaplaceScalar_backward(_lib.ptr(gk), _lib.ptr(gv), _lib.ptr(idx), _lib.ptr(vv), _lib.ptr(kappa))
    assert rel(gk, O.laplace_coo_backward(gv)) < TOL
    L.adfem_set_current_mesh(None)


def test_golden_fixture(gpulib):
    z = np.load(os.path.join(GOLD, "c_small.npz"))
    G = gpulib.Mesh(z["coords"], z["elems"])
    K = gpulib.compute_fem_laplace_matrix1(z["kappa"], G)
    Kg = sp.csc_matrix((z["K_data"], z["K_indices"], z["K_indptr"]))
    np.testing.assert_array_equal(K.indptr, Kg.indptr)
    np.testing.assert_array_equal(K.indices, Kg.indices)
    assert row_scaled_err(K, Kg) < TOL
    F = gpulib.compute_fem_source_term1(z["f"], G)
    assert rel(F, z["F"]) < TOL
    B, r = gpulib.impose_Dirichlet_boundary_conditions(K, F, z["bd"], np.zeros(z["bd"].size))
    u = gpulib.solve(B, r, rtol=1e-14)
    assert rel(u, z["u"]) < 1e-9


def test_error_paths(gpulib):
    from adfem_gpu import AdFemError

    coords, elems = synth.jittered_square(3, seed=0)
    G = gpulib.Mesh(coords, elems)
    with pytest.raises(AdFemError):
        gpulib.compute_fem_laplace_matrix1(np.ones(5), G)
    with pytest.raises(AdFemError):
        gpulib.Mesh(coords, elems, degree=3)
    bad = np.array([[1, 2, 2]])
    with pytest.raises(AdFemError):
        gpulib.Mesh(coords, bad)
    with pytest.raises(AdFemError):
        gpulib.Mesh(np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0]]), np.array([[1, 2, 3]]))  # zero area
