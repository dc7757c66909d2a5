"""Meshes with a vertex of high valence: a fan of k triangles around a centre vertex inside
rings of quads, so the centre's matrix row has k + 1 entries.  The row kernels keep a
row in shared memory and switch to their wide variants above 24 scalar entries (Laplace,
the fused Poisson system) or 16 (stiffness); mesh_build accepts up to 63 neighbours.  The
reference builds such meshes like any other (MFEM, src/MFEM/MFEM.jl:60-119), so the
operators and a resident Poisson system (forward, adjoint, kappa-gradient) are compared with
the oracle at the usual bars; resident elasticity systems, whose fused row pass stops at 16
entries, refuse them at creation with a status.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from adfem_gpu.synth import fan_mesh

pytestmark = pytest.mark.gpu
TOL = 1e-12


def row_scaled_err(A, B):
    A, B = sp.csr_matrix(A), sp.csr_matrix(B)
    d = abs(A - B).max(axis=1).toarray().ravel()
    s = abs(B).max(axis=1).toarray().ravel()
    s[s == 0] = 1.0
    return float(np.max(d / s))


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("k", [30, 63])
def test_wide_rows_laplace_source_stiffness(oracle, gpulib, k):
    """Rows of 31 and 64 scalar entries (62 and 128 in the stiffness operator): Laplace and
    stiffness CSC (the wide row kernels), the load, the COO ops, and K\\F on the wide
    operator, against the oracle."""
    import torch

    from adfem_gpu import system as S

    coords, elems = fan_mesh(k)
    O = oracle.OracleMesh(coords, elems)
    G = gpulib.Mesh(coords, elems)
    g = O.gauss_nodes()
    kappa = np.sin(g[:, 0]) * (1 + g[:, 1] ** 2) + 2
    B = O.laplace_csc(kappa)
    assert np.diff(B.indptr).max() == k + 1
    A = gpulib.compute_fem_laplace_matrix1(kappa, G)
    np.testing.assert_array_equal(A.indptr, B.indptr)
    np.testing.assert_array_equal(A.indices, B.indices)
    assert row_scaled_err(A, B) < TOL
    f = 1e5 * (g[:, 0] + g[:, 1])
    F = gpulib.compute_fem_source_term1(f, G)
    assert rel(F, O.source(f)) < TOL
    # device CSR values of the same operator
    v = S.laplace_csr(G, torch.tensor(kappa, device="cuda")).cpu().numpy()
    cp, rv = G.pattern()
    assert row_scaled_err(sp.csr_matrix((v, rv - 1, cp - 1), shape=A.shape), B) < TOL
    # stiffness, a non-symmetric D (checks the CSC transpose)
    rng = np.random.default_rng(k)
    D = rng.random((O.ngauss, 3, 3)) + np.eye(3)
    As = gpulib.compute_fem_stiffness_matrix(D, G)
    Bs = O.stiffness_csc(D)
    np.testing.assert_array_equal(As.indptr, Bs.indptr)
    np.testing.assert_array_equal(As.indices, Bs.indices)
    assert row_scaled_err(As, Bs) < TOL
    vs = S.stiffness_csr(G, torch.tensor(D.ravel(), device="cuda")).cpu().numpy()
    cpe, rve = G.pattern_elasticity()
    assert row_scaled_err(sp.csr_matrix((vs, rve - 1, cpe - 1), shape=As.shape), Bs) < TOL
    idx, vv = S.stiffness_coo(G, torch.tensor(D.ravel(), device="cuda"))
    oi, ov = O.stiffness_coo(D)
    np.testing.assert_array_equal(idx.cpu().numpy(), oi)
    assert rel(vv.cpu().numpy(), ov) < TOL
    # K\F on the Dirichlet-imposed wide operator (the solver's plain-loop SpMV)
    bd = O.bcnode()
    Kb, Fb = oracle.dirichlet_csc(B, O.source(f), bd, np.zeros(bd.size))
    u0 = oracle.spsolve(Kb, Fb)
    for prec, rtol in (("fp64", 1e-13), ("mixed", 1e-12)):
        u = gpulib.solve(Kb, Fb, precision=prec, rtol=rtol)
        assert rel(u, u0) < 1e-9, prec


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_wide_rows_resident_poisson_system(oracle, gpulib, precision):
    """A resident Poisson system on a fan mesh with a 64-entry row (the 64-wide fused row
    pass; the solver takes its scaled path above 24 entries): forward solve against the
    direct solve (1e-9), and the kappa-gradient of a misfit against the reference's backward
    chain (sparse-solve gradient, ImposeDirichlet backward, FemLaplaceScalar backward; 1e-7)."""
    import torch

    from test_solver_gpu import RTOL, oracle_kappa_gradient

    coords, elems = fan_mesh(63)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    kappa = np.sin(g[:, 0]) * (1 + g[:, 1] ** 2) + 2
    f = 1e5 * (g[:, 0] + g[:, 1])
    bd = O.bcnode()
    obs = np.arange(0, O.ndof, 7)
    uobs = np.random.default_rng(5).standard_normal(obs.size) * 1e-3
    gref, uref = oracle_kappa_gradient(oracle, O, kappa, f, bd, obs, uobs)
    S = gpulib.PoissonSystem(gpulib.Mesh(coords, elems))
    S.set_dirichlet(bd)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    assert S.solver_info()["banded"] == 0
    u = S.solve(precision=precision, rtol=RTOL[precision])
    assert S.last_stats.status == 0
    assert rel(u.cpu().numpy(), uref) < 1e-9
    ob = torch.tensor(obs, device="cuda")
    gu = torch.zeros_like(u)
    gu[ob] = 2 * (u[ob] - torch.tensor(uobs, device="cuda"))
    lam = S.adjoint(gu, precision=precision, rtol=RTOL[precision])
    assert rel(S.grad_kappa(u, lam).cpu().numpy(), gref) < 1e-7


def test_wide_rows_refused_by_resident_elasticity_systems(oracle, gpulib):
    """Resident elasticity systems fuse the rows with Dirichlet and the solver layout in a
    kernel that keeps 16 scalar entries per row: a 41-entry row is refused at creation with
    ADFEM_ERR_UNSUPPORTED and a message naming the limit, and the mesh and the library stay
    usable."""
    from adfem_gpu import _lib

    coords, elems = fan_mesh(40)
    G = gpulib.Mesh(coords, elems)
    with pytest.raises(gpulib.AdFemError) as ei:
        gpulib.ElasticitySystem(G)
    assert ei.value.status == _lib.ERR_UNSUPPORTED and "15 neighbours" in str(ei.value)
    O = oracle.OracleMesh(coords, elems)
    kappa = np.ones(O.ngauss)
    assert row_scaled_err(gpulib.compute_fem_laplace_matrix1(kappa, G), O.laplace_csc(kappa)) < TOL
