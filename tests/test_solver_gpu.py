"""GPU parity of K\\F, the fused resident systems and the adjoint.

Bars: solutions within 1e-9 relative (max norm) of the oracle's direct sparse
solve (scipy SuperLU on the oracle's matrices); gradients within 1e-7 relative
of the reference's backward chain (FemLaplaceScalar / ImposeDirichlet / sparse
solve gradients, restated in the oracle) and of central finite differences.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from adfem_gpu import synth

pytestmark = pytest.mark.gpu
# stopping tolerances on the FP64 (difference-form) residual of the Jacobi-scaled system
RTOL = {"fp64": 1e-13, "mixed": 1e-11}


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def poisson_case(oracle, m=64, seed=0):
    coords, elems = synth.jittered_square(m, seed=seed)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    kappa, f = synth.poisson_c1_fields(g[:, 0], g[:, 1])
    bd = O.bcnode()
    K = O.laplace_csc(kappa)
    F = O.source(f)
    B, r = oracle.dirichlet_csc(K, F, bd, np.zeros(bd.size))
    return coords, elems, O, kappa, f, bd, B, r


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_csc_solve_matches_direct(oracle, gpulib, precision):
    coords, elems, O, kappa, f, bd, B, r = poisson_case(oracle, 64)
    u0 = oracle.spsolve(B, r)
    u, st = gpulib.solve(B, r, precision=precision, rtol=RTOL[precision], return_stats=True)
    assert st.status == 0 and st.relres <= 1e-10
    assert rel(u, u0) < 1e-9


def scaled_relres(B, x, b, oracle):
    """||S (b - B x)|| / ||S b||, S = diag(B_ii)^-1/2: the solver's stopping quantity,
    recomputed on the CPU with the oracle's matrix in doubled precision."""
    s = 1.0 / np.sqrt(B.diagonal())
    r = oracle.residual_dd(B, x, b)
    return float(np.linalg.norm(s * r) / np.linalg.norm(s * b))


def test_fp64_cg_stops_on_true_residual(oracle, gpulib):
    """FP64 CG hands over to the true FP64 residual whenever its recurrence meets rtol (or
    has dropped 10x): the reported relres, and the same quantity recomputed on the CPU from
    the oracle's matrix, meet rtol; an unattainable rtol stops at the attainable floor."""
    coords, elems = synth.jittered_square(160, seed=0)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    G = synth.fourier_field(g[:, 0], g[:, 1], seed=1)
    kappa = 1 + np.exp(synth.contrast_sigma(G, 1e3) * G)
    bd = O.bcnode()
    B, r = oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(1e5 * (g[:, 0] + g[:, 1])), bd, np.zeros(bd.size))
    u0 = oracle.spsolve(B, r)
    for rtol in (1e-10, 1e-11):
        u, st = gpulib.solve(B, r, precision="fp64", rtol=rtol, return_stats=True)
        assert st.status == 0 and st.relres <= rtol and st.updates >= 1
        assert scaled_relres(B, u, r, oracle) <= 1.01 * rtol
        assert rel(u, u0) < 1e-9
    # rtol below what FP64 can represent: ends at the floor with status OK, well before max_iter
    u, st = gpulib.solve(B, r, precision="fp64", rtol=1e-18, max_iter=200000, return_stats=True)
    assert st.status == 0 and 1e-18 < st.relres < 1e-12 and st.iterations < 100000
    assert rel(u, u0) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_poisson_system_matches_oracle_pipeline(oracle, gpulib, precision):
    import torch

    coords, elems, O, kappa, f, bd, B, r = poisson_case(oracle, 64)
    G = gpulib.Mesh(coords, elems)
    S = gpulib.PoissonSystem(G)
    S.set_dirichlet(bd)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    assert rel(S.rhs().cpu().numpy(), r) < 1e-12
    u = S.solve(precision=precision, rtol=RTOL[precision])
    st = S.last_stats
    assert st.status == 0
    u0 = oracle.spsolve(B, r)
    assert rel(u.cpu().numpy(), u0) < 1e-9
    # the resident operator is the Dirichlet-imposed matrix
    x = np.random.default_rng(0).standard_normal(O.ndof)
    y = S.apply(torch.tensor(x, device="cuda")).cpu().numpy()
    assert rel(y, B @ x) < 1e-12
    # end-to-end host-buffer entry
    uh = S.solve_host(kappa, f, precision=precision, rtol=RTOL[precision])
    assert rel(uh, u0) < 1e-9


def test_nonzero_dirichlet_values(oracle, gpulib):
    import torch

    coords, elems = synth.jittered_square(24, seed=2)
    O = oracle.OracleMesh(coords, elems)
    rng = np.random.default_rng(8)
    kappa = 1 + rng.random(O.ngauss)
    f = rng.standard_normal(O.ngauss)
    bd = O.bcnode()
    bv = np.sin(3 * coords[bd - 1, 0]) + coords[bd - 1, 1]
    B, r = oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(f), bd, bv)
    G = gpulib.Mesh(coords, elems)
    S = gpulib.PoissonSystem(G)
    S.set_dirichlet(bd[::-1], bv[::-1])
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    assert rel(S.rhs().cpu().numpy(), r) < 1e-12
    u = S.solve(rtol=1e-14).cpu().numpy()
    assert rel(u, oracle.spsolve(B, r)) < 1e-9
    np.testing.assert_array_equal(u[bd - 1], bv)


def oracle_kappa_gradient(oracle, O, kappa, f, bd, obs, uobs):
    """dL/dkappa through the reference's backward ops: sparse-solve gradient, then
    ImposeDirichlet backward (ImposeDirichlet.h:63-93), then FemLaplaceScalar backward
    (FemLaplaceScalar.h:28-54)."""
    n = O.ndof
    idx, vv = O.laplace_coo(kappa)
    F = O.source(f)
    bv = np.zeros(bd.size)
    oi, ov, orhs = oracle.dirichlet_coo(idx, vv, bd, F, bv, n)
    A = sp.coo_matrix((ov, (oi[:, 0], oi[:, 1])), shape=(n, n)).tocsc()
    u = oracle.spsolve(A, orhs)
    g = np.zeros(n)
    g[obs] = 2 * (u[obs] - uobs)
    lam = oracle.spsolve(A.T.tocsc(), g)
    grad_ov = -lam[oi[:, 0]] * u[oi[:, 1]]  # x = A\b: dL/dA_ij = -lam_i x_j for each stored entry
    gvv, _, _ = oracle.dirichlet_coo_backward(grad_ov, lam, idx, vv, bd, bv, n)
    return O.laplace_coo_backward(gvv), u


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjoint_gradient_matches_reference_chain(oracle, gpulib, precision):
    import torch

    coords, elems = synth.jittered_square(32, seed=0)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    G0 = synth.fourier_field(g[:, 0], g[:, 1], seed=1)
    kappa = 1 + np.exp(0.5 * G0)
    f = 1e5 * (g[:, 0] + g[:, 1])
    bd = O.bcnode()
    obs = synth.observation_nodes(O.ndof, seed=3, frac=0.05)
    uobs = np.random.default_rng(5).standard_normal(obs.size) * 1e-3
    gref, uref = oracle_kappa_gradient(oracle, O, kappa, f, bd, obs, uobs)
    G = gpulib.Mesh(coords, elems)
    S = gpulib.PoissonSystem(G)
    S.set_dirichlet(bd)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    u = S.solve(precision=precision, rtol=RTOL[precision])
    assert rel(u.cpu().numpy(), uref) < 1e-9
    gu = torch.zeros_like(u)
    gu[torch.tensor(obs, device="cuda")] = 2 * (u[torch.tensor(obs, device="cuda")] -
                                                torch.tensor(uobs, device="cuda"))
    lam = S.adjoint(gu, precision=precision, rtol=RTOL[precision])
    gk = S.grad_kappa(u, lam).cpu().numpy()
    assert rel(gk, gref) < 1e-7


def test_gradient_central_differences(oracle, gpulib):
    import torch

    coords, elems = synth.jittered_square(16, seed=0)
    G = gpulib.Mesh(coords, elems)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    kappa = 1 + np.exp(0.5 * synth.fourier_field(g[:, 0], g[:, 1], seed=1))
    f = 1e5 * (g[:, 0] + g[:, 1])
    bd = O.bcnode()
    obs = synth.observation_nodes(O.ndof, seed=3, frac=0.1)
    uobs = np.zeros(obs.size)
    S = gpulib.PoissonSystem(G)
    S.set_dirichlet(bd)
    ft = torch.tensor(f, device="cuda")

    def loss(k):
        S.assemble(torch.tensor(k, device="cuda"), ft)
        u = S.solve(rtol=1e-15, max_iter=100000).cpu().numpy()
        return float(np.sum((u[obs] - uobs) ** 2)), u

    L0, u = loss(kappa)
    ut = torch.tensor(u, device="cuda")
    gu = torch.zeros_like(ut)
    gu[torch.tensor(obs, device="cuda")] = 2 * torch.tensor(u[obs] - uobs, device="cuda")
    lam = S.adjoint(gu, rtol=1e-15)
    gk = S.grad_kappa(ut, lam).cpu().numpy()
    rng = np.random.default_rng(233)
    for _ in range(4):
        v = rng.standard_normal(kappa.size)
        v /= np.linalg.norm(v)
        eps = 1e-4 * np.linalg.norm(kappa) / np.sqrt(kappa.size)
        fd = (loss(kappa + eps * v)[0] - loss(kappa - eps * v)[0]) / (2 * eps)
        assert abs(fd - gk @ v) <= 1e-6 * max(abs(fd), 1e-30) + 1e-12 * L0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_elasticity_system(oracle, gpulib, precision):
    import torch

    coords, elems = synth.jittered_square(24, seed=2)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    E = 1e9 * np.exp(0.3 * synth.fourier_field(g[:, 0], g[:, 1], seed=2))
    nu = np.full(O.ngauss, 0.3)
    D = oracle.plane_strain(E, nu, 0)
    K = O.stiffness_csc(D)
    fx = np.zeros(O.ngauss)
    fy = np.full(O.ngauss, -1e6)
    F = np.concatenate([O.source(fx), O.source(fy)])
    left = synth.left_edge_nodes(coords)
    bd = np.concatenate([left + 1, left + 1 + O.ndof])
    B, r = oracle.dirichlet_csc(K, F, bd, np.zeros(bd.size))
    u0 = oracle.spsolve(B, r)
    G = gpulib.Mesh(coords, elems)
    S = gpulib.ElasticitySystem(G)
    S.set_dirichlet(bd)
    t = lambda a: torch.tensor(a, device="cuda")  # noqa: E731
    S.assemble(t(E), t(nu), t(fx), t(fy))
    assert rel(S.rhs().cpu().numpy(), r) < 1e-12
    x = np.random.default_rng(0).standard_normal(2 * O.ndof)
    assert rel(S.apply(t(x)).cpu().numpy(), B @ x) < 1e-12
    u = S.solve(precision=precision, rtol=RTOL[precision])
    assert S.last_stats.status == 0
    assert rel(u.cpu().numpy(), u0) < 1e-9
    # adjoint gradient wrt E against central differences
    obs = synth.observation_nodes(O.ndof, seed=4, frac=0.05)
    oidx = np.concatenate([obs, obs + O.ndof])

    def loss(Ev):
        S.assemble(t(Ev), t(nu), t(fx), t(fy))
        uu = S.solve(rtol=1e-15).cpu().numpy()
        return float(np.sum(uu[oidx] ** 2)), uu

    L0, uu = loss(E)
    gu = np.zeros(2 * O.ndof)
    gu[oidx] = 2 * uu[oidx]
    lam = S.adjoint(t(gu), rtol=1e-15)
    gE = S.grad_E(t(uu), lam, t(E), t(nu)).cpu().numpy()
    rng = np.random.default_rng(233)
    for _ in range(3):
        v = rng.standard_normal(E.size)
        v /= np.linalg.norm(v)
        eps = 1e-5 * np.linalg.norm(E) / np.sqrt(E.size)
        fd = (loss(E + eps * v)[0] - loss(E - eps * v)[0]) / (2 * eps)
        assert abs(fd - gE @ v) <= 1e-6 * abs(fd) + 1e-12 * L0


def test_not_converged_and_breakdown_are_statuses(oracle, gpulib):
    import torch

    from adfem_gpu import AdFemError

    coords, elems = synth.jittered_square(32, seed=0)
    G = gpulib.Mesh(coords, elems)
    O = oracle.OracleMesh(coords, elems)
    S = gpulib.PoissonSystem(G)
    S.set_dirichlet(O.bcnode())
    k = torch.ones(O.ngauss, dtype=torch.float64, device="cuda")
    f = torch.ones(O.ngauss, dtype=torch.float64, device="cuda")
    S.assemble(k, f)
    with pytest.raises(AdFemError) as ei:
        S.solve(max_iter=3)
    assert ei.value.status == 4
    # the context stays usable
    u = S.solve(rtol=1e-12)
    assert S.last_stats.status == 0 and torch.isfinite(u).all()
    # a non-positive diagonal (negative conductivity) is rejected
    with pytest.raises(AdFemError) as ei:
        S.assemble(-k, f)
    assert ei.value.status in (5, 7)
    kn = k.clone()
    kn[5] = float("nan")
    with pytest.raises(AdFemError):
        S.assemble(kn, f)


@pytest.mark.parametrize("bdval", [False, True])
def test_pair_arithmetic_assembly(oracle, gpulib, monkeypatch, bdval):
    """The opt-in FP32-pair-arithmetic assembly of resident P1 Poisson systems
    (ADFEM_ASM_PAIRS=1): right-hand side and operator against the oracle's Dirichlet-imposed
    system at the 1e-12 value bar, and the FP64 and mixed solves against the direct solve."""
    import torch

    monkeypatch.setenv("ADFEM_ASM_PAIRS", "1")
    coords, elems = synth.jittered_square(48, seed=5)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    kappa, f = synth.poisson_c1_fields(g[:, 0], g[:, 1])
    bd = O.bcnode()
    bv = (np.sin(3 * coords[bd - 1, 0]) + coords[bd - 1, 1]) if bdval else np.zeros(bd.size)
    B, r = oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(f), bd, bv)
    S = gpulib.PoissonSystem(gpulib.Mesh(coords, elems))
    S.set_dirichlet(bd, bv)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    assert S.solver_info()["assembly_pairs"] == 1
    assert rel(S.rhs().cpu().numpy(), r) < 1e-12
    x = np.random.default_rng(1).standard_normal(O.ndof)
    assert rel(S.apply(torch.tensor(x, device="cuda")).cpu().numpy(), B @ x) < 1e-12
    u0 = oracle.spsolve(B, r)
    for prec in ("fp64", "mixed"):
        u = S.solve(precision=prec, rtol=RTOL[prec])
        assert S.last_stats.status == 0
        assert rel(u.cpu().numpy(), u0) < 1e-9


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_elasticity_gradient_matches_reference_chain(oracle, gpulib, precision):
    """dL/dE of a resident elasticity system against the reference's backward ops composed on
    the CPU: sparse-solve gradient -lam_i u_j per stored COO entry (lam zero on Dirichlet
    DOFs), ComputeFemStiffnessMatrixMfem backward (ComputeFemStiffnessMatrixMfem.h:50-81),
    then PlaneStrainAndStress backward (PlaneStrainAndStress.h:20-44)."""
    import torch

    coords, elems = synth.jittered_square(16, seed=3)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    E = 1e9 * np.exp(0.3 * synth.fourier_field(g[:, 0], g[:, 1], seed=5))
    nu = np.full(O.ngauss, 0.3)
    D = oracle.plane_strain(E, nu, 0)
    fx, fy = np.full(O.ngauss, 2e5), np.full(O.ngauss, -1e6)
    left = synth.left_edge_nodes(coords)
    bd = np.concatenate([left + 1, left + 1 + O.ndof])
    B, r = oracle.dirichlet_csc(O.stiffness_csc(D), np.concatenate([O.source(fx), O.source(fy)]), bd,
                                np.zeros(bd.size))
    u0 = oracle.spsolve(B, r)
    obs = synth.observation_nodes(2 * O.ndof, seed=9, frac=0.05)
    uobs = 1.01 * u0[obs]
    gu = np.zeros(2 * O.ndof)
    gu[obs] = 2 * (u0[obs] - uobs)
    gz = gu.copy()
    gz[bd - 1] = 0.0
    lam0 = oracle.spsolve(B.T.tocsc(), gz)
    lam0[bd - 1] = 0.0
    idx, _ = O.stiffness_coo(D)
    gD = O.stiffness_coo_backward(-lam0[idx[:, 0]] * u0[idx[:, 1]])
    gE_ref, _ = oracle.plane_strain_backward(gD.reshape(-1), E, nu, 0)

    S = gpulib.ElasticitySystem(gpulib.Mesh(coords, elems))
    S.set_dirichlet(bd)
    t = lambda a: torch.tensor(a, device="cuda")  # noqa: E731
    S.assemble(t(E), t(nu), t(fx), t(fy))
    u = S.solve(precision=precision, rtol=RTOL[precision])
    assert S.last_stats.status == 0 and rel(u.cpu().numpy(), u0) < 1e-9
    lam = S.adjoint(t(gu), precision=precision, rtol=RTOL[precision])
    assert S.last_stats.status == 0 and rel(lam.cpu().numpy(), lam0) < 1e-9
    gE = S.grad_E(u, lam, t(E), t(nu)).cpu().numpy()
    assert rel(gE, gE_ref) < 1e-7
