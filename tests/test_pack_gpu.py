"""Packed small-system solves (one launch; one thread block per system up to 16,384
DOFs, one cluster of eight blocks per system up to 65,536) against the oracle's direct
solve, and their independence from what they are packed with.

Bars: solutions and adjoints within 1e-9 relative of the direct solve at rtol 1e-11;
a system's packed result bit-identical alone and inside any pack.
"""
import numpy as np
import pytest

from adfem_gpu import synth

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def poisson(oracle, gpulib, m, seed):
    import torch

    coords, elems = synth.jittered_square(m, seed=seed)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    kappa = 1.0 + np.exp(synth.fourier_field(g[:, 0], g[:, 1], seed=seed) * 0.8)
    f = 1e3 * (1 + g[:, 0] - g[:, 1])
    bd = O.bcnode()
    bv = np.sin(3 * O.coords[bd - 1, 0]) + O.coords[bd - 1, 1]
    B, r = oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(f), bd, bv)
    G = gpulib.Mesh(coords, elems)
    S = gpulib.PoissonSystem(G)
    S.set_dirichlet(bd, bv)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    return G, S, B, r, bd


def elasticity(oracle, gpulib, m, seed):
    import torch

    coords, elems = synth.jittered_square(m, seed=seed)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    E = 1e9 * np.exp(0.3 * synth.fourier_field(g[:, 0], g[:, 1], seed=2))
    nu = np.full(O.ngauss, 0.3)
    K = O.stiffness_csc(oracle.plane_strain(E, nu, 0))
    fx, fy = np.zeros(O.ngauss), np.full(O.ngauss, -1e6)
    left = synth.left_edge_nodes(coords)
    bd = np.concatenate([left + 1, left + 1 + O.ndof])
    B, r = oracle.dirichlet_csc(K, np.concatenate([O.source(fx), O.source(fy)]), bd, np.zeros(bd.size))
    G = gpulib.Mesh(coords, elems)
    S = gpulib.ElasticitySystem(G)
    S.set_dirichlet(bd)
    t = lambda a: torch.tensor(a, device="cuda")  # noqa: E731
    S.assemble(t(E), t(nu), t(fx), t(fy))
    return G, S, B, r, bd


def test_packed_solves_match_direct(oracle, gpulib):
    from adfem_gpu import system as SY

    cases = [poisson(oracle, gpulib, m, s) for m, s in ((8, 0), (33, 1), (90, 2), (127, 3))]
    cases += [elasticity(oracle, gpulib, m, 4) for m in (10, 40)]
    systems = [c[1] for c in cases]
    us, stats = SY.solve_packed(systems, rtol=1e-11)
    for (G, S, B, r, bd), u, st in zip(cases, us, stats):
        assert st.status == 0 and st.relres <= 1e-10
        assert rel(u.cpu().numpy(), oracle.spsolve(B, r)) < 1e-9
    # adjoint: K lam = g with lam = 0 on the Dirichlet rows
    rng = np.random.default_rng(0)
    gs, want = [], []
    import torch

    for G, S, B, r, bd in cases:
        g = rng.standard_normal(S.ndof)
        gz = g.copy()
        gz[bd - 1] = 0.0
        want.append(oracle.spsolve(B, gz))
        gs.append(torch.tensor(g, device="cuda"))
    lams, st2 = SY.adjoint_packed(systems, gs, rtol=1e-11)
    for lam, w, (G, S, B, r, bd) in zip(lams, want, cases):
        lam = lam.cpu().numpy()
        assert np.all(lam[bd - 1] == 0.0)
        assert rel(lam, w) < 1e-9


def test_packed_result_independent_of_pack(oracle, gpulib):
    from adfem_gpu import system as SY

    cases = [poisson(oracle, gpulib, m, s) for m, s in ((20, 5), (64, 6), (100, 7))]
    alone = SY.solve_packed([cases[1][1]], rtol=1e-10)[0][0].cpu().numpy()
    packed = SY.solve_packed([c[1] for c in cases], rtol=1e-10)[0][1].cpu().numpy()
    reordered = SY.solve_packed([cases[2][1], cases[1][1]], rtol=1e-10)[0][1].cpu().numpy()
    np.testing.assert_array_equal(alone, packed)
    np.testing.assert_array_equal(alone, reordered)


def test_packed_warm_start_and_limits(oracle, gpulib):
    from adfem_gpu import AdFemError
    from adfem_gpu import system as SY

    G, S, B, r, bd = poisson(oracle, gpulib, 40, 8)
    (u,), (st,) = SY.solve_packed([S], rtol=1e-11)
    # a converged start meets a looser tolerance without iterating
    (u1,), (st1,) = SY.solve_packed([S], outs=[u.clone()], rtol=1e-9, warm_start=True)
    assert st1.iterations == 0 and st1.status == 0
    # a partly converged start needs fewer iterations than a cold solve
    (uc,), _ = SY.solve_packed([S], rtol=1e-5)
    (u2,), (st2,) = SY.solve_packed([S], outs=[uc], rtol=1e-11, warm_start=True)
    assert st2.iterations < st.iterations
    assert rel(u2.cpu().numpy(), oracle.spsolve(B, r)) < 1e-9
    big = poisson(oracle, gpulib, 256, 9)[1]  # 66,049 DOFs > 65,536
    with pytest.raises(AdFemError):
        SY.solve_packed([big])
    with pytest.raises(AdFemError):
        SY.solve_packed([S, S])  # the same system twice


def test_cluster_packed_solves_match_direct(oracle, gpulib):
    """Systems above 16,384 DOFs run on a cluster of eight blocks, mixed with one-block
    systems in the same launch; 255 x 255 (65,536 DOFs) is the largest packed size."""
    from adfem_gpu import system as SY

    cases = [poisson(oracle, gpulib, m, s) for m, s in ((130, 10), (200, 11), (255, 12), (50, 13))]
    cases += [elasticity(oracle, gpulib, 100, 14)]  # 20,402 DOFs
    systems = [c[1] for c in cases]
    us, stats = SY.solve_packed(systems, rtol=1e-11)
    for (G, S, B, r, bd), u, st in zip(cases, us, stats):
        assert st.status == 0 and st.relres <= 1e-10
        assert rel(u.cpu().numpy(), oracle.spsolve(B, r)) < 1e-9
    import torch

    rng = np.random.default_rng(1)
    gs, want = [], []
    for G, S, B, r, bd in cases[:2]:
        g = rng.standard_normal(S.ndof)
        gz = g.copy()
        gz[bd - 1] = 0.0
        want.append(oracle.spsolve(B, gz))
        gs.append(torch.tensor(g, device="cuda"))
    lams, _ = SY.adjoint_packed(systems[:2], gs, rtol=1e-11)
    for lam, w, (G, S, B, r, bd) in zip(lams, want, cases):
        lam = lam.cpu().numpy()
        assert np.all(lam[bd - 1] == 0.0)
        assert rel(lam, w) < 1e-9


def test_cluster_packed_result_independent_of_pack(oracle, gpulib):
    from adfem_gpu import system as SY

    cases = [poisson(oracle, gpulib, m, s) for m, s in ((30, 15), (150, 16), (180, 17))]
    alone = SY.solve_packed([cases[1][1]], rtol=1e-10)[0][0].cpu().numpy()
    packed = SY.solve_packed([c[1] for c in cases], rtol=1e-10)[0][1].cpu().numpy()
    reordered = SY.solve_packed([cases[2][1], cases[1][1]], rtol=1e-10)[0][1].cpu().numpy()
    np.testing.assert_array_equal(alone, packed)
    np.testing.assert_array_equal(alone, reordered)


def test_pack_kernel_boundary_warm_start_and_zero_rhs(oracle, gpulib):
    """3025 DOFs (largest one-block size below 3072) and 3136 DOFs (smallest cluster size
    here) both match the direct solve; on the cluster a converged warm start takes no
    iteration and a zero right-hand side gives u = 0 exactly."""
    import torch

    from adfem_gpu import system as SY

    block = poisson(oracle, gpulib, 54, 20)
    clus = poisson(oracle, gpulib, 55, 21)
    us, stats = SY.solve_packed([block[1], clus[1]], rtol=1e-11)
    for (G, S, B, r, bd), u, st in zip((block, clus), us, stats):
        assert st.status == 0
        assert rel(u.cpu().numpy(), oracle.spsolve(B, r)) < 1e-9
    (u1,), (st1,) = SY.solve_packed([clus[1]], outs=[us[1].clone()], rtol=1e-9, warm_start=True)
    assert st1.iterations == 0 and st1.status == 0
    S = clus[1]
    (lam,), (st2,) = SY.adjoint_packed([S], [torch.zeros(S.ndof, dtype=torch.float64, device="cuda")], rtol=1e-11)
    assert st2.status == 0 and st2.iterations == 0
    assert torch.count_nonzero(lam).item() == 0
