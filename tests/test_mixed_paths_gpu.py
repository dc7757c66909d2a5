"""The two mixed-precision iterations of the CG solver against the direct solve.

* banded path (one kernel per iteration, the band of each block's rows held in shared
  memory), chosen automatically when the band fits;
* scaled two-kernel path, the fallback for wide bands (forced with ADFEM_ZCG=0).

The path that ran is identified by the launch count per iteration (banded: one launch
per iteration plus the replacement checks; scaled: two plus the checks).  Bars as in
the mixed-precision target: 1e-10 relative error (max norm) against the FP64 direct solve
(SuperLU) on the oracle's matrices, or against an FP64 CG solve that stopped on its true
residual where the system is too large for the direct solve.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from adfem_gpu import synth

pytestmark = pytest.mark.gpu
RTOL_MIXED = 1e-11
ERR_BAR = 1e-10  # mixed solves: relative error against the FP64 solution


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def poisson(oracle, m, seed=0, contrast=None):
    coords, elems = synth.jittered_square(m, seed=seed)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    if contrast is None:
        kappa, f = synth.poisson_c1_fields(g[:, 0], g[:, 1])
    else:
        G = synth.fourier_field(g[:, 0], g[:, 1], seed=1)
        kappa = 1 + np.exp(synth.contrast_sigma(G, contrast) * G)
        f = 1e5 * (g[:, 0] + g[:, 1])
    bd = O.bcnode()
    return oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(f), bd, np.zeros(bd.size))


def launches_per_iter(st):
    return st.launches / max(st.iterations, 1)


@pytest.mark.parametrize("zcg", ["1", "0"])
def test_mixed_paths_match_direct(oracle, gpulib, monkeypatch, zcg):
    monkeypatch.setenv("ADFEM_ZCG", zcg)
    B, r = poisson(oracle, 64, contrast=1e3)
    u0 = oracle.spsolve(B, r)
    u, st = gpulib.solve(B, r, precision="mixed", rtol=RTOL_MIXED, return_stats=True)
    assert st.status == 0 and st.relres <= 1e-10
    assert rel(u, u0) < ERR_BAR
    lpi = launches_per_iter(st)
    assert (lpi < 1.9) if zcg == "1" else (lpi > 2.0), lpi


def test_banded_path_super_tiles_and_deterministic(oracle, gpulib, monkeypatch):
    # 361k DOF over a few hundred blocks, halos crossing block boundaries
    monkeypatch.delenv("ADFEM_ZCG", raising=False)
    monkeypatch.delenv("ADFEM_ZCG_SMAX", raising=False)
    B, r = poisson(oracle, 600, contrast=1e3)
    u64, s64 = gpulib.solve(B, r, precision="fp64", rtol=1e-13, return_stats=True)
    u1, s1 = gpulib.solve(B, r, precision="mixed", rtol=RTOL_MIXED, return_stats=True)
    u2, s2 = gpulib.solve(B, r, precision="mixed", rtol=RTOL_MIXED, return_stats=True)
    assert s64.status == 0 and s1.status == 0
    assert launches_per_iter(s1) < 1.9
    assert rel(u1, u64) < ERR_BAR
    # fixed grid, fixed reduction order, halos recomputed bit-identically
    assert s1.iterations == s2.iterations
    assert np.array_equal(u1, u2)
    # each block's range split into super-tiles of 512 rows (each with its own halo)
    monkeypatch.setenv("ADFEM_ZCG_SMAX", "512")
    u3, s3 = gpulib.solve(B, r, precision="mixed", rtol=RTOL_MIXED, return_stats=True)
    assert s3.status == 0 and launches_per_iter(s3) < 1.9
    assert rel(u3, u64) < ERR_BAR


def renumbered(m, seed=3):
    """Jittered square with a random node numbering: (coords, elems) in the original and the
    permuted numbering, and inv (new id of old node i)."""
    coords, elems = synth.jittered_square(m, seed=seed)
    perm = np.random.default_rng(5).permutation(coords.shape[0])
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.size)
    return coords, elems, coords[perm], inv[elems - 1] + 1, inv


@pytest.mark.parametrize("m", [40, 80])
def test_randomly_renumbered_mesh(oracle, gpulib, monkeypatch, m):
    # A random node numbering spreads the band over the whole matrix.  The resident system
    # renumbers its nodes (reverse Cuthill-McKee) so the banded mixed iteration applies;
    # every input and output stays in the caller's numbering.
    import torch

    from adfem_gpu import system as SY

    monkeypatch.delenv("ADFEM_ZCG", raising=False)
    coords, elems, coords_p, elems_p, inv = renumbered(m)
    O = oracle.OracleMesh(coords_p, elems_p)
    g = O.gauss_nodes()
    kappa, f = synth.poisson_c1_fields(g[:, 0], g[:, 1])
    bd = O.bcnode()
    bv = np.cos(2 * O.coords[bd - 1, 0])
    B, r = oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(f), bd, bv)
    t = lambda a: torch.tensor(a, device="cuda")  # noqa: E731
    S = gpulib.PoissonSystem(gpulib.Mesh(coords_p, elems_p))
    S.set_dirichlet(bd, bv)
    S.assemble(t(kappa), t(f))
    info = S.solver_info()
    assert info["renumbered"] == 1 and info["banded"] == 1, info
    assert info["band"] < 4 * m
    u0 = oracle.spsolve(B, r)
    for prec, rtol in (("mixed", RTOL_MIXED), ("fp64", 1e-12)):
        u = S.solve(precision=prec, rtol=rtol)
        assert S.last_stats.status == 0
        assert rel(u.cpu().numpy(), u0) < ERR_BAR
    assert rel(S.rhs().cpu().numpy(), r) < 1e-12
    x = np.random.default_rng(1).standard_normal(O.ndof)
    assert rel(S.apply(t(x)).cpu().numpy(), B @ x) < 1e-12
    (up,), _ = SY.solve_packed([S], rtol=1e-11)
    assert rel(up.cpu().numpy(), u0) < ERR_BAR
    # adjoint gradient against the same problem in the natural numbering (same elements,
    # same Gauss points): the gradients agree
    S2 = gpulib.PoissonSystem(gpulib.Mesh(coords, elems))
    S2.set_dirichlet(np.sort(np.argsort(inv)[bd - 1] + 1), bv[np.argsort(np.argsort(inv)[bd - 1])])
    S2.assemble(t(kappa), t(f))
    assert S2.solver_info()["renumbered"] == 0
    obs = np.arange(1, O.ndof + 1, 7)
    grads = []
    for SS, ob in ((S, obs), (S2, np.argsort(inv)[obs - 1] + 1)):
        uu = SS.solve(precision="fp64", rtol=1e-13)
        gu = torch.zeros_like(uu)
        gu[torch.tensor(ob - 1, device="cuda")] = 2 * uu[torch.tensor(ob - 1, device="cuda")]
        lam = SS.adjoint(gu, precision="fp64", rtol=1e-13)
        grads.append(SS.grad_kappa(uu, lam).cpu().numpy())
    assert rel(grads[0], grads[1]) < 1e-8


def test_renumbered_elasticity(oracle, gpulib, monkeypatch):
    import torch

    monkeypatch.delenv("ADFEM_ZCG", raising=False)
    coords, elems, coords_p, elems_p, inv = renumbered(30, seed=6)
    O = oracle.OracleMesh(coords_p, elems_p)
    g = O.gauss_nodes()
    E = 1e9 * np.exp(0.3 * synth.fourier_field(g[:, 0], g[:, 1], seed=2))
    nu = np.full(O.ngauss, 0.3)
    K = O.stiffness_csc(oracle.plane_strain(E, nu, 0))
    fx, fy = np.zeros(O.ngauss), np.full(O.ngauss, -1e6)
    left = synth.left_edge_nodes(coords_p)
    bd = np.concatenate([left + 1, left + 1 + O.ndof])
    B, r = oracle.dirichlet_csc(K, np.concatenate([O.source(fx), O.source(fy)]), bd, np.zeros(bd.size))
    S = gpulib.ElasticitySystem(gpulib.Mesh(coords_p, elems_p))
    S.set_dirichlet(bd)
    t = lambda a: torch.tensor(a, device="cuda")  # noqa: E731
    S.assemble(t(E), t(nu), t(fx), t(fy))
    info = S.solver_info()
    assert info["renumbered"] == 1 and info["banded"] == 1, info
    assert rel(S.rhs().cpu().numpy(), r) < 1e-12
    x = np.random.default_rng(2).standard_normal(2 * O.ndof)
    assert rel(S.apply(t(x)).cpu().numpy(), B @ x) < 1e-12
    u = S.solve(precision="mixed", rtol=RTOL_MIXED)
    assert S.last_stats.status == 0
    assert rel(u.cpu().numpy(), oracle.spsolve(B, r)) < ERR_BAR


def test_banded_path_warm_start_and_zero_rhs(oracle, gpulib, monkeypatch):
    monkeypatch.delenv("ADFEM_ZCG", raising=False)
    B, r = poisson(oracle, 48, seed=1)
    u0 = oracle.spsolve(B, r)
    z, st0 = gpulib.solve(B, np.zeros_like(r), precision="mixed", rtol=RTOL_MIXED, return_stats=True)
    assert st0.status == 0 and st0.iterations == 0 and not np.any(z)
    # warm start from the solution: converged by the first FP64 residual check
    uw, stw = gpulib.solve(B, r, precision="mixed", rtol=1e-8, u0=u0, return_stats=True)
    assert stw.status == 0 and stw.iterations == 0
    assert rel(uw, u0) < 1e-12


def test_system_reports_banded_layout(oracle, gpulib, monkeypatch):
    import torch

    monkeypatch.delenv("ADFEM_ZCG", raising=False)
    coords, elems = synth.jittered_square(32, seed=4)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    kappa, f = synth.poisson_c1_fields(g[:, 0], g[:, 1])
    S = gpulib.PoissonSystem(gpulib.Mesh(coords, elems))
    S.set_dirichlet(O.bcnode())
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    info = S.solver_info()
    B, r = oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(f), O.bcnode(), np.zeros(O.bcnode().size),
                                keep_zeros=True)
    C = sp.coo_matrix(B)
    assert info["rows"] == O.ndof and info["banded"] == 1
    assert info["band"] == int(np.max(np.abs(C.row - C.col)))  # the mesh's pattern, zeros kept
    assert info["blocks"] * info["rows_per_block"] >= info["rows"]
    assert info["ring"] >= 2 * info["band"] + 32
    u = S.solve(precision="mixed", rtol=RTOL_MIXED)
    assert rel(u.cpu().numpy(), oracle.spsolve(B, r)) < ERR_BAR


def _ring_system(gpulib, m):
    import torch

    coords, elems = synth.jittered_square(m, seed=2)
    mesh = gpulib.Mesh(coords, elems)
    g = gpulib.gauss_nodes(mesh)
    G = synth.fourier_field(g[:, 0], g[:, 1], seed=1)
    kappa = 1 + np.exp(synth.contrast_sigma(G, 1e3) * G)
    f = 1e5 * (g[:, 0] + g[:, 1])
    S = gpulib.PoissonSystem(mesh)
    S.set_dirichlet(gpulib.bcnode(mesh))
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    return S


@pytest.mark.parametrize("ring,smax,refill", [("3", "", "1"), ("2", "", "1"), ("3", "1504", "1"), ("2", "2080", "1"),
                                              ("2", "", "0")])
def test_matrix_ring_bit_identical_to_plain_variant(gpulib, monkeypatch, ring, smax, refill):
    """The opt-in ring variant of the banded mixed iteration (matrix values streamed into
    shared memory by bulk copies; refill 0: only the first stages) does the plain variant's
    arithmetic in the same order: same iterations, bit-identical solution.  1M DOF: several
    ring refills per block; with a super-tile cap the stages straddle no super-tile (partial
    stages at each tile's end).  Both variants run as programmatic dependent launches."""
    monkeypatch.delenv("ADFEM_ZCG", raising=False)
    monkeypatch.delenv("ADFEM_ZCG_PDL", raising=False)
    monkeypatch.setenv("ADFEM_ZCG_RING_REFILL", refill)
    if smax:
        monkeypatch.setenv("ADFEM_ZCG_SMAX", smax)
    else:
        monkeypatch.delenv("ADFEM_ZCG_SMAX", raising=False)
    monkeypatch.delenv("ADFEM_ZCG_RING", raising=False)
    plain = _ring_system(gpulib, 1000)
    monkeypatch.setenv("ADFEM_ZCG_RING", ring)
    ringed = _ring_system(gpulib, 1000)
    ip, ir = plain.solver_info(), ringed.solver_info()
    assert ip["banded"] == 1 and ip["ring_stages"] == 0
    assert ir["banded"] == 1 and ir["ring_stages"] == int(ring)
    assert ir["rows_per_block"] > 3 * 1024  # refills happen
    u0 = plain.solve(precision="mixed", rtol=RTOL_MIXED)
    s0 = plain.last_stats
    u1 = ringed.solve(precision="mixed", rtol=RTOL_MIXED)
    s1 = ringed.last_stats
    assert s0.status == 0 and s1.status == 0 and s0.relres <= 1e-10
    assert s1.iterations == s0.iterations and s1.updates == s0.updates
    assert np.array_equal(u1.cpu().numpy(), u0.cpu().numpy())


def test_dependent_launches_bit_identical(gpulib, monkeypatch):
    """Programmatic dependent launches of the banded iteration (the default) change only when
    a launch's blocks start: same iterations and bit-identical solution as plain launches."""
    monkeypatch.delenv("ADFEM_ZCG", raising=False)
    monkeypatch.delenv("ADFEM_ZCG_RING", raising=False)
    monkeypatch.delenv("ADFEM_ZCG_SMAX", raising=False)
    monkeypatch.setenv("ADFEM_ZCG_PDL", "0")
    plain = _ring_system(gpulib, 600)
    monkeypatch.delenv("ADFEM_ZCG_PDL", raising=False)
    dep = _ring_system(gpulib, 600)
    u0 = plain.solve(precision="mixed", rtol=RTOL_MIXED)
    u1 = dep.solve(precision="mixed", rtol=RTOL_MIXED)
    assert plain.last_stats.status == 0 and dep.last_stats.status == 0
    assert dep.last_stats.iterations == plain.last_stats.iterations
    assert np.array_equal(u1.cpu().numpy(), u0.cpu().numpy())


@pytest.mark.parametrize("smax", ["", "64"])
def test_elasticity_block_form_super_tiles(oracle, gpulib, monkeypatch, smax):
    """The interleaved 2-DOF (node-block Jacobi) banded variant with and without block ranges
    split into super-tiles (each with its own halo; the q^ stores deferred across tiles)."""
    import torch

    monkeypatch.delenv("ADFEM_ZCG", raising=False)
    if smax:
        monkeypatch.setenv("ADFEM_ZCG_SMAX", smax)
    else:
        monkeypatch.delenv("ADFEM_ZCG_SMAX", raising=False)
    coords, elems = synth.jittered_square(70, seed=8)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    E = 1e9 * np.exp(0.3 * synth.fourier_field(g[:, 0], g[:, 1], seed=2))
    nu = np.full(O.ngauss, 0.3)
    fx, fy = np.zeros(O.ngauss), np.full(O.ngauss, -1e6)
    left = synth.left_edge_nodes(coords)
    bd = np.concatenate([left + 1, left + 1 + O.ndof])
    B, r = oracle.dirichlet_csc(O.stiffness_csc(oracle.plane_strain(E, nu, 0)),
                                np.concatenate([O.source(fx), O.source(fy)]), bd, np.zeros(bd.size))
    S = gpulib.ElasticitySystem(gpulib.Mesh(coords, elems))
    S.set_dirichlet(bd)
    t = lambda a: torch.tensor(a, device="cuda")  # noqa: E731
    S.assemble(t(E), t(nu), t(fx), t(fy))
    info = S.solver_info()
    assert info["banded"] == 1
    if smax:
        assert info["rows_per_block"] > int(smax)  # several super-tiles per block
    u = S.solve(precision="mixed", rtol=RTOL_MIXED)
    assert S.last_stats.status == 0
    assert rel(u.cpu().numpy(), oracle.spsolve(B, r)) < ERR_BAR
