"""The two FP64 iterations of the CG solver against the direct solve and each other.

* banded FP64 path (one kernel per iteration: the mixed iteration's layout and fusion with
  FP64 values, vectors and dot products on the Jacobi-scaled operator), selected with
  ADFEM_ZCG64=1 when the system is created (the like-for-like FP64 counterpart of the
  mixed kernel; slower on GB300, where FP64 instructions bound both FP64 iterations);
* three-kernel FP64 path (SpMV, update, direction), the default.

The path that ran is identified by solver_info and by the launches per iteration.  Bars:
1e-10 relative (max norm) to SuperLU on the oracle's matrices where that fits, else to the
other FP64 path at rtol 1e-12.
"""
import numpy as np
import pytest
import torch

from adfem_gpu import synth

pytestmark = pytest.mark.gpu
ERR_BAR = 1e-10


def rel(a, b):
    a = a.cpu().numpy() if hasattr(a, "cpu") else np.asarray(a)
    b = b.cpu().numpy() if hasattr(b, "cpu") else np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def poisson_system(gpulib, oracle, m, contrast=1e3, seed=0):
    coords, elems = synth.jittered_square(m, seed=seed)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    G = synth.fourier_field(g[:, 0], g[:, 1], seed=1)
    kappa = 1 + np.exp(synth.contrast_sigma(G, contrast) * G)
    f = 1e5 * (g[:, 0] + g[:, 1])
    bd = O.bcnode()
    S = gpulib.PoissonSystem(gpulib.Mesh(coords, elems))
    S.set_dirichlet(bd)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    return S, O, kappa, f, bd


def test_default_fp64_path_is_three_kernel(oracle, gpulib, monkeypatch):
    monkeypatch.delenv("ADFEM_ZCG64", raising=False)
    S, *_ = poisson_system(gpulib, oracle, 32)
    assert S.solver_info()["banded_fp64"] == 0


@pytest.mark.parametrize("banded", ["1", "0"])
def test_fp64_paths_match_direct(oracle, gpulib, monkeypatch, banded):
    monkeypatch.setenv("ADFEM_ZCG64", banded)
    monkeypatch.delenv("ADFEM_ZCG_SMAX", raising=False)
    S, O, kappa, f, bd = poisson_system(gpulib, oracle, 64)
    assert S.solver_info()["banded_fp64"] == int(banded)
    B, r = oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(f), bd, np.zeros(bd.size))
    u0 = oracle.spsolve(B, r)
    u = S.solve(precision="fp64", rtol=1e-12)
    st = S.last_stats
    assert st.status == 0 and st.relres <= 1e-12
    assert rel(u, u0) < ERR_BAR
    lpi = st.launches / max(st.iterations, 1)
    assert (lpi < 1.9) if banded == "1" else (lpi > 3.0), lpi


def test_fp64_banded_super_tiles_deterministic(oracle, gpulib, monkeypatch):
    """361k DOF: halos across blocks, the FP64 window split into super-tiles (and forced
    into many more with ADFEM_ZCG_SMAX), bit-identical repeats, the same answer as the
    three-kernel FP64 path."""
    monkeypatch.setenv("ADFEM_ZCG64", "1")
    monkeypatch.delenv("ADFEM_ZCG_SMAX", raising=False)
    S, O, kappa, f, bd = poisson_system(gpulib, oracle, 600)
    info = S.solver_info()
    assert info["banded_fp64"] == 1 and info["fp64_tile_rows"] > 0, info
    u1 = S.solve(precision="fp64", rtol=1e-12)
    s1 = S.last_stats
    u2 = S.solve(precision="fp64", rtol=1e-12)
    assert s1.status == 0 and S.last_stats.iterations == s1.iterations
    assert torch.equal(u1, u2)
    monkeypatch.setenv("ADFEM_ZCG64", "0")
    S0, *_ = poisson_system(gpulib, oracle, 600)
    assert S0.solver_info()["banded_fp64"] == 0
    u0 = S0.solve(precision="fp64", rtol=1e-12)
    assert rel(u1, u0) < ERR_BAR
    # iteration counts agree within 8% at rtol 1e-10: the one-kernel form takes beta from the
    # one-step estimate rho_{k+1} = rho_k - 2 a r.q + a^2 q.q (the only way to fuse the
    # iteration).  (At 1e-12 both stop near the attainable accuracy of this system, where the
    # count depends on the last bits of the operator.)
    S.solve(precision="fp64", rtol=1e-10)
    n1 = S.last_stats.iterations
    S0.solve(precision="fp64", rtol=1e-10)
    n0 = S0.last_stats.iterations
    assert abs(n1 - n0) <= 0.08 * n0, (n1, n0)
    monkeypatch.setenv("ADFEM_ZCG64", "1")
    monkeypatch.setenv("ADFEM_ZCG_SMAX", "512")
    S3, *_ = poisson_system(gpulib, oracle, 600)
    assert S3.solver_info()["fp64_tile_rows"] == 512
    u3 = S3.solve(precision="fp64", rtol=1e-12)
    assert S3.last_stats.status == 0 and rel(u3, u0) < ERR_BAR


def test_fp64_banded_floor_and_adjoint(oracle, gpulib, monkeypatch):
    """An unattainable rtol ends at the FP64 floor with status OK; the adjoint through the
    banded FP64 path gives the gradient of the three-kernel path."""
    monkeypatch.setenv("ADFEM_ZCG64", "1")
    monkeypatch.delenv("ADFEM_ZCG_SMAX", raising=False)
    S, O, kappa, f, bd = poisson_system(gpulib, oracle, 96)
    u = S.solve(precision="fp64", rtol=1e-18, max_iter=200000)
    st = S.last_stats
    assert st.status == 0 and 1e-18 < st.relres < 1e-11 and st.iterations < 50000
    obs = torch.tensor(synth.observation_nodes(O.ndof, seed=3, frac=0.05), device="cuda")
    gu = torch.zeros_like(u)
    gu[obs] = 1.0
    lam = S.adjoint(gu, precision="fp64", rtol=1e-12)
    gk = S.grad_kappa(u, lam)
    monkeypatch.setenv("ADFEM_ZCG64", "0")
    S0, *_ = poisson_system(gpulib, oracle, 96)
    u0 = S0.solve(precision="fp64", rtol=1e-12)
    lam0 = S0.adjoint(gu, precision="fp64", rtol=1e-12)
    assert rel(lam, lam0) < ERR_BAR
    assert rel(gk, S0.grad_kappa(u0, lam0)) < 1e-9


def test_fp64_banded_elasticity(oracle, gpulib, monkeypatch):
    """The 16-wide variant (interleaved 2-DOF elasticity operator, point-Jacobi scaled)."""
    monkeypatch.delenv("ADFEM_ZCG_SMAX", raising=False)
    coords, elems = synth.jittered_square(48, seed=2)
    M = gpulib.Mesh(coords, elems)
    ng = gpulib.get_ngauss(M)
    g = torch.tensor(gpulib.gauss_nodes(M), device="cuda")
    E = (1e9 * torch.exp(0.3 * synth.fourier_field(g[:, 0], g[:, 1], seed=2))).contiguous()
    nu = torch.full((ng,), 0.3, dtype=torch.float64, device="cuda")
    fx = torch.zeros(ng, dtype=torch.float64, device="cuda")
    fy = torch.full((ng,), -1e6, dtype=torch.float64, device="cuda")
    left = synth.left_edge_nodes(coords) + 1
    out = {}
    for banded in ("1", "0"):
        monkeypatch.setenv("ADFEM_ZCG64", banded)
        S = gpulib.ElasticitySystem(M)
        S.set_dirichlet(np.concatenate([left, left + M.nnode]))
        S.assemble(E, nu, fx, fy)
        assert S.solver_info()["banded_fp64"] == int(banded)
        out[banded] = S.solve(precision="fp64", rtol=1e-9)
        assert S.last_stats.status == 0 and S.last_stats.relres <= 1e-9
        # rtol 1e-12 sits within 10x below this operator's FP64 floor: the solve must still end
        # (converged or at the floor), not run to max_iter
        S.solve(precision="fp64", rtol=1e-12, max_iter=20000)
        assert S.last_stats.status == 0 and S.last_stats.iterations < 5000
    assert rel(out["1"], out["0"]) < ERR_BAR
