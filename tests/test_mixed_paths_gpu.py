"""The two mixed-precision iterations of the CG solver against the direct solve.

* banded path (one kernel per iteration, the band of each block's rows held in shared
  memory), chosen automatically when the band fits;
* scaled two-kernel path, the fallback for wide bands (forced with ADFEM_ZCG=0).

The path that ran is identified by the launch count per iteration (banded: one launch
per iteration plus the replacement checks; scaled: two plus the checks).  Bars as in
test_solver_gpu.py: 1e-9 relative (max norm) to SuperLU on the oracle's matrices.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from adfem_gpu import synth

pytestmark = pytest.mark.gpu
RTOL_MIXED = 1e-11


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
    assert rel(u, u0) < 1e-9
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
    assert rel(u1, u64) < 1e-9
    # fixed grid, fixed reduction order, halos recomputed bit-identically
    assert s1.iterations == s2.iterations
    assert np.array_equal(u1, u2)
    # each block's range split into super-tiles of 512 rows (each with its own halo)
    monkeypatch.setenv("ADFEM_ZCG_SMAX", "512")
    u3, s3 = gpulib.solve(B, r, precision="mixed", rtol=RTOL_MIXED, return_stats=True)
    assert s3.status == 0 and launches_per_iter(s3) < 1.9
    assert rel(u3, u64) < 1e-9


@pytest.mark.parametrize("m,banded", [(40, 1), (80, 0)])
def test_randomly_renumbered_mesh(oracle, gpulib, monkeypatch, m, banded):
    # a random node numbering spreads the band over the whole matrix: at 1681 DOF a
    # super-tile still holds every column its rows need; at 6561 DOF the band exceeds
    # what shared memory can hold and the scaled two-kernel path takes over
    import torch

    monkeypatch.delenv("ADFEM_ZCG", raising=False)
    coords, elems = synth.jittered_square(m, seed=3)
    perm = np.random.default_rng(5).permutation(coords.shape[0])  # new id of old node i: inv[i]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.size)
    coords_p = coords[perm]
    elems_p = inv[elems - 1] + 1
    O = oracle.OracleMesh(coords_p, elems_p)
    g = O.gauss_nodes()
    kappa, f = synth.poisson_c1_fields(g[:, 0], g[:, 1])
    bd = O.bcnode()
    B, r = oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(f), bd, np.zeros(bd.size))
    S = gpulib.PoissonSystem(gpulib.Mesh(coords_p, elems_p))
    S.set_dirichlet(bd)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    info = S.solver_info()
    assert info["banded"] == banded, info
    u = S.solve(precision="mixed", rtol=RTOL_MIXED)
    assert S.last_stats.status == 0
    assert rel(u.cpu().numpy(), oracle.spsolve(B, r)) < 1e-9


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
    assert rel(u.cpu().numpy(), oracle.spsolve(B, r)) < 1e-9
