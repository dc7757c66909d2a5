"""Failure handling without a GPU fault: injected device-allocation failures.

adfem_debug_fail_alloc(k) makes the k-th following device allocation of the library fail
as if cudaMalloc had returned cudaErrorMemoryAllocation (nothing reaches the driver).  The
test walks k over every allocation a small Poisson pipeline makes (mesh, resident system,
assembly, mixed and FP64 solves, adjoint, gradient, Array-arm matrix, K\\F): each run either
completes with the reference results or fails with ADFEM_ERR_NOMEM (the status every
entry reports for cudaErrorMemoryAllocation) and the injected message -- never a crash or a wrong answer -- and after each failure the same pipeline runs
again to the same bits.
"""
import numpy as np
import pytest
import torch

from adfem_gpu import synth

pytestmark = pytest.mark.gpu


def _case(oracle, m=12):
    coords, elems = synth.jittered_square(m, seed=4)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    kappa, f = synth.poisson_c1_fields(g[:, 0], g[:, 1])
    return coords, elems, kappa, f, O.bcnode()


def _pipeline(A, coords, elems, kappa, f, bd):
    mesh = A.Mesh(coords, elems)
    S = A.PoissonSystem(mesh)
    S.set_dirichlet(bd)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    u = S.solve(precision="mixed", rtol=1e-11)
    u64 = S.solve(precision="fp64", rtol=1e-12)
    gu = torch.zeros_like(u)
    gu[::5] = 1.0
    lam = S.adjoint(gu, precision="fp64", rtol=1e-12)
    gk = S.grad_kappa(u64, lam)
    K = A.compute_fem_laplace_matrix1(kappa, mesh)
    F = A.compute_fem_source_term1(f, mesh)
    B, r = A.impose_Dirichlet_boundary_conditions(K, F, bd, np.zeros(bd.size))
    x = A.solve(B, r, rtol=1e-12)
    torch.cuda.synchronize()
    return [t.cpu().numpy() if hasattr(t, "cpu") else np.asarray(t) for t in (u, u64, lam, gk, K.data, x)]


def test_every_injected_allocation_failure_is_a_status(oracle, gpulib):
    from adfem_gpu import _lib

    L = _lib.load()
    case = _case(oracle)
    ref = _pipeline(gpulib, *case)
    failures = 0
    completed_at = None
    try:
        for k in range(400):
            L.adfem_debug_fail_alloc(k)
            try:
                got = _pipeline(gpulib, *case)
            except gpulib.AdFemError as e:
                assert e.status == _lib.ERR_NOMEM, str(e)
                assert "injected" in str(e), str(e)
                failures += 1
            else:
                # k beyond the pipeline's allocations: nothing failed, same results
                completed_at = k
                for a, b in zip(got, ref):
                    assert np.array_equal(a, b)
                break
            finally:
                L.adfem_debug_fail_alloc(-1)
            # the library stays usable after the failure: the same bits again
            again = _pipeline(gpulib, *case)
            for a, b in zip(again, ref):
                assert np.array_equal(a, b)
    finally:
        L.adfem_debug_fail_alloc(-1)
    assert completed_at is not None and failures == completed_at and failures >= 20, (failures, completed_at)
