"""The allocation-free solve entry point (adfem_csr_pcg_noalloc_d), through the C ABI.

It serves callers that cannot allocate device memory themselves (code running inside
another framework's memory pool, such as a TensorFlow/ADCME custom op or a CUDA.jl
task).  The test calls it twice in a row on the same system and compares both results
with the allocating entry point adfem_csc_solve (the GPU K\\F used everywhere else),
with the same 1e-9 relative solution tolerance as the other solver tests.  It lives in
its own file, collected last, and needs nothing from the other tests: it passes alone in
a fresh process and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


def _system(oracle, m=40):
    from adfem_gpu import synth

    coords, elems = synth.jittered_square(m, seed=7)
    O = oracle.OracleMesh(coords, elems)
    g = O.gauss_nodes()
    kappa, f = synth.poisson_c1_fields(g[:, 0], g[:, 1])
    bd = O.bcnode()
    B, r = oracle.dirichlet_csc(O.laplace_csc(kappa), O.source(f), bd, np.zeros(bd.size))
    return sp.csr_matrix(B), r


def test_noalloc_matches_allocating_solve_twice(oracle, gpulib):
    import torch

    from adfem_gpu import _lib

    L = _lib.load()
    B, rhs = _system(oracle)
    B.sort_indices()
    n = B.shape[0]
    ref = gpulib.solve(B, rhs, precision="fp64", rtol=1e-13)
    rp = torch.tensor(B.indptr.astype(np.int32), device="cuda")
    ci = torch.tensor(B.indices.astype(np.int32), device="cuda")
    va = torch.tensor(B.data, device="cuda")
    b = torch.tensor(rhs, device="cuda")
    for _ in range(2):  # two calls in a row share the static scratch
        u = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        it = ctypes.c_int()
        rr = ctypes.c_double()
        st = L.adfem_csr_pcg_noalloc_d(n, _lib.ptr(rp), _lib.ptr(ci), _lib.ptr(va), _lib.ptr(b), _lib.ptr(u), 1e-13,
                                       100000, ctypes.byref(it), ctypes.byref(rr), None)
        assert st == 0, L.adfem_last_error().decode()
        assert it.value > 0 and rr.value <= 1e-13
        got = u.cpu().numpy()
        assert np.max(np.abs(got - ref)) <= 1e-9 * np.max(np.abs(ref))


def test_noalloc_rejects_oversized_system(gpulib):
    from adfem_gpu import _lib

    L = _lib.load()
    dummy = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    st = L.adfem_csr_pcg_noalloc_d(131073, dummy, dummy, dummy, dummy, dummy, 1e-10, 10, None, None, None)
    assert st == _lib.ERR_INVALID
    assert "131072" in L.adfem_last_error().decode()
