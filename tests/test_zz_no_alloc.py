"""The allocation-free solve entry point (adfem_csr_pcg_noalloc_d), through the C ABI.

It serves callers that cannot allocate device memory themselves (code running inside
another framework's memory pool, such as a TensorFlow/ADCME custom op or a CUDA.jl
task).  The test calls it twice in a row on the same system and compares both results
with the allocating entry point adfem_csc_solve (the GPU K\\F used everywhere else) and
with the oracle's direct solve (SuperLU), with the 1e-9 relative solution tolerance of
the other solver tests.  It also covers the exits other than convergence (max_iter, a
zero right-hand side, an oversized system, a capturing stream) and checks that a warmed-up
call leaves the device's free memory unchanged.  It lives in its own file, collected
last, and needs nothing from the other tests: it passes alone in a fresh process and
after the rest of the suite.
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
    B = sp.csr_matrix(B)
    B.sort_indices()
    return B, r


def _device_csr(B, rhs):
    import torch

    return (torch.tensor(B.indptr.astype(np.int32), device="cuda"),
            torch.tensor(B.indices.astype(np.int32), device="cuda"),
            torch.tensor(B.data, device="cuda"), torch.tensor(rhs, device="cuda"))


def _call(L, n, bufs, u, rtol, max_iter, stream=None):
    from adfem_gpu import _lib

    rp, ci, va, b = bufs
    it = ctypes.c_int(-1)
    rr = ctypes.c_double(-1.0)
    st = L.adfem_csr_pcg_noalloc_d(n, _lib.ptr(rp), _lib.ptr(ci), _lib.ptr(va), _lib.ptr(b), _lib.ptr(u), rtol,
                                   max_iter, ctypes.byref(it), ctypes.byref(rr), stream)
    return st, it.value, rr.value


def test_noalloc_matches_allocating_solve_twice(oracle, gpulib):
    import torch

    from adfem_gpu import _lib

    L = _lib.load()
    B, rhs = _system(oracle)
    n = B.shape[0]
    ref = gpulib.solve(B, rhs, precision="fp64", rtol=1e-13)
    direct = oracle.spsolve(B, rhs)
    bufs = _device_csr(B, rhs)
    for _ in range(2):  # two calls in a row share the static scratch
        u = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        st, it, rr = _call(L, n, bufs, u, 1e-13, 100000)
        assert st == 0, L.adfem_last_error().decode()
        assert it > 0 and rr <= 1e-13
        got = u.cpu().numpy()
        assert np.max(np.abs(got - ref)) <= 1e-9 * np.max(np.abs(ref))
        assert np.max(np.abs(got - direct)) <= 1e-9 * np.max(np.abs(direct))


def test_noalloc_other_exits(oracle, gpulib):
    import torch

    from adfem_gpu import _lib

    L = _lib.load()
    B, rhs = _system(oracle, m=16)
    n = B.shape[0]
    bufs = _device_csr(B, rhs)
    u = torch.zeros(n, dtype=torch.float64, device="cuda")
    # max_iter reached: not converged, exactly max_iter iterations
    st, it, rr = _call(L, n, bufs, u, 1e-13, 3)
    assert st == _lib.ERR_NOT_CONVERGED and it == 3 and rr > 0.0
    # zero right-hand side: converged at the start, u = 0, no iterations
    zb = (bufs[0], bufs[1], bufs[2], torch.zeros(n, dtype=torch.float64, device="cuda"))
    u.fill_(7.0)
    st, it, rr = _call(L, n, zb, u, 1e-13, 100)
    assert st == 0 and it == 0 and rr == 0.0
    assert torch.count_nonzero(u).item() == 0


def test_noalloc_rejects_oversized_system(gpulib):
    import torch

    from adfem_gpu import _lib

    L = _lib.load()
    # real (small) device buffers: the size check comes first and nothing is read, but no
    # call here ever hands the library an address that is not a device allocation
    rp = torch.zeros(4, dtype=torch.int32, device="cuda")
    ci = torch.zeros(4, dtype=torch.int32, device="cuda")
    va = torch.zeros(4, dtype=torch.float64, device="cuda")
    b = torch.zeros(4, dtype=torch.float64, device="cuda")
    u = torch.zeros(4, dtype=torch.float64, device="cuda")
    st, _, _ = _call(L, 131073, (rp, ci, va, b), u, 1e-10, 10)
    assert st == _lib.ERR_INVALID
    assert "131072" in L.adfem_last_error().decode()


def test_noalloc_refuses_capturing_stream_and_allocates_nothing(oracle, gpulib):
    import torch

    from adfem_gpu import _lib

    L = _lib.load()
    B, rhs = _system(oracle, m=24)
    n = B.shape[0]
    bufs = _device_csr(B, rhs)
    u = torch.zeros(n, dtype=torch.float64, device="cuda")
    assert _call(L, n, bufs, u, 1e-12, 100000)[0] == 0  # warm-up: scratch address looked up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert _call(L, n, bufs, u, 1e-12, 100000)[0] == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0  # no device allocation by the calls
    # a capturing stream is refused before anything is enqueued; the capture stays valid
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    x = torch.zeros(8, device="cuda")
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        x.add_(1.0)
        st, _, _ = _call(L, n, bufs, u, 1e-12, 100000, stream=ctypes.c_void_p(s.cuda_stream))
        x.add_(1.0)
    assert st == _lib.ERR_UNSUPPORTED
    assert "captured" in L.adfem_last_error().decode()
    g.replay()  # (capturing records the two adds without running them)
    torch.cuda.synchronize()
    assert float(x[0]) == 2.0
