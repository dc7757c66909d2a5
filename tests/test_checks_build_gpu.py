"""The debug build (-DADFEM_CHECKS) through the solver paths, and a bad CSR column.

In the debug build the kernels check every index they compute before using it (matrix
columns of the SpMV and residual gathers, positions in the banded shared-memory window,
row slots of the assembly) and record the first failed check instead of faulting
(checks.cuh).  This test builds that variant, runs the solver paths through it in a child
process -- the banded and scaled mixed iterations, both FP64 iterations, elasticity, the
adjoint and K\\F -- and expects results within the usual bars and no failed check.  A column
index outside [0, n) handed to the allocation-free entry (the one entry that takes device
CSR arrays) is refused with a status before any gather uses it.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import os, sys
import numpy as np
sys.path.insert(0, "adfem.jl_gb300"); sys.path.insert(0, "oracle")
from adfem_gpu import _lib
_lib.LIB_PATH = sys.argv[1]
import torch
import adfem_gpu as A
import oracle as O
from adfem_gpu import synth

L = _lib.load()
assert L.adfem_debug_check_code() == 0
def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
coords, elems = synth.jittered_square(48, seed=0)
OM = O.OracleMesh(coords, elems)
g = OM.gauss_nodes()
G = synth.fourier_field(g[:, 0], g[:, 1], seed=1)
kappa = 1 + np.exp(synth.contrast_sigma(G, 1e3) * G)
f = 1e5 * (g[:, 0] + g[:, 1])
bd = OM.bcnode()
B, r = O.dirichlet_csc(OM.laplace_csc(kappa), OM.source(f), bd, np.zeros(bd.size))
u0 = O.spsolve(B, r)
for env in ({}, {"ADFEM_ZCG": "0"}, {"ADFEM_ZCG64": "1"}):
    for k in ("ADFEM_ZCG", "ADFEM_ZCG64"):
        os.environ.pop(k, None)
    os.environ.update(env)
    S = A.PoissonSystem(A.Mesh(coords, elems))
    S.set_dirichlet(bd)
    S.assemble(torch.tensor(kappa, device="cuda"), torch.tensor(f, device="cuda"))
    for prec, rtol in (("mixed", 1e-11), ("fp64", 1e-12)):
        u = S.solve(precision=prec, rtol=rtol)
        assert rel(u.cpu().numpy(), u0) < 1e-9, (env, prec)
    lam = S.adjoint(u.clone(), precision="mixed", rtol=1e-11)
    S.grad_kappa(u, lam)
    code = L.adfem_debug_check_code()
    assert code == 0, (env, code)
for k in ("ADFEM_ZCG", "ADFEM_ZCG64"):
    os.environ.pop(k, None)
x = A.solve(B, r, precision="mixed", rtol=1e-11)
assert rel(x, u0) < 1e-9
M = A.Mesh(coords, elems)
ng = A.get_ngauss(M)
gd = torch.tensor(A.gauss_nodes(M), device="cuda")
E = (1e9 * torch.exp(0.3 * synth.fourier_field(gd[:, 0], gd[:, 1], seed=2))).contiguous()
nu = torch.full((ng,), 0.3, dtype=torch.float64, device="cuda")
fx = torch.zeros(ng, dtype=torch.float64, device="cuda")
fy = torch.full((ng,), -1e6, dtype=torch.float64, device="cuda")
left = synth.left_edge_nodes(coords) + 1
SE = A.ElasticitySystem(M)
SE.set_dirichlet(np.concatenate([left, left + M.nnode]))
SE.assemble(E, nu, fx, fy)
ue = SE.solve(precision="mixed", rtol=1e-10)
ue64 = SE.solve(precision="fp64", rtol=1e-11)
assert rel(ue.cpu().numpy(), ue64.cpu().numpy()) < 1e-9
assert L.adfem_debug_check_code() == 0
torch.cuda.synchronize()
print("checks build ok")
'''


def test_checks_build_runs_the_solver_paths_without_a_failed_check(gpulib):
    import build as B

    lib = B.build(checks=True)
    r = subprocess.run([sys.executable, "-c", SCRIPT, lib], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0 and "checks build ok" in r.stdout, (r.stdout[-2000:], r.stderr[-4000:])


def test_release_build_reports_no_check(gpulib):
    from adfem_gpu import _lib

    assert _lib.load().adfem_debug_check_code() == 0


def test_bad_csr_column_is_refused_before_any_gather(oracle, gpulib):
    import ctypes

    import scipy.sparse as sp
    import torch

    from adfem_gpu import _lib, synth

    coords, elems = synth.jittered_square(8, seed=1)
    O = oracle.OracleMesh(coords, elems)
    bd = O.bcnode()
    Bm, rhs = oracle.dirichlet_csc(O.laplace_csc(np.ones(O.ngauss)), O.source(np.ones(O.ngauss)), bd,
                                   np.zeros(bd.size))
    Bm = sp.csr_matrix(Bm)
    n = Bm.shape[0]
    L = _lib.load()
    for bad in (n, n + 7, -1):
        ci = Bm.indices.astype(np.int32).copy()
        ci[len(ci) // 2] = bad
        rp = torch.tensor(Bm.indptr.astype(np.int32), device="cuda")
        cd = torch.tensor(ci, device="cuda")
        va = torch.tensor(Bm.data, device="cuda")
        b = torch.tensor(rhs, device="cuda")
        u = torch.zeros(n, dtype=torch.float64, device="cuda")
        it = ctypes.c_int(-1)
        rr = ctypes.c_double(-1.0)
        st = L.adfem_csr_pcg_noalloc_d(n, _lib.ptr(rp), _lib.ptr(cd), _lib.ptr(va), _lib.ptr(b), _lib.ptr(u), 1e-10,
                                       1000, ctypes.byref(it), ctypes.byref(rr), None)
        assert st == _lib.ERR_INVALID and "column" in L.adfem_last_error().decode()
        assert it.value == 0
    torch.cuda.synchronize()  # the context is intact
