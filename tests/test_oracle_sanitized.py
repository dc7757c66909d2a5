"""The oracle under AddressSanitizer and UndefinedBehaviorSanitizer (CPU).

The oracle is the parity yardstick, so an out-of-bounds read or an undefined shift in it
would make every comparison suspect.  This test builds oracle/fem_oracle.c with
-fsanitize=address,undefined (every finding aborts) and runs each restated routine on
small meshes, P1 and P2, in a child process with the sanitizer runtime preloaded.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import ctypes, os, sys
import numpy as np
sys.path.insert(0, "oracle"); sys.path.insert(0, "adfem.jl_gb300")
import oracle as O
from adfem_gpu import synth

assert O.lib()._name == os.environ["ADFEM_ORACLE_LIB"]  # the instrumented build is the one loaded
assert hasattr(ctypes.CDLL(None), "__asan_init")          # with the sanitizer runtime in the process
rng = np.random.default_rng(0)
coords, elems = synth.jittered_square(7, seed=1)
M = O.OracleMesh(coords, elems)
g = M.gauss_nodes()
M.edges()
bd = M.bcnode()
idx, vv = M.laplace_coo(1 + rng.random(M.ngauss))
M.laplace_coo_backward(rng.standard_normal(vv.size))
K = O.coo_to_csc(idx, vv, M.ndof)
K2 = O.coo_to_csc_sorted(idx, vv, M.ndof)
assert np.array_equal(K.data, K2.data)
F = M.source(rng.random(M.ngauss))
M.source_backward(rng.standard_normal(M.ndof))
D = O.plane_strain(1 + rng.random(M.ngauss), np.full(M.ngauss, 0.3))
O.plane_strain_backward(rng.standard_normal(D.size), 1 + rng.random(M.ngauss), np.full(M.ngauss, 0.3))
si, sv = M.stiffness_coo(D.reshape(-1))
M.stiffness_coo_backward(rng.standard_normal(sv.size))
oi, ov, orhs = O.dirichlet_coo(idx, vv, np.r_[bd, bd[:3]], F, np.zeros(bd.size + 3), M.ndof)
O.dirichlet_coo_backward(rng.standard_normal(ov.size), rng.standard_normal(M.ndof), idx, vv, bd, np.zeros(bd.size),
                         M.ndof)
B, r = O.dirichlet_csc(K, F, bd, np.ones(bd.size))
O.dirichlet_csc(K, F, bd, np.ones(bd.size), keep_zeros=True)
x, it, rr = O.pcg(B, r, rtol=1e-10, threads=2)
O.residual_dd(B, x, r)
for deg in (1, 2):
    Sp = O.OracleSpace(coords, elems, deg)
    k = 1 + rng.random(Sp.ngauss)
    Sp.laplace_csc(k); Sp.mass_csc(k); Sp.source(k)
    Sp.laplace_coo_backward(rng.standard_normal(Sp.laplace_coo(k)[1].size))
    Sp.mass_coo_backward(rng.standard_normal(Sp.mass_coo(k)[1].size))
    Sp.source_backward(rng.standard_normal(Sp.ndof))
    Ds = np.tile(np.array([2.0, 1.0, 0.0, 1.0, 2.0, 0.0, 0.0, 0.0, 0.5]), Sp.ngauss)
    Sp.stiffness_csc(Ds)
    Sp.stiffness_coo_backward(rng.standard_normal(Sp.stiffness_coo(Ds)[1].size))
    u = rng.standard_normal(Sp.ndof)
    Sp.dof_to_gauss(u); Sp.dof_to_gauss_backward(rng.standard_normal(Sp.ngauss))
    Sp.fem_to_gauss(u[:Sp.nnode]); Sp.fem_to_gauss_backward(rng.standard_normal(Sp.ngauss))
    Sp.pcl_laplace_jacobian(); Sp.bcnode()
ii, _ = M.laplace_coo(np.ones(M.ngauss))
O.pcl_dirichlet(ii[:50] + 1, bd, M.ndof)
print("sanitized oracle ok")
'''


def test_oracle_under_address_and_ub_sanitizers(oracle):
    try:
        asan = subprocess.check_output(["gcc", "-print-file-name=libasan.so"], text=True).strip()
        ubsan = subprocess.check_output(["gcc", "-print-file-name=libubsan.so"], text=True).strip()
    except (OSError, subprocess.CalledProcessError):
        pytest.skip("gcc sanitizer runtimes not available")
    if not (os.path.isabs(asan) and os.path.exists(asan)):
        pytest.skip("libasan not available")
    lib = oracle.build_sanitized()
    env = dict(os.environ, ADFEM_ORACLE_LIB=lib, LD_PRELOAD=asan + ((":" + ubsan) if os.path.exists(ubsan) else ""),
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=1", UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    r = subprocess.run([sys.executable, "-c", SCRIPT], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "sanitized oracle ok" in r.stdout, (r.stdout[-2000:], r.stderr[-4000:])
