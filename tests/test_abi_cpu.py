"""CPU checks of the drop-in boundary: the library builds, loads and exports every
entry point include/adfem_gpu.h declares; the Python mirror binds them all.
(No compute calls: this environment has no GPU.)"""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "adfem_gpu.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"ADFEM_API\s+[\w\s\*]+?\b(\w+)\s*\(", txt)))


def test_header_declares_reference_symbols():
    syms = declared_symbols()
    for s in ("init_nnfem_mesh", "mfem_get_ngauss", "mfem_get_gauss", "mfem_get_gauss_weights", "mfem_get_area",
              "mfem_get_elem_ndof", "mfem_get_ndof", "mfem_get_connectivity", "mfem_get_element_to_vertices",
              "FemLaplaceScalar_forward_Julia", "FemSourceScalar_forward_Julia",
              "ComputeFemStiffnessMatrixMfem_forward_Julia", "FemToGaussPointsMfem_Julia",
              "DofToGaussPointsMfem_forward_Julia"):
        assert s in syms, s


def test_library_exports_every_declared_symbol(gpulib):
    from adfem_gpu import _lib

    L = _lib.load()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    # every declared symbol is bound by the Python mirror with a signature
    unbound = [s for s in declared_symbols() if s not in _lib.SIGNATURES]
    assert not unbound, unbound
    assert L.adfem_version().decode().startswith("adfem_gpu")
    assert L.adfem_status_string(4).decode() == "not converged"


def test_errors_without_gpu_are_reported_not_crashing(gpulib):
    """With no current mesh the legacy getters record ADFEM_ERR_NO_MESH (no device needed)."""
    from adfem_gpu import _lib

    L = _lib.load()
    assert L.mfem_get_ngauss() == 0
    assert "no current mesh" in L.adfem_last_error().decode()
    o = _lib.SolverOpts()
    L.adfem_solver_opts_default(ctypes.byref(o))
    assert o.rtol == 1e-12 and o.precision == 0 and o.chunk == 32


def test_invalid_arguments_rejected_on_host(gpulib):
    from adfem_gpu import _lib

    L = _lib.load()
    h = ctypes.c_void_p()
    xyz = np.zeros(9)
    el = np.array([0, 1, 5], np.int32)  # vertex 5 out of range
    st = L.adfem_mesh_create(_lib.ptr(xyz), 3, _lib.ptr(el), 1, 1, ctypes.byref(h))
    assert st == _lib.ERR_INVALID
    st = L.adfem_mesh_create(_lib.ptr(xyz), 3, _lib.ptr(el), 1, 2, ctypes.byref(h))
    assert st == _lib.ERR_INVALID  # P2 meshes check their vertices the same way
    st = L.adfem_mesh_create(_lib.ptr(xyz), 3, _lib.ptr(el), 1, 3, ctypes.byref(h))
    assert st == _lib.ERR_UNSUPPORTED
    cnt = ctypes.c_longlong()
    cp = np.array([1, 2, 3], np.int64)
    rv = np.array([1, 2], np.int64)
    nz = np.ones(2)
    bd = np.array([3], np.int64)  # out of range for n = 2
    st = L.adfem_dirichlet_csc(2, _lib.ptr(cp), _lib.ptr(rv), _lib.ptr(nz), _lib.ptr(nz), _lib.ptr(bd), 1,
                               _lib.ptr(nz), 0, None, None, None, ctypes.byref(cnt), None)
    assert st == _lib.ERR_INVALID
    bd = np.array([1, 1], np.int64)  # duplicate
    st = L.adfem_dirichlet_csc(2, _lib.ptr(cp), _lib.ptr(rv), _lib.ptr(nz), _lib.ptr(nz), _lib.ptr(bd), 2,
                               _lib.ptr(nz), 0, None, None, None, ctypes.byref(cnt), None)
    assert st == _lib.ERR_INVALID


def test_csc_solve_refuses_non_symmetric_matrix_on_host(gpulib):
    """K\\F runs CG, which is only right for a symmetric K: a non-symmetric matrix (values,
    or a structural entry without its mirror) is refused before any device work, with
    ADFEM_ERR_UNSUPPORTED and a message, instead of being solved as its transpose."""
    import scipy.sparse as sp

    import adfem_gpu as A

    dense = np.array([[4.0, -1.0, 0.0], [-1.0, 4.0, -1.0], [0.0, -1.0, 4.0]])
    for bad in (dense + np.array([[0, 0.5, 0], [0, 0, 0], [0, 0, 0]]),   # values differ
                dense + np.array([[0, 0, 0.25], [0, 0, 0], [0, 0, 0]])):  # (1,3) without (3,1)
        with pytest.raises(A.AdFemError) as ei:
            A.solve(sp.csc_matrix(bad), np.ones(3))
        assert ei.value.status == _unsupported()
        assert "symmetric" in str(ei.value)


def _unsupported():
    from adfem_gpu import _lib

    return _lib.ERR_UNSUPPORTED


def test_synthetic_generator_properties():
    from adfem_gpu import synth

    c, e = synth.jittered_square(10, seed=0)
    assert c.shape == (121, 2) and e.shape == (200, 3) and e.min() == 1 and e.max() == 121
    c2, _ = synth.jittered_square(10, seed=0)
    np.testing.assert_array_equal(c, c2)
    b = np.isclose(c[:, 0], 0) | np.isclose(c[:, 0], 1) | np.isclose(c[:, 1], 0) | np.isclose(c[:, 1], 1)
    assert b.sum() == 40
    h = 0.1
    grid = np.stack(np.meshgrid(np.arange(11) * h, np.arange(11) * h), -1).reshape(-1, 2)
    assert np.max(np.abs(c - grid)) <= 0.2 * h + 1e-15
    g = synth.fourier_field(np.random.default_rng(1).random(20000), np.random.default_rng(2).random(20000), seed=1)
    assert abs(g.var() - 1) < 0.3
    s = synth.contrast_sigma(g, 1e3)
    k = synth.lognormal_kappa(g, s)
    assert abs(k.max() / k.min() - 1e3) < 1e-6 * 1e3
    obs = synth.observation_nodes(10000, seed=1)
    assert obs.size == 100 and np.unique(obs).size == 100
