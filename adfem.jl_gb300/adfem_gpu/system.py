"""Resident solver systems and device-pointer operators (torch tensors as buffers).

A system keeps one mesh's assembled, Dirichlet-imposed operator on the GPU
(sliced-ELL, FP64 plus a Jacobi-scaled FP32 copy) together with its right-hand
side and CG work vectors, so that forward solves, adjoint solves and gradients
reuse them.  torch is only used for device memory and streams; every kernel is
in libadfem_gpu.so.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import SolverStats, check, ptr, stream_ptr


def _torch():
    import torch

    return torch


def _dev(t, n=None, what="tensor"):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous():
        raise _lib.AdFemError(_lib.ERR_INVALID, "%s must be a contiguous float64 CUDA tensor" % what)
    if n is not None and t.numel() != n:
        raise _lib.AdFemError(_lib.ERR_INVALID, "%s must have %d entries (got %d)" % (what, n, t.numel()))
    return t


def _cur_stream():
    return stream_ptr(_torch().cuda.current_stream())


class _System:
    kind = None

    def __init__(self, mesh):
        from . import Mesh  # noqa: F401

        self.mesh = mesh
        h = ctypes.c_void_p()
        check(_lib.load().adfem_system_create(mesh.handle, self.kind, ctypes.byref(h)), "system_create")
        self._h = h
        self.ndof = mesh.ndof * (2 if self.kind == _lib.SYS_ELASTICITY else 1)
        self.last_stats = None

    def close(self):
        if getattr(self, "_h", None) is not None and _lib._LIB is not None:
            _lib._LIB.adfem_system_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_dirichlet(self, bd, bdval=None):
        """bd: 1-based DOF ids (reference ordering); bdval: values (default zero)."""
        bd = np.ascontiguousarray(bd, dtype=np.int64).ravel()
        bv = None if bdval is None else np.ascontiguousarray(bdval, dtype=np.float64).ravel()
        if bv is not None and bv.size != bd.size:
            raise _lib.AdFemError(_lib.ERR_INVALID, "bd and bdval lengths differ")
        check(_lib.load().adfem_system_set_dirichlet(self._h, ptr(bd), bd.size, ptr(bv)), "set_dirichlet")

    def solve(self, u=None, precision="fp64", rtol=1e-12, max_iter=200000, ru_delta=0.1, chunk=32, warm=False):
        from . import solver_opts

        torch = _torch()
        if u is None:
            u = torch.zeros(self.ndof, dtype=torch.float64, device="cuda")
        _dev(u, self.ndof, "u")
        o = solver_opts(precision, rtol, max_iter, ru_delta, chunk, warm)
        st = SolverStats()
        self.last_stats = st  # (filled in also when the solve reports an error status)
        check(_lib.load().adfem_system_solve_d(self._h, ptr(u), ctypes.byref(o), ctypes.byref(st), _cur_stream()),
              "system_solve")
        return u

    def adjoint(self, g, lam=None, precision="fp64", rtol=1e-12, max_iter=200000, ru_delta=0.1, chunk=32):
        from . import solver_opts

        torch = _torch()
        _dev(g, self.ndof, "g")
        if lam is None:
            lam = torch.zeros(self.ndof, dtype=torch.float64, device="cuda")
        o = solver_opts(precision, rtol, max_iter, ru_delta, chunk, False)
        st = SolverStats()
        self.last_stats = st
        check(_lib.load().adfem_system_adjoint_d(self._h, ptr(g), ptr(lam), ctypes.byref(o), ctypes.byref(st),
                                                 _cur_stream()), "system_adjoint")
        return lam

    def apply(self, x):
        torch = _torch()
        _dev(x, self.ndof, "x")
        y = torch.empty_like(x)
        check(_lib.load().adfem_system_apply_d(self._h, ptr(x), ptr(y), _cur_stream()), "system_apply")
        return y

    def rhs(self):
        torch = _torch()
        r = torch.empty(self.ndof, dtype=torch.float64, device="cuda")
        check(_lib.load().adfem_system_rhs_d(self._h, ptr(r), _cur_stream()), "system_rhs")
        return r

    def solver_info(self):
        """Operator layout and the mixed iteration used (dict of adfem_solver_info)."""
        info = _lib.SolverInfo()
        check(_lib.load().adfem_system_solver_info(self._h, ctypes.byref(info)), "system_solver_info")
        return {name: getattr(info, name) for name, _ in info._fields_}


class PoissonSystem(_System):
    """-div(kappa grad u) = f on a P1 or P2 mesh with u = bdval on the Dirichlet DOFs
    (kappa and f at the mesh's Gauss points: 3 per element for P1, 6 for P2)."""

    kind = _lib.SYS_POISSON

    def assemble(self, kappa, f):
        from . import get_ngauss

        ng = get_ngauss(self.mesh)
        _dev(kappa, ng, "kappa")
        _dev(f, ng, "f")
        check(_lib.load().adfem_system_assemble_poisson_d(self._h, ptr(kappa), ptr(f), _cur_stream()), "assemble")

    def grad_kappa(self, u, lam):
        from . import get_ngauss

        torch = _torch()
        _dev(u, self.ndof, "u")
        _dev(lam, self.ndof, "lam")
        g = torch.empty(get_ngauss(self.mesh), dtype=torch.float64, device="cuda")
        check(_lib.load().adfem_system_grad_kappa_d(self._h, ptr(u), ptr(lam), ptr(g), _cur_stream()), "grad_kappa")
        return g

    def solve_host(self, kappa, f, precision="fp64", rtol=1e-12, max_iter=200000):
        """End-to-end host-buffer call (adfem_poisson_solve): numpy in, numpy out."""
        from . import solver_opts

        kappa = np.ascontiguousarray(kappa, dtype=np.float64)
        f = np.ascontiguousarray(f, dtype=np.float64)
        u = np.zeros(self.ndof)
        o = solver_opts(precision, rtol, max_iter)
        st = SolverStats()
        check(_lib.load().adfem_poisson_solve(self._h, ptr(kappa), ptr(f), ptr(u), ctypes.byref(o), ctypes.byref(st)),
              "poisson_solve")
        self.last_stats = st
        return u


class ElasticitySystem(_System):
    """Plane-strain linear elasticity, DOFs [u_x; u_y] (reference ordering)."""

    kind = _lib.SYS_ELASTICITY

    def assemble(self, E, nu, fx, fy):
        ng = 3 * self.mesh.nelem
        for t, nm in ((E, "E"), (nu, "nu"), (fx, "fx"), (fy, "fy")):
            _dev(t, ng, nm)
        check(_lib.load().adfem_system_assemble_elasticity_d(self._h, ptr(E), ptr(nu), ptr(fx), ptr(fy),
                                                             _cur_stream()), "assemble")

    def grad_E(self, u, lam, E, nu):
        torch = _torch()
        g = torch.empty(3 * self.mesh.nelem, dtype=torch.float64, device="cuda")
        check(_lib.load().adfem_system_grad_E_d(self._h, ptr(u), ptr(lam), ptr(E), ptr(nu), ptr(g), _cur_stream()),
              "grad_E")
        return g


# --------------------------------------------------------------- packed solves
def _packed(systems, outs, gs, rtol, max_iter, warm_start, adjoint):
    torch = _torch()
    n = len(systems)
    if outs is None:
        outs = [torch.zeros(s.ndof, dtype=torch.float64, device="cuda") for s in systems]
    for s, u in zip(systems, outs):
        _dev(u, s.ndof, "u")
    o = _lib.SolverOpts()
    _lib.load().adfem_solver_opts_default(ctypes.byref(o))
    o.rtol, o.max_iter, o.warm_start = rtol, max_iter, int(warm_start)
    st = (SolverStats * n)()
    hs = (ctypes.c_void_p * n)(*[s.handle.value for s in systems])
    us = (ctypes.c_void_p * n)(*[u.data_ptr() for u in outs])
    L = _lib.load()
    if adjoint:
        for s, g in zip(systems, gs):
            _dev(g, s.ndof, "g")
        gp = (ctypes.c_void_p * n)(*[g.data_ptr() for g in gs])
        check(L.adfem_system_adjoint_packed_d(hs, n, gp, us, ctypes.byref(o), st, _cur_stream()), "adjoint_packed")
    else:
        check(L.adfem_system_solve_packed_d(hs, n, us, ctypes.byref(o), st, _cur_stream()), "solve_packed")
    return outs, list(st)


def solve_packed(systems, outs=None, rtol=1e-9, max_iter=200000, warm_start=False):
    """Solve assembled small systems (<= 65536 DOFs each) in one packed launch; returns (u list, stats list)."""
    return _packed(systems, outs, None, rtol, max_iter, warm_start, False)


def adjoint_packed(systems, gs, outs=None, rtol=1e-9, max_iter=200000):
    """Adjoint solves K^T lam = g of assembled small systems in one packed launch."""
    return _packed(systems, outs, gs, rtol, max_iter, False, True)


# --------------------------------------------------------------- device operators
def _ng(mesh):
    return (3 if mesh.degree == 1 else 6) * mesh.nelem


def laplace_coo(mesh, kappa):
    """FemLaplaceScalar forward on the device: (indices (N,2) int64, vv (N,)), N = elem_ndof^2 ngauss."""
    torch = _torch()
    ng, nd2 = _ng(mesh), mesh.elem_ndof ** 2
    _dev(kappa, ng, "kappa")
    idx = torch.empty((nd2 * ng, 2), dtype=torch.int64, device="cuda")
    vv = torch.empty(nd2 * ng, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_laplace_coo_d(mesh.handle, ptr(kappa), ptr(idx), ptr(vv), _cur_stream()), "laplace_coo")
    return idx, vv


def laplace_coo_backward(mesh, grad_vv):
    torch = _torch()
    ng = _ng(mesh)
    _dev(grad_vv, mesh.elem_ndof ** 2 * ng, "grad_vv")
    g = torch.empty(ng, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_laplace_coo_backward_d(mesh.handle, ptr(grad_vv), ptr(g), _cur_stream()), "laplace bwd")
    return g


def laplace_csr(mesh, kappa):
    torch = _torch()
    cp, rv = mesh.pattern()
    _dev(kappa, _ng(mesh), "kappa")
    v = torch.empty(rv.size, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_laplace_csr_d(mesh.handle, ptr(kappa), ptr(v), _cur_stream()), "laplace_csr")
    return v


def mass_coo(mesh, rho):
    """ComputeFemMassMatrix1 forward on the device (elem_ndof^2 entries per Gauss point)."""
    torch = _torch()
    ng, nd2 = _ng(mesh), mesh.elem_ndof ** 2
    _dev(rho, ng, "rho")
    idx = torch.empty((nd2 * ng, 2), dtype=torch.int64, device="cuda")
    vv = torch.empty(nd2 * ng, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_mass_coo_d(mesh.handle, ptr(rho), ptr(idx), ptr(vv), _cur_stream()), "mass_coo")
    return idx, vv


def mass_coo_backward(mesh, grad_vv):
    torch = _torch()
    ng = _ng(mesh)
    _dev(grad_vv, mesh.elem_ndof ** 2 * ng, "grad_vv")
    g = torch.empty(ng, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_mass_coo_backward_d(mesh.handle, ptr(grad_vv), ptr(g), _cur_stream()), "mass bwd")
    return g


def mass_csr(mesh, rho):
    torch = _torch()
    cp, rv = mesh.pattern()
    _dev(rho, _ng(mesh), "rho")
    v = torch.empty(rv.size, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_mass_csr_d(mesh.handle, ptr(rho), ptr(v), _cur_stream()), "mass_csr")
    return v


def source(mesh, f, rhs=None, accumulate=False):
    torch = _torch()
    _dev(f, _ng(mesh), "f")
    if rhs is None:
        rhs = torch.zeros(mesh.ndof, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_source_d(mesh.handle, ptr(f), ptr(rhs), int(accumulate), _cur_stream()), "source")
    return rhs


def source_backward(mesh, grad_rhs):
    torch = _torch()
    _dev(grad_rhs, mesh.ndof, "grad_rhs")
    g = torch.empty(_ng(mesh), dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_source_backward_d(mesh.handle, ptr(grad_rhs), ptr(g), _cur_stream()), "source bwd")
    return g


def stiffness_coo(mesh, D):
    torch = _torch()
    ng, n4 = _ng(mesh), 4 * mesh.elem_ndof ** 2
    _dev(D, 9 * ng, "D")
    idx = torch.empty((n4 * ng, 2), dtype=torch.int64, device="cuda")
    vv = torch.empty(n4 * ng, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_stiffness_coo_d(mesh.handle, ptr(D), ptr(idx), ptr(vv), _cur_stream()), "stiffness_coo")
    return idx, vv


def stiffness_coo_backward(mesh, grad_vv):
    torch = _torch()
    ng = _ng(mesh)
    _dev(grad_vv, 4 * mesh.elem_ndof ** 2 * ng, "grad_vv")
    g = torch.empty(9 * ng, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_stiffness_coo_backward_d(mesh.handle, ptr(grad_vv), ptr(g), _cur_stream()), "stiff bwd")
    return g


def stiffness_csr(mesh, D):
    torch = _torch()
    cp, rv = mesh.pattern_elasticity()
    _dev(D, 9 * _ng(mesh), "D")
    v = torch.empty(rv.size, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_stiffness_csr_d(mesh.handle, ptr(D), ptr(v), _cur_stream()), "stiffness_csr")
    return v


def fem_to_gauss(mesh, u):
    """fem_to_gauss_points on the device: nodal values (nnode) -> Gauss points."""
    torch = _torch()
    _dev(u, None, "u")
    out = torch.empty(_ng(mesh), dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_fem_to_gauss_d(mesh.handle, ptr(u), ptr(out), _cur_stream()), "fem_to_gauss")
    return out


def fem_to_gauss_backward(mesh, grad_out, nu=None, grad_u=None):
    """Transpose of fem_to_gauss: writes nu entries, or adds into grad_u when given."""
    torch = _torch()
    _dev(grad_out, _ng(mesh), "grad_out")
    acc = grad_u is not None
    if grad_u is None:
        grad_u = torch.empty(mesh.nnode if nu is None else nu, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_fem_to_gauss_backward_d(mesh.handle, ptr(grad_out), ptr(grad_u), grad_u.numel(),
                                                    int(acc), _cur_stream()), "fem_to_gauss backward")
    return grad_u


def dof_to_gauss(mesh, u):
    torch = _torch()
    _dev(u, mesh.ndof, "u")
    out = torch.empty(_ng(mesh), dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_dof_to_gauss_d(mesh.handle, ptr(u), ptr(out), _cur_stream()), "dof_to_gauss")
    return out


def dof_to_gauss_backward(mesh, grad_out, grad_u=None):
    torch = _torch()
    _dev(grad_out, _ng(mesh), "grad_out")
    acc = grad_u is not None
    if grad_u is None:
        grad_u = torch.empty(mesh.ndof, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_dof_to_gauss_backward_d(mesh.handle, ptr(grad_out), ptr(grad_u), grad_u.numel(),
                                                    int(acc), _cur_stream()), "dof_to_gauss backward")
    return grad_u


def plane_strain(E, nu, mode=0):
    torch = _torch()
    n = E.numel()
    _dev(E, n, "E")
    _dev(nu, n, "nu")
    D = torch.empty(9 * n, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_plane_strain_d(mode, n, ptr(E), ptr(nu), ptr(D), _cur_stream()), "plane_strain")
    return D


def plane_strain_backward(grad_D, E, nu, mode=0):
    torch = _torch()
    n = E.numel()
    gE = torch.empty(n, dtype=torch.float64, device="cuda")
    gn = torch.empty(n, dtype=torch.float64, device="cuda")
    check(_lib.load().adfem_plane_strain_backward_d(mode, n, ptr(grad_D), ptr(E), ptr(nu), ptr(gE), ptr(gn),
                                                    _cur_stream()), "plane_strain_backward")
    return gE, gn
