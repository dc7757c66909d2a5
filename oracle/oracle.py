"""Parity oracle for the triangle-element path (P1, P2) -- TEST INFRASTRUCTURE ONLY.

ctypes wrapper around ``fem_oracle.c`` (a serial C restatement of AdFem's
deps/MFEM kernels, each function citing the reference file:line it follows),
plus scipy's SuperLU direct solve standing in for Julia's ``K\\F``.  Only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module; the product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libfem_oracle.so")
SRC = os.path.join(HERE, "fem_oracle.c")

_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_longlong
_D = ctypes.c_double


SAN_LIB = os.path.join(BUILD, "libfem_oracle_san.so")


def build(force: bool = False) -> str:
    """Compile fem_oracle.c into oracle/_build/libfem_oracle.so (gcc, no FMA contraction)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp, SRC,
                               "-lm", "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


def build_sanitized() -> str:
    """The same library instrumented with AddressSanitizer and UndefinedBehaviorSanitizer
    (any finding aborts), for the memory-safety test of the oracle."""
    os.makedirs(BUILD, exist_ok=True)
    if not os.path.exists(SAN_LIB) or os.path.getmtime(SAN_LIB) < os.path.getmtime(SRC):
        tmp = SAN_LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O1", "-g", "-fPIC", "-shared", "-ffp-contract=off", "-fno-omit-frame-pointer",
                               "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-o", tmp, SRC,
                               "-lm", "-lpthread"])
        os.replace(tmp, SAN_LIB)
    return SAN_LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.environ.get("ADFEM_ORACLE_LIB")  # the sanitized build, for the memory-safety test
        if not path:
            build()
            path = LIB
        L = ctypes.CDLL(path)
        sig = {
            "orc_mesh_geometry": (_I, [_I, _P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
            "orc_mesh_edges": (_L, [_I, _I, _P, _P]),
            "orc_laplace_coo": (None, [_I, _P, _P, _P, _P, _P, _P, _P]),
            "orc_laplace_coo_backward": (None, [_I, _P, _P, _P, _P, _P]),
            "orc_source": (None, [_I, _P, _P, _P, _P, _P]),
            "orc_source_backward": (None, [_I, _P, _P, _P, _P, _P]),
            "orc_stiffness_coo": (None, [_I, _I, _P, _P, _P, _P, _P, _P, _P]),
            "orc_stiffness_coo_backward": (None, [_I, _P, _P, _P, _P, _P]),
            "orc_plane_strain_stress": (None, [_I, _L, _P, _P, _P]),
            "orc_plane_strain_stress_backward": (None, [_I, _L, _P, _P, _P, _P, _P]),
            "orc_dirichlet_coo": (_L, [_P, _P, _L, _P, _I, _P, _P, _L, _P, _P, _P]),
            "orc_dirichlet_coo_backward": (None, [_P, _P, _P, _P, _L, _P, _I, _P, _L, _P, _P, _P]),
            "orc_coo_to_csc_sorted": (_L, [_P, _P, _L, _L, _P, _P, _P]),
            "orc_coo_to_csc_alloc": (_L, [_P, _P, _L, _L, _P, _P, _P]),
            "orc_free": (None, [_P]),
            "orc_residual_csc_dd": (None, [_L, _P, _P, _P, _P, _P, _P]),
            "orc_dirichlet_csc": (_L, [_L, _P, _P, _P, _P, _P, _I, _P, _I, _P, _P, _P, _P]),
            "orc_bcnode": (_L, [_I, _I, _P, _P]),
            "orc_pcg": (_I, [_L, _P, _P, _P, _P, _P, _D, _I, _I, _P]),
            "orc_element_edges": (_L, [_I, _I, _P, _P]),
            "orc_space_tables": (None, [_I, _I, _P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
            "orc_gen_laplace_coo": (None, [_I, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
            "orc_gen_laplace_coo_backward": (None, [_I, _I, _I, _P, _P, _P, _P, _P]),
            "orc_gen_mass_coo": (None, [_I, _I, _I, _P, _P, _P, _P, _P, _P]),
            "orc_gen_mass_coo_backward": (None, [_I, _I, _I, _P, _P, _P, _P]),
            "orc_gen_source": (None, [_I, _I, _I, _P, _P, _P, _P, _P]),
            "orc_gen_source_backward": (None, [_I, _I, _I, _P, _P, _P, _P, _P]),
            "orc_gen_stiffness_coo": (None, [_I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
            "orc_gen_stiffness_coo_backward": (None, [_I, _I, _I, _P, _P, _P, _P, _P]),
            "orc_fem_to_gauss": (None, [_I, _I, _P, _P, _P, _P]),
            "orc_fem_to_gauss_backward": (None, [_I, _I, _P, _P, _P, _P]),
            "orc_dof_to_gauss": (None, [_I, _I, _I, _P, _P, _P, _P]),
            "orc_dof_to_gauss_backward": (None, [_I, _I, _I, _P, _P, _P, _P]),
            "orc_bcnode_p2": (_L, [_I, _I, _P, _P, _L, _P]),
            "orc_pcl_laplace_jacobian": (None, [_I, _I, _I, _P, _P, _P, _P]),
            "orc_pcl_dirichlet": (None, [_P, _P, _P, _I, _I]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class OracleMesh:
    """Restated NNFEM_Mesh (deps/MFEM/Common.cpp:20-142) for a P1 mesh.

    ``elems`` is 1-based (ne, 3) like the Julia constructor ``Mesh(coords, elems)``.
    """

    def __init__(self, coords, elems):
        coords = _c(coords, np.float64)
        elems = np.asarray(elems)
        self.nnode = coords.shape[0]
        self.nelem = elems.shape[0]
        self.ndof = self.nnode
        self.coords = coords
        xyz = np.zeros((self.nnode, 3))
        xyz[:, :2] = coords
        e0 = _c(elems - 1, np.int32)
        ne = self.nelem
        self.elem = np.empty((ne, 3), np.int32)
        self.area = np.empty(ne)
        self.w = np.empty((ne, 3))
        self.hx = np.empty((ne, 3))
        self.hy = np.empty((ne, 3))
        self.h = np.empty((ne, 3, 3))
        self.gx = np.empty((ne, 3))
        self.gy = np.empty((ne, 3))
        self.flipped = lib().orc_mesh_geometry(self.nnode, _p(xyz), ne, _p(e0), _p(self.elem), _p(self.area),
                                               _p(self.w), _p(self.hx), _p(self.hy), _p(self.h), _p(self.gx),
                                               _p(self.gy))
        self.ngauss = 3 * ne

    # --- getters (deps/MFEM/API.cpp:17-65) ---
    def gauss_nodes(self):
        return np.stack([self.gx.ravel(), self.gy.ravel()], axis=1)

    def edges(self):
        n = lib().orc_mesh_edges(self.nnode, self.nelem, _p(self.elem), None)
        out = np.empty(2 * n, np.int64)
        lib().orc_mesh_edges(self.nnode, self.nelem, _p(self.elem), _p(out))
        return out.reshape(2, n).T.copy()

    def elems1(self):
        return self.elem.astype(np.int64) + 1

    # --- operators ---
    def laplace_coo(self, kappa):
        kappa = _c(kappa, np.float64)
        N = 9 * self.ngauss
        idx = np.empty(2 * N, np.int64)
        vv = np.empty(N)
        lib().orc_laplace_coo(self.nelem, _p(self.elem), _p(self.w), _p(self.hx), _p(self.hy), _p(kappa), _p(idx),
                              _p(vv))
        return idx.reshape(N, 2), vv

    def laplace_coo_backward(self, grad_vv):
        g = _c(grad_vv, np.float64)
        out = np.empty(self.ngauss)
        lib().orc_laplace_coo_backward(self.nelem, _p(self.w), _p(self.hx), _p(self.hy), _p(g), _p(out))
        return out

    def laplace_csc(self, kappa):
        idx, vv = self.laplace_coo(kappa)
        return coo_to_csc(idx, vv, self.ndof)

    def source(self, f, rhs=None):
        f = _c(f, np.float64)
        out = np.zeros(self.ndof) if rhs is None else _c(rhs, np.float64).copy()
        lib().orc_source(self.nelem, _p(self.elem), _p(self.w), _p(self.h), _p(f), _p(out))
        return out

    def source_backward(self, grad_rhs):
        g = _c(grad_rhs, np.float64)
        out = np.empty(self.ngauss)
        lib().orc_source_backward(self.nelem, _p(self.elem), _p(self.w), _p(self.h), _p(g), _p(out))
        return out

    def stiffness_coo(self, D):
        D = _c(D, np.float64).reshape(-1)
        assert D.size == 9 * self.ngauss
        N = 36 * self.ngauss
        idx = np.empty(2 * N, np.int64)
        vv = np.empty(N)
        lib().orc_stiffness_coo(self.nelem, self.ndof, _p(self.elem), _p(self.w), _p(self.hx), _p(self.hy), _p(D),
                                _p(idx), _p(vv))
        return idx.reshape(N, 2), vv

    def stiffness_csc(self, D):
        idx, vv = self.stiffness_coo(D)
        return coo_to_csc(idx, vv, 2 * self.ndof)

    def stiffness_coo_backward(self, grad_vv):
        g = _c(grad_vv, np.float64)
        out = np.empty(9 * self.ngauss)
        lib().orc_stiffness_coo_backward(self.nelem, _p(self.w), _p(self.hx), _p(self.hy), _p(g), _p(out))
        return out.reshape(self.ngauss, 3, 3)

    def bcnode(self):
        n = lib().orc_bcnode(self.nnode, self.nelem, _p(self.elem), None)
        out = np.empty(n, np.int64)
        lib().orc_bcnode(self.nnode, self.nelem, _p(self.elem), _p(out))
        return out


class OracleSpace:
    """Restated NNFEM_Mesh tables for degree 1 (P1) or 2 (P2) Lagrange triangles.

    Follows deps/MFEM/Common.cpp:46-126: element DOFs (vertices, then nnode + edge of
    the local edges (0,1), (1,2), (2,0)), per-point weights, shape values and physical
    gradients on the default rule of the degree (order 2: 3 points; order 4: 6
    points).  The operator methods restate the reference loops over elem_ndof.
    """

    def __init__(self, coords, elems, degree: int = 1):
        if degree not in (1, 2):
            raise ValueError("degree must be 1 or 2")
        self.p1 = OracleMesh(coords, elems)
        m = self.p1
        self.degree = degree
        self.nnode, self.nelem = m.nnode, m.nelem
        ne = self.nelem
        self.eedge = np.empty((ne, 3), np.int32)
        self.nedge = int(lib().orc_element_edges(self.nnode, ne, _p(m.elem), _p(self.eedge)))
        nd = ng = 3 if degree == 1 else 6
        self.nd, self.ng = nd, ng
        self.ndof = self.nnode if degree == 1 else self.nnode + self.nedge
        self.ngauss = ng * ne
        xyz = np.zeros((self.nnode, 3))
        xyz[:, :2] = m.coords
        self.dof = np.empty((ne, nd), np.int32)
        self.w = np.empty((ne, ng))
        self.h = np.empty((ne, ng, nd))
        self.hx = np.empty((ne, ng, nd))
        self.hy = np.empty((ne, ng, nd))
        self.hs = np.empty((ne, ng, 3))
        self.gx = np.empty((ne, ng))
        self.gy = np.empty((ne, ng))
        lib().orc_space_tables(degree, self.nnode, _p(xyz), ne, _p(m.elem), _p(self.eedge), _p(m.area), _p(m.hx),
                               _p(m.hy), _p(self.dof), _p(self.w), _p(self.h), _p(self.hx), _p(self.hy), _p(self.hs),
                               _p(self.gx), _p(self.gy))

    def gauss_nodes(self):
        return np.stack([self.gx.ravel(), self.gy.ravel()], axis=1)

    def connectivity1(self):
        return self.dof.astype(np.int64) + 1

    def dof_nodes(self):
        """Coordinates of the DOFs: vertices, then edge midpoints (P2)."""
        xy = self.p1.coords
        if self.degree == 1:
            return xy.copy()
        mid = np.empty((self.nedge, 2))
        for j in range(3):
            a, b = self.p1.elem[:, j], self.p1.elem[:, (j + 1) % 3]
            mid[self.eedge[:, j]] = 0.5 * (xy[a] + xy[b])
        return np.concatenate([xy, mid])

    def _args(self):
        return self.nelem, self.nd, self.ng

    def laplace_coo(self, kappa):
        kappa = _c(kappa, np.float64)
        N = self.nd * self.nd * self.ngauss
        idx = np.empty(2 * N, np.int64)
        vv = np.empty(N)
        lib().orc_gen_laplace_coo(*self._args(), _p(self.dof), _p(self.w), _p(self.hx), _p(self.hy), _p(kappa),
                                  _p(idx), _p(vv))
        return idx.reshape(-1, 2), vv

    def laplace_coo_backward(self, grad_vv):
        g = _c(grad_vv, np.float64)
        out = np.empty(self.ngauss)
        lib().orc_gen_laplace_coo_backward(*self._args(), _p(self.w), _p(self.hx), _p(self.hy), _p(g), _p(out))
        return out

    def laplace_csc(self, kappa):
        idx, vv = self.laplace_coo(kappa)
        return coo_to_csc(idx, vv, self.ndof)

    def mass_coo(self, rho):
        rho = _c(rho, np.float64)
        N = self.nd * self.nd * self.ngauss
        idx = np.empty(2 * N, np.int64)
        vv = np.empty(N)
        lib().orc_gen_mass_coo(*self._args(), _p(self.dof), _p(self.w), _p(self.h), _p(rho), _p(idx), _p(vv))
        return idx.reshape(-1, 2), vv

    def mass_coo_backward(self, grad_vv):
        g = _c(grad_vv, np.float64)
        out = np.empty(self.ngauss)
        lib().orc_gen_mass_coo_backward(*self._args(), _p(self.w), _p(self.h), _p(g), _p(out))
        return out

    def mass_csc(self, rho):
        idx, vv = self.mass_coo(rho)
        return coo_to_csc(idx, vv, self.ndof)

    def source(self, f, rhs=None):
        f = _c(f, np.float64)
        out = np.zeros(self.ndof) if rhs is None else np.array(rhs, dtype=np.float64, copy=True)
        lib().orc_gen_source(*self._args(), _p(self.dof), _p(self.w), _p(self.h), _p(f), _p(out))
        return out

    def source_backward(self, grad_rhs):
        g = _c(grad_rhs, np.float64)
        out = np.empty(self.ngauss)
        lib().orc_gen_source_backward(*self._args(), _p(self.dof), _p(self.w), _p(self.h), _p(g), _p(out))
        return out

    def stiffness_coo(self, D):
        D = _c(D, np.float64)
        N = 4 * self.nd * self.nd * self.ngauss
        idx = np.empty(2 * N, np.int64)
        vv = np.empty(N)
        lib().orc_gen_stiffness_coo(*self._args(), self.ndof, _p(self.dof), _p(self.w), _p(self.hx), _p(self.hy),
                                    _p(D), _p(idx), _p(vv))
        return idx.reshape(-1, 2), vv

    def stiffness_coo_backward(self, grad_vv):
        g = _c(grad_vv, np.float64)
        out = np.empty(9 * self.ngauss)
        lib().orc_gen_stiffness_coo_backward(*self._args(), _p(self.w), _p(self.hx), _p(self.hy), _p(g), _p(out))
        return out

    def stiffness_csc(self, D):
        idx, vv = self.stiffness_coo(D)
        return coo_to_csc(idx, vv, 2 * self.ndof)

    def fem_to_gauss(self, u):
        u = _c(u, np.float64)
        out = np.empty(self.ngauss)
        lib().orc_fem_to_gauss(self.nelem, self.ng, _p(self.p1.elem), _p(self.hs), _p(u), _p(out))
        return out

    def fem_to_gauss_backward(self, grad_out, nu=None):
        g = _c(grad_out, np.float64)
        out = np.zeros(self.nnode if nu is None else nu)
        lib().orc_fem_to_gauss_backward(self.nelem, self.ng, _p(self.p1.elem), _p(self.hs), _p(g), _p(out))
        return out

    def dof_to_gauss(self, u):
        u = _c(u, np.float64)
        out = np.empty(self.ngauss)
        lib().orc_dof_to_gauss(*self._args(), _p(self.dof), _p(self.h), _p(u), _p(out))
        return out

    def dof_to_gauss_backward(self, grad_out):
        g = _c(grad_out, np.float64)
        out = np.zeros(self.ndof)
        lib().orc_dof_to_gauss_backward(*self._args(), _p(self.dof), _p(self.h), _p(g), _p(out))
        return out

    def pcl_laplace_jacobian(self):
        """pcl_compute_fem_laplace_matrix1 (src/pcl.jl:24-39): dense ngauss x nd^2 ngauss."""
        H = np.zeros((self.ngauss, self.nd * self.nd * self.ngauss), order="F")
        lib().orc_pcl_laplace_jacobian(*self._args(), _p(self.w), _p(self.hx), _p(self.hy), _p(H))
        return H

    def bcnode(self):
        if self.degree == 1:
            return self.p1.bcnode()
        n = lib().orc_bcnode_p2(self.nnode, self.nelem, _p(self.p1.elem), _p(self.eedge), self.nedge, None)
        out = np.empty(n, np.int64)
        lib().orc_bcnode_p2(self.nnode, self.nelem, _p(self.p1.elem), _p(self.eedge), self.nedge, _p(out))
        return out


def plane_strain(E, nu, mode: int = 0):
    E = _c(E, np.float64)
    nu = _c(nu, np.float64)
    out = np.empty((E.size, 3, 3))
    lib().orc_plane_strain_stress(mode, E.size, _p(E), _p(nu), _p(out))
    return out


def plane_strain_backward(grad_out, E, nu, mode: int = 0):
    g = _c(grad_out, np.float64)
    E = _c(E, np.float64)
    nu = _c(nu, np.float64)
    gE = np.empty(E.size)
    gn = np.empty(E.size)
    lib().orc_plane_strain_stress_backward(mode, E.size, _p(g), _p(E), _p(nu), _p(gE), _p(gn))
    return gE, gn


def coo_to_csc(indices, vv, n):
    """Julia ``sparse(I+1, J+1, V, n, n)`` (src/MFEM/MCore.jl:118-119) as a scipy CSC matrix
    (linear-time counting sorts; duplicates summed in input order)."""
    idx = _c(indices, np.int64).reshape(-1)
    vv = _c(vv, np.float64)
    N = vv.size
    cp, rv, nz = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    nnz = lib().orc_coo_to_csc_alloc(_p(idx), _p(vv), N, n, ctypes.byref(cp), ctypes.byref(rv), ctypes.byref(nz))
    if nnz < 0:
        raise MemoryError("orc_coo_to_csc_alloc: out of memory")

    def take(ptr, count, ctype, dtype):
        a = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctype)), shape=(max(count, 1),))[:count].copy()
        lib().orc_free(ptr)
        return a.astype(dtype, copy=False)

    colptr = take(cp, n + 1, ctypes.c_longlong, np.int64)
    rowval = take(rv, nnz, ctypes.c_longlong, np.int64)
    nzval = take(nz, nnz, ctypes.c_double, np.float64)
    return sp.csc_matrix((nzval, rowval, colptr), shape=(n, n))


def coo_to_csc_sorted(indices, vv, n):
    """The same conversion by a comparison sort of (col, row, position): the plain
    statement of the semantics, kept to check coo_to_csc bit for bit."""
    idx = _c(indices, np.int64).reshape(-1)
    vv = _c(vv, np.float64)
    N = vv.size
    nnz = lib().orc_coo_to_csc_sorted(_p(idx), _p(vv), N, n, None, None, None)
    colptr = np.empty(n + 1, np.int64)
    rowval = np.empty(nnz, np.int64)
    nzval = np.empty(nnz)
    lib().orc_coo_to_csc_sorted(_p(idx), _p(vv), N, n, _p(colptr), _p(rowval), _p(nzval))
    return sp.csc_matrix((nzval, rowval, colptr), shape=(n, n))


def residual_dd(A, x, b):
    """r = b - A x for the stored FP64 vector x, evaluated in doubled precision and rounded
    once (so that residuals at the FP64 rounding floor of x are resolved)."""
    A = sp.csc_matrix(A)
    n = A.shape[0]
    cp = _c(A.indptr, np.int64)
    rv = _c(A.indices, np.int64)
    nz = _c(A.data, np.float64)
    x = _c(x, np.float64)
    b = _c(b, np.float64)
    r = np.empty(n)
    lib().orc_residual_csc_dd(n, _p(cp), _p(rv), _p(nz), _p(x), _p(b), _p(r))
    return r


def dirichlet_coo(indices, vv, bd, rhs, bdval, n):
    """ImposeDirichlet forward (deps/MFEM/ImposeDirichlet/ImposeDirichlet.h:27-60); bd 1-based."""
    idx = _c(indices, np.int64).reshape(-1)
    vv = _c(vv, np.float64)
    bd = _c(bd, np.int64)
    rhs = _c(rhs, np.float64)
    bdval = _c(bdval, np.float64)
    z = lib().orc_dirichlet_coo(_p(idx), _p(vv), vv.size, _p(bd), bd.size, _p(rhs), _p(bdval), n, None, None, None)
    oi = np.empty(2 * z, np.int64)
    ov = np.empty(z)
    orhs = np.empty(n)
    lib().orc_dirichlet_coo(_p(idx), _p(vv), vv.size, _p(bd), bd.size, _p(rhs), _p(bdval), n, _p(oi), _p(ov),
                            _p(orhs))
    return oi.reshape(z, 2), ov, orhs


def dirichlet_coo_backward(grad_vv, grad_rhs, indices, vv, bd, bdval, n):
    """ImposeDirichlet backward (ImposeDirichlet.h:63-93)."""
    idx = _c(indices, np.int64).reshape(-1)
    vv = _c(vv, np.float64)
    bd = _c(bd, np.int64)
    bdval = _c(bdval, np.float64)
    g = _c(grad_vv, np.float64)
    gr = _c(grad_rhs, np.float64)
    gvi = np.empty(vv.size)
    gri = np.empty(n)
    gb = np.empty(bd.size)
    lib().orc_dirichlet_coo_backward(_p(g), _p(gr), _p(idx), _p(vv), vv.size, _p(bd), bd.size, _p(bdval), n,
                                     _p(gvi), _p(gri), _p(gb))
    return gvi, gri, gb


def dirichlet_csc(A, rhs, bd, bdval, keep_zeros: bool = False):
    """impose_Dirichlet_boundary_conditions, SparseMatrixCSC arm (src/MFEM/MUtils.jl:184-199)."""
    A = sp.csc_matrix(A)
    A.sort_indices()
    n = A.shape[0]
    colptr = _c(A.indptr, np.int64)
    rowval = _c(A.indices, np.int64)
    nzval = _c(A.data, np.float64)
    rhs = _c(rhs, np.float64)
    bd = _c(bd, np.int64)
    bdval = _c(bdval, np.float64)
    z = lib().orc_dirichlet_csc(n, _p(colptr), _p(rowval), _p(nzval), _p(rhs), _p(bd), bd.size, _p(bdval),
                                int(keep_zeros), None, None, None, None)
    oc = np.empty(n + 1, np.int64)
    orr = np.empty(z, np.int64)
    ov = np.empty(z)
    orhs = np.empty(n)
    lib().orc_dirichlet_csc(n, _p(colptr), _p(rowval), _p(nzval), _p(rhs), _p(bd), bd.size, _p(bdval),
                            int(keep_zeros), _p(oc), _p(orr), _p(ov), _p(orhs))
    return sp.csc_matrix((ov, orr, oc), shape=(n, n)), orhs


def pcl_dirichlet(indices1, bd, outdof):
    """pcl_impose_Dirichlet_boundary_conditions (src/pcl.jl:1-21): indices 1-based (sN, 2)."""
    idx = np.asfortranarray(np.asarray(indices1, dtype=np.int64))
    sN = idx.shape[0]
    bd = _c(bd, np.int64).ravel()
    J = np.zeros((sN, outdof), order="F")
    lib().orc_pcl_dirichlet(_p(J), idx.ctypes.data_as(ctypes.c_void_p), _p(bd), bd.size, sN)
    return J


def spsolve(A, b):
    """FP64 sparse direct solve (SuperLU) standing in for Julia's ``K\\F``."""
    return spla.spsolve(sp.csc_matrix(A), np.asarray(b, dtype=np.float64))


def pcg(A, b, rtol=1e-13, max_iter=100000, threads=1):
    """CPU Jacobi-PCG (FP64) from zero; returns (x, iterations, final relative residual)."""
    A = sp.csr_matrix(A)
    n = A.shape[0]
    rp = _c(A.indptr, np.int64)
    ci = _c(A.indices, np.int32)
    va = _c(A.data, np.float64)
    b = _c(b, np.float64)
    x = np.empty(n)
    rr = ctypes.c_double(0.0)
    it = lib().orc_pcg(n, _p(rp), _p(ci), _p(va), _p(b), _p(x), rtol, max_iter, threads, ctypes.byref(rr))
    return x, it, rr.value
