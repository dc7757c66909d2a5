"""adfem_gpu -- GB300 implementation of AdFem.jl's triangle-element forward/adjoint path.

This module mirrors the Julia operator API of AdFem on top of the C ABI of
libadfem_gpu.so (include/adfem_gpu.h): the same function names, argument
meaning, 1-based node numbering and sparse outputs (scipy CSC standing in for
Julia's SparseMatrixCSC).  All arithmetic runs in the CUDA library; this layer
only converts arguments.

    Mesh(coords, elems)                          src/MFEM/MFEM.jl:60-119
    Mesh(filename)                               src/MFEM/MUtils.jl:33-50
    Mesh.rectangle(m, n, h)                      src/MFEM/MFEM.jl:134-170
    get_ngauss / get_area / gauss_nodes          src/MFEM/MFEM.jl:207-232
    compute_fem_laplace_matrix1(kappa, mesh)     src/MFEM/MCore.jl:112-120
    compute_fem_source_term1(f, mesh)            src/MFEM/MCore.jl:77-82
    compute_fem_source_term(f1, f2, mesh)        src/MFEM/MCore.jl:87-94
    compute_fem_stiffness_matrix(D, mesh)        src/MFEM/MCore.jl:287-315
    compute_plane_strain_matrix(E, nu)           src/Core.jl:777-785
    compute_fem_mass_matrix1(rho, mesh)          src/MFEM/MCore.jl:170-193
    fem_to_gauss_points / dof_to_gauss_points    src/MFEM/MUtils.jl:231-275
    bcnode(mesh)                                 src/MFEM/MCore.jl:439-450
    impose_Dirichlet_boundary_conditions(...)    src/MFEM/MUtils.jl:184-199
    solve(K, F)  (K\\F)                          README.md:54
"""
from __future__ import annotations

import ctypes

import numpy as np
import scipy.sparse as sp

from . import _lib
from ._lib import AdFemError, SolverOpts, SolverStats, check, ptr

__all__ = [
    "AdFemError", "Mesh", "get_ngauss", "get_area", "gauss_nodes", "fem_nodes", "bcnode",
    "compute_fem_laplace_matrix1", "compute_fem_source_term1", "compute_fem_source_term",
    "compute_fem_stiffness_matrix", "compute_plane_strain_matrix", "compute_plane_stress_matrix",
    "impose_Dirichlet_boundary_conditions", "impose_Dirichlet_coo", "impose_Dirichlet_coo_backward",
    "solve", "solver_opts", "get_connectivity", "gauss_weights", "dof_nodes", "eval_f_on_gauss_pts",
    "eval_f_on_fem_pts", "eval_f_on_dof_pts", "compute_fem_mass_matrix1", "compute_fem_mass_matrix",
    "fem_to_gauss_points", "dof_to_gauss_points", "P1", "P2", "pcl_compute_fem_laplace_matrix1",
    "pcl_impose_Dirichlet_boundary_conditions",
]

P1 = 1
P2 = 2


def _lib_():
    return _lib.load()


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Mesh:
    """Triangle mesh resident on the GPU (mirror of AdFem's ``Mesh``).

    ``coords``: (nnode, 2) float; ``elems``: (nelem, 3) 1-based vertex ids; or
    ``Mesh(filename)`` for a .mat/.stl/.msh/.vtk mesh file (adfem_gpu.meshfile).  Degree 1
    (P1, order-2 rule) and degree 2 (P2, order-4 rule) are supported (``order=-1``
    selects these defaults, src/MFEM/MFEM.jl:71-77); BDM1 and other orders raise
    ``AdFemError`` with status ``ERR_UNSUPPORTED``.
    """

    def __init__(self, coords, elems=None, order: int = -1, degree: int = 1, lorder: int = -1,
                 file_format: str | None = None):
        if isinstance(coords, (str, bytes)) or hasattr(coords, "__fspath__"):
            # Mesh(filename) (src/MFEM/MUtils.jl:33-50)
            from .meshfile import read_mesh_file

            coords, elems = read_mesh_file(str(coords), file_format)
        if degree not in (1, 2):
            raise AdFemError(_lib.ERR_UNSUPPORTED, "degree 1 (P1) and 2 (P2) elements are implemented")
        if order not in (-1, 2 * degree):
            raise AdFemError(_lib.ERR_UNSUPPORTED, "P1 uses the order-2 rule and P2 the order-4 rule")
        L = _lib_()
        coords = _c(coords, np.float64)
        elems = np.asarray(elems)
        if coords.ndim != 2 or coords.shape[1] != 2 or elems.ndim != 2 or elems.shape[1] != 3:
            raise AdFemError(_lib.ERR_INVALID, "coords must be (n,2) and elems (m,3)")
        nv, ne = coords.shape[0], elems.shape[0]
        xyz = np.zeros((nv, 3))
        xyz[:, :2] = coords
        e0 = _c(elems - 1, np.int32)
        h = ctypes.c_void_p()
        check(L.adfem_mesh_create(ptr(xyz), nv, ptr(e0), ne, degree, ctypes.byref(h)), "Mesh")
        self._h = h
        self.nodes = coords
        self.nnode = nv
        self.nelem = ne
        self.degree = degree
        self.elem_type = P1 if degree == 1 else P2
        nd, ndof = ctypes.c_int(), ctypes.c_longlong()
        check(L.adfem_mesh_space(h, None, ctypes.byref(nd), None, ctypes.byref(ndof), None))
        self.ndof = ndof.value
        self.elem_ndof = nd.value
        self.lorder = 6 if lorder == -1 else lorder
        el = np.empty(3 * ne, np.int64)
        check(L.adfem_mesh_elements(h, ptr(el)))
        self.elems = el.reshape(ne, 3)
        conn = np.empty(self.elem_ndof * ne, np.int64)
        check(L.adfem_mesh_connectivity(h, ptr(conn)))
        self.conn = conn.reshape(ne, self.elem_ndof)
        nedge = ctypes.c_longlong()
        check(L.adfem_mesh_edges(h, None, ctypes.byref(nedge)))
        ed = np.empty(2 * nedge.value, np.int64)
        check(L.adfem_mesh_edges(h, ptr(ed), ctypes.byref(nedge)))
        self.nedge = nedge.value
        self.edges = ed.reshape(2, self.nedge).T.copy()
        self._pattern = None
        self._pattern_el = None

    @classmethod
    def rectangle(cls, m: int, n: int, h: float, version: int = 1, degree: int = 1):
        """``Mesh(m, n, h)``: m x n cells of size h, nodes x-fastest (MFEM.jl:134-170)."""
        if version not in (1, 2):
            raise AdFemError(_lib.ERR_UNSUPPORTED, "versions 1 and 2 are implemented")
        jj, ii = np.meshgrid(np.arange(m + 1), np.arange(n + 1))
        coords = np.stack([(jj * h).ravel(), (ii * h).ravel()], axis=1).astype(np.float64)
        i = np.arange(n)[:, None]
        j = np.arange(m)[None, :]
        a = (i * (m + 1) + j).ravel()
        b, c = a + 1, ((i + 1) * (m + 1) + j).ravel()
        d = c + 1
        el = np.empty((2 * m * n, 3), np.int64)
        if version == 1:
            el[0::2] = np.stack([a, b, c], 1)
            el[1::2] = np.stack([b, c, d], 1)
        else:
            el[0::2] = np.stack([a, d, c], 1)
            el[1::2] = np.stack([a, b, d], 1)
        return cls(coords, el + 1, degree=degree)

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and _lib._LIB is not None:
            _lib._LIB.adfem_mesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def pattern(self):
        """1-based CSC (colptr, rowval) of the scalar operator."""
        if self._pattern is None:
            L = _lib_()
            nnz = ctypes.c_longlong()
            check(L.adfem_mesh_sizes(self._h, None, None, None, ctypes.byref(nnz)))
            cp = np.empty(self.ndof + 1, np.int64)
            rv = np.empty(nnz.value, np.int64)
            check(L.adfem_mesh_pattern(self._h, ptr(cp), ptr(rv)))
            self._pattern = (cp, rv)
        return self._pattern

    def pattern_elasticity(self):
        if self._pattern_el is None:
            L = _lib_()
            cp0, rv0 = self.pattern()
            cp = np.empty(2 * self.ndof + 1, np.int64)
            rv = np.empty(4 * rv0.size, np.int64)
            check(L.adfem_mesh_pattern_elasticity(self._h, ptr(cp), ptr(rv)))
            self._pattern_el = (cp, rv)
        return self._pattern_el

    def __len__(self):
        return self.ndof


def get_ngauss(mesh: Mesh) -> int:
    return (3 if mesh.degree == 1 else 6) * mesh.nelem


def get_connectivity(mesh: Mesh):
    """ne x elem_ndof DOFs, 1-based: vertices, then nnode + edge for P2 (mfem_get_connectivity)."""
    return mesh.conn


def gauss_weights(mesh: Mesh):
    w = np.empty(get_ngauss(mesh))
    check(_lib_().adfem_mesh_gauss_weights(mesh.handle, ptr(w)))
    return w


def dof_nodes(mesh: Mesh):
    """Coordinates of the DOFs: the vertices, then (P2) the edge midpoints."""
    if mesh.degree == 1:
        return mesh.nodes
    mid = 0.5 * (mesh.nodes[mesh.edges[:, 0] - 1] + mesh.nodes[mesh.edges[:, 1] - 1])
    return np.concatenate([mesh.nodes, mid])


def eval_f_on_gauss_pts(f, mesh: Mesh):
    g = gauss_nodes(mesh)
    return np.asarray(f(g[:, 0], g[:, 1]), dtype=np.float64)


def eval_f_on_fem_pts(f, mesh: Mesh):
    return np.asarray(f(mesh.nodes[:, 0], mesh.nodes[:, 1]), dtype=np.float64)


def eval_f_on_dof_pts(f, mesh: Mesh):
    x = dof_nodes(mesh)
    return np.asarray(f(x[:, 0], x[:, 1]), dtype=np.float64)


def get_area(mesh: Mesh):
    a = np.empty(mesh.nelem)
    check(_lib_().adfem_mesh_area(mesh.handle, ptr(a)))
    return a


def gauss_nodes(mesh: Mesh):
    x = np.empty(get_ngauss(mesh))
    y = np.empty(get_ngauss(mesh))
    check(_lib_().adfem_mesh_gauss_nodes(mesh.handle, ptr(x), ptr(y)))
    return np.stack([x, y], axis=1)


def fem_nodes(mesh: Mesh):
    return mesh.nodes


def bcnode(mesh: Mesh):
    """Boundary DOFs, 1-based: ascending vertices (the reference returns Julia Set order),
    then for P2 the DOFs of the boundary edges."""
    L = _lib_()
    n = ctypes.c_longlong()
    check(L.adfem_mesh_bcnode(mesh.handle, None, ctypes.byref(n)))
    out = np.empty(n.value, np.int64)
    check(L.adfem_mesh_bcnode(mesh.handle, ptr(out), ctypes.byref(n)))
    return out


def _csc(nzval, cp1, rv1, n):
    return sp.csc_matrix((nzval, rv1 - 1, cp1 - 1), shape=(n, n))


def compute_fem_laplace_matrix1(kappa, mesh: Mesh):
    """Stiffness matrix of -div(kappa grad u) (SparseMatrixCSC arm), kappa at the Gauss points."""
    kappa = _c(kappa, np.float64).ravel()
    if kappa.size != get_ngauss(mesh):
        raise AdFemError(_lib.ERR_INVALID, "length(kappa) must equal get_ngauss(mesh)")
    cp, rv = mesh.pattern()
    nz = np.empty(rv.size)
    check(_lib_().adfem_laplace_csc(mesh.handle, ptr(kappa), kappa.size, ptr(nz)), "compute_fem_laplace_matrix1")
    return _csc(nz, cp, rv, mesh.ndof)


def compute_fem_source_term1(f, mesh: Mesh):
    f = _c(f, np.float64).ravel()
    if f.size != get_ngauss(mesh):
        raise AdFemError(_lib.ERR_INVALID, "length(f) must equal get_ngauss(mesh)")
    out = np.zeros(mesh.ndof)
    check(_lib_().adfem_source(mesh.handle, ptr(f), f.size, ptr(out), 0), "compute_fem_source_term1")
    return out


def compute_fem_source_term(f1, f2=None, mesh: Mesh | None = None):
    """[src(f1); src(f2)], or a single stacked vector of length 2 ngauss (MCore.jl:87-94)."""
    if mesh is None and isinstance(f2, Mesh):
        mesh, f = f2, _c(f1, np.float64).ravel()
        ng = get_ngauss(mesh)
        if f.size != 2 * ng:
            raise AdFemError(_lib.ERR_INVALID, "length(f) must be 2 ngauss")
        f1, f2 = f[:ng], f[ng:]
    return np.concatenate([compute_fem_source_term1(f1, mesh), compute_fem_source_term1(f2, mesh)])


def compute_fem_stiffness_matrix(D, mesh: Mesh):
    """Elasticity stiffness (2 ndof x 2 ndof, [x; y] DOF blocks); D is (3,3) or (ngauss,3,3)."""
    D = np.asarray(D, dtype=np.float64)
    ng = get_ngauss(mesh)
    if D.shape == (3, 3):
        D = np.broadcast_to(D, (ng, 3, 3))
    if D.shape != (ng, 3, 3):
        raise AdFemError(_lib.ERR_INVALID, "D must be (3,3) or (ngauss,3,3)")
    D = _c(D, np.float64).ravel()
    cp, rv = mesh.pattern_elasticity()
    nz = np.empty(rv.size)
    check(_lib_().adfem_stiffness_csc(mesh.handle, ptr(D), D.size, ptr(nz)), "compute_fem_stiffness_matrix")
    return _csc(nz, cp, rv, 2 * mesh.ndof)


def compute_fem_mass_matrix1(rho, mesh: Mesh | None = None):
    """Mass matrix sum_k rho_k w_k phi phi^T (SparseMatrixCSC arm), rho at the Gauss points;
    ``compute_fem_mass_matrix1(mesh)`` uses rho = 1 (MCore.jl:170-181)."""
    if mesh is None and isinstance(rho, Mesh):
        mesh, rho = rho, np.ones(get_ngauss(rho))
    rho = _c(rho, np.float64).ravel()
    if rho.size != get_ngauss(mesh):
        raise AdFemError(_lib.ERR_INVALID, "length(rho) must equal get_ngauss(mesh)")
    cp, rv = mesh.pattern()
    nz = np.empty(rv.size)
    check(_lib_().adfem_mass_csc(mesh.handle, ptr(rho), rho.size, ptr(nz)), "compute_fem_mass_matrix1")
    return _csc(nz, cp, rv, mesh.ndof)


def compute_fem_mass_matrix(rho, mesh: Mesh | None = None):
    """[M 0; 0 M] for the two displacement components (MCore.jl:183-193)."""
    M = compute_fem_mass_matrix1(rho, mesh)
    return sp.block_diag([M, M], format="csc")


def pcl_compute_fem_laplace_matrix1(mesh: Mesh):
    """J[i, j] = d v_j / d kappa_i for v the unsummed Laplace COO values (src/pcl.jl:24-39)."""
    ng = get_ngauss(mesh)
    J = np.zeros((ng, mesh.elem_ndof ** 2 * ng), order="F")
    check(_lib_().adfem_pcl_laplace_jacobian(mesh.handle, ptr(J)), "pcl_compute_fem_laplace_matrix1")
    return J


def pcl_impose_Dirichlet_boundary_conditions(indices, bdnode, outdof: int):
    """J[i, j] = d (v_B)_j / d (v_A)_i of the COO Dirichlet arm; indices 1-based (n_A, 2) (src/pcl.jl:1-21)."""
    idx = np.asarray(indices, dtype=np.int64)
    sN = idx.shape[0]
    i0 = _c(idx - 1, np.int64).reshape(-1)
    bd = _c(bdnode, np.int64).ravel()
    N = int(max(idx.max(initial=0), bd.max(initial=0)))
    pos = np.empty(sN, np.int64)
    nk = ctypes.c_longlong()
    check(_lib_().adfem_pcl_dirichlet(ptr(i0), sN, ptr(bd), bd.size, N, ptr(pos), ctypes.byref(nk)),
          "pcl_impose_Dirichlet_boundary_conditions")
    J = np.zeros((sN, outdof))
    k = np.nonzero(pos >= 0)[0]
    J[k, pos[k]] = 1.0
    return J


def fem_to_gauss_points(u, mesh: Mesh):
    """Nodal values (length nnode) at the Gauss points through the P1 shape (MUtils.jl:231-246)."""
    u = _c(u, np.float64).ravel()
    out = np.empty(get_ngauss(mesh))
    check(_lib_().adfem_fem_to_gauss(mesh.handle, ptr(u), u.size, ptr(out)), "fem_to_gauss_points")
    return out


def dof_to_gauss_points(u, mesh: Mesh):
    """DOF values (length ndof) at the Gauss points through every basis function (MUtils.jl:256-270)."""
    u = _c(u, np.float64).ravel()
    if u.size != mesh.ndof:
        raise AdFemError(_lib.ERR_INVALID, "length(u) must equal mesh.ndof")
    out = np.empty(get_ngauss(mesh))
    check(_lib_().adfem_dof_to_gauss(mesh.handle, ptr(u), u.size, ptr(out)), "dof_to_gauss_points")
    return out


def _plane(E, nu, fn):
    E = _c(E, np.float64).ravel()
    nu = _c(nu, np.float64).ravel()
    if E.size != nu.size:
        raise AdFemError(_lib.ERR_INVALID, "E and nu must have the same length")
    out = np.empty((E.size, 3, 3))
    getattr(_lib_(), fn)(ptr(out), ptr(E), ptr(nu), E.size)
    return out


def compute_plane_strain_matrix(E, nu):
    """Pointwise plane-strain matrices (N,3,3), the reference's nine-entry formula."""
    if np.isscalar(E) and np.isscalar(nu):
        return _plane([E], [nu], "PlaneStrainMatrix_forward")[0]
    return _plane(E, nu, "PlaneStrainMatrix_forward")


def compute_plane_stress_matrix(E, nu):
    if np.isscalar(E) and np.isscalar(nu):
        return _plane([E], [nu], "PlaneStressMatrix_forward")[0]
    return _plane(E, nu, "PlaneStressMatrix_forward")


def impose_Dirichlet_boundary_conditions(A, rhs, bdnode, bdval, keep_zeros: bool = False):
    """SparseMatrixCSC arm: returns (B, r) with B = [A_II 0; 0 I], r_I = rhs_I - A_IB bdval, r_B = bdval."""
    A = sp.csc_matrix(A)
    A.sort_indices()
    n = A.shape[0]
    if A.shape[1] != n or len(rhs) != n:
        raise AdFemError(_lib.ERR_INVALID, "A must be square and match rhs")
    cp = _c(A.indptr, np.int64) + 1
    rv = _c(A.indices, np.int64) + 1
    nz = _c(A.data, np.float64)
    rhs = _c(rhs, np.float64)
    bd = _c(bdnode, np.int64).ravel()
    bv = _c(bdval, np.float64).ravel()
    if bd.size != bv.size:
        raise AdFemError(_lib.ERR_INVALID, "length(bdnode) must equal length(bdval)")
    L = _lib_()
    onnz = ctypes.c_longlong()
    check(L.adfem_dirichlet_csc(n, ptr(cp), ptr(rv), ptr(nz), ptr(rhs), ptr(bd), bd.size, ptr(bv), int(keep_zeros),
                                None, None, None, ctypes.byref(onnz), None), "impose_Dirichlet_boundary_conditions")
    ocp = np.empty(n + 1, np.int64)
    orv = np.empty(onnz.value, np.int64)
    onz = np.empty(onnz.value)
    orhs = np.empty(n)
    check(L.adfem_dirichlet_csc(n, ptr(cp), ptr(rv), ptr(nz), ptr(rhs), ptr(bd), bd.size, ptr(bv), int(keep_zeros),
                                ptr(ocp), ptr(orv), ptr(onz), ctypes.byref(onnz), ptr(orhs)),
          "impose_Dirichlet_boundary_conditions")
    return _csc(onz, ocp, orv, n), orhs


def impose_Dirichlet_coo(indices, vv, n, rhs, bdnode, bdval):
    """SparseTensor arm (ImposeDirichlet op): indices (N,2) 0-based; returns (oindices, ov, orhs)."""
    idx = _c(indices, np.int64).reshape(-1)
    vv = _c(vv, np.float64)
    rhs = _c(rhs, np.float64)
    bd = _c(bdnode, np.int64).ravel()
    bv = _c(bdval, np.float64).ravel()
    L = _lib_()
    cnt = ctypes.c_longlong()
    check(L.adfem_dirichlet_coo(ptr(idx), ptr(vv), vv.size, ptr(bd), bd.size, ptr(rhs), ptr(bv), n, None, None, None,
                                ctypes.byref(cnt)), "impose_Dirichlet (COO)")
    oi = np.empty(2 * cnt.value, np.int64)
    ov = np.empty(cnt.value)
    orhs = np.empty(n)
    check(L.adfem_dirichlet_coo(ptr(idx), ptr(vv), vv.size, ptr(bd), bd.size, ptr(rhs), ptr(bv), n, ptr(oi), ptr(ov),
                                ptr(orhs), ctypes.byref(cnt)), "impose_Dirichlet (COO)")
    return oi.reshape(-1, 2), ov, orhs


def impose_Dirichlet_coo_backward(grad_vv, grad_rhs, indices, vv, n, bdnode, bdval):
    idx = _c(indices, np.int64).reshape(-1)
    vv = _c(vv, np.float64)
    g = _c(grad_vv, np.float64)
    gr = _c(grad_rhs, np.float64)
    bd = _c(bdnode, np.int64).ravel()
    bv = _c(bdval, np.float64).ravel()
    gvi = np.empty(vv.size)
    gri = np.empty(n)
    gb = np.empty(bd.size)
    check(_lib_().adfem_dirichlet_coo_backward(ptr(g), ptr(gr), ptr(idx), ptr(vv), vv.size, ptr(bd), bd.size, ptr(bv),
                                               n, ptr(gvi), ptr(gri), ptr(gb)), "impose_Dirichlet backward (COO)")
    return gvi, gri, gb


def solver_opts(precision: str = "fp64", rtol: float = 1e-12, max_iter: int = 200000, ru_delta: float = 0.1,
                chunk: int = 32, warm_start: bool = False) -> SolverOpts:
    o = SolverOpts()
    _lib_().adfem_solver_opts_default(ctypes.byref(o))
    o.rtol = rtol
    o.max_iter = max_iter
    o.precision = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}[precision]
    o.ru_delta = ru_delta
    o.chunk = chunk
    o.warm_start = int(warm_start)
    return o


def solve(K, F, precision: str = "fp64", rtol: float = 1e-12, max_iter: int = 200000, return_stats: bool = False,
          u0=None):
    """``K\\F`` for a symmetric positive definite sparse K (GPU Jacobi-CG); ``u0`` warm-starts."""
    K = sp.csc_matrix(K)
    K.sort_indices()
    n = K.shape[0]
    cp = _c(K.indptr, np.int64) + 1
    rv = _c(K.indices, np.int64) + 1
    nz = _c(K.data, np.float64)
    F = _c(F, np.float64)
    u = np.zeros(n) if u0 is None else np.array(u0, dtype=np.float64, copy=True)
    o = solver_opts(precision, rtol, max_iter, warm_start=u0 is not None)
    st = SolverStats()
    check(_lib_().adfem_csc_solve(n, ptr(cp), ptr(rv), ptr(nz), ptr(F), ptr(u), ctypes.byref(o), ctypes.byref(st)),
          "solve")
    return (u, st) if return_stats else u


from .server import Server  # noqa: E402
from .system import ElasticitySystem, PoissonSystem  # noqa: E402

__all__ += ["PoissonSystem", "ElasticitySystem", "Server"]
