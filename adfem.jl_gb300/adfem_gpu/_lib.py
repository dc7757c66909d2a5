"""ctypes binding of libadfem_gpu.so (the C ABI declared in include/adfem_gpu.h).

The library is built in-tree (adfem.jl_gb300/build.py) and loaded from
adfem.jl_gb300/lib.  There is no fallback: if the library is missing the
import of any compute entry point raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "lib", "libadfem_gpu.so")

c_p = ctypes.c_void_p
c_i = ctypes.c_int
c_ll = ctypes.c_longlong
c_d = ctypes.c_double
c_pp = ctypes.POINTER(ctypes.c_void_p)


class SolverOpts(ctypes.Structure):
    _fields_ = [("rtol", c_d), ("max_iter", c_i), ("precision", c_i), ("ru_delta", c_d), ("chunk", c_i),
                ("warm_start", c_i)]


class SolverStats(ctypes.Structure):
    _fields_ = [("iterations", c_i), ("updates", c_i), ("relres", c_d), ("ms", c_d), ("status", c_i),
                ("launches", c_ll)]


class SolverInfo(ctypes.Structure):
    _fields_ = [("rows", c_ll), ("stored", c_ll), ("uniform_entries", c_ll), ("slices", c_ll), ("band", c_ll),
                ("banded", c_i), ("blocks", c_i), ("rows_per_block", c_ll), ("ring", c_i), ("renumbered", c_i),
                ("banded_fp64", c_i), ("fp64_tile_rows", c_i), ("ring_stages", c_i),
                ("assembly_pairs", c_i)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", c_ll), ("workers", c_i), ("max_queue", c_i), ("opts", SolverOpts),
                ("pack_max_dof", c_i), ("pack_max", c_i)]


class Request(ctypes.Structure):
    _fields_ = [("mesh", c_p), ("kind", c_i), ("in_", c_p * 4), ("bd", c_p), ("nbd", c_ll), ("bdval", c_p),
                ("obs", c_p), ("nobs", c_ll), ("uobs", c_p), ("u", c_p), ("grad", c_p), ("deadline_ms", c_d),
                ("warm_start", c_i), ("precision", c_i)]


class Response(ctypes.Structure):
    _fields_ = [("status", c_i), ("iterations", c_i), ("adjoint_iterations", c_i), ("relres", c_d), ("loss", c_d),
                ("queue_ms", c_d), ("run_ms", c_d), ("total_ms", c_d), ("message", ctypes.c_char * 160),
                ("packed", c_i)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", c_ll), ("completed", c_ll), ("rejected", c_ll), ("timeouts", c_ll), ("failed", c_ll),
                ("cache_hits", c_ll), ("cache_misses", c_ll), ("evictions", c_ll), ("resident_systems", c_ll),
                ("device_bytes", c_ll), ("p50_ms", c_d), ("p99_ms", c_d), ("mean_ms", c_d), ("max_ms", c_d),
                ("p50_queue_ms", c_d), ("p99_queue_ms", c_d), ("packs", c_ll), ("packed_requests", c_ll)]


OK = 0
ERR_INVALID = 1
ERR_CUDA = 2
ERR_NOMEM = 3
ERR_NOT_CONVERGED = 4
ERR_BREAKDOWN = 5
ERR_NO_MESH = 6
ERR_NONFINITE = 7
ERR_UNSUPPORTED = 8
ERR_BUSY = 9
ERR_TIMEOUT = 10
PREC_FP64 = 0
PREC_MIXED = 1
SYS_POISSON = 0
SYS_ELASTICITY = 1

# name -> (restype, argtypes)
SIGNATURES = {
    "adfem_status_string": (ctypes.c_char_p, [c_i]),
    "adfem_last_error": (ctypes.c_char_p, []),
    "adfem_version": (ctypes.c_char_p, []),
    "adfem_debug_fail_alloc": (c_i, [c_ll]),
    "adfem_debug_check_code": (c_i, []),
    "init_nnfem_mesh": (ctypes.POINTER(c_ll), [c_p, c_i, c_p, c_i, c_i, c_i, c_i, c_p]),
    "mfem_get_ngauss": (c_i, []),
    "mfem_get_gauss": (None, [c_p, c_p]),
    "mfem_get_gauss_weights": (None, [c_p]),
    "mfem_get_area": (None, [c_p]),
    "mfem_get_elem_ndof": (c_i, []),
    "mfem_get_ndof": (c_i, []),
    "mfem_get_connectivity": (None, [c_p]),
    "mfem_get_element_to_vertices": (None, [c_p]),
    "FemLaplaceScalar_forward_Julia": (None, [c_p, c_p, c_p]),
    "FemSourceScalar_forward_Julia": (None, [c_p, c_p]),
    "ComputeFemStiffnessMatrixMfem_forward_Julia": (None, [c_p, c_p, c_p]),
    "FemLaplaceScalar_backward": (None, [c_p, c_p, c_p, c_p, c_p]),
    "FemSourceScalar_backward": (None, [c_p, c_p, c_p, c_p]),
    "ComputeFemStiffnessMatrixMfem_backward": (None, [c_p, c_p]),
    "ComputeFemMassMatrix1_forward": (None, [c_p, c_p, c_p]),
    "ComputeFemMassMatrix1_backward": (None, [c_p, c_p, c_p, c_p]),
    "FemToGaussPointsMfem_Julia": (None, [c_p, c_p]),
    "FemToGaussPointsMfem_forward": (None, [c_p, c_p]),
    "FemToGaussPointsMfem_backward": (None, [c_p, c_p, c_p, c_p]),
    "DofToGaussPointsMfem_forward_Julia": (None, [c_p, c_p]),
    "DofToGaussPointsMfem_forward": (None, [c_p, c_p]),
    "DofToGaussPointsMfem_backward": (None, [c_p, c_p, c_p, c_p]),
    "pcl_FemLaplaceScalar_Jacobian": (None, [c_p]),
    "pcl_ImposeDirichlet": (None, [c_p, c_p, c_p, c_i, c_i]),
    "PlaneStrainMatrix_forward": (None, [c_p, c_p, c_p, c_i]),
    "PlaneStrainMatrix_backward": (None, [c_p, c_p, c_p, c_p, c_p, c_i]),
    "PlaneStressMatrix_forward": (None, [c_p, c_p, c_p, c_i]),
    "PlaneStressMatrix_backward": (None, [c_p, c_p, c_p, c_p, c_p, c_i]),
    "adfem_mesh_create": (c_i, [c_p, c_ll, c_p, c_ll, c_i, c_pp]),
    "adfem_mesh_destroy": (c_i, [c_p]),
    "adfem_mesh_sizes": (c_i, [c_p, c_p, c_p, c_p, c_p]),
    "adfem_set_current_mesh": (c_i, [c_p]),
    "adfem_current_mesh": (c_p, []),
    "adfem_mesh_pattern": (c_i, [c_p, c_p, c_p]),
    "adfem_mesh_pattern_elasticity": (c_i, [c_p, c_p, c_p]),
    "adfem_mesh_bcnode": (c_i, [c_p, c_p, c_p]),
    "adfem_mesh_gauss_nodes": (c_i, [c_p, c_p, c_p]),
    "adfem_mesh_elements": (c_i, [c_p, c_p]),
    "adfem_mesh_area": (c_i, [c_p, c_p]),
    "adfem_mesh_edges": (c_i, [c_p, c_p, c_p]),
    "adfem_mesh_space": (c_i, [c_p, c_p, c_p, c_p, c_p, c_p]),
    "adfem_mesh_connectivity": (c_i, [c_p, c_p]),
    "adfem_mesh_gauss_weights": (c_i, [c_p, c_p]),
    "adfem_mass_csc": (c_i, [c_p, c_p, c_ll, c_p]),
    "adfem_mass_csr_d": (c_i, [c_p, c_p, c_p, c_p]),
    "adfem_mass_coo_d": (c_i, [c_p, c_p, c_p, c_p, c_p]),
    "adfem_mass_coo_backward_d": (c_i, [c_p, c_p, c_p, c_p]),
    "adfem_pcl_laplace_jacobian": (c_i, [c_p, c_p]),
    "adfem_pcl_laplace_jacobian_d": (c_i, [c_p, c_p, c_p]),
    "adfem_pcl_dirichlet": (c_i, [c_p, c_ll, c_p, c_ll, c_ll, c_p, c_p]),
    "adfem_fem_to_gauss": (c_i, [c_p, c_p, c_ll, c_p]),
    "adfem_dof_to_gauss": (c_i, [c_p, c_p, c_ll, c_p]),
    "adfem_fem_to_gauss_d": (c_i, [c_p, c_p, c_p, c_p]),
    "adfem_fem_to_gauss_backward_d": (c_i, [c_p, c_p, c_p, c_ll, c_i, c_p]),
    "adfem_dof_to_gauss_d": (c_i, [c_p, c_p, c_p, c_p]),
    "adfem_dof_to_gauss_backward_d": (c_i, [c_p, c_p, c_p, c_ll, c_i, c_p]),
    "adfem_laplace_csc": (c_i, [c_p, c_p, c_ll, c_p]),
    "adfem_laplace_csr_d": (c_i, [c_p, c_p, c_p, c_p]),
    "adfem_laplace_coo_d": (c_i, [c_p, c_p, c_p, c_p, c_p]),
    "adfem_laplace_coo_backward_d": (c_i, [c_p, c_p, c_p, c_p]),
    "adfem_source": (c_i, [c_p, c_p, c_ll, c_p, c_i]),
    "adfem_source_d": (c_i, [c_p, c_p, c_p, c_i, c_p]),
    "adfem_source_backward_d": (c_i, [c_p, c_p, c_p, c_p]),
    "adfem_stiffness_csc": (c_i, [c_p, c_p, c_ll, c_p]),
    "adfem_stiffness_csr_d": (c_i, [c_p, c_p, c_p, c_p]),
    "adfem_stiffness_coo_d": (c_i, [c_p, c_p, c_p, c_p, c_p]),
    "adfem_stiffness_coo_backward_d": (c_i, [c_p, c_p, c_p, c_p]),
    "adfem_plane_strain_d": (c_i, [c_i, c_ll, c_p, c_p, c_p, c_p]),
    "adfem_plane_strain_backward_d": (c_i, [c_i, c_ll, c_p, c_p, c_p, c_p, c_p, c_p]),
    "adfem_dirichlet_csc": (c_i, [c_ll, c_p, c_p, c_p, c_p, c_p, c_ll, c_p, c_i, c_p, c_p, c_p, c_p, c_p]),
    "adfem_dirichlet_coo": (c_i, [c_p, c_p, c_ll, c_p, c_ll, c_p, c_p, c_ll, c_p, c_p, c_p, c_p]),
    "adfem_dirichlet_coo_backward": (c_i, [c_p, c_p, c_p, c_p, c_ll, c_p, c_ll, c_p, c_ll, c_p, c_p, c_p]),
    "adfem_solver_opts_default": (None, [ctypes.POINTER(SolverOpts)]),
    "adfem_csc_solve": (c_i, [c_ll, c_p, c_p, c_p, c_p, c_p, ctypes.POINTER(SolverOpts),
                              ctypes.POINTER(SolverStats)]),
    "adfem_system_create": (c_i, [c_p, c_i, c_pp]),
    "adfem_system_destroy": (c_i, [c_p]),
    "adfem_system_set_dirichlet": (c_i, [c_p, c_p, c_ll, c_p]),
    "adfem_system_assemble_poisson_d": (c_i, [c_p, c_p, c_p, c_p]),
    "adfem_system_assemble_poisson_profiled_d": (c_i, [c_p, c_p, c_p, c_p, c_p]),
    "adfem_system_assemble_elasticity_d": (c_i, [c_p, c_p, c_p, c_p, c_p, c_p]),
    "adfem_system_solve_d": (c_i, [c_p, c_p, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats), c_p]),
    "adfem_system_adjoint_d": (c_i, [c_p, c_p, c_p, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats), c_p]),
    "adfem_system_grad_kappa_d": (c_i, [c_p, c_p, c_p, c_p, c_p]),
    "adfem_system_grad_E_d": (c_i, [c_p, c_p, c_p, c_p, c_p, c_p, c_p]),
    "adfem_system_apply_d": (c_i, [c_p, c_p, c_p, c_p]),
    "adfem_system_rhs_d": (c_i, [c_p, c_p, c_p]),
    "adfem_system_solve_profiled_d": (c_i, [c_p, c_p, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats), c_p,
                                            c_p, c_p]),
    "adfem_system_solver_info": (c_i, [c_p, ctypes.POINTER(SolverInfo)]),
    "adfem_system_solve_packed_d": (c_i, [c_p, c_i, c_p, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats),
                                          c_p]),
    "adfem_system_adjoint_packed_d": (c_i, [c_p, c_i, c_p, c_p, ctypes.POINTER(SolverOpts),
                                            ctypes.POINTER(SolverStats), c_p]),
    "adfem_server_config_default": (None, [ctypes.POINTER(ServerConfig)]),
    "adfem_server_create": (c_i, [ctypes.POINTER(ServerConfig), c_pp]),
    "adfem_server_destroy": (c_i, [c_p]),
    "adfem_server_submit": (c_i, [c_p, ctypes.POINTER(Request), ctypes.POINTER(c_ll)]),
    "adfem_server_wait": (c_i, [c_p, c_ll, c_d, ctypes.POINTER(Response)]),
    "adfem_server_get_stats": (c_i, [c_p, ctypes.POINTER(ServerStats)]),
    "adfem_server_reset_stats": (c_i, [c_p]),
    "adfem_poisson_solve": (c_i, [c_p, c_p, c_p, c_p, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats)]),
    "adfem_csr_pcg_noalloc_d": (c_i, [c_i, c_p, c_p, c_p, c_p, c_p, c_d, c_i, c_p, c_p, c_p]),
}


class AdFemError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


_LIB = None


def load():
    """Load libadfem_gpu.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libadfem_gpu.so not built: run `python adfem.jl_gb300/build.py` "
                              "(or __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def check(status: int, what: str = ""):
    if status != OK:
        L = load()
        msg = L.adfem_last_error().decode() or L.adfem_status_string(status).decode()
        raise AdFemError(status, (what + ": " if what else "") + msg)
    return status


def ptr(a):
    """Raw pointer of a numpy array or torch tensor (None -> NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


def stream_ptr(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return ctypes.c_void_p(stream.cuda_stream)
    return ctypes.c_void_p(int(stream))
