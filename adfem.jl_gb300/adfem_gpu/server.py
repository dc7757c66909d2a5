"""Request server over libadfem_gpu's serving loop (adfem_server_* in include/adfem_gpu.h).

A request is one forward solve on a mesh (Poisson: kappa, f; plane-strain elasticity:
E, nu, fx, fy, all at the Gauss points) with its Dirichlet DOFs, optionally with
observations whose misfit gradient with respect to kappa (or E) comes back through
the adjoint.  Worker threads in the library run requests concurrently on their own
CUDA streams and keep the systems of recently used meshes resident; see the C header
for admission and eviction.  Host numpy arrays in and out.

Tracing: ``Server(trace=path_or_file)`` appends one JSON line per completed request (when
``wait`` returns it): ticket, kind, DOFs, observation count, requested precision, and the
library's response (status, iterations, residual, misfit, queue / run / total ms, whether it
ran in a packed launch, message).
"""
from __future__ import annotations

import ctypes
import json

import numpy as np

from . import _lib
from ._lib import AdFemError, check, ptr


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Server:
    def __init__(self, hbm_budget_bytes: int = 0, workers: int = 8, max_queue: int = 0, precision: str = "mixed",
                 rtol: float = 1e-10, max_iter: int = 200000, ru_delta: float = 0.1, chunk: int = 32,
                 pack_max_dof: int = 0, pack_max: int = 0, trace=None):
        """pack_max_dof: mixed-precision requests up to this many DOFs are solved in packed
        launches (0: the library default, 16384; -1: never); pack_max: systems per pack;
        trace: a path (opened for appending) or a writable text file for the per-request
        JSON lines, None for no trace."""
        from . import solver_opts

        L = _lib.load()
        cfg = _lib.ServerConfig()
        L.adfem_server_config_default(ctypes.byref(cfg))
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.workers = int(workers)
        cfg.max_queue = int(max_queue)
        cfg.opts = solver_opts(precision, rtol, max_iter, ru_delta, chunk)
        cfg.pack_max_dof = int(pack_max_dof)
        cfg.pack_max = int(pack_max)
        h = ctypes.c_void_p()
        check(L.adfem_server_create(ctypes.byref(cfg), ctypes.byref(h)), "server_create")
        self._h = h
        self._live = {}  # ticket -> arrays the request points at (kept alive until it completes)
        self._meta = {}  # ticket -> request description for the trace
        self._trace_owned = isinstance(trace, str)
        self._trace = open(trace, "a") if self._trace_owned else trace

    # ------------------------------------------------------------------ requests
    def submit(self, mesh, kind: int, fields, bd, bdval=None, obs=None, uobs=None, deadline_ms: float = 0.0,
               warm_start: bool = False, precision=None) -> int:
        """Queue one request; returns its ticket.  ``kind``: ``_lib.SYS_POISSON`` with
        ``fields = (kappa, f)`` or ``_lib.SYS_ELASTICITY`` with ``(E, nu, fx, fy)``; ``bd``
        1-based DOF ids; ``obs`` 1-based DOF ids with observed values ``uobs``."""
        nin = 4 if kind == _lib.SYS_ELASTICITY else 2
        if len(fields) != nin:
            raise AdFemError(_lib.ERR_INVALID, "request needs %d input fields" % nin)
        ng = 3 * mesh.nelem
        ndof = mesh.nnode * (2 if kind == _lib.SYS_ELASTICITY else 1)
        ins = [_f64(f) for f in fields]
        for a in ins:
            if a.size != ng:
                raise AdFemError(_lib.ERR_INVALID, "input fields must have %d entries (one per Gauss point)" % ng)
        bd = np.ascontiguousarray(bd, dtype=np.int64).ravel()
        bv = None if bdval is None else _f64(bdval).ravel()
        u = np.empty(ndof)
        keep = [ins, bd, bv, u]
        r = _lib.Request()
        r.mesh = mesh.handle
        r.kind = kind
        for i, a in enumerate(ins):
            r.in_[i] = a.ctypes.data
        r.bd = bd.ctypes.data if bd.size else None
        r.nbd = bd.size
        r.bdval = None if bv is None else bv.ctypes.data
        grad = None
        if obs is not None and len(obs) > 0:
            ob = np.ascontiguousarray(obs, dtype=np.int64).ravel()
            uo = _f64(uobs).ravel()
            if uo.size != ob.size:
                raise AdFemError(_lib.ERR_INVALID, "obs and uobs lengths differ")
            grad = np.empty(ng)
            r.obs, r.nobs, r.uobs, r.grad = ob.ctypes.data, ob.size, uo.ctypes.data, grad.ctypes.data
            keep += [ob, uo, grad]
        r.u = u.ctypes.data
        r.deadline_ms = float(deadline_ms)
        r.warm_start = int(bool(warm_start))
        r.precision = -1 if precision is None else {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}[precision]
        t = ctypes.c_longlong()
        check(_lib.load().adfem_server_submit(self._h, ctypes.byref(r), ctypes.byref(t)), "server_submit")
        self._live[t.value] = (keep, u, grad)
        if self._trace is not None:
            self._meta[t.value] = {"kind": "elasticity" if kind == _lib.SYS_ELASTICITY else "poisson",
                                   "ndof": int(ndof), "nobs": int(r.nobs), "precision": precision or "server"}
        return t.value

    def wait(self, ticket: int, timeout_ms: float = -1.0):
        """(response dict, u, grad or None) once the request completed; raises
        AdFemError(ERR_TIMEOUT) if it is still running after timeout_ms."""
        resp = _lib.Response()
        check(_lib.load().adfem_server_wait(self._h, ticket, float(timeout_ms), ctypes.byref(resp)), "server_wait")
        _, u, grad = self._live.pop(ticket)
        out = {name: getattr(resp, name) for name, _ in resp._fields_}
        out["message"] = out["message"].decode(errors="replace")
        if self._trace is not None:
            rec = {"ticket": int(ticket)}
            rec.update(self._meta.pop(ticket, {}))
            rec.update(out)
            self._trace.write(json.dumps(rec) + "\n")
            self._trace.flush()
        return out, u, grad

    def stats(self) -> dict:
        s = _lib.ServerStats()
        check(_lib.load().adfem_server_get_stats(self._h, ctypes.byref(s)), "server_stats")
        return {name: getattr(s, name) for name, _ in s._fields_}

    def reset_stats(self):
        check(_lib.load().adfem_server_reset_stats(self._h), "server_reset_stats")

    def close(self):
        if getattr(self, "_h", None) is not None and _lib._LIB is not None:
            _lib._LIB.adfem_server_destroy(self._h)
            self._h = None
            self._live.clear()
            self._meta.clear()
        if getattr(self, "_trace_owned", False) and self._trace is not None:
            self._trace.close()
            self._trace = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
