"""The Python request-server wrapper (adfem_gpu.Server) on CPU, against a stand-in for the
library's adfem_server_* entry points: requests are marshalled into the C request struct,
tickets map back to their output arrays, and the optional JSONL trace gets one line per
completed request with the request's description and the library's response.  (The
serving loop itself runs on the GPU: tests/test_server_gpu.py.)"""
import ctypes
import json
import types

import numpy as np
import pytest


class FakeServerLib:
    """Implements the adfem_server_* calls the wrapper makes; `wait` answers with a
    response derived from the submitted request."""

    def __init__(self):
        self.requests = {}
        self.next = 41
        self.destroyed = False

    def adfem_solver_opts_default(self, o):
        o._obj.rtol, o._obj.max_iter, o._obj.ru_delta, o._obj.chunk = 1e-12, 200000, 0.1, 32
        return None

    def adfem_server_config_default(self, cfg):
        return None

    def adfem_server_create(self, cfg, out):
        self.cfg = cfg._obj
        out._obj.value = 1234
        return 0

    def adfem_server_submit(self, h, req, ticket):
        r = req._obj
        self.next += 1
        self.requests[self.next] = {"kind": r.kind, "nbd": r.nbd, "nobs": r.nobs, "precision": r.precision,
                                    "u": r.u}
        ticket._obj.value = self.next
        return 0

    def adfem_server_wait(self, h, ticket, timeout_ms, resp):
        q = self.requests.pop(ticket)
        out = resp._obj
        out.status = 0
        out.iterations = 7 * ticket
        out.adjoint_iterations = 3 if q["nobs"] else 0
        out.relres = 1e-11
        out.queue_ms, out.run_ms, out.total_ms = 0.5, 2.0, 2.5
        out.packed = int(q["kind"] == 0)
        out.message = b""
        # the library writes the solution through the request's u pointer
        ctypes.memmove(q["u"], np.full(4, float(ticket)).ctypes.data, 8)
        return 0

    def adfem_server_destroy(self, h):
        self.destroyed = True
        return 0


@pytest.fixture
def fake(monkeypatch):
    from adfem_gpu import _lib

    lib = FakeServerLib()
    monkeypatch.setattr(_lib, "_LIB", lib)
    monkeypatch.setattr(_lib, "load", lambda: lib)
    return lib


def test_requests_round_trip_and_trace(fake, tmp_path):
    from adfem_gpu import Server, _lib

    mesh = types.SimpleNamespace(handle=ctypes.c_void_p(99), nelem=2, nnode=4)
    ng = 3 * mesh.nelem
    path = tmp_path / "trace.jsonl"
    srv = Server(precision="fp64", rtol=1e-10, trace=str(path))
    assert fake.cfg.opts.rtol == 1e-10 and fake.cfg.opts.precision == _lib.PREC_FP64
    t1 = srv.submit(mesh, _lib.SYS_POISSON, (np.ones(ng), np.zeros(ng)), bd=[1, 2])
    t2 = srv.submit(mesh, _lib.SYS_ELASTICITY, [np.ones(ng)] * 4, bd=[1, 5], obs=[3], uobs=[0.1],
                    precision="mixed")
    assert fake.requests[t2]["nobs"] == 1 and fake.requests[t2]["precision"] == _lib.PREC_MIXED
    r2, u2, g2 = srv.wait(t2)
    r1, u1, g1 = srv.wait(t1)
    assert r1["status"] == 0 and r1["iterations"] == 7 * t1 and g1 is None
    assert u1.shape == (4,) and u1[0] == t1 and u2.shape == (8,) and u2[0] == t2 and g2.shape == (ng,)
    srv.close()
    assert fake.destroyed
    lines = [json.loads(x) for x in path.read_text().splitlines()]
    assert [x["ticket"] for x in lines] == [t2, t1]
    assert lines[0]["kind"] == "elasticity" and lines[0]["ndof"] == 8 and lines[0]["nobs"] == 1
    assert lines[0]["precision"] == "mixed" and lines[0]["adjoint_iterations"] == 3 and lines[0]["packed"] == 0
    assert lines[1]["kind"] == "poisson" and lines[1]["ndof"] == 4 and lines[1]["precision"] == "server"
    for x in lines:
        assert x["status"] == 0 and x["total_ms"] == 2.5 and x["message"] == ""


def test_no_trace_by_default_and_bad_requests(fake):
    from adfem_gpu import AdFemError, Server, _lib

    mesh = types.SimpleNamespace(handle=ctypes.c_void_p(99), nelem=2, nnode=4)
    with Server() as srv:
        with pytest.raises(AdFemError):
            srv.submit(mesh, _lib.SYS_POISSON, (np.ones(6),), bd=[1])  # one field missing
        with pytest.raises(AdFemError):
            srv.submit(mesh, _lib.SYS_POISSON, (np.ones(5), np.ones(5)), bd=[1])  # wrong length
        t = srv.submit(mesh, _lib.SYS_POISSON, (np.ones(6), np.ones(6)), bd=[1])
        r, u, _ = srv.wait(t)
        assert r["status"] == 0 and not srv._meta
