"""Serving loop (adfem_server_*): results, batch invariance, admission, deadlines.

Requests go through the library's worker threads and resident systems; their
solutions must equal the resident-system path run alone (same kernels, same options:
bit-identical) -- the per-system solver with packing off, the packed solver for small
mixed-precision requests with packing on -- match the direct solve within 1e-9, and not
depend on the other requests in flight.
"""
import numpy as np
import pytest

from adfem_gpu import synth

pytestmark = pytest.mark.gpu
RTOL = 1e-11


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


class Case:
    """A Poisson or elasticity request on a jittered m x m mesh, fields from `seed`."""

    def __init__(self, gpulib, m, kind, seed, obs_frac=0.0):
        self.m, self.kind, self.seed = m, kind, seed
        coords, elems = synth.jittered_square(m, seed=0)
        self.coords, self.elems = coords, elems
        self.mesh = gpulib.Mesh(coords, elems)
        g = gpulib.gauss_nodes(self.mesh)
        G = synth.fourier_field(g[:, 0], g[:, 1], seed=seed)
        if kind == gpulib._lib.SYS_POISSON:
            self.fields = (1.0 + np.exp(0.5 * G), 1e5 * (g[:, 0] + g[:, 1]))
            self.bd = gpulib.bcnode(self.mesh)
            ndof = self.mesh.nnode
        else:
            ng = g.shape[0]
            self.fields = (1e9 * np.exp(0.3 * G), np.full(ng, 0.3), np.zeros(ng), np.full(ng, -1e6))
            left = synth.left_edge_nodes(coords) + 1  # 1-based x DOFs; y DOFs follow after nv
            self.bd = np.concatenate([left, left + self.mesh.nnode])
            ndof = 2 * self.mesh.nnode
        self.obs = self.uobs = None
        if obs_frac > 0:
            rng = np.random.default_rng(seed + 100)
            self.obs = np.sort(rng.choice(np.arange(1, ndof + 1), max(1, int(obs_frac * ndof)), replace=False))
            self.uobs = rng.standard_normal(self.obs.size) * 1e-3

    def submit(self, srv, **kw):
        return srv.submit(self.mesh, self.kind, self.fields, self.bd, obs=self.obs, uobs=self.uobs, **kw)

    def system_solve(self, gpulib, precision="mixed"):
        """Same request through a resident system on the caller's stream (no server)."""
        import torch

        cls = gpulib.PoissonSystem if self.kind == gpulib._lib.SYS_POISSON else gpulib.ElasticitySystem
        S = cls(self.mesh)
        S.set_dirichlet(self.bd)
        t = [torch.tensor(f, device="cuda") for f in self.fields]
        S.assemble(*t)
        u = S.solve(precision=precision, rtol=RTOL)
        grad = None
        if self.obs is not None:
            uh = u.cpu().numpy()
            gu = np.zeros(uh.size)
            np.add.at(gu, self.obs - 1, 2 * (uh[self.obs - 1] - self.uobs))
            lam = S.adjoint(torch.tensor(gu, device="cuda"), precision=precision, rtol=RTOL)
            if self.kind == gpulib._lib.SYS_POISSON:
                grad = S.grad_kappa(u, lam).cpu().numpy()
            else:
                grad = S.grad_E(u, lam, t[0], t[1]).cpu().numpy()
        return u.cpu().numpy(), grad

    def packed_solve(self, gpulib):
        """Same request through a resident system and the packed solver (no server)."""
        import torch

        from adfem_gpu import system as SY

        cls = gpulib.PoissonSystem if self.kind == gpulib._lib.SYS_POISSON else gpulib.ElasticitySystem
        S = cls(self.mesh)
        S.set_dirichlet(self.bd)
        t = [torch.tensor(f, device="cuda") for f in self.fields]
        S.assemble(*t)
        (u,), _ = SY.solve_packed([S], rtol=RTOL)
        grad = None
        if self.obs is not None:
            uh = u.cpu().numpy()
            gu = np.zeros(uh.size)
            np.add.at(gu, self.obs - 1, 2 * (uh[self.obs - 1] - self.uobs))
            (lam,), _ = SY.adjoint_packed([S], [torch.tensor(gu, device="cuda")], rtol=RTOL)
            if self.kind == gpulib._lib.SYS_POISSON:
                grad = S.grad_kappa(u, lam).cpu().numpy()
            else:
                grad = S.grad_E(u, lam, t[0], t[1]).cpu().numpy()
        return u.cpu().numpy(), grad


def test_server_matches_resident_system_and_direct(oracle, gpulib):
    P, E = gpulib._lib.SYS_POISSON, gpulib._lib.SYS_ELASTICITY
    cases = [Case(gpulib, 16, P, 1), Case(gpulib, 40, P, 2, obs_frac=0.05), Case(gpulib, 24, E, 3),
             Case(gpulib, 20, E, 4, obs_frac=0.05)]
    with gpulib.Server(workers=4, precision="mixed", rtol=RTOL, pack_max_dof=-1) as srv:
        tickets = [c.submit(srv) for c in cases]
        out = [srv.wait(t) for t in tickets]
    for c, (resp, u, grad) in zip(cases, out):
        assert resp["status"] == 0, resp
        assert resp["packed"] == 0
        u_sys, g_sys = c.system_solve(gpulib)
        assert np.array_equal(u, u_sys)
        if c.obs is not None:
            assert resp["adjoint_iterations"] > 0
            assert np.array_equal(grad, g_sys)
            assert resp["loss"] == pytest.approx(float(np.sum((u[c.obs - 1] - c.uobs) ** 2)), rel=1e-12)
    # the Poisson cases against the oracle's direct solve
    for c, (resp, u, _) in zip(cases[:2], out[:2]):
        O = oracle.OracleMesh(c.coords, c.elems)
        B, r = oracle.dirichlet_csc(O.laplace_csc(c.fields[0]), O.source(c.fields[1]), c.bd, np.zeros(c.bd.size))
        assert rel(u, oracle.spsolve(B, r)) < 1e-9


@pytest.mark.parametrize("pack", [0, -1])
def test_server_batch_invariance(gpulib, pack):
    """A request's u and gradient are bit-identical alone and in a concurrent mix (packed
    with the other small requests, or on its own worker)."""
    P, E = gpulib._lib.SYS_POISSON, gpulib._lib.SYS_ELASTICITY
    x = Case(gpulib, 48, P, 7, obs_frac=0.02)
    with gpulib.Server(workers=1, rtol=RTOL, pack_max_dof=pack) as srv:
        r1, u1, g1 = srv.wait(x.submit(srv))
    mix = [Case(gpulib, m, P if i % 5 else E, 20 + i, obs_frac=0.02 if i % 2 else 0.0)
           for i, m in enumerate([16, 64, 24, 96, 32, 20, 80, 40, 12, 56])]
    with gpulib.Server(workers=8, rtol=RTOL, pack_max_dof=pack) as srv:
        tk = [c.submit(srv) for c in mix[:5]] + [x.submit(srv)] + [c.submit(srv) for c in mix[5:]]
        res = [srv.wait(t) for t in tk]
    r2, u2, g2 = res[5]
    assert all(r[0]["status"] == 0 for r in res), [(r[0]["status"], r[0]["message"]) for r in res]
    assert r1["status"] == 0, r1
    assert r1["iterations"] == r2["iterations"]
    assert r1["packed"] == r2["packed"] == (1 if pack == 0 else 0)
    assert np.array_equal(u1, u2) and np.array_equal(g1, g2)


def test_server_packs_small_requests(oracle, gpulib):
    """Small mixed-precision requests are solved in packed launches (one thread block per
    system); results equal the packed solver run alone and the direct solve; requests
    above pack_max_dof and FP64 requests keep the per-system solver."""
    P, E = gpulib._lib.SYS_POISSON, gpulib._lib.SYS_ELASTICITY
    cases = [Case(gpulib, m, P, 30 + i, obs_frac=0.03 if i % 2 else 0.0) for i, m in enumerate([12, 30, 50, 70])]
    cases += [Case(gpulib, 20, E, 40, obs_frac=0.03), Case(gpulib, 140, P, 41)]  # 19,881 DOFs: not packed
    with gpulib.Server(workers=6, rtol=RTOL, pack_max_dof=16384) as srv:
        tk = [c.submit(srv) for c in cases]
        res = [srv.wait(t) for t in tk]
        fp64 = srv.wait(cases[0].submit(srv, precision="fp64"))[0]
        st = srv.stats()
    for c, (resp, u, grad) in zip(cases[:5], res[:5]):
        assert resp["status"] == 0 and resp["packed"] == 1, resp
        u_p, g_p = c.packed_solve(gpulib)
        assert np.array_equal(u, u_p)
        if c.obs is not None:
            assert np.array_equal(grad, g_p)
    assert res[5][0]["status"] == 0 and res[5][0]["packed"] == 0
    assert fp64["status"] == 0 and fp64["packed"] == 0
    assert st["packed_requests"] == 5 and 1 <= st["packs"] <= 8
    for c, (resp, u, _) in zip(cases[:4], res[:4]):
        O = oracle.OracleMesh(c.coords, c.elems)
        B, r = oracle.dirichlet_csc(O.laplace_csc(c.fields[0]), O.source(c.fields[1]), c.bd, np.zeros(c.bd.size))
        assert rel(u, oracle.spsolve(B, r)) < 1e-9


def test_server_warm_start_and_resident_reuse(gpulib):
    c = Case(gpulib, 40, gpulib._lib.SYS_POISSON, 5)
    with gpulib.Server(workers=2, rtol=1e-10, pack_max_dof=-1) as srv:
        r0, u0, _ = srv.wait(c.submit(srv))
        r1, u1, _ = srv.wait(c.submit(srv, warm_start=True))
        st = srv.stats()
    assert r0["status"] == 0 and r1["status"] == 0
    assert r0["iterations"] > 0 and r1["iterations"] == 0  # same inputs: the warm start is the solution
    assert rel(u1, u0) < 1e-12
    assert st["cache_misses"] == 1 and st["cache_hits"] == 1 and st["completed"] == 2


def test_server_admission_and_eviction(gpulib):
    small = Case(gpulib, 8, gpulib._lib.SYS_POISSON, 1)
    big = Case(gpulib, 64, gpulib._lib.SYS_POISSON, 1)
    with gpulib.Server(hbm_budget_bytes=1 << 20, workers=1) as srv:
        r, _, _ = srv.wait(small.submit(srv))
        assert r["status"] == 0
        with pytest.raises(gpulib.AdFemError) as e:
            big.submit(srv)
        assert e.value.status == gpulib._lib.ERR_BUSY
        assert srv.stats()["rejected"] == 1
    # room for one 48x48 system but not two: the second mesh evicts the first
    a = Case(gpulib, 48, gpulib._lib.SYS_POISSON, 1)
    b = Case(gpulib, 48, gpulib._lib.SYS_POISSON, 2)
    b.mesh = gpulib.Mesh(*synth.jittered_square(48, seed=9))
    with gpulib.Server(hbm_budget_bytes=2_500_000, workers=1) as srv:
        ra = srv.wait(a.submit(srv))[0]
        rb = srv.wait(b.submit(srv))[0]
        st = srv.stats()
    assert ra["status"] == 0 and rb["status"] == 0
    assert st["evictions"] == 1 and st["resident_systems"] == 1
    assert 0 < st["device_bytes"] <= 2_500_000


def test_server_deadline_and_bad_requests(gpulib):
    slow = Case(gpulib, 160, gpulib._lib.SYS_POISSON, 3)
    quick = Case(gpulib, 8, gpulib._lib.SYS_POISSON, 3)
    with gpulib.Server(workers=1, precision="fp64", rtol=1e-12) as srv:
        t0 = slow.submit(srv)
        t1 = quick.submit(srv, deadline_ms=1e-3)  # waits behind the slow request
        r0 = srv.wait(t0)[0]
        r1 = srv.wait(t1)[0]
        assert r0["status"] == 0
        assert r1["status"] == gpulib._lib.ERR_TIMEOUT
        with pytest.raises(gpulib.AdFemError) as e:
            srv.submit(quick.mesh, gpulib._lib.SYS_POISSON, quick.fields, quick.bd, obs=[10**9], uobs=[0.0])
        assert e.value.status == gpulib._lib.ERR_INVALID
        st = srv.stats()
    assert st["timeouts"] == 1 and st["completed"] == 1
    assert st["p50_ms"] > 0 and st["p99_ms"] >= st["p50_ms"]
