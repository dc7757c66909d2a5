#!/usr/bin/env python
"""Benchmark: Poisson forward (+adjoint) of AdFem's P1 path at 4M DOF on GB300.

Workload (one "step"): the 2000x2000-cell jittered unit square (8M triangles,
4,004,001 DOF), kappa = 1 + exp(sigma G) with G a 64-mode random Fourier field
(seed 1) and sigma set so max/min kappa = 1e3, f = 1e5 (x + y), u = 0 on the
boundary.  A step assembles the Laplace matrix and load vector, imposes the
Dirichlet condition (one fused pass) and solves with the mixed-precision
Jacobi-CG (FP32 inner iteration, FP64 residual replacement and stop test) to
the residual tolerance that gives <= 1e-10 relative error against the FP64
reference solution.  Inputs are resident in HBM; the working set (about 700 MB
of matrix and vectors) is larger than L2 (129 MB), so no flush is needed.

Printed: one JSON line (rank 0) with value = solves/s over all ranks, the
FP64-CG comparison, grads/s, roofline of the dominant kernel, the end-to-end
rate through the host-buffer C ABI call, the CPU baseline, SM clocks and the
serving workload ("serve": a stream of independent Poisson/elasticity requests of
16x16 to 1024x1024 cells through the library's request server, saturation
throughput and p50/p99 latency under open-loop Poisson arrivals).
``--impl reference`` times the CPU restatement of the reference path instead.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "adfem.jl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "solves/s & grads/s at 4M DOF, mixed vs FP64 @1e-10; serve p50/p99 ms"
UNIT = "solves/s"
# FP64 Jacobi-CG iterations this workload needs at the default rtol on GB300; the
# reference arm times a bounded number of CPU iterations and scales to this count.
FP64_ITERS_DEFAULT = 14346


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.th = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.th is not None:
            self.th.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for nm, v in zip(names, r[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- workload
def make_workload(m, seed_mesh=0, seed_field=1, contrast=1e3):
    """Mesh, Gauss points and the C3 fields (kappa on the device)."""
    import torch

    import adfem_gpu as A
    from adfem_gpu import synth

    coords, elems = synth.jittered_square(m, seed=seed_mesh)
    mesh = A.Mesh(coords, elems)
    g = A.gauss_nodes(mesh)
    gx = torch.tensor(g[:, 0], device="cuda")
    gy = torch.tensor(g[:, 1], device="cuda")
    G = synth.fourier_field(gx, gy, seed=seed_field)
    sigma = synth.contrast_sigma(G.cpu().numpy(), contrast)
    kappa = synth.lognormal_kappa(G, sigma).contiguous()
    f = (1e5 * (gx + gy)).contiguous()
    bd = A.bcnode(mesh)
    return mesh, coords, elems, kappa, f, bd, sigma


def spmv32_bytes(mesh_nent, n, nslices):
    # values (4 B) + int16 column deltas (2 B) per stored entry, slice pointers,
    # r and p_old gathered once, p_new and q written
    return 6 * mesh_nent + 4 * (nslices + 1) + 16 * n


def zcg_bytes(info):
    """Algorithmic bytes of one banded mixed iteration (k_zcg_iter), averaged over an even
    and an odd launch: per row Z, q^, P of the previous iteration read (12 B), Z, P, q^
    written (12 B), the diagonal (4 B), and the Y hi+lo pair read and written with
    P_{k-2} read on even launches only (20 B every other launch: 10 B); per stored entry
    its FP32 value (4 B) plus the int16 column delta outside slices with a stored pattern
    (2 B); slice pointer and pattern index per slice (8 B).  Halo re-reads are not counted."""
    return (38 * info["rows"] + 4 * info["stored"] + 2 * (info["stored"] - info["uniform_entries"])
            + 8 * info["slices"])


def profiled_traffic(kernel, m):
    """DRAM bytes per launch of `kernel` on the m x m workload (dram__bytes_read.sum +
    dram__bytes_write.sum of one ncu capture, averaged over the launches captured), from
    profiles/traffic.json, which records each figure with the command that measured it;
    None when no capture of that kernel and size is recorded."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
    except (OSError, ValueError):
        return None
    e = d.get(kernel)
    if not e or int(e.get("m", -1)) != int(m):
        return None
    return int(e["bytes_per_launch"])


def bench_config(m, world):
    """The workload description both arms print (same dict, so the lines compare)."""
    n = (m + 1) ** 2
    return {"workload": "poisson-%dx%d-jittered-%s-dof-contrast1e3" % (m, m, "4M" if m == 2000 else str(n)),
            "m": m, "dof": n, "nnz": n + 2 * (3 * m * m + 2 * m), "kappa_contrast": 1e3,
            "l2": "working set > L2 (no flush needed)", "parallelism": "single" if world == 1 else "replicas"}


def dcg_bytes(info):
    """Algorithmic bytes of one banded FP64 iteration (k_dcg_iter), averaged over an even and
    an odd launch: per row r, q, p of the previous iteration read (24 B) and r, p, q written
    (24 B), the correction z read and written with p_{k-2} read on even launches only (24 B
    every other launch: 12 B); per stored entry its FP64 value (8 B) plus the int16 column
    delta outside slices with a stored pattern (2 B); per slice its two offsets and its
    pattern index (12 B).  Halo re-reads are not counted."""
    return (60 * info["rows"] + 8 * info["stored"] + 2 * (info["stored"] - info["uniform_entries"])
            + 12 * info["slices"])


def dcg_flops(info):
    """FP64 operations of one banded FP64 iteration (an FMA counts 2): per stored entry the
    SpMV FMA; per row r_k and p_k (2 FMA), r.r, p.q and q.q (3 FMA) and half of the two-step
    z update (2 FMA every other launch)."""
    return 2 * info["stored"] + 2 * (2 + 3 + 1) * info["rows"]


def spmv64_bytes(mesh_nent, n, nslices):
    return 10 * mesh_nent + 4 * (nslices + 1) + 16 * n


def sell_entries(mesh):
    """Stored entries (incl. padding) of the sliced-ELL operator of the mesh's scalar pattern."""
    cp, rv = mesh.pattern()
    lens = np.diff(cp)
    n = lens.size
    ns = (n + 31) // 32
    pad = np.zeros(ns * 32, np.int64)
    pad[:n] = lens
    w = pad.reshape(ns, 32).max(axis=1)
    return int(32 * w.sum()), n, ns


# ----------------------------------------------------------------------------- CPU leg
def oracle_system(coords, elems, kappa, f, abs_sum=False):
    """The oracle's Array-arm pipeline on the full mesh (serial C restatement of the reference):
    unsummed COO of FemLaplaceScalar -> Julia sparse() CSC -> FemSourceScalar load -> CSC
    Dirichlet arm with u = 0 on bcnode.  The mesh geometry is set up first and not timed (the
    reference builds its mesh once); t_assembly_s times the per-solve part, on one core.
    abs_sum: also (untimed) the matrix of sums of |summand| per stored entry, the scale of
    the rounding any summation order of that entry can carry."""
    import oracle as O

    O.build()
    M = O.OracleMesh(coords, elems)
    bd = M.bcnode()
    t0 = time.perf_counter()
    idx, vv = M.laplace_coo(kappa)
    K = O.coo_to_csc(idx, vv, M.ndof)
    F = M.source(f)
    B, Fb = O.dirichlet_csc(K, F, bd, np.zeros(bd.size))
    t_asm = time.perf_counter() - t0
    Kabs = O.coo_to_csc(idx, np.abs(vv), M.ndof) if abs_sum else None
    del idx, vv
    return {"mesh": M, "K": K, "F": F, "B": B, "Fb": Fb, "bd": bd, "t_assembly_s": t_asm, "Kabs": Kabs}


def cpu_pcg_iter_s(B, b, iters, threads):
    """Seconds per Jacobi-PCG iteration of the oracle (FP64, `threads` pthreads) on B, timed
    over `iters` iterations from zero."""
    import oracle as O

    t0 = time.perf_counter()
    O.pcg(B, b, rtol=0.0, max_iter=iters, threads=threads)
    return (time.perf_counter() - t0) / iters


def matrix_parity(Kg, Ko, Kabs=None):
    """Entry-by-entry comparison of two CSC matrices of one pattern: pattern equality, the
    largest difference over the largest entry of its column (row-scaled; the matrices are
    symmetric), the largest elementwise relative difference over entries at least 1e-10 of
    their column's largest entry, and how many of those exceed 1e-12 (and how large they are
    relative to their column).  With Kabs (per entry, the sum of |summand| of the reference's
    COO duplicates): the largest difference over that sum, the rounding scale of a sum whose
    terms cancel (entries between two elements of a jittered mesh can nearly vanish)."""
    Kg, Ko = Kg.tocsc(), Ko.tocsc()
    Kg.sort_indices()
    Ko.sort_indices()
    same = Kg.shape == Ko.shape and np.array_equal(Kg.indptr, Ko.indptr) and np.array_equal(Kg.indices, Ko.indices)
    if not same:
        return {"pattern_equal": False}
    d = np.abs(Kg.data - Ko.data)
    a = np.abs(Ko.data)
    lens = np.diff(Ko.indptr)
    nzc = np.flatnonzero(lens)
    cmax = np.zeros(Ko.shape[1])
    cmax[nzc] = np.maximum.reduceat(a, Ko.indptr[nzc])
    colmax = np.repeat(cmax, lens)
    big = a >= 1e-10 * colmax
    rel = np.zeros_like(d)
    rel[big] = d[big] / a[big]
    over = rel > 1e-12
    out = {"pattern_equal": True, "nnz": int(Ko.nnz),
           "max_err_row_scaled": float(np.max(d / np.maximum(colmax, 1e-300))) if d.size else 0.0,
           "max_err_elementwise": float(rel.max()) if d.size else 0.0,
           "entries_compared_elementwise": int(big.sum()),
           "entries_over_1e-12_elementwise": int(over.sum()),
           "largest_such_entry_over_row_max": float(np.max(a[over] / colmax[over])) if over.any() else 0.0}
    if Kabs is not None:
        Kabs = Kabs.tocsc()
        Kabs.sort_indices()
        if np.array_equal(Kabs.indices, Ko.indices):
            out["max_err_over_abs_summand_sum"] = float(np.max(d / np.maximum(Kabs.data, 1e-300))) if d.size else 0.0
    return out


def vector_parity(g, o):
    d = np.abs(np.asarray(g) - np.asarray(o))
    a = np.abs(np.asarray(o))
    big = a >= 1e-10 * a.max()
    return {"max_err_scaled": float(d.max() / max(a.max(), 1e-300)),
            "max_err_elementwise": float(np.max(d[big] / a[big])) if big.any() else 0.0}


def residual_report(B, x, b, oracle_mod):
    """Residual of a solution against the oracle's operator, in doubled precision: relres in
    the solver's own measure (Jacobi-scaled 2-norm), plain relres, and the normwise backward
    error ||r||_inf / (|| |B| |x| ||_inf + ||b||_inf)."""
    r = oracle_mod.residual_dd(B, x, b)
    s = 1.0 / np.sqrt(B.diagonal())
    absbx = abs(B) @ np.abs(x)
    return r, {"relres_scaled": float(np.linalg.norm(s * r) / np.linalg.norm(s * b)),
               "relres": float(np.linalg.norm(r) / np.linalg.norm(b)),
               "backward_error": float(np.abs(r).max() / (absbx.max() + np.abs(b).max()))}


def accuracy_c3(A, S, mesh, coords, elems, kappa, f, u_ref, sols):
    """Independent CPU checks of the 4M-DOF workload against the oracle (run once, after the
    timed legs):
    (a) the oracle's full-size assembly (oracle_system), timed on one core;
    (b) entry-by-entry parity of the GPU's Array-arm outputs (compute_fem_laplace_matrix1,
        compute_fem_source_term1) with (a);
    (c) the residual of each GPU solution against (a) in doubled precision;
    (d) a forward-error estimate of the FP64 reference by one refinement step: the correction
        delta = B^-1 r_ref (r_ref from (c), solved on the GPU in FP64) estimates u* - u_ref,
        and every solution's error is measured against u_ref + delta.
    sols: {name: device solution}.  Returns (report, oracle system)."""
    import torch

    import oracle as O

    kap = kappa.cpu().numpy()
    fh = f.cpu().numpy()
    osys = oracle_system(coords, elems, kap, fh, abs_sum=True)
    B, Fb = osys["B"], osys["Fb"]
    Kg = A.compute_fem_laplace_matrix1(kap, mesh)
    Fg = A.compute_fem_source_term1(fh, mesh)
    rep = {"oracle": "serial C restatement: unsummed COO -> Julia sparse() CSC -> load -> CSC Dirichlet arm, "
                     "%d DOF, %d stored entries; residuals in doubled precision" % (B.shape[0], osys["K"].nnz),
           "matrix_parity": matrix_parity(Kg, osys["K"], osys["Kabs"]), "load_parity": vector_parity(Fg, osys["F"])}
    del Kg
    osys["Kabs"] = None
    ur = u_ref.cpu().numpy()
    r_ref, rr = residual_report(B, ur, Fb, O)
    delta = S.adjoint(torch.tensor(r_ref, device="cuda"), precision="fp64", rtol=1e-10).cpu().numpy()
    scale = float(np.abs(ur).max())
    rr["forward_error_estimate"] = float(np.abs(delta).max() / scale)
    rep["fp64_reference"] = rr
    for name, u in sols.items():
        uh = u.cpu().numpy()
        _, rs = residual_report(B, uh, Fb, O)
        rs["rel_err_vs_refined_reference"] = float(np.abs((uh - ur) - delta).max() / scale)
        rep[name] = rs
    return rep, osys


# ----------------------------------------------------------------------------- reference arm
def c3_fields_cpu(m, threads):
    """The C3 fields on the host (torch on the CPU threads, no GPU): mesh, Gauss points,
    kappa = 1 + exp(sigma G) with max/min = 1e3, f = 1e5 (x + y)."""
    import torch

    from adfem_gpu import synth

    import oracle as O

    torch.set_num_threads(threads)
    coords, elems = synth.jittered_square(m, seed=0)
    M = O.OracleMesh(coords, elems)
    g = M.gauss_nodes()
    G = synth.fourier_field(torch.from_numpy(g[:, 0].copy()), torch.from_numpy(g[:, 1].copy()), seed=1).numpy()
    sigma = synth.contrast_sigma(G, 1e3)
    return coords, elems, synth.lognormal_kappa(G, sigma), 1e5 * (g[:, 0] + g[:, 1])


def run_reference(args, rank, world):
    """The reference's CPU path (the oracle port; the reference itself cannot be built here):
    the full-size Array-arm assembly timed once, serially as in the reference, then each step
    = `ref_iters` Jacobi-PCG iterations on the full Dirichlet-imposed operator with every host
    thread, timed.  solves/s = 1 / (assembly + fp64_iters x per-iteration time): the assembly is
    measured whole, only the iteration count is extrapolated (factor printed)."""
    if rank != 0:
        return 0
    import scipy.sparse as sp

    threads = os.cpu_count() or 1
    coords, elems, kappa, f = c3_fields_cpu(args.m, threads)
    osys = oracle_system(coords, elems, kappa, f)
    B = sp.csr_matrix(osys["B"])
    b = osys["Fb"]
    steps = []
    for i in range(args.warmup + args.steps):
        t = cpu_pcg_iter_s(B, b, args.ref_iters, threads)
        if i >= args.warmup:
            steps.append(t * args.ref_iters)
    t_step = statistics.median(steps)
    t_iter = t_step / args.ref_iters
    t_solve = osys["t_assembly_s"] + args.fp64_iters * t_iter
    v = 1.0 / t_solve
    sample = ("oracle port of the reference path: full %dx%d assembly (COO -> Julia sparse() CSC -> load -> "
              "Dirichlet) timed once on 1 core (%.2f s), plus Jacobi-PCG on the full %d-DOF operator with %d threads, "
              "%d iterations per step (%.1f ms per iteration), extrapolated to the %d FP64 iterations the solve needs"
              % (args.m, args.m, osys["t_assembly_s"], B.shape[0], threads, args.ref_iters, 1e3 * t_iter,
                 args.fp64_iters))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(args.m, world),
            "impl": "reference",
            "step": "%d Jacobi-PCG iterations (ms_per_step); one solve = assembly + %d iterations"
                    % (args.ref_iters, args.fp64_iters),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "t_assembly_s": osys["t_assembly_s"], "t_iter_s": t_iter,
                             "extrapolated": {"assembly_x": 1, "iters_x": args.fp64_iters / args.ref_iters}},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------- replicas
def max_over_ranks(dist, x):
    """Largest value of x over all ranks (the slowest replica sets the job's time); the
    tensor lives on the GPU for NCCL and on the CPU for gloo."""
    if dist is None:
        return float(x)
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard(items, rank, world):
    """Request-level dispatch to replicas: rank r takes items r, r + world, ..."""
    return items[rank::world]


def replica_rate(world, units_per_rank, seconds):
    """Whole-job rate: all ranks' units over the slowest rank's time."""
    return world * units_per_rank / seconds


# ----------------------------------------------------------------------------- serving (C5)
SERVE_SIZES = sorted({int(round(16 * 2 ** (k / 4))) for k in range(25)})  # 16 .. 1024, ratio 2^(1/4)


class ServeCatalog:
    """Meshes of the serving workload, prepared before any timing: per mesh size m (jittered
    m x m square, seed 0) the Dirichlet sets (Poisson: boundary; elasticity: left edge
    clamped in x and y), 1% observation DOFs and the shared fields (f = 1e5(x+y); nu = 0.3,
    body force (0, -1e6)).  Each request's own field (kappa = 1 + exp(0.5 G) or
    E = 1e9 exp(0.3 G), G a unit-variance 64-mode Fourier field) is drawn from the request's
    seed by `fields`, also before the timing."""

    def __init__(self, A, sizes):
        import torch
        from adfem_gpu import synth

        self.A = A
        self.sizes = sizes
        self.items = {}
        for m in sizes:
            coords, elems = synth.jittered_square(m, seed=0)
            mesh = A.Mesh(coords, elems)
            g = torch.tensor(A.gauss_nodes(mesh), device="cuda")
            ng = g.shape[0]
            nv = mesh.nnode
            left = synth.left_edge_nodes(coords) + 1
            rng = np.random.default_rng(m)
            it = {"mesh": mesh, "ndof": (nv, 2 * nv), "g": g,
                  "bd": (A.bcnode(mesh), np.concatenate([left, left + nv])),
                  "f": (1e5 * (g[:, 0] + g[:, 1])).cpu().numpy(),
                  "nu": np.full(ng, 0.3), "fx": np.zeros(ng), "fy": np.full(ng, -1e6), "obs": []}
            for nd in it["ndof"]:
                ob = np.sort(rng.choice(np.arange(1, nd + 1), max(1, nd // 100), replace=False))
                it["obs"].append((ob, 1e-3 * rng.standard_normal(ob.size)))
            self.items[m] = it

    def requests(self, count, seed):
        """(m, kind, field seed, with_gradient) for `count` requests with per-request draws:
        m log-uniform in [16, 1024] (to the nearest catalog size), 80/20 Poisson/elasticity,
        50% with a gradient, and a field seed of the request's own."""
        rng = np.random.default_rng(seed)
        lo, hi = math.log(16), math.log(1024)
        out = []
        for _ in range(count):
            mc = math.exp(rng.uniform(lo, hi))
            m = min(self.sizes, key=lambda s: abs(math.log(s) - math.log(mc)))
            kind = 0 if rng.random() < 0.8 else 1
            out.append((m, kind, int(rng.integers(1 << 31)), bool(rng.random() < 0.5)))
        return out

    def fields(self, req):
        """The request's input fields (host arrays) from its seed."""
        import torch
        from adfem_gpu import synth

        m, kind, seed, _ = req
        it = self.items[m]
        G = synth.fourier_field(it["g"][:, 0], it["g"][:, 1], seed=seed)
        if kind == 0:
            return ((1.0 + torch.exp(0.5 * G)).cpu().numpy(), it["f"])
        return ((1e9 * torch.exp(0.3 * G)).cpu().numpy(), it["nu"], it["fx"], it["fy"])

    def submit(self, srv, req, fields):
        m, kind, _, grad = req
        it = self.items[m]
        ob, uo = it["obs"][kind] if grad else (None, None)
        return srv.submit(it["mesh"], kind, fields, it["bd"][kind], obs=ob, uobs=uo)

    def dof(self, req):
        return self.items[req[0]]["ndof"][req[1]]

    def reference(self, req, fields, rtol=1e-13):
        """FP64 solution of the request's system at rtol 1e-13 (or its attainable floor)."""
        import torch

        m, kind, _, _ = req
        it = self.items[m]
        dev = [torch.tensor(np.ascontiguousarray(a), device="cuda") for a in fields]
        S = self.A.PoissonSystem(it["mesh"]) if kind == 0 else self.A.ElasticitySystem(it["mesh"])
        S.set_dirichlet(it["bd"][kind])
        S.assemble(*dev)
        return S.solve(precision="fp64", rtol=rtol).cpu().numpy()


def _serve_arm(cat, args, precision, rank, world, dist, reqs_sat, sweeps, fields):
    """One serving arm (all requests at `precision`): warm-up over every (size, kind), a
    saturation run (every request queued at t = 0), then open-loop Poisson arrivals at
    fractions of the saturation throughput.  Returns (report, saturation-run solutions)."""
    A = cat.A
    with A.Server(workers=args.serve_workers, precision=precision, rtol=args.serve_rtol,
                  pack_max_dof=args.serve_pack_max_dof) as srv:
        warm = [(m, k, 0, True) for m in SERVE_SIZES for k in (0, 1)]
        for t in [cat.submit(srv, r, cat.fields(r)) for r in warm]:
            srv.wait(t)
        srv.reset_stats()
        ts = time.perf_counter()
        tickets = [cat.submit(srv, r, fields[i]) for i, r in reqs_sat]
        outs = [srv.wait(t) for t in tickets]
        wall = max_over_ranks(dist, time.perf_counter() - ts)
        st = srv.stats()
        sat = {"requests": len(reqs_sat) * world, "wall_s": wall,
               "throughput_req_s": replica_rate(world, len(reqs_sat), wall),
               "dof_per_s": replica_rate(world, sum(cat.dof(r) for _, r in reqs_sat), wall),
               "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "failed": sum(1 for o in outs if o[0]["status"] != 0),
               "gradients": sum(1 for _, r in reqs_sat if r[3]), "packs": st["packs"],
               "packed_requests": st["packed_requests"]}
        sols = {i: o[1] for (i, _), o in zip(reqs_sat, outs)}
        sweep = []
        for frac, sub in sweeps:
            rate = frac * sat["throughput_req_s"]
            gaps = np.random.default_rng(int(1000 * frac) + rank).exponential(world / rate, len(sub))
            srv.reset_stats()
            ts = time.perf_counter()
            nxt = ts
            tickets = []
            for (i, r), gap in zip(sub, gaps):
                nxt += gap
                dt = nxt - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                tickets.append(cat.submit(srv, r, fields[i]))
            rs = [srv.wait(t)[0] for t in tickets]
            wall = max_over_ranks(dist, time.perf_counter() - ts)
            s = srv.stats()
            sweep.append({"offered_req_s": rate, "load": frac, "requests": len(sub) * world,
                          "achieved_req_s": replica_rate(world, len(sub), wall),
                          "p50_ms": s["p50_ms"], "p99_ms": s["p99_ms"], "p50_queue_ms": s["p50_queue_ms"],
                          "failed": sum(1 for r in rs if r["status"] != 0), "packs": s["packs"],
                          "packed_requests": s["packed_requests"]})
        cache = srv.stats()
    ref = min(sweep, key=lambda x: abs(x["load"] - 0.5)) if sweep else None
    return {"precision": precision, "rtol": args.serve_rtol,
            "p50_ms": ref["p50_ms"] if ref else sat["p50_ms"], "p99_ms": ref["p99_ms"] if ref else sat["p99_ms"],
            "latency_at_load": ref["load"] if ref else 1.0, "saturation": sat, "sweep": sweep,
            "resident_systems": cache["resident_systems"], "device_bytes": cache["device_bytes"]}, sols


def run_serve(A, args, rank=0, world=1, dist=None):
    """C5 serving workload through adfem_gpu.Server, a mixed-precision arm and an FP64 arm on
    the same request streams: per-request seeded fields, a saturation run of
    `serve_requests` requests and open-loop Poisson arrivals (`serve_sweep_requests` each) at
    the `serve_loads` fractions of each arm's saturation throughput.  The error of a sample of
    the saturation run's solutions (both arms) is measured against an FP64 solve of the same
    request at rtol 1e-13.  With several ranks each runs a server replica on its GPU and takes
    its share of every stream (`shard`); throughput is all requests over the slowest
    replica's time, latency percentiles are rank 0's."""
    t0 = time.perf_counter()
    cat = ServeCatalog(A, SERVE_SIZES)
    all_reqs = cat.requests(args.serve_requests, seed=11)
    sat_reqs = shard(list(enumerate(all_reqs)), rank, world)
    streams, base = [], len(all_reqs)
    for frac in args.serve_loads:
        sub = cat.requests(args.serve_sweep_requests, seed=int(100 * frac))
        streams.append((frac, [(base + j, r) for j, r in enumerate(sub)]))
        base += len(sub)
    sweeps = [(frac, shard(sub, rank, world)) for frac, sub in streams]
    fields = {}
    for i, r in sat_reqs + [x for _, sub in sweeps for x in sub]:
        fields[i] = cat.fields(r)
    setup_s = time.perf_counter() - t0
    arms, sols = {}, {}
    for prec in args.serve_precisions:
        arms[prec], sols[prec] = _serve_arm(cat, args, prec, rank, world, dist, sat_reqs, sweeps, fields)
    # accuracy of a sample of the served solutions against FP64 at rtol 1e-13
    acc = None
    if rank == 0 and args.serve_check > 0 and sat_reqs:
        rng = np.random.default_rng(5)
        pick = [sat_reqs[j] for j in sorted(rng.choice(len(sat_reqs), min(args.serve_check, len(sat_reqs)),
                                                       replace=False))]
        errs = {p: [] for p in sols}
        for i, r in pick:
            uref = cat.reference(r, fields[i])
            sc = max(float(np.abs(uref).max()), 1e-300)
            for p in sols:
                errs[p].append(float(np.abs(sols[p][i] - uref).max()) / sc)
        acc = {"sample": len(pick), "reference": "FP64 solve of the same request at rtol 1e-13",
               **{p: {"max_rel_err": max(v), "median_rel_err": statistics.median(v)} for p, v in errs.items()}}
    out = {"workload": "C5 mix: 80/20 Poisson/elasticity, m log-uniform in [16,1024] (to the nearest of %d sizes, "
                       "ratio 2^(1/4)), 50%% with a misfit gradient (1%% observations), each request's kappa or E "
                       "from its own seed" % len(SERVE_SIZES),
           "workers": args.serve_workers, "rtol": args.serve_rtol,
           "pack_max_dof": args.serve_pack_max_dof if args.serve_pack_max_dof != 0 else 16384,
           "setup_s": setup_s, "arms": arms, "accuracy_vs_fp64": acc}
    head = arms.get("mixed") or next(iter(arms.values()))
    out.update({"p50_ms": head["p50_ms"], "p99_ms": head["p99_ms"], "latency_at_load": head["latency_at_load"],
                "saturation": head["saturation"], "sweep": head["sweep"]})
    return out


# ----------------------------------------------------------------------------- C2, C4
def run_c2(A, args):
    """Inverse Poisson at m x m cells (C2, m = 1000: 1,002,001 DOF, 6M Gauss points).
    kappa_true = 1 + exp(0.5 G) (G: unit-variance 64-mode Fourier field, seed 1), f = 1e5(x+y),
    u = 0 on the boundary; observations at 1% of the nodes (seed 3) of the true solution
    plus N(0, 1e-3^2) noise (seed 4); L = sum (u[obs] - uobs)^2.  The gradient dL/dkappa at
    all Gauss points is taken at the iterate kappa0 = kappa_true (1 + 0.1 G2) (G2 seed 5)
    by one mixed forward and one mixed adjoint solve; grads/s is timed over `c2_steps`
    such gradients.  Checks:
    * the FP64 adjoint gradient against the reference's backward chain at full size, with
      the oracle (sparse-solve gradient -lam_i u_j per stored entry of the Dirichlet-imposed
      COO, ImposeDirichlet backward, FemLaplaceScalar backward) fed the GPU's FP64 u and lam,
      whose residuals against the oracle's operator are reported beside it;
    * central differences of L (FP64 solves at rtol 1e-13, warm-started from u(kappa0)) along
      `c2_dirs` random unit directions d, steps eps = 1e-4 ||kappa0|| and eps/2, and their
      Richardson combination (4 D(eps/2) - D(eps)) / 3, against d.grad; errors relative to
      |d.grad| and to ||grad|| (d.grad can be small for a random d, so the relative error of
      the worst direction is set by the solves' rounding noise over |d.grad|)."""
    import torch
    from adfem_gpu import synth

    m = args.c2_m
    coords, elems = synth.jittered_square(m, seed=0)
    mesh = A.Mesh(coords, elems)
    g = torch.tensor(A.gauss_nodes(mesh), device="cuda")
    G = synth.fourier_field(g[:, 0], g[:, 1], seed=1)
    G2 = synth.fourier_field(g[:, 0], g[:, 1], seed=5)
    kap_true = (1.0 + torch.exp(0.5 * G)).contiguous()
    kap0 = (kap_true * (1.0 + 0.1 * G2)).contiguous()
    f = (1e5 * (g[:, 0] + g[:, 1])).contiguous()
    S = A.PoissonSystem(mesh)
    bd = A.bcnode(mesh)
    S.set_dirichlet(bd)
    S.assemble(kap_true, f)
    u_true = S.solve(precision="fp64", rtol=1e-13)
    obs = torch.tensor(synth.observation_nodes(mesh.nnode, seed=3), device="cuda")
    noise = torch.randn(obs.numel(), dtype=torch.float64, device="cuda",
                        generator=torch.Generator(device="cuda").manual_seed(4))
    uobs = u_true[obs] + 1e-3 * noise

    def loss_grad(kap, precision, rtol, grad=True, u0=None):
        S.assemble(kap, f)
        if u0 is None:
            u = S.solve(precision=precision, rtol=rtol)
        else:
            u = u0.clone()
            S.solve(u, precision=precision, rtol=rtol, warm=True)
        r = u[obs] - uobs
        L = float((r * r).sum())
        if not grad:
            return L, None, u, None
        gu = torch.zeros_like(u)
        gu[obs] = 2 * r
        lam = S.adjoint(gu, precision=precision, rtol=rtol)
        return L, S.grad_kappa(u, lam), u, lam

    loss_grad(kap0, "mixed", args.rtol)  # warm-up (graph capture)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.c2_steps):
        L, gk, _, _ = loss_grad(kap0, "mixed", args.rtol)
    torch.cuda.synchronize()
    grads_s = args.c2_steps / (time.perf_counter() - t0)
    L0, g64, u64, lam64 = loss_grad(kap0, "fp64", 1e-13)
    out = {"workload": "inverse Poisson %dx%d jittered, %d DOF, %d Gauss-point parameters, 1%% observations"
                       % (m, m, mesh.nnode, kap0.numel()),
           "grads_per_s": grads_s, "loss": L, "grad_mixed_vs_fp64_rel": float((gk - g64).norm() / g64.norm())}
    # finite differences (FP64 solves) at eps and eps/2, Richardson-combined
    eps = 1e-4 * float(kap0.norm())
    gen = torch.Generator(device="cuda").manual_seed(6)
    gnorm = float(g64.norm())
    e1, e2, er, en = [], [], [], []
    for _ in range(args.c2_dirs):
        d = torch.randn(kap0.numel(), dtype=torch.float64, device="cuda", generator=gen)
        d /= d.norm()
        an = float((g64 * d).sum())
        D = []
        for h in (eps, eps / 2):
            # warm-started from u(kappa0): the perturbed solves only add a small correction,
            # so their rounding noise scales with the correction, not with u
            lp = loss_grad(kap0 + h * d, "fp64", 1e-13, grad=False, u0=u64)[0]
            lm = loss_grad(kap0 - h * d, "fp64", 1e-13, grad=False, u0=u64)[0]
            D.append((lp - lm) / (2 * h))
        rich = (4 * D[1] - D[0]) / 3
        e1.append(abs(D[0] - an) / max(abs(an), 1e-300))
        e2.append(abs(D[1] - an) / max(abs(an), 1e-300))
        er.append(abs(rich - an) / max(abs(an), 1e-300))
        en.append(abs(rich - an) / gnorm)
    out["fd_check"] = {"directions": args.c2_dirs, "eps": eps,
                       "max_rel_err": max(e1) if e1 else None,
                       "median_rel_err": statistics.median(e1) if e1 else None,
                       "max_rel_err_half_eps": max(e2) if e2 else None,
                       "max_rel_err_richardson": max(er) if er else None,
                       "median_rel_err_richardson": statistics.median(er) if er else None,
                       "max_err_richardson_over_grad_norm": max(en) if en else None}
    # the reference's backward chain at full size (oracle), fed the GPU's FP64 u and lam
    if not args.no_cpu:
        import scipy.sparse as sp

        import oracle as O

        t0 = time.perf_counter()
        kh = kap0.cpu().numpy()
        osys = oracle_system(coords, elems, kh, f.cpu().numpy())
        M, Bo, Fb = osys["mesh"], osys["B"], osys["Fb"]
        uh, lh = u64.cpu().numpy(), lam64.cpu().numpy()
        gu = np.zeros(M.ndof)
        oi = obs.cpu().numpy()
        gu[oi] = 2 * (uh[oi] - uobs.cpu().numpy())
        _, ru = residual_report(Bo, uh, Fb, O)
        gz = gu.copy()
        gz[bd - 1] = 0.0  # the adjoint solve takes lambda = 0 on Dirichlet rows
        _, rl = residual_report(Bo, lh, gz, O)
        idx, vv = M.laplace_coo(kh)
        bv = np.zeros(bd.size)
        oi2, ov, _ = O.dirichlet_coo(idx, vv, bd, osys["F"], bv, M.ndof)
        grad_ov = -lh[oi2[:, 0]] * uh[oi2[:, 1]]
        del oi2, ov
        gvv, _, _ = O.dirichlet_coo_backward(grad_ov, lh, idx, vv, bd, bv, M.ndof)
        del idx, vv, grad_ov
        gref = M.laplace_coo_backward(gvv)
        gg = g64.cpu().numpy()
        out["grad_vs_oracle_chain"] = {
            "chain": "sparse-solve gradient -> ImposeDirichlet backward -> FemLaplaceScalar backward (oracle, "
                     "%d Gauss points), fed the GPU's FP64 u and lambda" % gg.size,
            "max_rel_err": float(np.abs(gg - gref).max() / np.abs(gref).max()),
            "rel_err_2norm": float(np.linalg.norm(gg - gref) / np.linalg.norm(gref)),
            "u_residual": ru, "lambda_residual": rl, "cpu_s": time.perf_counter() - t0}
        del osys, Bo
    return out


def run_c4(A, args):
    """Plane-strain elasticity at m x m cells, 2 DOF per node (C4, m = 1000: 2,004,002 DOF).
    E = 1e9 exp(0.3 G) (G: unit-variance Fourier field, seed 2), nu = 0.3 with the
    reference's plane-strain matrix, body force (0, -1e6), nodes on x = 0 clamped in both
    components.  FP64 and mixed solves/s (each against an FP64 reference at rtol 1e-12)
    and grads/s of a misfit at 1% of the DOFs with respect to E at every Gauss point."""
    import torch
    from adfem_gpu import synth

    m = args.c4_m
    coords, elems = synth.jittered_square(m, seed=0)
    mesh = A.Mesh(coords, elems)
    g = torch.tensor(A.gauss_nodes(mesh), device="cuda")
    ng = g.shape[0]
    E = (1e9 * torch.exp(0.3 * synth.fourier_field(g[:, 0], g[:, 1], seed=2))).contiguous()
    nu = torch.full((ng,), 0.3, dtype=torch.float64, device="cuda")
    fx = torch.zeros(ng, dtype=torch.float64, device="cuda")
    fy = torch.full((ng,), -1e6, dtype=torch.float64, device="cuda")
    S = A.ElasticitySystem(mesh)
    left = synth.left_edge_nodes(coords) + 1
    S.set_dirichlet(np.concatenate([left, left + mesh.nnode]))
    S.assemble(E, nu, fx, fy)
    u_ref = S.solve(precision="fp64", rtol=1e-12)
    ref_iters = S.last_stats.iterations
    out = {"workload": "plane-strain elasticity %dx%d jittered, %d DOF, left edge clamped" % (m, m, 2 * mesh.nnode),
           "fp64_reference": {"rtol": 1e-12, "iters": ref_iters}}
    u = torch.zeros_like(u_ref)
    for prec, rtol in (("fp64", args.rtol_fp64), ("mixed", args.rtol)):
        S.solve(u, precision=prec, rtol=rtol)  # warm-up (graph capture)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.c4_steps):
            S.assemble(E, nu, fx, fy)
            S.solve(u, precision=prec, rtol=rtol)
        torch.cuda.synchronize()
        out[prec] = {"solves_per_s": args.c4_steps / (time.perf_counter() - t0), "rtol": rtol,
                     "iters": S.last_stats.iterations,
                     "rel_err_vs_fp64_ref": float((u - u_ref).abs().max() / u_ref.abs().max())}
    out["speedup_mixed_over_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    obs = torch.tensor(synth.observation_nodes(2 * mesh.nnode, seed=7), device="cuda")
    uobs = u_ref[obs] * 1.01
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.c4_steps):
        S.assemble(E, nu, fx, fy)
        S.solve(u, precision="mixed", rtol=args.rtol)
        gu = torch.zeros_like(u)
        gu[obs] = 2 * (u[obs] - uobs)
        lam = S.adjoint(gu, precision="mixed", rtol=args.rtol)
        gE = S.grad_E(u, lam, E, nu)
    torch.cuda.synchronize()
    out["grads_per_s"] = args.c4_steps / (time.perf_counter() - t0)
    out["grad_norm"] = float(gE.norm())
    # the E-gradient at full size: FP64 adjoint gradient against central differences of the
    # misfit (FP64 solves at rtol 1e-13, warm-started from the unperturbed solution) along
    # random unit directions, and the mixed gradient against the FP64 one
    if args.c4_dirs > 0:
        def loss(Ev, grad):
            S.assemble(Ev, nu, fx, fy)
            uu = u_ref.clone()
            S.solve(uu, precision="fp64", rtol=1e-13, warm=True)
            r = uu[obs] - uobs
            if not grad:
                return float((r * r).sum()), None
            g = torch.zeros_like(uu)
            g[obs] = 2 * r
            lm = S.adjoint(g, precision="fp64", rtol=1e-13)
            return float((r * r).sum()), S.grad_E(uu, lm, Ev, nu)

        _, g64 = loss(E, True)
        eps = 1e-4 * float(E.norm())
        gen = torch.Generator(device="cuda").manual_seed(8)
        errs, errs_n = [], []
        for _ in range(args.c4_dirs):
            d = torch.randn(E.numel(), dtype=torch.float64, device="cuda", generator=gen)
            d /= d.norm()
            an = float((g64 * d).sum())
            fd = (loss(E + eps * d, False)[0] - loss(E - eps * d, False)[0]) / (2 * eps)
            errs.append(abs(fd - an) / max(abs(an), 1e-300))
            errs_n.append(abs(fd - an) / float(g64.norm()))
        S.assemble(E, nu, fx, fy)
        out["grad_check"] = {"directions": args.c4_dirs, "eps": eps, "max_rel_err": max(errs),
                             "median_rel_err": statistics.median(errs), "max_err_over_grad_norm": max(errs_n),
                             "grad_mixed_vs_fp64_rel": float((gE - g64).norm() / g64.norm())}
    return out


def run_p2(A, args):
    """P2 elements, mass matrix and Gauss-point interpolation on the m x m jittered square
    (m = 1000: 4,004,001 P2 DOF, 46,016,001 stored entries, 12M Gauss points).

    Device time of each op through the C ABI (CUDA events on the current stream, inputs
    resident), the roofline of the P2 Laplace assembly (FP64-instruction bound on GB300:
    738 flops per element for the 6-point element matrix plus 36 adds per element in the
    row gather, against the nominal 1.25 TFLOP/s FP64 rate; and its algorithmic bytes
    against the measured copy peak), a bounded serial oracle sample of the same Array-arm
    op (COO loop + sparse() sum, Julia semantics) scaled by element count, and one
    end-to-end P2 solve (assembly, load, Dirichlet, K\\F) of -lap u = -6 with
    u = 1 + x^2 + 2y^2 on the boundary, whose P2 solution is exact."""
    import torch
    from adfem_gpu import synth
    from adfem_gpu import system as S

    m = args.p2_m
    coords, elems = synth.jittered_square(m, seed=0)
    mesh = A.Mesh(coords, elems, degree=2)
    ng = A.get_ngauss(mesh)
    g = torch.tensor(A.gauss_nodes(mesh), device="cuda")
    kappa = (1.0 + synth.fourier_field(g[:, 0], g[:, 1], seed=1).exp()).contiguous()
    D = torch.tensor([[2.0, 1.0, 0.0], [1.0, 2.0, 0.0], [0.0, 0.0, 0.5]], dtype=torch.float64,
                     device="cuda").repeat(ng, 1).reshape(-1).contiguous()
    u = torch.rand(mesh.ndof, dtype=torch.float64, device="cuda")
    nnz = int(mesh.pattern()[1].size)

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    ops = {
        "laplace_csr_ms": timed(lambda: S.laplace_csr(mesh, kappa)),
        "mass_csr_ms": timed(lambda: S.mass_csr(mesh, kappa)),
        "stiffness_csr_ms": timed(lambda: S.stiffness_csr(mesh, D), 1),
        "source_ms": timed(lambda: S.source(mesh, kappa)),
        "source_backward_ms": timed(lambda: S.source_backward(mesh, u)),
        "dof_to_gauss_ms": timed(lambda: S.dof_to_gauss(mesh, u)),
        "dof_to_gauss_backward_ms": timed(lambda: S.dof_to_gauss_backward(mesh, kappa)),
        "fem_to_gauss_ms": timed(lambda: S.fem_to_gauss(mesh, u[:mesh.nnode].contiguous())),
    }
    ne = mesh.nelem
    lap_s = ops["laplace_csr_ms"] * 1e-3
    flops = (738 + 36) * ne
    bytes_alg = 8 * ng + 56 * ne + 16 * 6 * ne + 4 * (mesh.ndof + 1) * 2 + 8 * nnz
    hbm, kind = peaks()
    out = {"workload": "P2 Lagrange %dx%d jittered square, %d DOF, %d stored entries" % (m, m, mesh.ndof, nnz),
           "ndof": mesh.ndof, "nnz": nnz, "ngauss": ng, "device_ms": ops,
           "laplace_roofline": {"bound": "fp64", "achieved_tflops": flops / lap_s / 1e12, "peak_tflops": 1.25,
                                "peak_kind": "nominal GB300 FP64", "frac": flops / lap_s / 1e12 / 1.25,
                                "flops_per_element": 774, "bytes": bytes_alg, "achieved_gbs": bytes_alg / lap_s / 1e9,
                                "hbm_frac": bytes_alg / lap_s / 1e9 / hbm, "hbm_peak_kind": kind}}
    # serial oracle sample of the same Array-arm op, scaled by element count
    if not args.no_cpu:
        import oracle as O

        ms = args.p2_cpu_m
        c2, e2 = synth.jittered_square(ms, seed=0)
        Os = O.OracleSpace(c2, e2, 2)
        kk = 1.0 + np.random.default_rng(0).random(Os.ngauss)
        t0 = time.perf_counter()
        Os.laplace_csc(kk)
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"laplace_csc_s": tc * ne / Os.nelem, "cores": 1, "kind": "port",
                               "sample": "serial oracle COO loop + sparse() sum on the %dx%d P2 mesh, scaled x%.0f by "
                                         "element count" % (ms, ms, ne / Os.nelem),
                               "gpu_speedup": tc * ne / Os.nelem / lap_s}
    # end-to-end P2 solve with a known exact answer
    ms = args.p2_solve_m
    c3, e3 = synth.jittered_square(ms, seed=3)
    M3 = A.Mesh(c3, e3, degree=2)
    n3 = A.get_ngauss(M3)
    t0 = time.perf_counter()
    K = A.compute_fem_laplace_matrix1(np.ones(n3), M3)
    F = A.compute_fem_source_term1(np.full(n3, -6.0), M3)
    ue = A.eval_f_on_dof_pts(lambda x, y: 1 + x ** 2 + 2 * y ** 2, M3)
    bd = A.bcnode(M3)
    Kb, Fb = A.impose_Dirichlet_boundary_conditions(K, F, bd, ue[bd - 1])
    sol, st = A.solve(Kb, Fb, rtol=1e-12, return_stats=True)
    out["solve_exact_quadratic"] = {"m": ms, "ndof": M3.ndof, "seconds": time.perf_counter() - t0,
                                    "cg_iterations": st.iterations, "max_abs_err": float(np.abs(sol - ue).max())}
    # the same exact solution through a resident P2 system (banded mixed solve)
    R3 = A.PoissonSystem(M3)
    R3.set_dirichlet(bd, ue[bd - 1])
    R3.assemble(torch.ones(n3, dtype=torch.float64, device="cuda"),
                torch.full((n3,), -6.0, dtype=torch.float64, device="cuda"))
    u3 = R3.solve(precision="mixed", rtol=1e-12).cpu().numpy()
    out["system_exact_quadratic"] = {"m": ms, "ndof": M3.ndof, "precision": "mixed", "rtol": 1e-12,
                                     "iterations": R3.last_stats.iterations, "banded": R3.solver_info()["banded"],
                                     "max_abs_err": float(np.abs(u3 - ue).max())}
    # resident P2 Poisson system at full size: assembly, mixed forward solve, adjoint and
    # kappa gradient (kappa with contrast 1e3, f = 1e5 (x + y), u = 0 on the boundary)
    R = A.PoissonSystem(mesh)
    R.set_dirichlet(A.bcnode(mesh))
    G = synth.fourier_field(g[:, 0], g[:, 1], seed=1)
    kap = synth.lognormal_kappa(G, synth.contrast_sigma(G.cpu().numpy(), 1e3)).contiguous()
    f2 = (1e5 * (g[:, 0] + g[:, 1])).contiguous()
    asm_ms = timed(lambda: R.assemble(kap, f2))
    info = R.solver_info()
    R.solve(precision="mixed", rtol=args.rtol)
    uu = torch.zeros(mesh.ndof, dtype=torch.float64, device="cuda")
    solve_ms = timed(lambda: R.solve(uu, precision="mixed", rtol=args.rtol), 1)
    st_f = R.last_stats
    obs = torch.tensor(synth.observation_nodes(mesh.ndof, seed=3), device="cuda")
    gu = torch.zeros_like(uu)
    gu[obs] = 1.0

    def grad_step():
        lam = R.adjoint(gu, precision="mixed", rtol=args.rtol)
        return R.grad_kappa(uu, lam)

    grad_ms = timed(grad_step, 1)
    out["system_4M"] = {"workload": "resident P2 Poisson system, %d DOF, kappa contrast 1e3" % mesh.ndof,
                        "assemble_ms": asm_ms, "solve_ms": solve_ms, "adjoint_and_grad_ms": grad_ms,
                        "rtol": args.rtol, "iterations": st_f.iterations, "relres": st_f.relres,
                        "banded": info["banded"], "band": info["band"], "stored": info["stored"],
                        "us_per_iteration": 1e3 * solve_ms / max(st_f.iterations, 1),
                        "solves_per_s": 1e3 / (asm_ms + solve_ms)}
    return out


# ----------------------------------------------------------------------------- our arm
def run_ours(args, rank, world, dist):
    import torch

    import adfem_gpu as A

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    mesh, coords, elems, kappa, f, bd, sigma = make_workload(args.m)
    n = mesh.ndof
    S = A.PoissonSystem(mesh)
    S.set_dirichlet(bd)
    if args.trace_iters > 0:
        # short run of the same step for profiler captures: one assembly, then the
        # mixed and the FP64 solve stopped after trace_iters iterations
        S.assemble(kappa, f)
        u = torch.zeros(n, dtype=torch.float64, device="cuda")
        for prec in ("mixed", "fp64"):
            try:
                S.solve(u, precision=prec, rtol=args.rtol, max_iter=args.trace_iters, chunk=8)
            except A.AdFemError as e:
                if e.status != 4:
                    raise
        torch.cuda.synchronize()
        print(json.dumps({"trace_iters": args.trace_iters, "m": args.m}))
        return 0

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # FP64 reference solution (untimed): the error bar of both solves is measured against it
    S.assemble(kappa, f)
    u_ref = S.solve(precision="fp64", rtol=args.ref_rtol)
    ref_stats = S.last_stats

    def step(prec, u):
        S.assemble(kappa, f)
        S.solve(u, precision=prec, rtol=args.rtol if prec == "mixed" else args.rtol_fp64)
        return S.last_stats

    u = torch.zeros(n, dtype=torch.float64, device="cuda")
    # ------------------------------------------------------------------ mixed (headline)
    for _ in range(args.warmup):
        step("mixed", u)
    barrier()
    clk = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    launches = 0
    mixed_stats = []
    for _ in range(args.steps):
        st = step("mixed", u)
        mixed_stats.append((st.iterations, st.updates, st.relres))
        launches += st.launches + 4  # + prepass, system, scale_diag, scale_values
    e1.record()
    barrier()
    clocks = clk.stop()
    ms = max_over_ranks(dist, e0.elapsed_time(e1))
    err_mixed = float((u - u_ref).abs().max() / u_ref.abs().max())
    value = replica_rate(world, args.steps, ms / 1000.0)

    # ------------------------------------------------------------------ FP64 CG comparison
    u64 = torch.zeros_like(u)
    for _ in range(max(1, args.warmup // 2)):
        step("fp64", u64)
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    fp64_stats = []
    for _ in range(args.fp64_steps):
        st = step("fp64", u64)
        fp64_stats.append((st.iterations, st.relres))
    f1.record()
    barrier()
    ms64 = f0.elapsed_time(f1)
    err_fp64 = float((u64 - u_ref).abs().max() / u_ref.abs().max())
    ms64 = max_over_ranks(dist, ms64)
    fp64_value = replica_rate(world, args.fp64_steps, ms64 / 1000.0)

    # the banded one-kernel FP64 iteration on the same operator (the like-for-like FP64
    # counterpart of the mixed kernel; a system created with ADFEM_ZCG64=1)
    os.environ["ADFEM_ZCG64"] = "1"
    try:
        S0 = A.PoissonSystem(mesh)
    finally:
        del os.environ["ADFEM_ZCG64"]
    S0.set_dirichlet(bd)
    u64b = torch.zeros_like(u)

    def step_banded(uu):
        S0.assemble(kappa, f)
        S0.solve(uu, precision="fp64", rtol=args.rtol_fp64)
        return S0.last_stats

    step_banded(u64b)
    barrier()
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h0.record()
    fp64b_stats = []
    for _ in range(args.fp64_steps):
        st = step_banded(u64b)
        fp64b_stats.append((st.iterations, st.relres))
    h1.record()
    barrier()
    fp64b_value = replica_rate(world, args.fp64_steps, max_over_ranks(dist, h0.elapsed_time(h1)) / 1000.0)

    # ------------------------------------------------------------------ grads/s (mixed)
    from adfem_gpu import synth

    obs = torch.tensor(synth.observation_nodes(n, seed=3), device="cuda")
    uobs = u_ref[obs] + 1e-3 * torch.randn(obs.numel(), dtype=torch.float64, device="cuda",
                                           generator=torch.Generator(device="cuda").manual_seed(4))
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    g0.record()
    for _ in range(args.grad_steps):
        S.assemble(kappa, f)
        S.solve(u, precision="mixed", rtol=args.rtol)
        gu = torch.zeros_like(u)
        gu[obs] = 2 * (u[obs] - uobs)
        lam = S.adjoint(gu, precision="mixed", rtol=args.rtol)
        gk = S.grad_kappa(u, lam)
    g1.record()
    barrier()
    grads_value = replica_rate(world, args.grad_steps, max_over_ranks(dist, g0.elapsed_time(g1)) / 1000.0)

    # ------------------------------------------------------------------ roofline (profiled solve)
    import ctypes

    from adfem_gpu import _lib

    S.assemble(kappa, f)
    kms = (ctypes.c_double * 4)()
    kn = (ctypes.c_longlong * 4)()
    o = A.solver_opts("mixed", args.rtol)
    pst = _lib.SolverStats()
    up = torch.zeros_like(u)
    _lib.check(_lib.load().adfem_system_solve_profiled_d(S.handle, _lib.ptr(up), ctypes.byref(o), ctypes.byref(pst),
                                                         kms, kn, _lib.stream_ptr(torch.cuda.current_stream())))
    nent, nrow, nsl = sell_entries(mesh)
    info = S.solver_info()
    spmv_ms = kms[0] / max(kn[0], 1)
    upd_ms = kms[1] / max(kn[1], 1)
    hbm, peak_kind = peaks()
    traffic = None
    if info["banded"]:
        kname, b32 = "k_zcg_iter", zcg_bytes(info)
        traffic = profiled_traffic("k_zcg_iter", args.m)
        others = {"k_fold": kms[2] / max(kn[2], 1), "k_zres64": kms[3] / max(kn[3], 1)}
    else:
        kname, b32 = "k_cg32_spmv", spmv32_bytes(nent, nrow, nsl)
        others = {"k_cg32_update": upd_ms, "k_fold": kms[2] / max(kn[2], 1), "k_residual64": kms[3] / max(kn[3], 1)}
    achieved = b32 / (spmv_ms * 1e-3) / 1e9
    # the banded FP64 iteration's kernel, timed the same way (profiled FP64 solve)
    fp64_kernel = None
    info0 = S0.solver_info()
    if info0.get("banded_fp64"):
        S0.assemble(kappa, f)
        kms64 = (ctypes.c_double * 4)()
        kn64 = (ctypes.c_longlong * 4)()
        o64 = A.solver_opts("fp64", args.rtol_fp64)
        _lib.check(_lib.load().adfem_system_solve_profiled_d(S0.handle, _lib.ptr(up), ctypes.byref(o64),
                                                             ctypes.byref(pst), kms64, kn64,
                                                             _lib.stream_ptr(torch.cuda.current_stream())))
        d_ms = kms64[0] / max(kn64[0], 1)
        b64 = dcg_bytes(info0)
        fl64 = dcg_flops(info0)
        fp64_kernel = {"kernel": "k_dcg_iter", "avg_launch_ms": d_ms, "launches": int(kn64[0]),
                       "bytes_per_launch": b64, "achieved_gbs": b64 / (d_ms * 1e-3) / 1e9,
                       "hbm_frac": b64 / (d_ms * 1e-3) / 1e9 / peaks()[0],
                       "fp64_flops_per_launch": fl64, "achieved_fp64_tflops": fl64 / (d_ms * 1e-3) / 1e12,
                       "fp64_frac_of_nominal": fl64 / (d_ms * 1e-3) / 1e12 / 1.25,
                       "tile_rows": info0.get("fp64_tile_rows")}
    del S0
    # assembly phases (CUDA events inside the library): element pass, fused Laplace + load +
    # Dirichlet rows, operator conversion for the solver; median of 3
    phases = []
    for _ in range(3):
        ms3 = (ctypes.c_double * 3)()
        _lib.check(_lib.load().adfem_system_assemble_poisson_profiled_d(
            S.handle, _lib.ptr(kappa), _lib.ptr(f), ms3, _lib.stream_ptr(torch.cuda.current_stream())))
        phases.append(list(ms3))
    ph = [statistics.median(p[k] for p in phases) for k in range(3)]
    asm_ms = sum(ph)
    ne_ = mesh.nelem
    ng_ = 3 * ne_
    # algorithmic bytes of the assembly proper (element pass + rows): kappa and f at the
    # Gauss points, per-element geometry (32 B as FP64; 40 B as the FP32 pairs of the
    # pair-arithmetic kernel) and the three incidence records (24 B), the operator values
    # (8 B per stored entry) and the load vector
    pairs_asm = bool(S.solver_info().get("assembly_pairs", 0))
    asm_bytes = 16 * ng_ + ((40 if pairs_asm else 32) + 24) * ne_ + 8 * nent + 8 * n
    asm_s = (ph[0] + ph[1]) * 1e-3
    # the Laplace-assembly byte model of the scope table: kappa at the Gauss points, node
    # coordinates, connectivity, a 36-byte element-to-CSR-slot map, each CSR value written once
    nnz_ = int(mesh.pattern()[1].size)
    laplace_bytes = 8 * ng_ + 16 * n + 12 * ne_ + 36 * ne_ + 8 * nnz_
    # FP64 kernels: element pass 8 per element (sigma, and the load terms without the weight);
    # rows: 2 FMA per incidence, diagonal, load gather (one FMA per incidence applies the
    # weight).  Pair kernel: one FP64 add per output value (the pair -> FP64 conversion)
    fp64_ops = (nent + n) if pairs_asm else 8 * ne_ + 24 * n
    # DRAM traffic of the FP64 element pass and row pass from one ncu capture of this
    # workload (profiles/traffic.json): the bytes the kernels actually move, including the
    # per-element intermediate (sigma and the load terms, written and read back) that the
    # algorithmic model leaves out
    asm_traffic = None
    if not pairs_asm:
        tr = [profiled_traffic(k, args.m) for k in ("k_element_prepass", "k_poisson_system")]
        if None not in tr:
            asm_traffic = {"bytes": sum(tr), "element_pass": tr[0], "rows": tr[1],
                           "achieved_gbs": sum(tr) / asm_s / 1e9, "hbm_frac": sum(tr) / asm_s / 1e9 / hbm}
    assembly = {"arithmetic": "fp32 pairs, one pass" if pairs_asm else "fp64, element pass + rows",
                "element_pass_ms": ph[0], "rows_ms": ph[1], "solver_conversion_ms": ph[2], "total_ms": asm_ms,
                "bytes": asm_bytes, "achieved_gbs": asm_bytes / asm_s / 1e9, "hbm_frac": asm_bytes / asm_s / 1e9 / hbm,
                "laplace_model_bytes": laplace_bytes,
                "hbm_frac_laplace_model": laplace_bytes / asm_s / 1e9 / hbm,
                "fp64_ops": fp64_ops, "fp64_tops": fp64_ops / asm_s / 1e12,
                "fp64_frac_of_nominal": fp64_ops / asm_s / 1e12 / 0.625,
                "dram_traffic": asm_traffic,
                "dof_per_s": n / asm_s, "elements_per_s": ne_ / asm_s}

    # ------------------------------------------------------------------ e2e through host buffers
    kh = kappa.cpu().pin_memory()
    fh = f.cpu().pin_memory()
    uh = torch.zeros(n, dtype=torch.float64).pin_memory()
    import numpy as _np

    kn_ = kh.numpy()
    fn_ = fh.numpy()
    S.solve_host(kn_, fn_, precision="mixed", rtol=args.rtol)
    barrier()
    t0 = time.perf_counter()
    o = A.solver_opts("mixed", args.rtol)
    est = _lib.SolverStats()
    for _ in range(args.steps):
        _lib.check(_lib.load().adfem_poisson_solve(S.handle, _lib.ptr(kh), _lib.ptr(fh), _lib.ptr(uh),
                                                   ctypes.byref(o), ctypes.byref(est)))
    barrier()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e_value = replica_rate(world, args.steps, e2e_s)
    err_e2e = float(_np.max(_np.abs(uh.numpy() - u_ref.cpu().numpy())) / float(u_ref.abs().max()))

    # ------------------------------------------------------------------ serving (C5)
    serve = run_serve(A, args, rank, world, dist) if args.serve_requests > 0 else None
    c2 = run_c2(A, args) if args.c2_m > 0 else None
    c4 = run_c4(A, args) if args.c4_m > 0 else None
    p2 = run_p2(A, args) if args.p2_m > 0 else None

    # ------------------------------------------------------------------ CPU checks and baseline (rank 0, N=1)
    cpu = None
    accuracy = None
    if rank == 0 and world == 1 and not args.no_cpu:
        import scipy.sparse as sp

        accuracy, osys = accuracy_c3(A, S, mesh, coords, elems, kappa, f, u_ref,
                                     {"mixed": u, "fp64": u64, "fp64_banded": u64b})
        fp64_iters = int(round(statistics.median([s_[0] for s_ in fp64_stats])))
        t_it = cpu_pcg_iter_s(sp.csr_matrix(osys["B"]), osys["Fb"], args.cpu_iters, 1)
        t_asm = osys["t_assembly_s"]
        cv = 1.0 / (t_asm + fp64_iters * t_it)
        cpu = {"value": cv, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "oracle port, 1 core: full %dx%d assembly (COO -> Julia sparse() CSC -> load -> Dirichlet) "
                         "timed once (%.2f s) + %d Jacobi-PCG iterations on the full %d-DOF operator (%.1f ms each), "
                         "extrapolated to the %d FP64 iterations of this run"
                         % (args.m, args.m, t_asm, args.cpu_iters, n, 1e3 * t_it, fp64_iters),
               "t_assembly_s": t_asm, "t_iter_s": t_it,
               "extrapolated": {"assembly_x": 1, "iters_x": fp64_iters / args.cpu_iters}}
        del osys

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": bench_config(args.m, world),
            "kappa_sigma": sigma,
            "mixed": {"solves_per_s": value, "rtol": args.rtol, "iters": [s[0] for s in mixed_stats],
                      "fp64_residual_evals": [s[1] for s in mixed_stats], "relres": mixed_stats[-1][2],
                      "rel_err_vs_fp64_ref": err_mixed,
                      "rel_err_vs_oracle": accuracy["mixed"]["rel_err_vs_refined_reference"] if accuracy else None},
            "fp64": {"solves_per_s": fp64_value, "rtol": args.rtol_fp64, "iters": [s[0] for s in fp64_stats],
                     "relres": fp64_stats[-1][1], "rel_err_vs_fp64_ref": err_fp64,
                     "rel_err_vs_oracle": accuracy["fp64"]["rel_err_vs_refined_reference"] if accuracy else None,
                     "iteration": "three-kernel FP64 CG (SpMV + p.q, update + r.r, direction): the library's "
                                  "FP64 path and the fastest FP64 iteration here",
                     "speedup_mixed_over_fp64": value / fp64_value},
            "fp64_banded": {"solves_per_s": fp64b_value, "rtol": args.rtol_fp64,
                            "iters": [s[0] for s in fp64b_stats], "relres": fp64b_stats[-1][1],
                            "rel_err_vs_oracle": accuracy["fp64_banded"]["rel_err_vs_refined_reference"]
                            if accuracy else None,
                            "iteration": "banded one-kernel FP64 CG (k_dcg_iter): the mixed iteration's layout "
                                         "and fusion with FP64 values, vectors and dot products",
                            "kernel": fp64_kernel,
                            "speedup_mixed_over_fp64_banded": value / fp64b_value},
            "accuracy_vs_oracle": accuracy,
            "grads_per_s": grads_value,
            "dof_per_s": value * n,
            "assembly": assembly,
            "fp64_reference": {"rtol": args.ref_rtol, "iters": ref_stats.iterations, "relres": ref_stats.relres,
                               "true_residual_replacements": ref_stats.updates},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": traffic, "kernel": kname, "bytes_per_launch": b32,
                         "avg_launch_ms": spmv_ms, "launches": int(kn[0]), "peak_kind": peak_kind,
                         "other_kernels_avg_ms": others, "assembly_ms": asm_ms,
                         "solver_layout": info},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * int(kappa.numel()),
                    "d2h_bytes_per_step": 8 * n, "rel_err_vs_fp64_ref": err_e2e},
            "gpu_launches": launches,
            "clocks": clocks,
            "cpu_baseline": cpu,
            "serve": serve,
            "inverse_poisson_1M": c2,
            "elasticity_2M": c4,
            "p2_4M": p2,
        }
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--m", type=int, default=2000)
    ap.add_argument("--rtol", type=float, default=3e-10, help="mixed-precision stopping tolerance")
    ap.add_argument("--rtol-fp64", type=float, default=1e-9, help="FP64 CG stopping tolerance")
    ap.add_argument("--ref-rtol", type=float, default=1e-14)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--grad-steps", type=int, default=2)
    ap.add_argument("--cpu-iters", type=int, default=200, help="CPU baseline: single-thread PCG iterations timed")
    ap.add_argument("--ref-iters", type=int, default=200, help="reference arm: PCG iterations per step")
    ap.add_argument("--fp64-iters", type=int, default=FP64_ITERS_DEFAULT)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=400,
                    help="serving workload: requests of the saturation run (0 skips serving)")
    ap.add_argument("--serve-sweep-requests", type=int, default=300)
    ap.add_argument("--serve-precisions", nargs="*", default=["mixed", "fp64"])
    ap.add_argument("--serve-check", type=int, default=24, help="served solutions checked against FP64 at rtol 1e-13")
    ap.add_argument("--serve-loads", type=float, nargs="*", default=[0.5, 0.8])
    ap.add_argument("--serve-workers", type=int, default=8)
    ap.add_argument("--serve-rtol", type=float, default=1e-10)
    ap.add_argument("--serve-pack-max-dof", type=int, default=0,
                    help="requests up to this many DOFs are solved in packed launches (0: library default; -1: off)")
    ap.add_argument("--only-serve", action="store_true", help="run only the serving leg and print it")
    ap.add_argument("--c2-m", type=int, default=1000, help="inverse Poisson cells per side (0 skips)")
    ap.add_argument("--c2-steps", type=int, default=2)
    ap.add_argument("--c2-dirs", type=int, default=32, help="finite-difference directions of the gradient check")
    ap.add_argument("--c4-m", type=int, default=1000, help="elasticity cells per side (0 skips)")
    ap.add_argument("--c4-steps", type=int, default=1)
    ap.add_argument("--c4-dirs", type=int, default=4, help="finite-difference directions of the E-gradient check")
    ap.add_argument("--p2-m", type=int, default=1000, help="P2 / mass / interpolation ops cells per side (0 skips)")
    ap.add_argument("--p2-cpu-m", type=int, default=120, help="P2 oracle sample cells per side")
    ap.add_argument("--p2-solve-m", type=int, default=200, help="P2 exact-solution solve cells per side")
    ap.add_argument("--only-p2", action="store_true",
                    help="profiling aid: run only the P2 / mass / interpolation leg and print it")
    ap.add_argument("--only-c4", action="store_true",
                    help="profiling aid: run only the elasticity leg and print it")
    ap.add_argument("--trace-iters", type=int, default=0,
                    help="profiling aid: run one truncated step (this many CG iterations) and exit")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.only_p2 or args.only_serve or args.only_c4:
        import adfem_gpu as A

        if args.only_p2:
            out = {"p2_4M": run_p2(A, args)}
        elif args.only_c4:
            out = {"elasticity_2M": run_c4(A, args)}
        else:
            out = {"serve": run_serve(A, args)}
        print(json.dumps(out), flush=True)
        return 0
    if world > 1:
        import torch
        import torch.distributed as td

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        td.init_process_group("nccl")
        dist = td
    r = run_ours(args, rank, world, dist)
    if dist is not None:
        dist.destroy_process_group()
    return r


if __name__ == "__main__":
    sys.exit(main())
