"""Seeded synthetic inputs for the P1-triangle Poisson and elasticity workloads.

Meshes follow ``Mesh(m, n, h)`` in src/MFEM/MFEM.jl:134-170 (nodes numbered
x-fastest, each cell split into two triangles with the "version 1" split of
MFEM.jl:143-144), on the unit square, with interior nodes jittered uniformly by
up to +-0.2 h in x and y.  Coefficient fields are random Fourier fields

    g(x) = sqrt(2 / M) * sum_{j<M} cos(k_j . x + phi_j),

with wavenumbers k_j uniform in the disk |k| <= kmax and phases uniform in
[0, 2 pi); g has unit variance in expectation.  All randomness comes from numpy's
PCG64 generator (``numpy.random.default_rng(seed)``), so a seed gives the same
inputs on every machine.  No dataset is involved: these stand in for the meshes
and fields a user would build in Julia.
"""
from __future__ import annotations

import math

import numpy as np

__all__ = [
    "jittered_square",
    "fan_mesh",
    "fourier_modes",
    "fourier_field",
    "poisson_c1_fields",
    "lognormal_kappa",
    "contrast_sigma",
    "observation_nodes",
    "left_edge_nodes",
]


def jittered_square(m: int, seed: int = 0, jitter: float = 0.2, n: int | None = None):
    """Unit square with m x n cells (n defaults to m).

    Returns ``(coords, elems)``: coords float64 (Nn, 2); elems int64 (Ne, 3),
    1-based like the Julia ``Mesh(coords, elems)`` constructor expects.
    """
    n = m if n is None else n
    if m < 1 or n < 1:
        raise ValueError("need at least one cell per side")
    hx, hy = 1.0 / m, 1.0 / n
    jj, ii = np.meshgrid(np.arange(m + 1), np.arange(n + 1))
    x = (jj * hx).astype(np.float64).ravel()
    y = (ii * hy).astype(np.float64).ravel()
    rng = np.random.default_rng(seed)
    d = rng.uniform(-jitter, jitter, size=(x.size, 2))
    interior = ((jj > 0) & (jj < m) & (ii > 0) & (ii < n)).ravel()
    x = x + np.where(interior, d[:, 0] * hx, 0.0)
    y = y + np.where(interior, d[:, 1] * hy, 0.0)
    coords = np.stack([x, y], axis=1)
    # version-1 split (MFEM.jl:143-144), 0-based then shifted to 1-based
    i = np.arange(n)[:, None]
    j = np.arange(m)[None, :]
    a = (i * (m + 1) + j).ravel()
    b = a + 1
    c = ((i + 1) * (m + 1) + j).ravel()
    d2 = c + 1
    elems = np.empty((2 * m * n, 3), dtype=np.int64)
    elems[0::2] = np.stack([a, b, c], axis=1)
    elems[1::2] = np.stack([b, c, d2], axis=1)
    return coords, elems + 1


def fan_mesh(k: int = 40, rings: int = 3, seed: int = 0):
    """A disk whose centre vertex has k neighbours: vertex 0 at the origin, ``rings`` rings
    of k vertices at radius r / rings (inner rings jittered radially by up to 2.5 %, odd
    rings rotated half a step), a fan of k triangles around the centre and two triangles
    per quad between consecutive rings.  The centre's matrix row has k + 1 entries, far
    above the 7 of a structured triangulation.

    Returns ``(coords, elems)`` as ``jittered_square`` does (elems 1-based)."""
    rng = np.random.default_rng(seed)
    pts = [(0.0, 0.0)]
    for r in range(1, rings + 1):
        rad = r / rings
        for j in range(k):
            t = 2 * math.pi * (j + 0.5 * (r % 2)) / k
            rr = rad * (1 + 0.05 * (rng.random() - 0.5)) if r < rings else rad
            pts.append((rr * math.cos(t), rr * math.sin(t)))

    def ring(r, j):
        return 1 + (r - 1) * k + (j % k)

    el = [(0, ring(1, j), ring(1, j + 1)) for j in range(k)]
    for r in range(1, rings):
        for j in range(k):
            a, b, c, d = ring(r, j), ring(r, j + 1), ring(r + 1, j), ring(r + 1, j + 1)
            el += [(a, c, d), (a, d, b)]
    return np.array(pts), np.array(el, dtype=np.int64) + 1


def fourier_modes(seed: int, nmodes: int = 64, kmax: float = 16 * math.pi):
    """Wavenumbers (nmodes, 2) uniform in the disk |k|<=kmax and phases (nmodes,)."""
    rng = np.random.default_rng(seed)
    r = kmax * np.sqrt(rng.uniform(0.0, 1.0, nmodes))
    th = rng.uniform(0.0, 2 * math.pi, nmodes)
    k = np.stack([r * np.cos(th), r * np.sin(th)], axis=1)
    phi = rng.uniform(0.0, 2 * math.pi, nmodes)
    return k, phi


def fourier_field(x, y, seed: int, nmodes: int = 64, kmax: float = 16 * math.pi, chunk: int = 1 << 20):
    """Unit-variance random Fourier field g evaluated at points (x, y).

    ``x``/``y`` may be numpy arrays or torch tensors (any device); the result has the
    same type.  The modes come from ``fourier_modes(seed)``.
    """
    k, phi = fourier_modes(seed, nmodes, kmax)
    amp = math.sqrt(2.0 / nmodes)
    if isinstance(x, np.ndarray):
        out = np.empty(x.shape, dtype=np.float64)
        xf, yf, of = x.ravel(), y.ravel(), out.ravel()
        for s in range(0, xf.size, chunk):
            ph = np.outer(xf[s:s + chunk], k[:, 0]) + np.outer(yf[s:s + chunk], k[:, 1]) + phi[None, :]
            of[s:s + chunk] = amp * np.cos(ph).sum(axis=1)
        return out
    import torch  # torch path: evaluation on the tensor's device

    kt = torch.as_tensor(k, dtype=torch.float64, device=x.device)
    pt = torch.as_tensor(phi, dtype=torch.float64, device=x.device)
    out = torch.empty_like(x, dtype=torch.float64)
    xf, yf, of = x.reshape(-1), y.reshape(-1), out.view(-1)
    for s in range(0, xf.numel(), chunk):
        ph = torch.outer(xf[s:s + chunk], kt[:, 0]) + torch.outer(yf[s:s + chunk], kt[:, 1]) + pt[None, :]
        of[s:s + chunk] = amp * torch.cos(ph).sum(dim=1)
    return out


def poisson_c1_fields(gx, gy):
    """kappa = sin(x)(1+y^2)+1 and f = 1e5 (x+y) at the Gauss points (64x64 Poisson case)."""
    lib = np if isinstance(gx, np.ndarray) else __import__("torch")
    kappa = lib.sin(gx) * (1 + gy * gy) + 1
    f = 1e5 * (gx + gy)
    return kappa, f


def contrast_sigma(g, target: float = 1e3):
    """Scale sigma so that (1+exp(sigma*max g)) / (1+exp(sigma*min g)) == target (bisection)."""
    gmax, gmin = float(g.max()), float(g.min())

    def contrast(s):
        return (1 + math.exp(s * gmax)) / (1 + math.exp(s * gmin))

    lo, hi = 0.0, 1.0
    while contrast(hi) < target:
        hi *= 2
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if contrast(mid) < target:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def lognormal_kappa(g, sigma: float):
    """kappa = 1 + exp(sigma g)."""
    lib = np if isinstance(g, np.ndarray) else __import__("torch")
    return 1 + lib.exp(sigma * g)


def observation_nodes(nnode: int, seed: int, frac: float = 0.01):
    """1% of the nodes, drawn without replacement, sorted (0-based)."""
    rng = np.random.default_rng(seed)
    k = max(1, int(round(frac * nnode)))
    return np.sort(rng.choice(nnode, size=k, replace=False)).astype(np.int64)


def left_edge_nodes(coords, tol: float = 1e-12):
    """0-based ids of nodes on x = 0."""
    return np.nonzero(np.abs(coords[:, 0]) <= tol)[0].astype(np.int64)
