"""The library's host mesh code under AddressSanitizer and UndefinedBehaviorSanitizer (CPU).

adfem.jl_gb300/csrc/mesh.cpp does all of a mesh's host work before anything reaches the
GPU: orientation fix, geometry, node->element incidence, the CSR pattern and its
sliced-ELL copy, edges, boundary nodes and the P2 space.  tests/host_mesh_harness.cpp
links it with host-memory stand-ins for the four CUDA runtime calls it makes, instrumented
(-fsanitize=address,undefined, every finding aborts).  A child process then:
  * builds structured, jittered, fan (63-neighbour vertex) and reoriented meshes and checks
    the pattern, boundary nodes, edges, areas, Gauss points and P2 space against the oracle,
    and every stored entry of the sliced-ELL copy against the pattern;
  * renumbers a shuffled mesh by reverse Cuthill-McKee (the solver's DOF order) and checks
    the permutation and the band it reports;
  * lays out the interleaved 2-DOF pattern of an elasticity operator (slice-uniform column
    patterns per row parity) and a pattern with a band beyond int16 (int32 columns) in
    sliced ELL, and decodes every stored entry;
  * feeds the invalid meshes the entry rejects (vertex index out of range, a degenerate
    triangle, a vertex in no element, a vertex with 70 neighbours) and checks the statuses;
  * makes each device allocation of a mesh build fail in turn (adfem_debug_fail_alloc) and
    checks that every one is reported as ADFEM_ERR_NOMEM with nothing leaked into a crash.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "adfem.jl_gb300", "csrc")

SCRIPT = r'''
import ctypes, os, sys
import numpy as np
sys.path.insert(0, "oracle"); sys.path.insert(0, "adfem.jl_gb300")
import oracle as O
from adfem_gpu import synth

assert hasattr(ctypes.CDLL(None), "__asan_init")  # the sanitizer runtime is in the process
H = ctypes.CDLL(os.environ["HOST_MESH_LIB"])
vp, ll = ctypes.c_void_p, ctypes.c_longlong
H.hm_build.argtypes = [vp, ll, vp, ll, ctypes.POINTER(vp)]
H.hm_error.restype = ctypes.c_char_p
H.hm_destroy.argtypes = [vp]
H.hm_sizes.argtypes = [vp, vp, vp, vp]
H.hm_pattern.argtypes = [vp, vp, vp]
H.hm_bcnode.argtypes = [vp, vp]; H.hm_bcnode.restype = ll
H.hm_edges.argtypes = [vp, vp]; H.hm_edges.restype = ll
H.hm_area.argtypes = [vp, vp]
H.hm_gauss.argtypes = [vp, vp, vp]
H.hm_sell.argtypes = [vp, vp, vp, vp, vp, vp]
H.hm_space.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp]
H.adfem_debug_fail_alloc.argtypes = [ll]
H.hm_rcm.argtypes = [vp, vp]; H.hm_rcm.restype = ll
H.hm_make_p2.argtypes = [vp]
H.hm_gauss_weights.argtypes = [vp, vp]
H.hm_sell_build.argtypes = [ll, vp, vp, ctypes.c_int, vp, vp, vp, vp, vp, vp]

def P(a):
    return a.ctypes.data

def build(coords, elems1):
    n = coords.shape[0]
    xyz = np.zeros((n, 3)); xyz[:, :2] = coords
    e0 = np.ascontiguousarray(np.asarray(elems1) - 1, dtype=np.int32)
    h = vp()
    st = H.hm_build(P(xyz), n, P(e0), e0.shape[0], ctypes.byref(h))
    return st, h

def check_mesh(coords, elems):
    st, h = build(coords, elems)
    assert st == 0, H.hm_error()
    M = O.OracleMesh(coords, elems)
    n = M.ndof
    nnz, maxrow, flipped = ctypes.c_longlong(), ctypes.c_int(), ctypes.c_int()
    H.hm_sizes(h, ctypes.byref(nnz), ctypes.byref(maxrow), ctypes.byref(flipped))
    rp = np.empty(n + 1, np.int32); ci = np.empty(nnz.value, np.int32)
    H.hm_pattern(h, P(rp), P(ci))
    K = M.laplace_csc(np.ones(M.ngauss))
    assert np.array_equal(rp, K.indptr) and np.array_equal(ci, K.indices)
    assert maxrow.value == np.diff(rp).max() and flipped.value == M.flipped
    nb = H.hm_bcnode(h, None); bd = np.empty(nb, np.int64); H.hm_bcnode(h, P(bd))
    assert np.array_equal(bd, M.bcnode())
    ne = H.hm_edges(h, None); ed = np.empty(2 * ne, np.int64); H.hm_edges(h, P(ed))
    assert np.array_equal(ed.reshape(2, ne).T, M.edges())
    a = np.empty(M.nelem); H.hm_area(h, P(a))
    assert np.allclose(a, M.area, rtol=1e-15, atol=0)
    gx = np.empty(M.ngauss); gy = np.empty(M.ngauss); H.hm_gauss(h, P(gx), P(gy))
    assert np.allclose(np.stack([gx, gy], 1), M.gauss_nodes(), rtol=0, atol=1e-15)
    # sliced-ELL copy: row r of slice r // 32 holds its pattern row, then padding on the diagonal
    ns, nent, maxw = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
    H.hm_sell(h, ctypes.byref(ns), ctypes.byref(nent), ctypes.byref(maxw), None, None)
    assert ns.value == (n + 31) // 32 and maxw.value == maxrow.value
    sp = np.empty(ns.value + 1, np.int32); col = np.empty(max(nent.value, 1), np.int32)
    H.hm_sell(h, ctypes.byref(ns), ctypes.byref(nent), ctypes.byref(maxw), P(sp), P(col))
    for r in range(n):
        s = r // 32; w = (sp[s + 1] - sp[s]) // 32
        got = col[sp[s] + 32 * np.arange(w) + (r % 32)]
        row = ci[rp[r]:rp[r + 1]]
        assert np.array_equal(got[:row.size], row) and np.all(got[row.size:] == r), r
    # the P2 space on the same mesh
    nd, nz, mr = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
    assert H.hm_space(h, 2, ctypes.byref(nd), ctypes.byref(nz), ctypes.byref(mr), None, None) == 0
    S = O.OracleSpace(coords, elems, 2)
    rp2 = np.empty(nd.value + 1, np.int32); ci2 = np.empty(nz.value, np.int32)
    H.hm_space(h, 2, ctypes.byref(nd), ctypes.byref(nz), ctypes.byref(mr), P(rp2), P(ci2))
    K2 = S.laplace_csc(np.ones(S.ngauss))
    assert nd.value == S.ndof and np.array_equal(rp2, K2.indptr) and np.array_equal(ci2, K2.indices)
    H.hm_destroy(h)
    # the same mesh as a degree-2 mesh: 6 Gauss points per element (order-4 rule), boundary
    # DOFs with the boundary edges' DOFs after the vertices
    st, h = build(coords, elems)
    assert st == 0 and H.hm_make_p2(h) == 0
    g6x = np.empty(S.ngauss); g6y = np.empty(S.ngauss); H.hm_gauss(h, P(g6x), P(g6y))
    assert np.allclose(np.stack([g6x, g6y], 1), S.gauss_nodes(), rtol=0, atol=1e-15)
    w6 = np.empty(S.ngauss); H.hm_gauss_weights(h, P(w6))
    assert abs(w6.sum() - M.area.sum()) < 1e-13 * M.area.sum()  # the weights integrate 1
    nb = H.hm_bcnode(h, None); bd2 = np.empty(nb, np.int64); H.hm_bcnode(h, P(bd2))
    assert np.array_equal(bd2, S.bcnode())
    H.hm_destroy(h)

cases = [synth.jittered_square(1, seed=0, jitter=0.0), synth.jittered_square(2, seed=0, jitter=0.0),
         synth.jittered_square(7, seed=3), synth.jittered_square(40, seed=1), synth.fan_mesh(30),
         synth.fan_mesh(63)]
c, e = synth.jittered_square(5, seed=2)
cases.append((c, e[:, ::-1].copy()))  # every triangle clockwise: all reoriented
for c, e in cases:
    check_mesh(c, e)

# reverse Cuthill-McKee on a mesh whose nodes were shuffled: a permutation, the band it
# reports is the band of the renumbered pattern, and far below the shuffled one
c, e = synth.jittered_square(30, seed=5)
perm = np.random.default_rng(6).permutation(c.shape[0])
inv = np.argsort(perm)
cs, es = c[perm], inv[e - 1] + 1
st, h = build(cs, es); assert st == 0
n = cs.shape[0]
nnz, maxrow, flipped = ctypes.c_longlong(), ctypes.c_int(), ctypes.c_int()
H.hm_sizes(h, ctypes.byref(nnz), ctypes.byref(maxrow), ctypes.byref(flipped))
rp = np.empty(n + 1, np.int32); ci = np.empty(nnz.value, np.int32); H.hm_pattern(h, P(rp), P(ci))
pi = np.empty(n, np.int32)
band = H.hm_rcm(h, P(pi))
assert np.array_equal(np.sort(pi), np.arange(n))
rows = np.repeat(np.arange(n), np.diff(rp))
assert band == np.abs(pi[rows] - pi[ci]).max()
assert band <= np.abs(rows - ci).max() // 4 and band <= 2 * 31 + 8, band
H.hm_destroy(h)

# sliced-ELL layouts of other patterns: the interleaved 2-DOF pattern of an elasticity
# operator (slice-uniform patterns per row parity) and a pattern whose band exceeds the
# int16 deltas (int32 columns, padding on the diagonal)
def sell_check(rp, ci, period):
    n = rp.size - 1
    ns, nent, maxw = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
    info = np.zeros(3, np.int64)
    assert H.hm_sell_build(n, P(rp), P(ci), period, ctypes.byref(ns), ctypes.byref(nent), ctypes.byref(maxw),
                           P(info), None, None) == 0
    sp = np.empty(ns.value + 1, np.int32); col = np.empty(max(nent.value, 1), np.int32)
    H.hm_sell_build(n, P(rp), P(ci), period, ctypes.byref(ns), ctypes.byref(nent), ctypes.byref(maxw), P(info),
                    P(sp), P(col))
    for r in range(n):
        s = r // 32; w = (sp[s + 1] - sp[s]) // 32
        got = col[sp[s] + 32 * np.arange(w) + (r % 32)]
        row = ci[rp[r]:rp[r + 1]]
        assert np.array_equal(got[:row.size], row) and np.all(got[row.size:] == r), r
    return info

c, e = synth.jittered_square(100, seed=7)
st, h = build(c, e); assert st == 0
n = c.shape[0]
nnz, maxrow, flipped = ctypes.c_longlong(), ctypes.c_int(), ctypes.c_int()
H.hm_sizes(h, ctypes.byref(nnz), ctypes.byref(maxrow), ctypes.byref(flipped))
rp = np.empty(n + 1, np.int32); ci = np.empty(nnz.value, np.int32); H.hm_pattern(h, P(rp), P(ci))
H.hm_destroy(h)
rows2 = [np.sort(np.r_[2 * ci[rp[i]:rp[i + 1]], 2 * ci[rp[i]:rp[i + 1]] + 1]) for i in range(n) for _ in (0, 1)]
rp2 = np.r_[0, np.cumsum([r.size for r in rows2])].astype(np.int32)
ci2 = np.concatenate(rows2).astype(np.int32)
info = sell_check(rp2, ci2, 2)
assert info[0] == 1 and info[1] > 0  # int16 deltas; interior slices share a pattern
far = 40000
rows3 = [sorted({max(i - 1, 0), i, min(i + 1, far - 1)} | ({i + 35000} if i < 5000 else set())
                | ({i - 35000} if i >= 35000 else set())) for i in range(far)]
rp3 = np.r_[0, np.cumsum([len(r) for r in rows3])].astype(np.int32)
ci3 = np.concatenate([np.array(r) for r in rows3]).astype(np.int32)
info = sell_check(rp3, ci3, 1)
assert info[0] == 0 and info[2] == 35000

# invalid meshes: a status and a message, no crash
c, e = synth.jittered_square(3, seed=0)
bad = e.copy(); bad[4, 1] = c.shape[0] + 1
st, _ = build(c, bad); assert st == 1 and b"out of range" in H.hm_error()
bad = e.copy(); bad[2, 2] = bad[2, 0]
st, _ = build(c, bad); assert st == 1 and b"degenerate" in H.hm_error()
st, _ = build(np.vstack([c, [[5.0, 5.0]]]), e); assert st == 1 and b"no element" in H.hm_error()
st, _ = build(*synth.fan_mesh(70)); assert st == 8 and b"63" in H.hm_error()

# each device allocation of a build fails in turn
c, e = synth.jittered_square(6, seed=4)
walked = 0
for k in range(200):
    H.adfem_debug_fail_alloc(k)
    st, h = build(c, e)
    if st == 0:
        H.hm_destroy(h)
        break
    assert st == 3 and not h.value, (k, st, H.hm_error())
    walked += 1
H.adfem_debug_fail_alloc(-1)
assert 5 <= walked < 200, walked
st, h = build(c, e); assert st == 0; H.hm_destroy(h)
print("host mesh ok", walked)
'''


def _runtimes():
    try:
        asan = subprocess.check_output(["gcc", "-print-file-name=libasan.so"], text=True).strip()
        ubsan = subprocess.check_output(["gcc", "-print-file-name=libubsan.so"], text=True).strip()
    except (OSError, subprocess.CalledProcessError):
        return None, None
    return (asan if os.path.isabs(asan) and os.path.exists(asan) else None,
            ubsan if os.path.isabs(ubsan) and os.path.exists(ubsan) else None)


def test_host_mesh_code_under_sanitizers(oracle, tmp_path):
    asan, ubsan = _runtimes()
    if asan is None:
        pytest.skip("gcc sanitizer runtimes not available")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("CUDA headers not available")
    lib = str(tmp_path / "libhostmesh.so")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-g", "-fPIC", "-shared", "-pthread", "-fno-omit-frame-pointer",
                           "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-I", cuda_inc, "-I", CSRC,
                           "-I", os.path.join(ROOT, "include"), "-o", lib,
                           os.path.join(ROOT, "tests", "host_mesh_harness.cpp"), os.path.join(CSRC, "mesh.cpp")])
    env = dict(os.environ, HOST_MESH_LIB=lib, LD_PRELOAD=asan + ((":" + ubsan) if ubsan else ""),
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=1", UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    r = subprocess.run([sys.executable, "-c", SCRIPT], cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0 and "host mesh ok" in r.stdout, (r.stdout[-2000:], r.stderr[-4000:])
