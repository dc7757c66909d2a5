"""Writes the golden fixtures under tests/golden.

kats.json: known answers transcribed from the reference's own tests
  - test/MFEM2.jl:7-27   Mesh(2,2,0.5): node coordinates, get_ngauss == 24, every area 0.125
  - test/mfem.jl:78-87    impose_Dirichlet: dense (Array) arm == SparseTensor arm, bd=[5;2;3],
                          bdval=[1;2;3] on a 5x5 matrix (the test draws rand(5,5); the case here
                          fixes a seeded draw so both arms can be compared exactly)
  - deps/MFEM/FemSource1/ftest.jl:5-14   source(f=c) == mass * c
c_small.npz: oracle outputs for the jittered 8x8 Poisson case (seed 0), used as a
  regression pin for the oracle and as fixed vectors for the GPU parity tests.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "adfem.jl_gb300"))

import oracle as O  # noqa: E402
from adfem_gpu import synth  # noqa: E402


def main():
    kats = {
        "mfem2_mesh_2_2_0.5": {
            "source": "test/MFEM2.jl:7-27",
            "nodes": [[0.0, 0.0], [0.5, 0.0], [1.0, 0.0], [0.0, 0.5], [0.5, 0.5], [1.0, 0.5],
                      [0.0, 1.0], [0.5, 1.0], [1.0, 1.0]],
            "ngauss": 24,
            "area": [0.125] * 8,
        },
        "dirichlet_dense_vs_sparse": {
            "source": "test/mfem.jl:78-87",
            "seed": 233,
            "n": 5,
            "bd": [5, 2, 3],
            "bdval": [1.0, 2.0, 3.0],
            "tol": 1e-5,
        },
        "source_equals_mass_times_constant": {"source": "deps/MFEM/FemSource1/ftest.jl:5-14", "c": 2.5},
    }
    with open(os.path.join(HERE, "kats.json"), "w") as f:
        json.dump(kats, f, indent=1)

    coords, elems = synth.jittered_square(8, seed=0)
    M = O.OracleMesh(coords, elems)
    g = M.gauss_nodes()
    kappa, fsrc = synth.poisson_c1_fields(g[:, 0], g[:, 1])
    K = M.laplace_csc(kappa)
    F = M.source(fsrc)
    bd = M.bcnode()
    B, r = O.dirichlet_csc(K, F, bd, np.zeros(bd.size))
    u = O.spsolve(B, r)
    np.savez_compressed(os.path.join(HERE, "c_small.npz"), coords=coords, elems=elems, kappa=kappa, f=fsrc,
                        K_indptr=K.indptr, K_indices=K.indices, K_data=K.data, F=F, bd=bd,
                        B_indptr=B.indptr, B_indices=B.indices, B_data=B.data, r=r, u=u,
                        area=M.area, gx=g[:, 0], gy=g[:, 1])
    print("wrote", os.path.join(HERE, "kats.json"), os.path.join(HERE, "c_small.npz"))


if __name__ == "__main__":
    main()
