"""Writes tests/golden/mtj_small.npz: small seeded inputs and the oracle's
outputs for them (CompRowMatrix products, preconditioner applies, solver
iterates and residual histories).

The reference ships no golden vectors (its fixtures come from unseeded
Math.random), so these fixtures pin the oracle, which is itself checked bit
for bit against the independent restatement in tests/pyref.py, and give the
GPU tests fixed expected values.  Inputs are stored next to the outputs, so
the fixture does not depend on any generator staying the same.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "matrix-toolkits-java_gb300"))

import oracle as O  # noqa: E402
from mtjg import workloads  # noqa: E402

OUT = os.path.join(HERE, "mtj_small.npz")


def random_csr(rng, n, m, density):
    dense = rng.uniform(-1, 1, (n, m)) * (rng.random((n, m)) < density)
    dense[rng.integers(0, n, 3)] = 0.0  # a few empty rows
    rp, ci, v = [0], [], []
    for i in range(n):
        nz = np.nonzero(dense[i])[0]
        ci.extend(nz.tolist())
        v.extend(dense[i, nz].tolist())
        rp.append(len(ci))
    return np.array(rp, np.int32), np.array(ci, np.int32), np.array(v)


def put_csr(d, key, n, m, rp, ci, v):
    d[key + "/shape"] = np.array([n, m], np.int64)
    d[key + "/rowptr"] = np.asarray(rp, np.int32)
    d[key + "/colind"] = np.asarray(ci, np.int32)
    d[key + "/val"] = np.asarray(v, np.float64)


def main():
    O.build()
    rng = np.random.default_rng(20240601)
    d = {}
    # ---- products
    n, m = 60, 45
    rp, ci, v = random_csr(rng, n, m, 0.2)
    put_csr(d, "prod/A", n, m, rp, ci, v)
    A = O.Csr(n, m, rp, ci, v)
    x, y, xt, yt = rng.uniform(-1, 1, m), rng.uniform(-1, 1, n), rng.uniform(-1, 1, n), rng.uniform(-1, 1, m)
    d.update({"prod/x": x, "prod/y": y, "prod/xt": xt, "prod/yt": yt, "prod/alpha": np.array([-0.75])})
    d["prod/mult"] = O.mult(A, x)
    d["prod/mult_add"] = O.mult_add(A, -0.75, x, y)
    d["prod/trans_mult"] = O.trans_mult(A, xt)
    d["prod/trans_mult_add"] = O.trans_mult_add(A, -0.75, xt, yt)
    # ---- systems: SPD 2D Poisson and nonsymmetric 3D convection-diffusion
    systems = {"poisson": workloads.poisson2d(12), "convdiff": workloads.convdiff3d(6)}
    for name, (n, rp, ci, v) in systems.items():
        put_csr(d, name + "/A", n, n, rp, ci, v)
        A = O.Csr(n, n, rp, ci, v)
        xt = rng.uniform(-1, 1, n)
        b = O.mult(A, xt)
        d[name + "/b"] = b
        kinds = [("jacobi", O.PC_JACOBI), ("ilu", O.PC_ILU)] + ([("icc", O.PC_ICC)] if name == "poisson" else [])
        for pname, pk in kinds:
            pc = O.Precond(pk, n)
            assert pc.set_matrix(A) == O.OK
            d[f"{name}/{pname}/apply"] = pc.apply(b)
            if pk != O.PC_JACOBI:
                d[f"{name}/{pname}/trans_apply"] = pc.trans_apply(b)
        runs = ([("cg_jacobi", O.CG, O.PC_JACOBI, 30), ("cg_icc", O.CG, O.PC_ICC, 30)] if name == "poisson" else
                [("bicgstab_ilu", O.BICGSTAB, O.PC_ILU, 30), ("gmres_ilu", O.GMRES, O.PC_ILU, 30),
                 ("gmres5_identity", O.GMRES, O.PC_IDENTITY, 5)])
        for rname, kind, pk, restart in runs:
            pc = O.Precond(pk, n)
            assert pc.set_matrix(A) == O.OK
            xs, res, hr, hi = O.solve(kind, A, b, np.zeros(n), pc, max_iter=2000, rtol=1e-10, restart=restart)
            assert res.status == O.OK, (name, rname, res.status)
            d[f"{name}/{rname}/x"] = xs
            d[f"{name}/{rname}/iterations"] = np.array([res.iterations], np.int64)
            d[f"{name}/{rname}/hist_r"] = hr
            d[f"{name}/{rname}/hist_it"] = hi.astype(np.int64)
            d[f"{name}/{rname}/restart"] = np.array([restart], np.int64)
    np.savez_compressed(OUT, **d)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
