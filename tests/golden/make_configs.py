"""Writes tests/golden/mtj_configs.npz: the oracle's outcome on the full-size
benchmark systems, for the GPU parity tests at those sizes.

  c1       2D 5-point Poisson 128^2, CG + DiagonalPreconditioner, seed 1
  c2jac    3D 7-point Poisson 128^3, CG + DiagonalPreconditioner, seed 2
  c2icc    3D 7-point Poisson 128^3, CG + ICC, seed 2 (and the ICC factor)
  c3gmres  3D upwind convection-diffusion 96^3, GMRES(30) + ILU, seed 3
  c3bicg   3D upwind convection-diffusion 96^3, BiCGstab + ILU, seed 3

b = A x_true with x_true ~ U[-1, 1) from the seed, x0 = 0, rtol 1e-10,
atol 1e-50, dtol 1e5.  For each run the fixture keeps SHA-256 hashes of the
inputs (rowptr, colind, data and b: the GPU test regenerates them and checks
the hashes first, so a generator that changed fails loudly), the oracle's
status, iteration count and full residual history, and x at 4096 fixed
indices.  c2icc adds the SHA-256 of the oracle's ICC factor (the data array
of ICC's private copy of A, S/ICC.java:79-139) -- the reach-based oracle
factor of this matrix takes minutes on one core, so the GPU test compares a
hash instead of running it.  c3bicg adds the summation-order envelope of
BiCGstab's history: how far the oracle's own relative residuals r_k / r_0
move when only the order of its dot products and norms changes (blocks of
16, 64, 256 and 1024 entries summed pairwise, oracle.sum_order).

Run from the repository root (about six minutes, most of it the ICC factor):
    python tests/golden/make_configs.py
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "matrix-toolkits-java_gb300"))

import oracle as O  # noqa: E402
from mtjg import workloads  # noqa: E402

OUT = os.path.join(HERE, "mtj_configs.npz")
SAMPLES = 4096

# name: (generator, grid, seed, solver, preconditioner, max iterations)
CONFIGS = {
    "c1": ("poisson2d", 128, 1, O.CG, O.PC_JACOBI, 2000),
    "c2jac": ("poisson3d", 128, 2, O.CG, O.PC_JACOBI, 5000),
    "c2icc": ("poisson3d", 128, 2, O.CG, O.PC_ICC, 5000),
    "c3gmres": ("convdiff3d", 96, 3, O.GMRES, O.PC_ILU, 5000),
    "c3bicg": ("convdiff3d", 96, 3, O.BICGSTAB, O.PC_ILU, 5000),
}


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def sample_index(n):
    return np.unique(np.linspace(0, n - 1, SAMPLES).astype(np.int64))


def system(gen, N, seed):
    n, rp, ci, v = getattr(workloads, gen)(N)
    A = O.Csr(n, n, rp, ci, v)
    b = O.mult(A, workloads.uniform(n, seed))
    return n, rp, ci, v, A, b


def main():
    O.build()
    d = {}
    cache = {}
    for name, (gen, N, seed, kind, pk, max_iter) in CONFIGS.items():
        t0 = time.perf_counter()
        key = (gen, N, seed)
        if key not in cache:
            cache = {key: system(gen, N, seed)}
        n, rp, ci, v, A, b = cache[key]
        pc = O.Precond(pk, n)
        st = pc.set_matrix(A)
        assert st == O.OK, (name, st)
        if pk == O.PC_ICC:
            d[name + "/factor_sha256"] = np.array(sha(pc.values()))
        x, res, hr, hi = O.solve(kind, A, b, np.zeros(n), pc, max_iter=max_iter, rtol=1e-10, atol=1e-50,
                                 dtol=1e5, restart=30)
        idx = sample_index(n)
        d[name + "/input_sha256"] = np.array(sha(np.asarray(rp, np.int32), np.asarray(ci, np.int32),
                                                 np.asarray(v, np.float64), b))
        d[name + "/n"] = np.array([n], np.int64)
        d[name + "/status"] = np.array([res.status], np.int32)
        d[name + "/iterations"] = np.array([res.iterations], np.int32)
        d[name + "/hist_r"] = hr
        d[name + "/hist_it"] = hi
        d[name + "/x_index"] = idx
        d[name + "/x_sample"] = x[idx]
        if kind == O.BICGSTAB:
            env = 0.0
            for block in (16, 64, 256, 1024):
                with O.sum_order(block):
                    _, _, h_blk, _ = O.solve(kind, A, b, np.zeros(n), pc, max_iter=max_iter, rtol=1e-10,
                                             restart=30)
                k = min(len(hr), len(h_blk))
                env = max(env, float(np.max(np.abs(hr[:k] - h_blk[:k])) / hr[0]))
            d[name + "/order_envelope"] = np.array([env])
        print(f"{name}: n={n} status={res.status} iterations={res.iterations} "
              f"history={len(hr)} ({time.perf_counter() - t0:.1f} s)", flush=True)
    np.savez_compressed(OUT, **d)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
