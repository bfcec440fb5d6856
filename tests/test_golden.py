"""Golden fixtures (tests/golden/mtj_small.npz, written by
tests/golden/make_golden.py from the oracle).

CPU: the oracle reproduces every fixture bit for bit.
GPU: in STRICT numerics the CSR products and preconditioner applies equal
the fixtures bit for bit; the solvers meet the parity bar (iteration count
within 2, relative residual history within 1e-10 of r_0 -- BiCGstab within
four times its own summation-order envelope -- and x within 1e-8)."""
import os

import numpy as np
import pytest

import oracle as O

GOLD = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mtj_small.npz"))

RUNS = [("poisson", "cg_jacobi", O.CG, O.PC_JACOBI), ("poisson", "cg_icc", O.CG, O.PC_ICC),
        ("convdiff", "bicgstab_ilu", O.BICGSTAB, O.PC_ILU), ("convdiff", "gmres_ilu", O.GMRES, O.PC_ILU),
        ("convdiff", "gmres5_identity", O.GMRES, O.PC_IDENTITY)]
PCS = [("poisson", "jacobi", O.PC_JACOBI), ("poisson", "ilu", O.PC_ILU), ("poisson", "icc", O.PC_ICC),
       ("convdiff", "jacobi", O.PC_JACOBI), ("convdiff", "ilu", O.PC_ILU)]


def _csr(key):
    n, m = (int(t) for t in GOLD[key + "/shape"])
    return n, m, GOLD[key + "/rowptr"], GOLD[key + "/colind"], GOLD[key + "/val"]


# ------------------------------------------------------------------ CPU
def test_oracle_products_match_fixture():
    A = O.Csr(*_csr("prod/A"))
    a = float(GOLD["prod/alpha"][0])
    assert np.array_equal(O.mult(A, GOLD["prod/x"]), GOLD["prod/mult"])
    assert np.array_equal(O.mult_add(A, a, GOLD["prod/x"], GOLD["prod/y"]), GOLD["prod/mult_add"])
    assert np.array_equal(O.trans_mult(A, GOLD["prod/xt"]), GOLD["prod/trans_mult"])
    assert np.array_equal(O.trans_mult_add(A, a, GOLD["prod/xt"], GOLD["prod/yt"]), GOLD["prod/trans_mult_add"])


@pytest.mark.parametrize("sysname,pname,pk", PCS)
def test_oracle_preconditioners_match_fixture(sysname, pname, pk):
    n, _, rp, ci, v = _csr(sysname + "/A")
    pc = O.Precond(pk, n)
    assert pc.set_matrix(O.Csr(n, n, rp, ci, v)) == O.OK
    b = GOLD[sysname + "/b"]
    assert np.array_equal(pc.apply(b), GOLD[f"{sysname}/{pname}/apply"])
    if pk != O.PC_JACOBI:
        assert np.array_equal(pc.trans_apply(b), GOLD[f"{sysname}/{pname}/trans_apply"])


@pytest.mark.parametrize("sysname,rname,kind,pk", RUNS)
def test_oracle_solves_match_fixture(sysname, rname, kind, pk):
    n, _, rp, ci, v = _csr(sysname + "/A")
    A = O.Csr(n, n, rp, ci, v)
    pc = O.Precond(pk, n)
    assert pc.set_matrix(A) == O.OK
    restart = int(GOLD[f"{sysname}/{rname}/restart"][0])
    x, res, hr, hi = O.solve(kind, A, GOLD[sysname + "/b"], np.zeros(n), pc, max_iter=2000, rtol=1e-10,
                             restart=restart)
    key = f"{sysname}/{rname}"
    assert res.status == O.OK and res.iterations == int(GOLD[key + "/iterations"][0])
    assert np.array_equal(x, GOLD[key + "/x"])
    assert np.array_equal(hr, GOLD[key + "/hist_r"]) and np.array_equal(hi, GOLD[key + "/hist_it"])


# ------------------------------------------------------------------ GPU
@pytest.fixture(scope="module")
def strict_ctx():
    from mtjg import _lib as L
    from mtjg import sparse
    c = sparse.Context(0, L.NUMERICS_STRICT)
    yield c


@pytest.mark.gpu
def test_gpu_products_equal_fixture(strict_ctx):
    from mtjg import sparse
    A = sparse.CompRowMatrix(*_csr("prod/A"), ctx=strict_ctx)
    a = float(GOLD["prod/alpha"][0])
    assert np.array_equal(A.mult(GOLD["prod/x"]), GOLD["prod/mult"])
    assert np.array_equal(A.multAdd(a, GOLD["prod/x"], GOLD["prod/y"].copy()), GOLD["prod/mult_add"])
    assert np.array_equal(A.transMult(GOLD["prod/xt"]), GOLD["prod/trans_mult"])
    assert np.array_equal(A.transMultAdd(a, GOLD["prod/xt"], GOLD["prod/yt"].copy()), GOLD["prod/trans_mult_add"])


@pytest.mark.gpu
@pytest.mark.parametrize("sysname,pname,pk", PCS)
def test_gpu_preconditioners_equal_fixture(strict_ctx, sysname, pname, pk):
    from mtjg import sparse
    n, _, rp, ci, v = _csr(sysname + "/A")
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx=strict_ctx)
    M = {O.PC_JACOBI: sparse.DiagonalPreconditioner, O.PC_ILU: sparse.ILU, O.PC_ICC: sparse.ICC}[pk](n, strict_ctx)
    M.setMatrix(A)
    b = GOLD[sysname + "/b"]
    assert np.array_equal(M.apply(b), GOLD[f"{sysname}/{pname}/apply"])
    if pk != O.PC_JACOBI:
        assert np.array_equal(M.transApply(b), GOLD[f"{sysname}/{pname}/trans_apply"])


def _order_envelope(kind, pk, n, rp, ci, v, b, restart):
    """How far the oracle's own relative residual history moves when its
    dot products are summed in blocks instead of sequentially."""
    A = O.Csr(n, n, rp, ci, v)
    pc = O.Precond(pk, n)
    pc.set_matrix(A)
    _, _, h_seq, _ = O.solve(kind, A, b, np.zeros(n), pc, max_iter=2000, rtol=1e-10, restart=restart)
    env = 0.0
    for block in (16, 64, 256, 1024):
        with O.sum_order(block):
            _, _, h_blk, _ = O.solve(kind, A, b, np.zeros(n), pc, max_iter=2000, rtol=1e-10, restart=restart)
        k = min(len(h_seq), len(h_blk))
        env = max(env, float(np.max(np.abs(h_seq[:k] - h_blk[:k])) / h_seq[0]))
    return env


@pytest.mark.gpu
@pytest.mark.parametrize("numerics", [0, 1], ids=["fast", "strict"])
@pytest.mark.parametrize("sysname,rname,kind,pk", RUNS)
def test_gpu_solves_meet_parity_bar_on_fixture(ctx, numerics, sysname, rname, kind, pk):
    from mtjg import sparse
    n, _, rp, ci, v = _csr(sysname + "/A")
    key = f"{sysname}/{rname}"
    restart = int(GOLD[key + "/restart"][0])
    ctx.setNumerics(numerics)
    try:
        A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
        cls = {O.CG: sparse.CG, O.BICGSTAB: sparse.BiCGstab, O.GMRES: sparse.GMRES}[kind]
        solver = cls(n, restart=restart, ctx=ctx) if kind == O.GMRES else cls(n, ctx=ctx)
        if pk != O.PC_IDENTITY:
            M = {O.PC_JACOBI: sparse.DiagonalPreconditioner, O.PC_ILU: sparse.ILU, O.PC_ICC: sparse.ICC}[pk](n, ctx)
            M.setMatrix(A)
            solver.setPreconditioner(M)
        mon = sparse.DefaultIterationMonitor(2000, 1e-10, 1e-50, 1e5)
        mon.setIterationReporter(sparse.IterationReporter(), history_cap=8192)
        solver.setIterationMonitor(mon)
        x = np.zeros(n)
        b = GOLD[sysname + "/b"]
        solver.solve(A, b, x)
    finally:
        ctx.setNumerics(0)
    it = solver.getIterationMonitor().iterations()
    assert abs(it - int(GOLD[key + "/iterations"][0])) <= 2
    gr, gi = solver.history
    hr, hi = GOLD[key + "/hist_r"], GOLD[key + "/hist_it"]
    k = min(len(gr), len(hr))
    assert np.array_equal(gi[:k], hi[:k])
    rel = float(np.max(np.abs(gr[:k] - hr[:k])) / hr[0])
    bar = 1e-10
    if kind == O.BICGSTAB:
        bar = max(bar, 4.0 * _order_envelope(kind, pk, n, rp, ci, v, b, restart))
    assert rel <= bar, (rel, bar)
    xo = GOLD[key + "/x"]
    assert np.max(np.abs(x - xo)) <= 1e-8 * max(1.0, np.max(np.abs(xo)))


# ------------------------------------------------- full-size configurations
CONF_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mtj_configs.npz")


def test_config_fixture_inputs_and_c1_reproduce():
    """The full-size fixture (tests/golden/make_configs.py): the generators
    give the same 2D Poisson 128^2 system here, and the oracle reproduces its
    CG + Jacobi history and x bit for bit (the larger runs take minutes on
    one core and are checked by the GPU tests through the fixture)."""
    import hashlib

    from mtjg import workloads

    conf = np.load(CONF_PATH)
    n, rp, ci, v = workloads.poisson2d(128)
    A = O.Csr(n, n, rp, ci, v)
    b = O.mult(A, workloads.uniform(n, 1))
    h = hashlib.sha256()
    for a in (rp, ci, v, b):
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == str(conf["c1/input_sha256"])
    pc = O.Precond(O.PC_JACOBI, n)
    assert pc.set_matrix(A) == O.OK
    x, res, hr, hi = O.solve(O.CG, A, b, np.zeros(n), pc, max_iter=2000, rtol=1e-10)
    assert res.status == int(conf["c1/status"][0]) and res.iterations == int(conf["c1/iterations"][0])
    assert np.array_equal(hr, conf["c1/hist_r"]) and np.array_equal(hi, conf["c1/hist_it"])
    assert np.array_equal(x[conf["c1/x_index"]], conf["c1/x_sample"])
    for name in ("c2jac", "c2icc", "c3gmres", "c3bicg"):
        assert int(conf[name + "/status"][0]) == 0
        assert len(conf[name + "/hist_r"]) == len(conf[name + "/hist_it"]) > 1
