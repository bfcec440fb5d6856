"""Matrix Market input (mtjg_csr_parse_matrix_market_host, the parse behind
mtjg_csr_read_matrix_market) against a plain-Python restatement of MTJ's
reader: CompRowMatrix(MatrixVectorReader) (S/CompRowMatrix.java:86-166),
DenseVector(MatrixVectorReader) (M/DenseVector.java:52-96) and the
tokenizer of M/io/MatrixVectorReader.java.  No GPU: these run the host
parse.  The device path (upload, then a solve) is in test_gpu_mmio.py."""
import io
import re

import numpy as np
import pytest

from mtjg import sparse

scipy_io = pytest.importorskip("scipy.io")


# ------------------------------------------------ the restatement (checker)
def _tokens(text: str):
    # StreamTokenizer: '%' comments to end of line; whitespace ' ' and \t..\x0e
    body = re.sub(r"%[^\n\r]*", " ", text)
    return [t for t in re.split(r"[ \t\n\x0b\x0c\r\x0e]+", body) if t]


def _java_double(tok: str) -> float:
    s = tok.strip().lower()
    if s and s[-1] in "df":
        s = s[:-1]
    if not re.fullmatch(r"[+-]?(\d+\.?\d*|\.\d+)(e[+-]?\d+)?", s) and \
            not re.fullmatch(r"[+-]?0x([0-9a-f]+\.?[0-9a-f]*|\.[0-9a-f]+)p[+-]?\d+", s):
        raise IOError("For input string: " + tok)
    return float.fromhex(s) if "x" in s else float(s)


def _java_int(tok: str) -> int:
    d = _java_double(tok)
    if d != d:
        return 0
    return int(max(min(d, 2 ** 31 - 1), -2 ** 31))


def mtj_read(text: str):
    """(n, m, rowptr, colind, data) as MTJ builds them, or raises."""
    lines = text.splitlines()
    first = lines[0].strip() if lines else ""
    comp = [c for c in first.split(" ") if c] if first else [""]
    sym = "general"
    if comp[0].lower() == "%%matrixmarket":
        if len(comp) != 5:
            raise IOError("5 tokens")
        if comp[2].lower() == "array":
            raise sparse.UnsupportedOperationException("Dense")
        if comp[3].lower() in ("pattern", "complex"):
            raise sparse.UnsupportedOperationException(comp[3])
        sym = comp[4].lower()
        rest = text[len(lines[0]):]
    else:
        rest = text
    toks = _tokens(rest)
    n, m, ne = (_java_int(t) for t in toks[:3])
    ent = []
    for k in range(ne):
        r, c, v = toks[3 + 3 * k:6 + 3 * k]
        ent.append((_java_int(r) - 1, _java_int(c) - 1, _java_double(v)))
    for r, c, _ in ent:
        if not 0 <= r < n:
            raise IndexError(r)
    seq = list(ent)
    if sym in ("symmetric", "skew-symmetric"):
        seq += [(c, r, -v if sym == "skew-symmetric" else v) for r, c, v in ent if r != c]
    for r, c, _ in seq:
        if not 0 <= c < m:
            raise ValueError(c)
    val = {}
    for r, c, v in seq:  # CompRowMatrix.set overwrites: the last assignment wins
        val[(r, c)] = v
    rows = [sorted(c for (r, c) in val if r == i) for i in range(n)]
    rp = np.zeros(n + 1, dtype=np.int32)
    rp[1:] = np.cumsum([len(x) for x in rows])
    ci = np.array([c for x in rows for c in x], dtype=np.int32)
    dv = np.array([val[(i, c)] for i, x in enumerate(rows) for c in x], dtype=np.float64)
    return n, m, rp, ci, dv


def _same(got, want):
    n, m, rp, ci, v = got
    wn, wm, wrp, wci, wv = want
    assert (n, m) == (wn, wm)
    assert np.array_equal(rp, wrp) and np.array_equal(ci, wci)
    assert np.array_equal(v, wv)


# ------------------------------------------------------------------- cases
CASES = {
    "general": "%%MatrixMarket matrix coordinate real general\n% a comment\n3 4 4\n1 1 2.5\n2 4 -1e-3\n3 2 7\n1 3 .5\n",
    "symmetric": "%%MatrixMarket matrix coordinate real symmetric\n3 3 4\n1 1 4\n2 1 -1\n3 2 -2\n3 3 6\n",
    "skew": "%%MatrixMarket matrix coordinate real skew-symmetric\n3 3 2\n2 1 1.5\n3 1 -2\n",
    "integer_upper_case_header": "%%MATRIXMARKET Matrix COORDINATE Integer GENERAL\n2 2 3\n1 1 3\n2 2 4\n1 2 -5\n",
    "no_header": "2 3 2\n1 3 1.0\n2 1 2.0\n",
    "duplicates_last_wins": "%%MatrixMarket matrix coordinate real general\n2 2 4\n1 1 1\n1 1 2\n2 2 3\n1 1 9\n",
    "symmetric_mirror_after_direct": "%%MatrixMarket matrix coordinate real symmetric\n2 2 3\n1 2 5\n2 1 7\n1 1 1\n",
    "tokens_across_lines_and_comments": "%%MatrixMarket matrix coordinate real general\n2 2 2 1\n1 % c\n 3.0 2\n2\n4d\n",
    "explicit_zero_and_empty_row": "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 0\n3 3 1.0f\n",
    "no_entries": "%%MatrixMarket matrix coordinate real general\n4 4 0\n",
    "hex_and_exponents": "%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 0x1.8p1\n2 2 1E+2\n1.0e0 2 -0.25\n",
    "crlf": "%%MatrixMarket matrix coordinate real general\r\n2 2 2\r\n1 1 1.5\r\n2 2 2.5\r\n",
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_parse_matches_restatement(name):
    text = CASES[name]
    _same(sparse.parseMatrixMarket(text.encode()), mtj_read(text))


def test_parse_matches_scipy_on_files_without_duplicates():
    rng = np.random.default_rng(7)
    for sym in ("general", "symmetric", "skew-symmetric"):
        n = 40
        A = (rng.random((n, n)) < 0.15) * rng.uniform(-3, 3, (n, n))
        if sym == "symmetric":
            A = np.tril(A) + np.tril(A, -1).T
        elif sym == "skew-symmetric":
            A = np.tril(A, -1) - np.tril(A, -1).T
        buf = io.BytesIO()
        import scipy.sparse as sp
        scipy_io.mmwrite(buf, sp.coo_matrix(A), symmetry=sym)
        text = buf.getvalue()
        n2, m2, rp, ci, v = sparse.parseMatrixMarket(text)
        B = sp.csr_array((v, ci, rp), shape=(n2, m2)).toarray()
        assert np.array_equal(B, scipy_io.mmread(io.BytesIO(text), spmatrix=False).toarray())
        _same((n2, m2, rp, ci, v), mtj_read(text.decode()))


def test_large_file_parses_in_parallel_the_same():
    # several MB of text: the tokenizer splits it over threads at line ends
    rng = np.random.default_rng(11)
    n, ne = 20000, 300000
    r = rng.integers(1, n + 1, ne)
    c = rng.integers(1, n + 1, ne)
    v = rng.standard_normal(ne)
    lines = ["%%MatrixMarket matrix coordinate real general", "% generated", f"{n} {n} {ne}"]
    lines += [f"{a} {b} {float(x)!r}" for a, b, x in zip(r, c, v)]
    text = "\n".join(lines) + "\n"
    assert len(text) > 8 << 20
    got = sparse.parseMatrixMarket(text.encode())
    # restatement through a dict: the last assignment of each position wins
    val = {}
    for a, b, x in zip(r - 1, c - 1, v):
        val[(int(a), int(b))] = float(x)
    keys = sorted(val)
    rp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rp, np.array([k[0] for k in keys]) + 1, 1)
    rp = np.cumsum(rp)
    assert np.array_equal(got[2], rp)
    assert np.array_equal(got[3], np.array([k[1] for k in keys]))
    assert np.array_equal(got[4], np.array([val[k] for k in keys]))


@pytest.mark.parametrize("text,exc", [
    ("%%MatrixMarket matrix coordinate pattern general\n2 2 1\n1 1\n", sparse.UnsupportedOperationException),
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", sparse.UnsupportedOperationException),
    ("%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1 0\n", sparse.UnsupportedOperationException),
    ("%%MatrixMarket matrix coordinate real\n1 1 1\n1 1 1\n", IOError),
    ("%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1\n2 2 2\n", IOError),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 Infinity\n", IOError),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1.5D+00\n", IOError),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n", sparse.IndexOutOfBoundsException),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 3 1\n", sparse.IllegalArgumentException),
    ("%%MatrixMarket matrix coordinate real unknown\n2 2 1\n1 1 1\n", IOError),
])
def test_errors_map_to_mtj_exceptions(text, exc):
    with pytest.raises(exc):
        sparse.parseMatrixMarket(text.encode())


@pytest.mark.parametrize("text,want", [
    ("%%MatrixMarket vector array real\n3\n1.5\n-2\n4e1\n", [1.5, -2.0, 40.0]),
    ("%%MatrixMarket vector coordinate real\n4 2\n2 3.5\n4 -1\n", [0.0, 3.5, 0.0, -1.0]),
    ("%%MatrixMarket vector coordinate integer\n3 1\n1 7\n", [7.0, 0.0, 0.0]),
    ("3 2\n1 1.0\n3 2.0\n", [1.0, 0.0, 2.0]),
])
def test_dense_vector_reader(text, want):
    assert np.array_equal(sparse.readVector(text.encode()), np.array(want))


def test_dense_vector_reader_rejects_pattern_and_complex():
    with pytest.raises(sparse.UnsupportedOperationException):
        sparse.readVector(b"%%MatrixMarket vector coordinate pattern\n3 1\n1\n")
    with pytest.raises(sparse.UnsupportedOperationException):
        sparse.readVector(b"%%MatrixMarket vector array complex\n1\n1 2\n")


def test_reads_files_from_disk(tmp_path):
    p = tmp_path / "a.mtx"
    p.write_text(CASES["symmetric"])
    v = tmp_path / "b.mtx"
    v.write_text("%%MatrixMarket vector array real\n2\n1\n2\n")
    assert np.array_equal(sparse.readVector(str(v)), np.array([1.0, 2.0]))
    with pytest.raises(IOError):
        sparse.readVector(str(tmp_path / "missing.mtx"))


def _mtj_writer_coordinate(n, m, rows, cols, vals):
    """The text MatrixVectorWriter writes for a coordinate real general matrix
    (M/io/MatrixVectorWriter.java: printMatrixInfo, printMatrixSize with
    "%10d %10d %19d", printCoordinate with "%10d %10d % .12e", 1-based)."""
    out = ["%%MatrixMarket matrix coordinate real general\n", "%10d %10d %19d\n" % (n, m, len(vals))]
    for r, c, v in zip(rows, cols, vals):
        out.append("%10d %10d % .12e\n" % (r + 1, c + 1, v))
    return "".join(out)


def test_reference_sparse_write_read_round_trip():
    """The reference's known-answer test (MatrixVectorIoTest.testSparseWriteRead):
    a 3x3 CompRowMatrix with pattern {{1, 2}, {0, 2}, {1}} and values 1..5,
    written by MTJ's writer and read back, equals the original."""
    rows, cols, vals = [0, 0, 1, 1, 2], [1, 2, 0, 2, 1], [1.0, 2.0, 3.0, 4.0, 5.0]
    text = _mtj_writer_coordinate(3, 3, rows, cols, vals)
    n, m, rp, ci, v = sparse.parseMatrixMarket(text.encode())
    assert (n, m) == (3, 3)
    assert np.array_equal(rp, [0, 2, 4, 5]) and np.array_equal(ci, cols) and np.array_equal(v, vals)
    _same((n, m, rp, ci, v), mtj_read(text))


def test_writer_format_round_trips_every_double_exactly():
    """MTJ's writer keeps 13 significant digits ("% .12e"); reading its text
    gives the double nearest to each printed decimal, as Java's parser does."""
    rng = np.random.default_rng(11)
    vals = list(rng.standard_normal(200) * 10.0 ** rng.integers(-30, 30, 200))
    rows = list(range(200))
    text = _mtj_writer_coordinate(200, 200, rows, rows, vals)
    n, m, rp, ci, v = sparse.parseMatrixMarket(text.encode())
    want = [float("%.12e" % x) for x in vals]
    assert np.array_equal(v, want)
