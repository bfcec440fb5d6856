// mmio.cpp -- Matrix Market input: CompRowMatrix(MatrixVectorReader)
// (S/CompRowMatrix.java:86-166) and DenseVector(MatrixVectorReader)
// (M/DenseVector.java:52-96), with the tokenizer rules of
// M/io/MatrixVectorReader.java:
//   * an optional first line "%%MatrixMarket matrix <layout> <field> <symmetry>"
//     (5 tokens split on spaces, case-insensitive; vectors: 4 tokens); without
//     it a matrix is coordinate real general and a vector coordinate real;
//   * after it, tokens are maximal runs of characters other than whitespace
//     (' ', '\t'..'\x0e') and '%', which starts a comment to the end of the
//     line; lines carry no meaning;
//   * integers are read as Double.valueOf(token).intValue() (truncation,
//     saturation, NaN -> 0), values as Double.parseDouble(token) of the
//     lower-cased token (a trailing 'd' or 'f' is allowed).
// Matrices: pattern, array (dense) and complex files are unsupported, as in
// MTJ.  Entries become a CSR with sorted unique columns per row; the value of
// a position is the last one assigned, in MTJ's order: every entry of the
// file in file order, then (symmetric / skew-symmetric) every off-diagonal
// entry mirrored (negated when skew), again in file order.
//
// The text is tokenized by up to 16 threads: chunks end at newlines, which
// end any token and any comment, so each chunk tokenizes on its own.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <locale.h>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"

namespace mtjg {
namespace {

constexpr int kMaxThreads = 16;

bool is_ws(unsigned char c) { return c == ' ' || (c >= 0x09 && c <= 0x0e); }

struct Text {
    const char *p;
    int64_t n;
};

// The first line, as BufferedReader.readLine().trim() gives it.
std::string first_line(const Text &t, int64_t *after)
{
    int64_t e = 0;
    while (e < t.n && t.p[e] != '\n' && t.p[e] != '\r') ++e;
    int64_t next = e;
    if (next < t.n && t.p[next] == '\r') ++next;
    if (next < t.n && t.p[next] == '\n' && (next == e || t.p[next - 1] == '\r')) ++next;
    *after = next;
    int64_t b = 0, f = e;
    while (b < f && (unsigned char)t.p[b] <= ' ') ++b;
    while (f > b && (unsigned char)t.p[f - 1] <= ' ') --f;
    return std::string(t.p + b, (size_t)(f - b));
}

// String.split(" +") of a trimmed line
std::vector<std::string> split_spaces(const std::string &s)
{
    std::vector<std::string> out;
    size_t i = 0;
    while (i < s.size()) {
        size_t j = s.find(' ', i);
        if (j == std::string::npos) j = s.size();
        out.push_back(s.substr(i, j - i));
        i = j;
        while (i < s.size() && s[i] == ' ') ++i;
    }
    return out;
}

bool ieq(const std::string &a, const char *b)
{
    size_t n = std::strlen(b);
    if (a.size() != n) return false;
    for (size_t i = 0; i < n; ++i)
        if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
    return true;
}

struct Tok {
    int64_t b, e;
};

// Tokens of [b, e) (b and e at line starts / text end).
void tokenize(const Text &t, int64_t b, int64_t e, std::vector<Tok> &out)
{
    int64_t i = b;
    while (i < e) {
        const unsigned char c = (unsigned char)t.p[i];
        if (is_ws(c)) {
            ++i;
        } else if (c == '%') {
            while (i < e && t.p[i] != '\n' && t.p[i] != '\r') ++i;
        } else {
            const int64_t s = i;
            while (i < e && !is_ws((unsigned char)t.p[i]) && t.p[i] != '%') ++i;
            out.push_back(Tok{s, i});
        }
    }
}

std::vector<Tok> tokenize_all(const Text &t, int64_t start)
{
    const int64_t len = t.n - start;
    int nt = (int)std::min<int64_t>(kMaxThreads, std::max<int64_t>(1, len / (1 << 20)));
    nt = std::max(1, std::min<int>(nt, (int)std::thread::hardware_concurrency()));
    std::vector<int64_t> cut = {start};
    for (int k = 1; k < nt; ++k) {
        int64_t c = start + len * k / nt;
        while (c < t.n && t.p[c] != '\n') ++c;
        if (c < t.n) ++c;
        cut.push_back(std::max(c, cut.back()));
    }
    cut.push_back(t.n);
    std::vector<std::vector<Tok>> parts(nt);
    std::vector<std::thread> th;
    for (int k = 0; k < nt; ++k) th.emplace_back([&, k] { tokenize(t, cut[k], cut[k + 1], parts[k]); });
    for (auto &x : th) x.join();
    std::vector<Tok> all;
    size_t tot = 0;
    for (auto &p : parts) tot += p.size();
    all.reserve(tot);
    for (auto &p : parts) all.insert(all.end(), p.begin(), p.end());
    return all;
}

locale_t c_locale()
{
    static locale_t loc = newlocale(LC_NUMERIC_MASK, "C", (locale_t)0);
    return loc;
}

// Double.parseDouble of the lower-cased token (java.lang.Double's grammar):
// after String.trim(), an optional sign, then a decimal literal
// (digits[.digits] or .digits, optional e[sign]digits) or a hexadecimal one
// (0x mantissa p[sign]digits), then an optional 'd' or 'f'.  The lower-cased
// words "nan" and "infinity" are not numbers to Java (it expects "NaN" and
// "Infinity"), so they are rejected too.
bool parse_double(const Text &t, const Tok &k, double *out)
{
    const char *src = t.p + k.b;
    size_t n = (size_t)(k.e - k.b);
    while (n && (unsigned char)src[0] <= ' ') ++src, --n;
    while (n && (unsigned char)src[n - 1] <= ' ') --n;
    char buf[96];
    std::string big;
    char *p = buf;
    if (n + 1 > sizeof(buf)) {
        big.resize(n + 1);
        p = &big[0];
    }
    for (size_t i = 0; i < n; ++i) p[i] = (char)std::tolower((unsigned char)src[i]);
    size_t len = n;
    if (len && (p[len - 1] == 'd' || p[len - 1] == 'f')) --len;
    p[len] = 0;
    size_t i = 0;
    if (i < len && (p[i] == '+' || p[i] == '-')) ++i;
    auto digits = [&](bool hex) {
        size_t c = 0;
        while (i < len && (std::isdigit((unsigned char)p[i]) || (hex && p[i] >= 'a' && p[i] <= 'f'))) ++i, ++c;
        return c;
    };
    const bool hex = i + 1 < len && p[i] == '0' && p[i + 1] == 'x';
    if (hex) i += 2;
    size_t mant = digits(hex);
    if (i < len && p[i] == '.') {
        ++i;
        mant += digits(hex);
    }
    if (mant == 0) return false;
    if (i < len && p[i] == (hex ? 'p' : 'e')) {
        ++i;
        if (i < len && (p[i] == '+' || p[i] == '-')) ++i;
        if (digits(false) == 0) return false;
    } else if (hex) {
        return false;  // a hexadecimal literal needs its binary exponent
    }
    if (i != len) return false;
    char *end = nullptr;
    const double v = strtod_l(p, &end, c_locale());
    if (end != p + len) return false;
    *out = v;
    return true;
}

// Double.valueOf(token).intValue()
bool parse_int(const Text &t, const Tok &k, int *out)
{
    double d;
    if (!parse_double(t, k, &d)) return false;
    if (d != d) *out = 0;
    else if (d >= 2147483647.0) *out = 2147483647;
    else if (d <= -2147483648.0) *out = -2147483647 - 1;
    else *out = (int)d;
    return true;
}

int io_fail(const std::string &m) { return fail(MTJG_ERR_IO, m); }

struct Header {
    bool coordinate = true;
    int field = 0;     // 0 real, 1 integer, 2 complex, 3 pattern
    int symmetry = 0;  // 0 general, 1 symmetric, 2 skew-symmetric, 3 Hermitian
};

// MatrixVectorReader.hasInfo / readMatrixInfo / readVectorInfo
// (M/io/MatrixVectorReader.java:122-240); *start receives the first
// character the tokenizer reads.
int read_header(const Text &t, bool vector, Header *h, int64_t *start)
{
    int64_t after = 0;
    const std::string line = first_line(t, &after);
    const std::vector<std::string> c = split_spaces(line);
    *start = 0;
    if (c.empty() || !ieq(c[0], "%%MatrixMarket")) return MTJG_OK;  // no info: the defaults
    *start = after;
    const size_t want = vector ? 4 : 5;
    if (c.size() != want)
        return io_fail("Current line unparsable. It must consist of " + std::to_string(want) + " tokens");
    if (!ieq(c[1], vector ? "vector" : "matrix"))
        return io_fail(std::string("Expected \"") + (vector ? "vector" : "matrix") + "\", got " + c[1]);
    if (ieq(c[2], "coordinate")) h->coordinate = true;
    else if (ieq(c[2], "array")) h->coordinate = false;
    else return io_fail("Unknown layout " + c[2]);
    if (ieq(c[3], "real")) h->field = 0;
    else if (ieq(c[3], "integer")) h->field = 1;
    else if (ieq(c[3], "complex")) h->field = 2;
    else if (ieq(c[3], "pattern")) h->field = 3;
    else return io_fail("Unknown field specification " + c[3]);
    if (!vector) {
        if (ieq(c[4], "general")) h->symmetry = 0;
        else if (ieq(c[4], "symmetric")) h->symmetry = 1;
        else if (ieq(c[4], "skew-symmetric")) h->symmetry = 2;
        else if (ieq(c[4], "Hermitian")) h->symmetry = 3;
        else return io_fail("Unknown symmetry specification " + c[4]);
    }
    return MTJG_OK;
}

struct TokReader {
    const Text &t;
    const std::vector<Tok> &tok;
    size_t k = 0;
    int next_int(int *v)
    {
        if (k >= tok.size()) return io_fail("End-of-File encountered during parsing");
        if (!parse_int(t, tok[k], v))
            return fail(MTJG_ERR_IO, "For input string: \"" + std::string(t.p + tok[k].b, (size_t)(tok[k].e - tok[k].b)) + "\"");
        ++k;
        return MTJG_OK;
    }
    int next_double(double *v)
    {
        if (k >= tok.size()) return io_fail("End-of-File encountered during parsing");
        if (!parse_double(t, tok[k], v))
            return fail(MTJG_ERR_IO, "For input string: \"" + std::string(t.p + tok[k].b, (size_t)(tok[k].e - tok[k].b)) + "\"");
        ++k;
        return MTJG_OK;
    }
};

// The CSR of CompRowMatrix(MatrixVectorReader).
int parse_matrix(const Text &t, int *n_out, int *m_out, std::vector<int> &rowptr, std::vector<int> &colind,
                 std::vector<double> &val)
{
    Header h;
    int64_t start = 0;
    int st = read_header(t, false, &h, &start);
    if (st != MTJG_OK) return st;
    if (h.field == 3) return fail(MTJG_ERR_UNSUPPORTED, "Pattern matrices are not supported");
    if (!h.coordinate) return fail(MTJG_ERR_UNSUPPORTED, "Dense matrices are not supported");
    if (h.field == 2) return fail(MTJG_ERR_UNSUPPORTED, "Complex matrices are not supported");
    const std::vector<Tok> tok = tokenize_all(t, start);
    TokReader r{t, tok};
    int n = 0, m = 0, ne = 0;
    if ((st = r.next_int(&n)) != MTJG_OK || (st = r.next_int(&m)) != MTJG_OK || (st = r.next_int(&ne)) != MTJG_OK)
        return st;
    if (n < 0 || m < 0 || ne < 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "negative matrix size or entry count");
    if (tok.size() - r.k < (size_t)ne * 3) return io_fail("End-of-File encountered during parsing");
    // entries in file order (1-based indices shifted to 0-based)
    std::vector<int> row(ne), col(ne);
    std::vector<double> ent(ne);
    {
        const size_t base = r.k;
        int nt = std::max(1, std::min(kMaxThreads, ne / 65536));
        std::vector<int> err(nt, MTJG_OK);
        std::vector<std::string> msg(nt);
        std::vector<std::thread> th;
        for (int w = 0; w < nt; ++w)
            th.emplace_back([&, w] {
                const int a = (int)((int64_t)ne * w / nt), b = (int)((int64_t)ne * (w + 1) / nt);
                TokReader q{t, tok, base + 3 * (size_t)a};
                for (int i = a; i < b; ++i) {
                    int st2 = q.next_int(&row[i]);
                    if (st2 == MTJG_OK) st2 = q.next_int(&col[i]);
                    if (st2 == MTJG_OK) st2 = q.next_double(&ent[i]);
                    if (st2 != MTJG_OK) {
                        err[w] = st2;
                        msg[w] = mtjg_last_error();
                        return;
                    }
                    row[i] -= 1;
                    col[i] -= 1;
                }
            });
        for (auto &x : th) x.join();
        for (int w = 0; w < nt; ++w)
            if (err[w] != MTJG_OK) return fail(err[w], msg[w]);
    }
    // rows first (ArrayList.get in file order), then columns (construct)
    for (int i = 0; i < ne; ++i)
        if (row[i] < 0 || row[i] >= n)
            return fail(MTJG_ERR_INDEX_OUT_OF_BOUNDS, "Index: " + std::to_string(row[i]) + ", Size: " + std::to_string(n));
    const bool mirror = h.symmetry == 1 || h.symmetry == 2;
    if (mirror)
        for (int i = 0; i < ne; ++i)
            if (row[i] != col[i] && (col[i] < 0 || col[i] >= n))
                return fail(MTJG_ERR_INDEX_OUT_OF_BOUNDS,
                            "Index: " + std::to_string(col[i]) + ", Size: " + std::to_string(n));
    for (int i = 0; i < ne; ++i)
        if (col[i] < 0 || col[i] >= m)
            return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "nz[" + std::to_string(row[i]) + "]=" + std::to_string(col[i]) +
                                                       ", which is not a valid column index");
    // assignment sequence: entries, then mirrors; per row, a stable counting
    // sort keeps assignments in sequence order
    std::vector<int64_t> cnt((size_t)n + 1, 0);
    for (int i = 0; i < ne; ++i) {
        cnt[(size_t)row[i] + 1]++;
        if (mirror && row[i] != col[i]) cnt[(size_t)col[i] + 1]++;
    }
    for (int i = 0; i < n; ++i) cnt[(size_t)i + 1] += cnt[i];
    const int64_t total = cnt[(size_t)n];
    std::vector<int> acol((size_t)total);
    std::vector<double> aval((size_t)total);
    std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
    for (int i = 0; i < ne; ++i) {
        const int64_t p = pos[(size_t)row[i]]++;
        acol[(size_t)p] = col[i];
        aval[(size_t)p] = ent[i];
    }
    if (mirror)
        for (int i = 0; i < ne; ++i)
            if (row[i] != col[i]) {
                const int64_t p = pos[(size_t)col[i]]++;
                acol[(size_t)p] = row[i];
                aval[(size_t)p] = h.symmetry == 2 ? -ent[i] : ent[i];
            }
    // per row: stable sort by column, keep each column's last assignment
    std::vector<int> rlen((size_t)n, 0);
    {
        int nt = std::max(1, std::min(kMaxThreads, n / 16384));
        std::vector<std::thread> th;
        for (int w = 0; w < nt; ++w)
            th.emplace_back([&, w] {
                const int a = (int)((int64_t)n * w / nt), b = (int)((int64_t)n * (w + 1) / nt);
                std::vector<int> idx;
                std::vector<int> c2;
                std::vector<double> v2;
                for (int i = a; i < b; ++i) {
                    const int64_t s = cnt[i], e = cnt[(size_t)i + 1];
                    const int L = (int)(e - s);
                    idx.resize(L);
                    for (int q = 0; q < L; ++q) idx[q] = q;
                    std::stable_sort(idx.begin(), idx.end(),
                                     [&](int x, int y) { return acol[(size_t)(s + x)] < acol[(size_t)(s + y)]; });
                    c2.clear();
                    v2.clear();
                    for (int q = 0; q < L; ++q) {
                        const int c = acol[(size_t)(s + idx[q])];
                        const double v = aval[(size_t)(s + idx[q])];
                        if (!c2.empty() && c2.back() == c) v2.back() = v;
                        else {
                            c2.push_back(c);
                            v2.push_back(v);
                        }
                    }
                    for (size_t q = 0; q < c2.size(); ++q) {
                        acol[(size_t)s + q] = c2[q];
                        aval[(size_t)s + q] = v2[q];
                    }
                    rlen[i] = (int)c2.size();
                }
            });
        for (auto &x : th) x.join();
    }
    int64_t nnz = 0;
    for (int i = 0; i < n; ++i) nnz += rlen[i];
    if (nnz >= (1LL << 31)) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "more than 2^31 - 1 stored entries");
    rowptr.assign((size_t)n + 1, 0);
    colind.resize((size_t)nnz);
    val.resize((size_t)nnz);
    for (int i = 0; i < n; ++i) {
        rowptr[(size_t)i + 1] = rowptr[i] + rlen[i];
        std::copy(acol.begin() + cnt[i], acol.begin() + cnt[i] + rlen[i], colind.begin() + rowptr[i]);
        std::copy(aval.begin() + cnt[i], aval.begin() + cnt[i] + rlen[i], val.begin() + rowptr[i]);
    }
    *n_out = n;
    *m_out = m;
    return MTJG_OK;
}

// DenseVector(MatrixVectorReader)
int parse_vector(const Text &t, std::vector<double> &out)
{
    Header h;
    int64_t start = 0;
    int st = read_header(t, true, &h, &start);
    if (st != MTJG_OK) return st;
    const std::vector<Tok> tok = tokenize_all(t, start);
    TokReader r{t, tok};
    int size = 0, ne = 0;
    if ((st = r.next_int(&size)) != MTJG_OK) return st;
    if (h.coordinate && (st = r.next_int(&ne)) != MTJG_OK) return st;
    if (size < 0 || ne < 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "negative vector size or entry count");
    if (h.field == 3) return fail(MTJG_ERR_UNSUPPORTED, "Pattern vectors are not supported");
    if (h.field == 2) return fail(MTJG_ERR_UNSUPPORTED, "Complex vectors are not supported");
    out.assign((size_t)size, 0.0);
    if (h.coordinate) {
        std::vector<int> idx(ne);
        std::vector<double> ent(ne);
        for (int i = 0; i < ne; ++i) {
            if ((st = r.next_int(&idx[i])) != MTJG_OK || (st = r.next_double(&ent[i])) != MTJG_OK) return st;
            idx[i] -= 1;
        }
        for (int i = 0; i < ne; ++i) {
            if (idx[i] < 0 || idx[i] >= size)
                return fail(MTJG_ERR_INDEX_OUT_OF_BOUNDS, "index " + std::to_string(idx[i]) + ", size " +
                                                              std::to_string(size));
            out[(size_t)idx[i]] = ent[i];
        }
    } else {
        for (int i = 0; i < size; ++i)
            if ((st = r.next_double(&out[(size_t)i])) != MTJG_OK) return st;
    }
    return MTJG_OK;
}

int read_file(const char *path, std::vector<char> &buf)
{
    if (!path) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL path");
    FILE *f = std::fopen(path, "rb");
    if (!f) return io_fail(std::string(path) + " (No such file or directory)");
    std::fseek(f, 0, SEEK_END);
    const long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize(sz > 0 ? (size_t)sz : 0);
    const size_t got = sz > 0 ? std::fread(buf.data(), 1, (size_t)sz, f) : 0;
    std::fclose(f);
    if (got != buf.size()) return io_fail(std::string("reading ") + path + " failed");
    return MTJG_OK;
}

int matrix_from_text(mtjg_ctx *ctx, const Text &t, mtjg_csr **out)
{
    if (!ctx || !out) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    *out = nullptr;
    int n = 0, m = 0;
    std::vector<int> rp, ci;
    std::vector<double> v;
    const int st = parse_matrix(t, &n, &m, rp, ci, v);
    if (st != MTJG_OK) return st;
    return mtjg_csr_upload(ctx, n, m, rp.data(), ci.data(), v.data(), out);
}

int vector_out(const std::vector<double> &v, double *out, int64_t cap, int64_t *size)
{
    if (size) *size = (int64_t)v.size();
    if (out) std::memcpy(out, v.data(), sizeof(double) * (size_t)std::min<int64_t>(cap, (int64_t)v.size()));
    return MTJG_OK;
}

}  // namespace
}  // namespace mtjg

using namespace mtjg;

extern "C" MTJG_API int mtjg_csr_read_matrix_market(mtjg_ctx *ctx, const char *path, mtjg_csr **out)
{
    std::vector<char> buf;
    const int st = read_file(path, buf);
    if (st != MTJG_OK) return st;
    return matrix_from_text(ctx, Text{buf.data(), (int64_t)buf.size()}, out);
}

extern "C" MTJG_API int mtjg_csr_parse_matrix_market(mtjg_ctx *ctx, const char *text, int64_t len, mtjg_csr **out)
{
    if (!text && len > 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL text");
    return matrix_from_text(ctx, Text{text, len}, out);
}

extern "C" MTJG_API int mtjg_vector_read_matrix_market(const char *path, double *out, int64_t cap, int64_t *size)
{
    std::vector<char> buf;
    int st = read_file(path, buf);
    if (st != MTJG_OK) return st;
    std::vector<double> v;
    st = parse_vector(Text{buf.data(), (int64_t)buf.size()}, v);
    if (st != MTJG_OK) return st;
    return vector_out(v, out, cap, size);
}

extern "C" MTJG_API int mtjg_vector_parse_matrix_market(const char *text, int64_t len, double *out, int64_t cap,
                                                        int64_t *size)
{
    if (!text && len > 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL text");
    std::vector<double> v;
    const int st = parse_vector(Text{text, len}, v);
    if (st != MTJG_OK) return st;
    return vector_out(v, out, cap, size);
}

extern "C" MTJG_API int mtjg_csr_parse_matrix_market_host(const char *text, int64_t len, int *num_rows,
                                                          int *num_cols, int64_t *nnz, int *rowptr, int *colind,
                                                          double *val, int64_t cap)
{
    if (!text && len > 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL text");
    int n = 0, m = 0;
    std::vector<int> rp, ci;
    std::vector<double> v;
    const int st = parse_matrix(Text{text, len}, &n, &m, rp, ci, v);
    if (st != MTJG_OK) return st;
    if (num_rows) *num_rows = n;
    if (num_cols) *num_cols = m;
    if (nnz) *nnz = (int64_t)ci.size();
    if (rowptr) std::memcpy(rowptr, rp.data(), sizeof(int) * rp.size());
    const size_t k = (size_t)std::min<int64_t>(cap, (int64_t)ci.size());
    if (colind) std::memcpy(colind, ci.data(), sizeof(int) * k);
    if (val) std::memcpy(val, v.data(), sizeof(double) * k);
    return MTJG_OK;
}
