// host_io.cpp -- host-side loaders, TSP distances and seeded instance
// generators of the C ABI (no device needed).
//
// sbx_load_mtx follows CSR::from_file + construct_csr (src/csr.cpp:15-192):
// header words until "symmetric"/"general" ("pattern" switches to unweighted
// entries), '%' comment lines, "M N L", L entries with the diagonal dropped,
// W = sum of the file's weights, mirrored entries for symmetric files, rows
// sorted by (column, value) and duplicates kept.  Unlike the reference it
// keeps empty rows (src/csr.cpp:168-186 drops their row pointer) and returns
// an error where the reference loops forever on a missing or malformed file.
#include "../../include/sbx.h"
#include "host_par.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

struct Text {
    std::vector<char> buf;
    size_t pos = 0;
    bool load(const char *path)
    {
        FILE *f = fopen(path, "rb");
        if (!f) return false;
        fseek(f, 0, SEEK_END);
        long sz = ftell(f);
        fseek(f, 0, SEEK_SET);
        buf.resize(sz > 0 ? (size_t)sz + 1 : 1);
        size_t got = sz > 0 ? fread(buf.data(), 1, (size_t)sz, f) : 0;
        fclose(f);
        buf.resize(got + 1);
        buf[got] = 0;
        return true;
    }
    size_t size() const { return buf.size() - 1; }
    static bool ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }
    // operator>>(std::string)
    bool word(std::string &out)
    {
        while (pos < size() && ws(buf[pos])) pos++;
        if (pos >= size()) return false;
        size_t b = pos;
        while (pos < size() && !ws(buf[pos])) pos++;
        out.assign(&buf[b], pos - b);
        return true;
    }
    bool integer(long long &v)
    {
        while (pos < size() && ws(buf[pos])) pos++;
        if (pos >= size()) return false;
        char *end;
        v = strtoll(&buf[pos], &end, 10);
        if (end == &buf[pos]) return false;
        pos = (size_t)(end - buf.data());
        return true;
    }
    bool real(double &v)
    {
        while (pos < size() && ws(buf[pos])) pos++;
        if (pos >= size()) return false;
        char *end;
        v = strtod(&buf[pos], &end);
        if (end == &buf[pos]) return false;
        pos = (size_t)(end - buf.data());
        return true;
    }
    // istream::ignore(2048, '\n')
    void skip_line()
    {
        size_t k = 0;
        while (pos < size() && k < 2048) {
            k++;
            if (buf[pos++] == '\n') break;
        }
    }
    int peek() const { return pos < size() ? (unsigned char)buf[pos] : -1; }
};

struct Entry {
    int32_t r, c;
    double v;
};

using sbx::host_threads;
using sbx::parallel;

// construct_csr with every row kept: counting sort by row, then (col, value)
// within the row, which is the order of std::sort on the tuples
// (src/csr.cpp:157-192).  The rows are sorted by host threads in parallel.
void to_csr(int64_t n, std::vector<Entry> &t, int32_t *rowptr, int32_t *col, double *val)
{
    std::vector<int64_t> cnt((size_t)n + 1, 0);
    for (auto &e : t) cnt[(size_t)e.r + 1]++;
    for (int64_t i = 0; i < n; i++) cnt[i + 1] += cnt[i];
    std::vector<Entry> s(t.size());
    std::vector<int64_t> at(cnt.begin(), cnt.end() - 1);
    for (auto &e : t) s[(size_t)at[e.r]++] = e;
    const int T = t.size() > (1u << 20) ? host_threads() : 1;
    parallel(T, [&](int k, int K) {
        const int64_t r0 = n * k / K, r1 = n * (k + 1) / K;
        for (int64_t i = r0; i < r1; i++)
            std::sort(s.begin() + cnt[i], s.begin() + cnt[i + 1], [](const Entry &a, const Entry &b) {
                return a.c != b.c ? a.c < b.c : a.v < b.v;
            });
        for (int64_t k2 = cnt[r0]; k2 < cnt[r1]; k2++) {
            col[k2] = s[(size_t)k2].c;
            val[k2] = s[(size_t)k2].v;
        }
    });
    for (int64_t i = 0; i <= n; i++) rowptr[i] = (int32_t)cnt[i];
}

// The L entries "r c [v]" of an .mtx body from text position pos, the
// diagonal dropped, in file order.  Large bodies are cut at newlines into
// one piece per host thread and parsed in parallel; a piece that does not
// end on an entry boundary (an entry spread over lines) sends the whole body
// to the sequential parse, which reads tokens like istream's operator>>.
// Returns SBX_OK, SBX_ERR_FORMAT (short or malformed body, index out of range).
int parse_entries(Text &f, long long M, long long L, bool pattern, std::vector<Entry> &out)
{
    const size_t body = f.pos, end = f.size();
    const int T = (end - body) > (8u << 20) ? host_threads() : 1;
    if (T > 1) {
        std::vector<size_t> cut((size_t)T + 1);
        cut[0] = body;
        cut[(size_t)T] = end;
        for (int t = 1; t < T; t++) {
            size_t c = body + (end - body) * (size_t)t / (size_t)T;
            while (c < end && f.buf[c] != '\n') c++;
            cut[(size_t)t] = std::max(c, cut[(size_t)t - 1]);
        }
        std::vector<std::vector<Entry>> part((size_t)T);
        std::vector<long long> nread((size_t)T, 0);
        std::vector<int> bad((size_t)T, 0);
        parallel(T, [&](int t, int) {
            Text g;   // a view of the piece: parse with the same tokenizer
            g.buf.assign(f.buf.begin() + (long)cut[(size_t)t], f.buf.begin() + (long)cut[(size_t)t + 1]);
            g.buf.push_back(0);
            auto &v = part[(size_t)t];
            for (;;) {
                long long r, c;
                double d = 1;
                const size_t before = g.pos;
                if (!g.integer(r)) {
                    // only whitespace may remain
                    while (g.pos < g.size() && Text::ws(g.buf[g.pos])) g.pos++;
                    if (g.pos < g.size()) bad[(size_t)t] = 1;
                    break;
                }
                if (!g.integer(c) || (!pattern && !g.real(d))) {
                    bad[(size_t)t] = 1;   // entry split across pieces or malformed
                    g.pos = before;
                    break;
                }
                nread[(size_t)t]++;
                v.push_back({(int32_t)(r < 1 || r > M ? -1 : r - 1), (int32_t)(c < 1 || c > M ? -1 : c - 1), d});
            }
        });
        bool ok = true;
        for (int t = 0; t < T; t++) ok = ok && !bad[(size_t)t];
        if (ok) {
            long long total = 0;
            for (int t = 0; t < T; t++) total += nread[(size_t)t];
            if (total < L) return SBX_ERR_FORMAT;
            out.clear();
            out.reserve((size_t)L);
            long long taken = 0;
            for (int t = 0; t < T && taken < L; t++)
                for (const Entry &e : part[(size_t)t]) {
                    if (taken == L) break;
                    taken++;
                    if (e.r < 0 || e.c < 0) return SBX_ERR_FORMAT;
                    if (e.r != e.c) out.push_back(e);
                }
            return SBX_OK;
        }
    }
    out.clear();
    for (long long l = 0; l < L; l++) {
        long long r, c;
        double d = 1;
        if (!f.integer(r) || !f.integer(c) || (!pattern && !f.real(d))) return SBX_ERR_FORMAT;
        if (r < 1 || r > M || c < 1 || c > M) return SBX_ERR_FORMAT;
        if (r != c) out.push_back({(int32_t)(r - 1), (int32_t)(c - 1), d});
    }
    return SBX_OK;
}

// splitmix64: the seeded generator of the synthetic instances.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// Undirected edge list (u != v) -> symmetric CSR; W = sum over edges.
int finish(int64_t n, std::vector<Entry> &edges, int64_t *nnz, int32_t *rowptr, int32_t *col,
           double *val, double *wsum)
{
    double W = 0;
    for (auto &e : edges) W += e.v;
    *nnz = (int64_t)edges.size() * 2;
    if (wsum) *wsum = W;
    if (!rowptr || !col || !val) return SBX_OK;
    std::vector<Entry> t;
    t.reserve(edges.size() * 2);
    for (auto &e : edges) {
        t.push_back(e);
        t.push_back({e.c, e.r, e.v});
    }
    to_csr(n, t, rowptr, col, val);
    return SBX_OK;
}

}  // namespace

extern "C" {

int sbx_load_mtx(const char *path, int64_t *n_out, int64_t *nnz_out, int32_t *rowptr, int32_t *col,
                 double *val, double *wsum)
{
    if (!path || !n_out || !nnz_out) return SBX_ERR_ARG;
    Text f;
    if (!f.load(path)) return SBX_ERR_IO;
    bool symmetric = true, pattern = false, found = false;
    std::string w;
    while (!found) {
        if (!f.word(w)) return SBX_ERR_FORMAT;
        if (w == "symmetric") symmetric = found = true;
        else if (w == "pattern") pattern = true;
        else if (w == "integer") pattern = false;
        else if (w == "general") {
            symmetric = false;
            found = true;
        }
    }
    f.skip_line();
    while (f.peek() == '%') f.skip_line();
    long long M, N, L;
    if (!f.integer(M) || !f.integer(N) || !f.integer(L) || M <= 0 || L < 0 || M > INT32_MAX - 1)
        return SBX_ERR_FORMAT;
    std::vector<Entry> t;
    t.reserve((size_t)L * (symmetric ? 2 : 1));
    const int prc = parse_entries(f, M, L, pattern, t);
    if (prc) return prc;
    // W in file order, as the reference accumulates it (src/csr.cpp:69)
    double sum = 0;
    for (const Entry &e : t) sum += e.v;
    if (symmetric) {
        const size_t m0 = t.size();
        for (size_t i = 0; i < m0; i++) t.push_back({t[i].c, t[i].r, t[i].v});
    }
    if ((int64_t)t.size() > INT32_MAX) return SBX_ERR_UNSUPPORTED;
    *n_out = M;
    *nnz_out = (int64_t)t.size();
    if (wsum) *wsum = sum;
    if (rowptr && col && val) to_csr(M, t, rowptr, col, val);
    return SBX_OK;
}

// TSP_CPU::read_file (src/tsp_cpu.cpp:9-45): the line starting with 'D'
// (DIMENSION), the line starting with 'E' (EDGE_WEIGHT_TYPE: EUC_2D or GEO),
// then N "id x y" lines from the first line starting with '1'; GEO converts
// DDD.MM to radians.  "KEY : value" is accepted too (the reference hangs).
int sbx_load_tsplib(const char *path, int32_t *N_out, double *xc, double *yc, int32_t *kind)
{
    if (!path || !N_out || !kind) return SBX_ERR_ARG;
    Text f;
    if (!f.load(path)) return SBX_ERR_IO;
    std::string w;
    long long N;
    while (f.peek() != 'D') {
        if (f.peek() < 0) return SBX_ERR_FORMAT;
        f.skip_line();
    }
    if (!f.word(w)) return SBX_ERR_FORMAT;
    if (w == "DIMENSION" && !f.word(w)) return SBX_ERR_FORMAT;
    if (!f.integer(N) || N < 2 || N > 100000) return SBX_ERR_FORMAT;
    while (f.peek() != 'E') {
        if (f.peek() < 0) return SBX_ERR_FORMAT;
        f.skip_line();
    }
    if (!f.word(w)) return SBX_ERR_FORMAT;
    if (w == "EDGE_WEIGHT_TYPE" && !f.word(w)) return SBX_ERR_FORMAT;
    if (!f.word(w)) return SBX_ERR_FORMAT;
    if (w == "GEO") *kind = SBX_DIST_GEO;
    else if (w == "EUC_2D") *kind = SBX_DIST_EUC_2D;
    else return SBX_ERR_UNSUPPORTED;
    *N_out = (int32_t)N;
    if (!xc || !yc) return SBX_OK;
    while (f.peek() != '1') {
        if (f.peek() < 0) return SBX_ERR_FORMAT;
        f.skip_line();
    }
    const double PI = 3.14159265358979323846;
    for (long long i = 0; i < N; i++) {
        double id, la, lo;
        if (!f.real(id) || !f.real(la) || !f.real(lo)) return SBX_ERR_FORMAT;
        if (*kind == SBX_DIST_GEO) {
            int lat_deg = (int)la, long_deg = (int)lo;
            double lat_min = la - lat_deg, long_min = lo - long_deg;
            la = PI * (lat_deg + 5.0 * lat_min / 3.0) / 180.0;
            lo = PI * (long_deg + 5.0 * long_min / 3.0) / 180.0;
        }
        xc[i] = la;
        yc[i] = lo;
    }
    return SBX_OK;
}

// TSP_distances_EUC_2D / _GEO (src/kernels.cu:404-442) on the host, packed
// upper triangle, (int) truncation as the reference; EUC_2D_FLOAT keeps it.
int sbx_tsp_distances(int32_t N, const double *xc, const double *yc, int32_t kind, double *packed)
{
    if (N < 2 || !xc || !yc || !packed) return SBX_ERR_ARG;
    for (int32_t c1 = 0; c1 < N; c1++)
        for (int32_t c2 = c1 + 1; c2 < N; c2++) {
            double d;
            if (kind == SBX_DIST_GEO) {
                const double R = 6378.388;
                const double q1 = cos(yc[c1] - yc[c2]);
                const double q2 = cos(xc[c1] - xc[c2]);
                const double q3 = cos(xc[c1] + xc[c2]);
                d = (double)(int)(R * acos(0.5 * ((1.0 + q1) * q2 - (1.0 - q1) * q3)) + 1.0);
            } else {
                const double xd = xc[c1] - xc[c2], yd = yc[c1] - yc[c2];
                d = pow(xd * xd + yd * yd, 0.5);
                if (kind == SBX_DIST_EUC_2D) d = (double)(int)d;
            }
            packed[(int64_t)c2 + (int64_t)c1 * N - (int64_t)(c1 + 2) * (c1 + 1) / 2] = d;
        }
    return SBX_OK;
}

int sbx_gen_er(int64_t n, double p, int32_t pm1, uint64_t seed, int64_t *nnz, int32_t *rowptr,
               int32_t *col, double *val, double *wsum)
{
    if (n < 1 || n > INT32_MAX - 1 || !(p >= 0 && p <= 1) || !nnz) return SBX_ERR_ARG;
    Rng g(seed);
    std::vector<Entry> e;
    // Geometric skips over the pairs (i < j) in row-major order.
    if (p > 0) {
        const double lq = std::log(1.0 - std::min(p, 1.0 - 1e-15));
        int64_t i = 0, j = 0;   // current pair index (i, j), j > i
        for (;;) {
            const double u = g.uniform();
            int64_t skip = p >= 1.0 ? 0 : (int64_t)std::floor(std::log(1.0 - u) / lq);
            j += skip + 1;
            while (i < n && j >= n) {
                j = j - n + i + 2;
                i++;
            }
            if (i >= n - 1) break;
            const double w = pm1 ? ((g.next() >> 63) ? 1.0 : -1.0) : 1.0;
            e.push_back({(int32_t)i, (int32_t)j, w});
        }
    }
    return finish(n, e, nnz, rowptr, col, val, wsum);
}

int sbx_gen_torus(int32_t rows, int32_t cols, uint64_t seed, int64_t *nnz, int32_t *rowptr,
                  int32_t *col, double *val, double *wsum)
{
    if (rows < 3 || cols < 3 || (int64_t)rows * cols > INT32_MAX / 4 || !nnz) return SBX_ERR_ARG;
    Rng g(seed);
    std::vector<Entry> e;
    for (int32_t r = 0; r < rows; r++)
        for (int32_t c = 0; c < cols; c++) {
            const int32_t v = r * cols + c;
            const int32_t right = r * cols + (c + 1) % cols, down = ((r + 1) % rows) * cols + c;
            e.push_back({v, right, (g.next() >> 63) ? 1.0 : -1.0});
            e.push_back({v, down, (g.next() >> 63) ? 1.0 : -1.0});
        }
    return finish((int64_t)rows * cols, e, nnz, rowptr, col, val, wsum);
}

int sbx_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                 int64_t *nnz, int32_t *rowptr, int32_t *col, double *val, double *wsum)
{
    if (scale < 1 || scale > 30 || edge_factor < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1 || !nnz)
        return SBX_ERR_ARG;
    const int64_t n = 1ll << scale, m = (int64_t)edge_factor << scale;
    Rng g(seed);
    std::vector<uint64_t> keys;
    keys.reserve((size_t)m);
    for (int64_t k = 0; k < m; k++) {
        uint64_t u = 0, v = 0;
        for (int l = 0; l < scale; l++) {
            const double x = g.uniform();
            const int q = x < a ? 0 : x < a + b ? 1 : x < a + b + c ? 2 : 3;
            u = (u << 1) | (uint64_t)(q >> 1);
            v = (v << 1) | (uint64_t)(q & 1);
        }
        if (u == v) continue;   // self loop
        const uint64_t lo = std::min(u, v), hi = std::max(u, v);
        keys.push_back((lo << 32) | hi);
    }
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    std::vector<Entry> e;
    e.reserve(keys.size());
    for (uint64_t k : keys) e.push_back({(int32_t)(k >> 32), (int32_t)(k & 0xffffffffu), 1.0});
    return finish(n, e, nnz, rowptr, col, val, wsum);
}

int sbx_gen_rgg(int64_t n, double avg_degree, uint64_t seed, int64_t *nnz, int32_t *rowptr,
                int32_t *col, double *val, double *wsum)
{
    if (n < 2 || n > (1 << 26) || !(avg_degree > 0) || !nnz) return SBX_ERR_ARG;
    Rng g(seed);
    std::vector<double> px((size_t)n), py((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        px[i] = g.uniform();
        py[i] = g.uniform();
    }
    const double rad = std::sqrt(avg_degree / ((double)n * 3.14159265358979323846));
    const int cells = std::max(1, (int)std::floor(1.0 / rad));
    std::vector<std::vector<int32_t>> grid((size_t)cells * cells);
    for (int64_t i = 0; i < n; i++) {
        const int cx = std::min(cells - 1, (int)(px[i] * cells)), cy = std::min(cells - 1, (int)(py[i] * cells));
        grid[(size_t)cy * cells + cx].push_back((int32_t)i);
    }
    std::vector<Entry> e;
    const double r2 = rad * rad;
    for (int cy = 0; cy < cells; cy++)
        for (int cx = 0; cx < cells; cx++)
            for (int32_t i : grid[(size_t)cy * cells + cx])
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        const int nx = cx + dx, ny = cy + dy;
                        if (nx < 0 || ny < 0 || nx >= cells || ny >= cells) continue;
                        for (int32_t j : grid[(size_t)ny * cells + nx]) {
                            if (j <= i) continue;
                            const double ddx = px[i] - px[j], ddy = py[i] - py[j];
                            if (ddx * ddx + ddy * ddy <= r2) e.push_back({i, j, 0.0});
                        }
                    }
    std::sort(e.begin(), e.end(), [](const Entry &a, const Entry &b) { return a.r != b.r ? a.r < b.r : a.c < b.c; });
    for (auto &x : e) x.v = (g.next() >> 63) ? 1.0 : -1.0;
    return finish(n, e, nnz, rowptr, col, val, wsum);
}

int sbx_gen_cities(int32_t N, double scale, uint64_t seed, double *xc, double *yc)
{
    if (N < 2 || !xc || !yc || !(scale > 0)) return SBX_ERR_ARG;
    Rng g(seed);
    for (int32_t i = 0; i < N; i++) {
        xc[i] = g.uniform() * scale;
        yc[i] = g.uniform() * scale;
    }
    return SBX_OK;
}

}  // extern "C"
