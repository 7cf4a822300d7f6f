// emv_host.cpp -- host side of the EMV solver: STP reader, CSR builder,
// admission checks, instance generators and STP writer (C ABI, include/emv.h).
//
// Reference counterparts (reader/reader-el.c unless stated):
//   graph_load        R:473-618   -> emv_stp_parse / emv_stp_load
//   root_build        R:706-899   -> emv_csr_build (no virtual vertices)
//   gen-unique        graph-gen/gen-unique.c:480-557 -> emv_gen_regular / emv_gen_mixed
//   graph_out_dimacs  graph-gen/gen-unique.c:244-273 -> emv_stp_write
#include "emv_internal.h"

#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

// ------------------------------------------------------------------ errors

static thread_local std::string g_last_error;

int emv_fail(int status, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

extern "C" const char *emv_last_error(void) { return g_last_error.c_str(); }

extern "C" const char *emv_status_str(int status)
{
    switch (status) {
    case EMV_OK: return "ok";
    case EMV_ERR_BAD_INPUT: return "bad input";
    case EMV_ERR_PARSE: return "parse error";
    case EMV_ERR_OOM: return "out of memory";
    case EMV_ERR_OVER_BUDGET: return "over admission budget";
    case EMV_ERR_TIMEOUT: return "device loop timeout";
    case EMV_ERR_CUDA: return "cuda error";
    case EMV_ERR_DISCONNECTED: return "graph not connected";
    case EMV_ERR_OVERFLOW: return "values would reach the int32 sentinel";
    case EMV_ERR_NOT_READY: return "not ready";
    case EMV_ERR_CANCELLED: return "cancelled";
    case EMV_ERR_INTERNAL: return "internal error";
    default: return "unknown status";
    }
}

// -------------------------------------------------------------- STP parser

namespace {

struct StpBuilder {
    int64_t n = 0, m = 0, k = 0, cost = -1;
    bool has_graph = false, has_terminals = false, term_alloc = false;
    std::vector<int64_t> edges;
    std::vector<int64_t> terms;
};

// One line of the grammar of graph_load (R:494-589).  `line` holds the line
// as fgets would return it (terminating '\n' included when present).
int parse_line(StpBuilder &b, const char *line, int &in_section, int64_t lineno)
{
    char buf[1024];
    std::strncpy(buf, line, sizeof(buf) - 1);
    buf[sizeof(buf) - 1] = '\0';
    char *save = nullptr;
    char *c = strtok_r(buf, " ", &save);
    if (c == nullptr) return EMV_OK;  // only spaces: the reference would crash here
    long a = 0, bb = 0, cc = 0;
    if (!std::strcmp(c, "section")) {
        if (in_section) return emv_fail(EMV_ERR_PARSE, "line %lld: nested sections", (long long)lineno);
        in_section = 1;
        char section[256];
        if (std::sscanf(line, "section %255s", section) != 1)
            return emv_fail(EMV_ERR_PARSE, "line %lld: invalid section line", (long long)lineno);
        if (!std::strcmp(section, "comment")) {
        } else if (!std::strcmp(section, "graph")) {
            b.has_graph = true;
        } else if (!std::strcmp(section, "terminals")) {
            b.has_terminals = true;
        } else if (!std::strcmp(section, "coordinates")) {
        } else {
            return emv_fail(EMV_ERR_PARSE, "line %lld: invalid section", (long long)lineno);
        }
    } else if (!std::strcmp(c, "end\n")) {
        if (!in_section) return emv_fail(EMV_ERR_PARSE, "line %lld: no section to end", (long long)lineno);
        in_section = 0;
    } else if (!std::strcmp(c, "nodes")) {
        if (std::sscanf(line, "nodes %ld", &a) != 1)
            return emv_fail(EMV_ERR_PARSE, "line %lld: invalid nodes line", (long long)lineno);
        b.n = a;
    } else if (!std::strcmp(c, "edges")) {
        if (std::sscanf(line, "edges %ld", &a) != 1)
            return emv_fail(EMV_ERR_PARSE, "line %lld: invalid edges line", (long long)lineno);
        b.m = a;
        if (a > 0 && a < (int64_t)1 << 40) b.edges.reserve(3 * (size_t)a);
    } else if (!std::strcmp(c, "terminals")) {
        if (std::sscanf(line, "terminals %ld", &a) != 1)
            return emv_fail(EMV_ERR_PARSE, "line %lld: invalid terminals line", (long long)lineno);
        b.k = a;
        b.term_alloc = true;
        b.terms.clear();
    } else if (!std::strcmp(c, "coordinates")) {
        // R:540-548 rejects this token unconditionally.
        return emv_fail(EMV_ERR_PARSE, "line %lld: duplicate section coordinates", (long long)lineno);
    } else if (!std::strcmp(c, "e")) {
        if (std::sscanf(line, "e %ld %ld %ld", &a, &bb, &cc) != 3)
            return emv_fail(EMV_ERR_PARSE, "line %lld: invalid edge line", (long long)lineno);
        int64_t u = a - 1, v = bb - 1;
        if (u < 0 || v < 0 || u >= b.n || v >= b.n)
            return emv_fail(EMV_ERR_PARSE, "line %lld: edge endpoint out of range", (long long)lineno);
        b.edges.push_back(u);
        b.edges.push_back(v);
        b.edges.push_back(cc);
    } else if (!std::strcmp(c, "t")) {
        if (std::sscanf(line, "t %ld", &a) != 1)
            return emv_fail(EMV_ERR_PARSE, "line %lld: invalid terminal line", (long long)lineno);
        if (!b.term_alloc)
            return emv_fail(EMV_ERR_PARSE, "line %lld: section terminals not initialised", (long long)lineno);
        int64_t u = a - 1;
        if (u < 0 || u >= b.n)
            return emv_fail(EMV_ERR_PARSE, "line %lld: terminal out of range", (long long)lineno);
        if ((int64_t)b.terms.size() + 1 > b.k)
            return emv_fail(EMV_ERR_PARSE, "line %lld: more terminals than declared", (long long)lineno);
        b.terms.push_back(u);
    } else if (!std::strcmp(c, "cost")) {
        if (std::sscanf(line, "cost %ld", &a) != 1)
            return emv_fail(EMV_ERR_PARSE, "line %lld: invalid cost line", (long long)lineno);
        b.cost = a;
    }
    // "dd", "eof" and every other line are ignored (R:579-589).
    return EMV_OK;
}

int finish(StpBuilder &b, emv_stp **out)
{
    // Final checks of R:597-600.
    if (b.n == 0) return emv_fail(EMV_ERR_PARSE, "no nodes");
    if (b.m == 0 || b.m != (int64_t)(b.edges.size() / 3))
        return emv_fail(EMV_ERR_PARSE, "edge count %lld does not match edges line %lld",
                        (long long)(b.edges.size() / 3), (long long)b.m);
    if (b.k == 0 || b.k != (int64_t)b.terms.size())
        return emv_fail(EMV_ERR_PARSE, "terminal count %lld does not match terminals line %lld",
                        (long long)b.terms.size(), (long long)b.k);
    if (!b.has_graph || !b.has_terminals)
        return emv_fail(EMV_ERR_PARSE, "missing graph or terminals section");
    emv_stp *g = (emv_stp *)std::calloc(1, sizeof(emv_stp));
    if (!g) return emv_fail(EMV_ERR_OOM, "stp alloc");
    g->n = b.n; g->m = b.m; g->k = b.k; g->cost = b.cost;
    g->edges = (int64_t *)std::malloc(sizeof(int64_t) * b.edges.size());
    g->terminals = (int64_t *)std::malloc(sizeof(int64_t) * (b.terms.size() ? b.terms.size() : 1));
    if (!g->edges || !g->terminals) { emv_stp_free(g); return emv_fail(EMV_ERR_OOM, "stp alloc"); }
    std::memcpy(g->edges, b.edges.data(), sizeof(int64_t) * b.edges.size());
    std::memcpy(g->terminals, b.terms.data(), sizeof(int64_t) * b.terms.size());
    *out = g;
    return EMV_OK;
}

}  // namespace

extern "C" int emv_stp_parse(const char *text, int64_t len, emv_stp **out)
{
    if (!text || len < 0 || !out) return emv_fail(EMV_ERR_BAD_INPUT, "null argument");
    *out = nullptr;
    StpBuilder b;
    int in_section = 0;
    int64_t lineno = 0, i = 0;
    char line[1024];
    while (i < len) {
        // fgets semantics (R:491): at most 1023 bytes, '\n' kept.
        int64_t j = 0;
        while (i < len && j < 1023) {
            char ch = text[i++];
            line[j++] = ch;
            if (ch == '\n') break;
        }
        line[j] = '\0';
        lineno++;
        if (std::strlen(line) != (size_t)j)
            return emv_fail(EMV_ERR_PARSE, "line %lld: NUL byte", (long long)lineno);
        int st = parse_line(b, line, in_section, lineno);
        if (st != EMV_OK) return st;
    }
    return finish(b, out);
}

extern "C" int emv_stp_load(const char *path, emv_stp **out)
{
    if (!out) return emv_fail(EMV_ERR_BAD_INPUT, "null argument");
    FILE *f = path ? std::fopen(path, "rb") : stdin;
    if (!f) return emv_fail(EMV_ERR_PARSE, "unable to open file '%s'", path);
    std::string text;
    char buf[1 << 16];
    size_t r;
    while ((r = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, r);
    if (path) std::fclose(f);
    return emv_stp_parse(text.data(), (int64_t)text.size(), out);
}

extern "C" void emv_stp_free(emv_stp *g)
{
    if (!g) return;
    std::free(g->edges);
    std::free(g->terminals);
    std::free(g);
}

extern "C" int emv_stp_write(const emv_stp *g, const char *path)
{
    if (!g || !path) return emv_fail(EMV_ERR_BAD_INPUT, "null argument");
    FILE *f = std::fopen(path, "wb");
    if (!f) return emv_fail(EMV_ERR_BAD_INPUT, "cannot write '%s'", path);
    std::string s;
    s.reserve(64 + (size_t)g->m * 24);
    char line[128];
    s += "33d32945 stp file, stp format version 1.0\n\nsection comment\n";
    s += "name    \"generated\"\ncreator \"emv-gb300\"\nend\n\nsection graph\n";
    std::snprintf(line, sizeof line, "nodes %lld\nedges %lld\n", (long long)g->n, (long long)g->m);
    s += line;
    for (int64_t e = 0; e < g->m; e++) {
        std::snprintf(line, sizeof line, "e %lld %lld %lld\n", (long long)g->edges[3 * e] + 1,
                      (long long)g->edges[3 * e + 1] + 1, (long long)g->edges[3 * e + 2]);
        s += line;
    }
    std::snprintf(line, sizeof line, "end\n\nsection terminals\nterminals %lld\n", (long long)g->k);
    s += line;
    for (int64_t t = 0; t < g->k; t++) {
        std::snprintf(line, sizeof line, "t %lld\n", (long long)g->terminals[t] + 1);
        s += line;
    }
    s += "end\n\n";
    if (g->cost >= 0) {
        std::snprintf(line, sizeof line, "cost %lld\n", (long long)g->cost);
        s += line;
    }
    s += "eof\n";
    size_t wr = std::fwrite(s.data(), 1, s.size(), f);
    std::fclose(f);
    return wr == s.size() ? EMV_OK : emv_fail(EMV_ERR_BAD_INPUT, "short write");
}

// --------------------------------------------------------------------- CSR

// Degree count and prefix sum (R:750-792): row_ptr only.
static int csr_pos(int64_t n, int64_t m, const int64_t *edges, int32_t *row_ptr)
{
    if (n <= 0 || n >= INT32_MAX || m < 0 || 2 * m >= INT32_MAX || (m > 0 && !edges) || !row_ptr)
        return emv_fail(EMV_ERR_BAD_INPUT, "csr: bad sizes");
    for (int64_t e = 0; e < m; e++) {
        int64_t u = edges[3 * e], v = edges[3 * e + 1], x = edges[3 * e + 2];
        if (u < 0 || v < 0 || u >= n || v >= n) return emv_fail(EMV_ERR_BAD_INPUT, "csr: endpoint out of range");
        if (x < 0) return emv_fail(EMV_ERR_BAD_INPUT, "csr: negative weight");
        if (x >= EMV_INF32) return emv_fail(EMV_ERR_OVERFLOW, "csr: weight %lld reaches 2^30", (long long)x);
    }
    std::vector<int64_t> deg((size_t)n + 1, 0);
    for (int64_t e = 0; e < m; e++) {
        deg[(size_t)edges[3 * e]]++;
        deg[(size_t)edges[3 * e + 1]]++;
    }
    int64_t run = 0;
    for (int64_t u = 0; u < n; u++) {
        row_ptr[u] = (int32_t)run;
        run += deg[(size_t)u];
    }
    row_ptr[n] = (int32_t)run;
    return EMV_OK;
}

// The fill in edge order (R:794-826), both arcs of every edge.
static int csr_adj(int64_t n, int64_t m, const int64_t *edges, const int32_t *row_ptr, int32_t *col, int32_t *w)
{
    if (m > 0 && (!col || !w)) return emv_fail(EMV_ERR_BAD_INPUT, "csr: bad sizes");
    std::vector<int64_t> fill(row_ptr, row_ptr + n);
    for (int64_t e = 0; e < m; e++) {
        int64_t u = edges[3 * e], v = edges[3 * e + 1];
        int32_t x = (int32_t)edges[3 * e + 2];
        col[fill[(size_t)u]] = (int32_t)v; w[fill[(size_t)u]++] = x;
        col[fill[(size_t)v]] = (int32_t)u; w[fill[(size_t)v]++] = x;
    }
    return EMV_OK;
}

extern "C" int emv_csr_build(int64_t n, int64_t m, const int64_t *edges, int32_t *row_ptr,
                             int32_t *col, int32_t *w)
{
    int st = csr_pos(n, m, edges, row_ptr);
    return st ? st : csr_adj(n, m, edges, row_ptr, col, w);
}

int emv_csr_build_timed(int64_t n, int64_t m, const int64_t *edges, int32_t *row_ptr, int32_t *col, int32_t *w,
                        double *pos_ms, double *adj_ms)
{
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    int st = csr_pos(n, m, edges, row_ptr);
    const auto t1 = clk::now();
    if (!st) st = csr_adj(n, m, edges, row_ptr, col, w);
    const auto t2 = clk::now();
    if (pos_ms) *pos_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    if (adj_ms) *adj_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
    return st;
}

int emv_graph_validate(const emv_graph *g)
{
    if (!g || g->n <= 0 || g->arcs < 0 || !g->row_ptr || (g->arcs > 0 && (!g->col || !g->w)))
        return emv_fail(EMV_ERR_BAD_INPUT, "graph: null array or bad size");
    if (g->arcs >= INT32_MAX) return emv_fail(EMV_ERR_BAD_INPUT, "graph: too many arcs");
    return EMV_OK;
}

extern "C" int emv_graph_check(const emv_graph *g, int64_t *bound_out)
{
    int st = emv_graph_validate(g);
    if (st) return st;
    const int32_t n = g->n;
    if (g->row_ptr[0] != 0 || g->row_ptr[n] != g->arcs) return emv_fail(EMV_ERR_BAD_INPUT, "graph: row_ptr ends");
    for (int32_t u = 0; u < n; u++)
        if (g->row_ptr[u + 1] < g->row_ptr[u]) return emv_fail(EMV_ERR_BAD_INPUT, "graph: row_ptr not monotone");
    int64_t maxw = 0, sumw = 0;
    for (int64_t e = 0; e < g->arcs; e++) {
        int32_t v = g->col[e], x = g->w[e];
        if (v < 0 || v >= n) return emv_fail(EMV_ERR_BAD_INPUT, "graph: arc head out of range");
        if (x < 0) return emv_fail(EMV_ERR_BAD_INPUT, "graph: negative weight");
        if (x > maxw) maxw = x;
        sumw += x;
    }
    // Connectivity by BFS from vertex 0.
    std::vector<int32_t> queue((size_t)n);
    std::vector<uint8_t> seen((size_t)n, 0);
    int64_t head = 0, tail = 0;
    queue[tail++] = 0;
    seen[0] = 1;
    while (head < tail) {
        int32_t u = queue[(size_t)head++];
        for (int32_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; e++) {
            int32_t v = g->col[e];
            if (!seen[(size_t)v]) { seen[(size_t)v] = 1; queue[(size_t)tail++] = v; }
        }
    }
    if (tail != n) return emv_fail(EMV_ERR_DISCONNECTED, "graph: %lld of %d vertices reachable from vertex 1",
                                   (long long)tail, n);
    // Every finite d[X][v] is the weight of a Steiner tree, at most the weight of
    // a spanning tree: at most (n-1)*max_w and at most the sum of all weights
    // (each edge appears as two arcs, so the arc sum is halved).
    int64_t bound = std::min<int64_t>((int64_t)(n - 1) * maxw, sumw / 2);
    if (bound_out) *bound_out = bound;
    if (bound >= EMV_INF32)
        return emv_fail(EMV_ERR_OVERFLOW, "graph: table values may reach 2^30 (bound %lld)", (long long)bound);
    return EMV_OK;
}

// --------------------------------------------------------------- generator

namespace {

uint64_t splitmix64(uint64_t &x)
{
    uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// xoshiro256** (Blackman & Vigna), seeded through splitmix64.
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed)
    {
        uint64_t x = seed;
        for (auto &w : s) w = splitmix64(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next()
    {
        uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    // Uniform integer in [0, range) by Lemire's multiply-and-reject.
    uint64_t below(uint64_t range)
    {
        uint64_t x = next();
        __uint128_t mm = (__uint128_t)x * range;
        uint64_t lo = (uint64_t)mm;
        if (lo < range) {
            uint64_t thr = (0 - range) % range;
            while (lo < thr) {
                x = next();
                mm = (__uint128_t)x * range;
                lo = (uint64_t)mm;
            }
        }
        return (uint64_t)(mm >> 64);
    }
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
};

// exp2 for x in [0, 64) from +, *, / only, so that x86-64 and aarch64 give
// the same bits (host code is compiled with -ffp-contract=off).
double det_exp2(double x)
{
    int ip = (int)x;
    double f = (x - ip) * 0.69314718055994530942;  // f * ln 2, in [0, ln 2)
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 30; i++) {
        term = term * f / i;
        sum += term;
    }
    return std::ldexp(sum, ip);
}

// log2 for x > 0 from frexp and the atanh series.
double det_log2(double x)
{
    int e;
    double mnt = std::frexp(x, &e);  // x = mnt * 2^e, mnt in [0.5, 1)
    double z = (mnt - 1.0) / (mnt + 1.0), z2 = z * z, term = z, sum = 0.0;
    for (int i = 1; i < 60; i += 2) {
        sum += term / i;
        term *= z2;
    }
    return e + 2.0 * sum / 0.69314718055994530942;
}

struct Dsu {
    std::vector<int64_t> p;
    explicit Dsu(int64_t n) : p((size_t)n) { for (int64_t i = 0; i < n; i++) p[(size_t)i] = i; }
    int64_t find(int64_t x)
    {
        while (p[(size_t)x] != x) { p[(size_t)x] = p[(size_t)p[(size_t)x]]; x = p[(size_t)x]; }
        return x;
    }
    bool join(int64_t a, int64_t b)
    {
        a = find(a); b = find(b);
        if (a == b) return false;
        p[(size_t)a] = b;
        return true;
    }
};

// Configuration-model pairing of the stubs of a degree sequence (vertex v
// holds deg[v] stubs), redrawn from the same stream until connected.
int config_edges(Rng &rng, const std::vector<int32_t> &deg, int32_t wmin, int32_t wmax, std::vector<int64_t> &edges)
{
    const int64_t n = (int64_t)deg.size();
    int64_t stubs = 0;
    for (int32_t d : deg) stubs += d;
    const int64_t m = stubs / 2;
    std::vector<int32_t> st((size_t)stubs), owner((size_t)stubs);
    for (int64_t v = 0, pos = 0; v < n; v++)
        for (int32_t j = 0; j < deg[(size_t)v]; j++) owner[(size_t)pos++] = (int32_t)v;
    for (int attempt = 0; attempt < 1000; attempt++) {
        for (int64_t i = 0; i < stubs; i++) st[(size_t)i] = owner[(size_t)i];
        for (int64_t i = stubs - 1; i > 0; i--) {
            int64_t j = (int64_t)rng.below((uint64_t)i + 1);
            std::swap(st[(size_t)i], st[(size_t)j]);
        }
        edges.assign((size_t)(3 * m), 0);
        Dsu dsu(n);
        int64_t comps = n;
        for (int64_t e = 0; e < m; e++) {
            int64_t u = st[(size_t)(2 * e)], v = st[(size_t)(2 * e + 1)];
            edges[(size_t)(3 * e)] = u;
            edges[(size_t)(3 * e + 1)] = v;
            edges[(size_t)(3 * e + 2)] = wmin + (int64_t)rng.below((uint64_t)(wmax - wmin) + 1);
            if (dsu.join(u, v)) comps--;
        }
        if (comps == 1) return EMV_OK;
    }
    return emv_fail(EMV_ERR_DISCONNECTED, "generator: no connected pairing in 1000 draws");
}

int regular_edges(Rng &rng, int64_t n, int32_t d, int32_t wmin, int32_t wmax, std::vector<int64_t> &edges)
{
    return config_edges(rng, std::vector<int32_t>((size_t)n, d), wmin, wmax, edges);
}

double det_pow(double x, double y) { return det_exp2(y * det_log2(x)); }  // x > 0

// Power-law degree sequence with `classes` degree classes (gen-unique.c's
// mkpowlawdist, graph-gen/gen-unique.c:409-470, restated): class sizes grow
// geometrically, f_j ~ b^j with sum n (b by bisection); degrees follow
// f_j^alpha scaled so that the mean degree is d; the total is made even.
int powlaw_degrees(int64_t n, int32_t d, double alpha, int32_t classes, std::vector<int32_t> &deg)
{
    double lo = 1.0, hi = det_exp2(det_log2((double)n) / (double)(classes - 1)), b = lo;
    for (int it = 0; it < 200; it++) {
        b = 0.5 * (lo + hi);
        double s = 0, p = 1;
        for (int32_t j = 0; j < classes; j++) { s += p; p *= b; }
        if (s < (double)n) lo = b; else hi = b;
    }
    std::vector<int64_t> freq((size_t)classes);
    int64_t fsum = 0;
    double p = b;
    for (int32_t j = 0; j < classes; j++) {
        const double cum = (1.0 - p) / (1.0 - b);
        freq[(size_t)j] = std::max<int64_t>(1, (int64_t)(cum - (double)fsum + 0.5));
        fsum += freq[(size_t)j];
        p *= b;
    }
    freq[(size_t)classes - 1] += n - fsum;  // exact total n
    if (freq[(size_t)classes - 1] < 1) return emv_fail(EMV_ERR_BAD_INPUT, "generator: too many degree classes");
    double norm = 0;
    for (int64_t f : freq) norm += det_pow((double)f, alpha + 1.0);
    const double scale = (double)d * (double)n / norm;
    std::vector<int32_t> cdeg((size_t)classes);
    for (int32_t j = 0; j < classes; j++) {
        const double x = scale * det_pow((double)freq[(size_t)j], alpha);
        cdeg[(size_t)j] = (int32_t)std::min<double>(std::max<double>(1.0, x + 0.5), (double)(n - 1));
    }
    deg.clear();
    int64_t total = 0;
    for (int32_t j = 0; j < classes; j++)
        for (int64_t i = 0; i < freq[(size_t)j]; i++) {
            deg.push_back(cdeg[(size_t)j]);
            total += cdeg[(size_t)j];
        }
    if (total % 2) deg[0]++;
    return EMV_OK;
}

void sample_distinct(Rng &rng, int64_t n, int32_t k, std::vector<int64_t> &out)
{
    // Partial Fisher-Yates over a lazily materialised identity permutation.
    std::vector<int64_t> perm((size_t)n);
    for (int64_t i = 0; i < n; i++) perm[(size_t)i] = i;
    out.resize((size_t)k);
    for (int32_t i = 0; i < k; i++) {
        int64_t j = i + (int64_t)rng.below((uint64_t)(n - i));
        std::swap(perm[(size_t)i], perm[(size_t)j]);
        out[(size_t)i] = perm[(size_t)i];
    }
}

int make_stp(int64_t n, const std::vector<int64_t> &edges, const std::vector<int64_t> &terms, emv_stp **out)
{
    emv_stp *g = (emv_stp *)std::calloc(1, sizeof(emv_stp));
    if (!g) return emv_fail(EMV_ERR_OOM, "stp alloc");
    g->n = n;
    g->m = (int64_t)edges.size() / 3;
    g->k = (int64_t)terms.size();
    g->cost = -1;
    g->edges = (int64_t *)std::malloc(sizeof(int64_t) * (edges.size() ? edges.size() : 1));
    g->terminals = (int64_t *)std::malloc(sizeof(int64_t) * (terms.size() ? terms.size() : 1));
    if (!g->edges || !g->terminals) { emv_stp_free(g); return emv_fail(EMV_ERR_OOM, "stp alloc"); }
    std::memcpy(g->edges, edges.data(), sizeof(int64_t) * edges.size());
    std::memcpy(g->terminals, terms.data(), sizeof(int64_t) * terms.size());
    *out = g;
    return EMV_OK;
}

}  // namespace

extern "C" int emv_gen_regular(int64_t n, int32_t degree, int32_t wmin, int32_t wmax, int32_t k, uint64_t seed,
                               emv_stp **out)
{
    if (!out) return emv_fail(EMV_ERR_BAD_INPUT, "null argument");
    *out = nullptr;
    if (n < 2 || n >= INT32_MAX || degree < 1 || (n * degree) % 2 != 0 || n * degree >= INT32_MAX)
        return emv_fail(EMV_ERR_BAD_INPUT, "generator: need n*degree even and in range");
    if (wmin < 0 || wmax < wmin || wmax >= EMV_INF32) return emv_fail(EMV_ERR_BAD_INPUT, "generator: weight range");
    if (k < 1 || k > n) return emv_fail(EMV_ERR_BAD_INPUT, "generator: k out of range");
    Rng rng(seed);
    std::vector<int64_t> edges, terms;
    int st = regular_edges(rng, n, degree, wmin, wmax, edges);
    if (st) return st;
    sample_distinct(rng, n, k, terms);
    return make_stp(n, edges, terms, out);
}

extern "C" int emv_gen_mixed(uint64_t base_seed, int64_t index, int32_t nmin, int32_t nmax, int32_t kmin,
                             int32_t kmax, int32_t group_pct, emv_stp **out)
{
    if (!out) return emv_fail(EMV_ERR_BAD_INPUT, "null argument");
    *out = nullptr;
    if (nmin < 16 || nmax < nmin || kmin < 1 || kmax < kmin || kmax > nmin || group_pct < 0 || group_pct > 100 ||
        index < 0)
        return emv_fail(EMV_ERR_BAD_INPUT, "generator: bad mixed parameters");
    Rng rng(base_seed + (uint64_t)index);
    static const int32_t degrees[4] = {3, 4, 6, 8};
    double ln_ratio = det_log2((double)nmax / (double)nmin);
    int64_t n = (int64_t)(nmin * det_exp2(ln_ratio * rng.unit()) + 0.5);
    if (n < nmin) n = nmin;
    if (n > nmax) n = nmax;
    int32_t d = degrees[rng.below(4)];
    if ((n * d) % 2) n = (n + 1 <= nmax) ? n + 1 : n - 1;
    int32_t k = kmin + (int32_t)rng.below((uint64_t)(kmax - kmin) + 1);
    bool group = (int32_t)rng.below(100) < group_pct;
    std::vector<int64_t> edges, terms;
    int st = regular_edges(rng, n, d, 1, 1000, edges);
    if (st) return st;
    if (!group) {
        sample_distinct(rng, n, k, terms);
        return make_stp(n, edges, terms, out);
    }
    // Group instance: 6 groups of 1..8 distinct vertices, root n+g joined to
    // each member by a zero-weight edge; the roots are the terminals.
    const int32_t groups = 6;
    for (int32_t g = 0; g < groups; g++) {
        int32_t size = 1 + (int32_t)rng.below(8);
        std::vector<int64_t> members;
        sample_distinct(rng, n, size, members);
        for (int64_t v : members) {
            edges.push_back(n + g);
            edges.push_back(v);
            edges.push_back(0);
        }
        terms.push_back(n + g);
    }
    return make_stp(n + groups, edges, terms, out);
}

extern "C" int emv_gen_powlaw(int64_t n, int32_t degree, double alpha, int32_t classes, int32_t wmin, int32_t wmax,
                              int32_t k, uint64_t seed, emv_stp **out)
{
    if (!out) return emv_fail(EMV_ERR_BAD_INPUT, "null argument");
    *out = nullptr;
    if (n < 2 || n >= INT32_MAX / 64 || degree < 1 || !(alpha < 0.0) || classes < 2 || classes > n)
        return emv_fail(EMV_ERR_BAD_INPUT, "generator: need alpha < 0, 2 <= classes <= n");
    if (wmin < 0 || wmax < wmin || wmax >= EMV_INF32) return emv_fail(EMV_ERR_BAD_INPUT, "generator: weight range");
    if (k < 1 || k > n) return emv_fail(EMV_ERR_BAD_INPUT, "generator: k out of range");
    std::vector<int32_t> deg;
    int st = powlaw_degrees(n, degree, alpha, classes, deg);
    if (st) return st;
    Rng rng(seed);
    // vertex ids are shuffled so that degree does not follow the id
    std::vector<int64_t> perm;
    sample_distinct(rng, n, (int32_t)n, perm);
    std::vector<int32_t> pdeg((size_t)n);
    for (int64_t i = 0; i < n; i++) pdeg[(size_t)perm[(size_t)i]] = deg[(size_t)i];
    std::vector<int64_t> edges, terms;
    st = config_edges(rng, pdeg, wmin, wmax, edges);
    if (st) return st;
    sample_distinct(rng, n, k, terms);
    return make_stp(n, edges, terms, out);
}

extern "C" int emv_gen_clique(int64_t n, int32_t wmin, int32_t wmax, int32_t k, uint64_t seed, emv_stp **out)
{
    if (!out) return emv_fail(EMV_ERR_BAD_INPUT, "null argument");
    *out = nullptr;
    if (n < 2 || n > 46341) return emv_fail(EMV_ERR_BAD_INPUT, "generator: clique of n in [2, 46341]");
    if (wmin < 0 || wmax < wmin || wmax >= EMV_INF32) return emv_fail(EMV_ERR_BAD_INPUT, "generator: weight range");
    if (k < 1 || k > n) return emv_fail(EMV_ERR_BAD_INPUT, "generator: k out of range");
    Rng rng(seed);
    std::vector<int64_t> edges, terms;
    edges.reserve((size_t)(n * (n - 1) / 2 * 3));
    for (int64_t u = 0; u < n; u++)
        for (int64_t v = u + 1; v < n; v++) {
            edges.push_back(u);
            edges.push_back(v);
            edges.push_back(wmin + (int64_t)rng.below((uint64_t)(wmax - wmin) + 1));
        }
    sample_distinct(rng, n, k, terms);
    return make_stp(n, edges, terms, out);
}
