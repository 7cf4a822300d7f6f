// emv_bin.cpp -- packed binary container of solver inputs (no text parse on
// ingress).
//
// The reference's experiment driver asks its generator and reader for "-bin"
// graph files (experiments/report.py:265-266, 457-470), but neither
// graph-gen/gen-unique.c nor reader/reader-el.c implements a binary format:
// the generator always prints STP text (gen-unique.c:244-273, 643).  This
// container is therefore new.  It stores each instance in the form the
// solver consumes -- the int32 CSR of emv_csr_build (both arcs of every edge)
// plus the terminals -- so loading is a read and a bounds check, and
// optionally the STP edge list, so an instance converts back to STP exactly.
//
// Layout (little-endian, every array padded to 8 bytes):
//   "EMVBIN01"  u64 count  u64 offset[count]
//   instance at offset[i]: i64 n, m, k, cost (-1: none), flags (bit 0: edges)
//                          i32 row_ptr[n+1], col[2m], w[2m], terminals[k],
//                          [i32 edges[3m]: u, v, w]
#include "emv_internal.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

namespace {

constexpr char BIN_MAGIC[8] = {'E', 'M', 'V', 'B', 'I', 'N', '0', '1'};
constexpr int64_t REC_HEAD = 5 * 8;

int64_t pad8(int64_t bytes) { return (bytes + 7) / 8 * 8; }

bool little_endian()
{
    const uint32_t x = 1;
    unsigned char b;
    std::memcpy(&b, &x, 1);
    return b == 1;
}

struct RecView {
    int64_t n, m, k, cost, flags;
    const int32_t *row_ptr, *col, *w, *terms, *edges;
};

}  // namespace

struct emv_bin {
    std::vector<uint64_t> words;  // the whole file, 8-byte aligned
    int64_t bytes = 0;
    int64_t count = 0;
    std::vector<char> checked;    // instance i passed the full check
    const unsigned char *base() const { return reinterpret_cast<const unsigned char *>(words.data()); }
};

static int rec_bytes(int64_t n, int64_t m, int64_t k, int64_t flags, int64_t *out)
{
    if (n <= 0 || n >= INT32_MAX || m < 0 || 2 * m >= INT32_MAX || k <= 0 || k >= INT32_MAX / 4 || (flags & ~1LL))
        return emv_fail(EMV_ERR_PARSE, "bin: bad instance sizes n=%lld m=%lld k=%lld flags=%lld", (long long)n,
                        (long long)m, (long long)k, (long long)flags);
    int64_t b = REC_HEAD + pad8(4 * (n + 1)) + 2 * pad8(8 * m) + pad8(4 * k);
    if (flags & 1) b += pad8(12 * m);
    *out = b;
    return EMV_OK;
}

// Header and array views of record i, with every size checked against the file.
static int rec_view(const emv_bin *b, int64_t i, RecView *v)
{
    if (i < 0 || i >= b->count) return emv_fail(EMV_ERR_BAD_INPUT, "bin: index %lld of %lld", (long long)i,
                                                (long long)b->count);
    uint64_t off;
    std::memcpy(&off, b->base() + 16 + 8 * i, 8);
    if (off % 8 || off < (uint64_t)(16 + 8 * b->count) || off > (uint64_t)b->bytes ||
        (uint64_t)b->bytes - off < (uint64_t)REC_HEAD)
        return emv_fail(EMV_ERR_PARSE, "bin: instance %lld offset %llu outside the file", (long long)i,
                        (unsigned long long)off);
    const unsigned char *p = b->base() + off;
    int64_t h[5];
    std::memcpy(h, p, sizeof h);
    int64_t need;
    int r = rec_bytes(h[0], h[1], h[2], h[4], &need);
    if (r) return r;
    if ((uint64_t)b->bytes - off < (uint64_t)need)
        return emv_fail(EMV_ERR_PARSE, "bin: instance %lld truncated", (long long)i);
    v->n = h[0]; v->m = h[1]; v->k = h[2]; v->cost = h[3]; v->flags = h[4];
    const unsigned char *q = p + REC_HEAD;
    v->row_ptr = reinterpret_cast<const int32_t *>(q); q += pad8(4 * (v->n + 1));
    v->col = reinterpret_cast<const int32_t *>(q); q += pad8(8 * v->m);
    v->w = reinterpret_cast<const int32_t *>(q); q += pad8(8 * v->m);
    v->terms = reinterpret_cast<const int32_t *>(q); q += pad8(4 * v->k);
    v->edges = (v->flags & 1) ? reinterpret_cast<const int32_t *>(q) : nullptr;
    return EMV_OK;
}

// Contents of record i: a CSR that emv_csr_build could have produced
// (prefix sums from 0 to 2m, heads in range, weights in [0, 2^30)), terminals
// in range, and an edge list consistent with the CSR's degrees.
static int rec_check(const RecView &v)
{
    const int64_t arcs = 2 * v.m;
    if (v.row_ptr[0] != 0 || v.row_ptr[v.n] != arcs) return emv_fail(EMV_ERR_PARSE, "bin: row_ptr ends");
    for (int64_t u = 0; u < v.n; u++)
        if (v.row_ptr[u + 1] < v.row_ptr[u]) return emv_fail(EMV_ERR_PARSE, "bin: row_ptr decreases at %lld",
                                                             (long long)u);
    for (int64_t e = 0; e < arcs; e++) {
        if (v.col[e] < 0 || v.col[e] >= v.n) return emv_fail(EMV_ERR_PARSE, "bin: arc %lld head out of range",
                                                              (long long)e);
        if (v.w[e] < 0 || v.w[e] >= EMV_INF32) return emv_fail(EMV_ERR_PARSE, "bin: arc %lld weight out of range",
                                                                (long long)e);
    }
    for (int64_t t = 0; t < v.k; t++)
        if (v.terms[t] < 0 || v.terms[t] >= v.n) return emv_fail(EMV_ERR_PARSE, "bin: terminal out of range");
    if (v.edges) {
        std::vector<int64_t> deg((size_t)v.n, 0);
        for (int64_t e = 0; e < v.m; e++) {
            const int32_t a = v.edges[3 * e], c = v.edges[3 * e + 1], x = v.edges[3 * e + 2];
            if (a < 0 || a >= v.n || c < 0 || c >= v.n || x < 0 || x >= EMV_INF32)
                return emv_fail(EMV_ERR_PARSE, "bin: edge %lld out of range", (long long)e);
            deg[(size_t)a]++;
            deg[(size_t)c]++;
        }
        for (int64_t u = 0; u < v.n; u++)
            if (deg[(size_t)u] != v.row_ptr[u + 1] - v.row_ptr[u])
                return emv_fail(EMV_ERR_PARSE, "bin: edge list and CSR disagree at vertex %lld", (long long)u);
    }
    return EMV_OK;
}

static bool put(std::FILE *f, const void *p, int64_t bytes)
{
    static const unsigned char zero[8] = {};
    if (bytes > 0 && std::fwrite(p, 1, (size_t)bytes, f) != (size_t)bytes) return false;
    const int64_t pad = pad8(bytes) - bytes;
    return pad == 0 || std::fwrite(zero, 1, (size_t)pad, f) == (size_t)pad;
}

extern "C" int emv_bin_write(const char *path, const emv_stp *const *insts, int32_t count, int32_t with_edges)
{
    if (!path || !insts || count <= 0) return emv_fail(EMV_ERR_BAD_INPUT, "bin write: null argument or count");
    if (!little_endian()) return emv_fail(EMV_ERR_BAD_INPUT, "bin write: big-endian host");
    const int64_t flags = with_edges ? 1 : 0;
    std::vector<uint64_t> offs((size_t)count);
    uint64_t off = 16 + 8 * (uint64_t)count;
    for (int32_t i = 0; i < count; i++) {
        const emv_stp *g = insts[i];
        if (!g) return emv_fail(EMV_ERR_BAD_INPUT, "bin write: instance %d is null", i);
        for (int64_t t = 0; t < g->k; t++)
            if (g->terminals[t] < 0 || g->terminals[t] >= g->n)
                return emv_fail(EMV_ERR_BAD_INPUT, "bin write: instance %d terminal out of range", i);
        int64_t b;
        int r = rec_bytes(g->n, g->m, g->k, flags, &b);
        if (r) return emv_fail(EMV_ERR_BAD_INPUT, "bin write: instance %d: %s", i, emv_last_error());
        offs[(size_t)i] = off;
        off += (uint64_t)b;
    }
    std::FILE *f = std::fopen(path, "wb");
    if (!f) return emv_fail(EMV_ERR_BAD_INPUT, "bin write: cannot open '%s'", path);
    const uint64_t cnt = (uint64_t)count;
    bool ok = put(f, BIN_MAGIC, 8) && put(f, &cnt, 8) && put(f, offs.data(), 8 * (int64_t)count);
    std::vector<int32_t> row, col, w, terms, edges;
    for (int32_t i = 0; ok && i < count; i++) {
        const emv_stp *g = insts[i];
        row.assign((size_t)g->n + 1, 0);
        col.assign((size_t)std::max<int64_t>(1, 2 * g->m), 0);
        w.assign(col.size(), 0);
        int r = emv_csr_build(g->n, g->m, g->edges, row.data(), col.data(), w.data());
        if (r) {
            std::fclose(f);
            std::remove(path);
            return r;
        }
        terms.assign((size_t)g->k, 0);
        for (int64_t t = 0; t < g->k; t++) terms[(size_t)t] = (int32_t)g->terminals[t];
        const int64_t head[5] = {g->n, g->m, g->k, g->cost, flags};
        ok = put(f, head, sizeof head) && put(f, row.data(), 4 * (g->n + 1)) && put(f, col.data(), 8 * g->m) &&
             put(f, w.data(), 8 * g->m) && put(f, terms.data(), 4 * g->k);
        if (ok && flags) {
            edges.resize((size_t)(3 * g->m));
            for (int64_t e = 0; e < 3 * g->m; e++) edges[(size_t)e] = (int32_t)g->edges[e];
            ok = put(f, edges.data(), 12 * g->m);
        }
    }
    if (std::fclose(f) != 0) ok = false;
    if (!ok) {
        std::remove(path);
        return emv_fail(EMV_ERR_BAD_INPUT, "bin write: short write to '%s'", path);
    }
    return EMV_OK;
}

extern "C" int emv_bin_open(const char *path, emv_bin **out)
{
    if (!path || !out) return emv_fail(EMV_ERR_BAD_INPUT, "bin open: null argument");
    *out = nullptr;
    if (!little_endian()) return emv_fail(EMV_ERR_BAD_INPUT, "bin open: big-endian host");
    std::FILE *f = std::fopen(path, "rb");
    if (!f) return emv_fail(EMV_ERR_BAD_INPUT, "bin open: cannot open '%s'", path);
    emv_bin *b = new (std::nothrow) emv_bin();
    if (!b) {
        std::fclose(f);
        return emv_fail(EMV_ERR_OOM, "bin open");
    }
    std::vector<unsigned char> chunk(1 << 20);
    std::vector<unsigned char> all;
    size_t r;
    while ((r = std::fread(chunk.data(), 1, chunk.size(), f)) > 0) all.insert(all.end(), chunk.begin(), chunk.begin() + (long)r);
    std::fclose(f);
    b->bytes = (int64_t)all.size();
    b->words.assign((all.size() + 7) / 8, 0);
    if (!all.empty()) std::memcpy(b->words.data(), all.data(), all.size());
    uint64_t cnt = 0;
    if (b->bytes < 16 || std::memcmp(b->base(), BIN_MAGIC, 8) != 0) {
        delete b;
        return emv_fail(EMV_ERR_PARSE, "bin open: '%s' is not an EMVBIN01 container", path);
    }
    std::memcpy(&cnt, b->base() + 8, 8);
    if (cnt == 0 || cnt > (uint64_t)(b->bytes - 16) / 8 || cnt > (uint64_t)INT32_MAX) {
        delete b;
        return emv_fail(EMV_ERR_PARSE, "bin open: bad instance count %llu", (unsigned long long)cnt);
    }
    b->count = (int64_t)cnt;
    b->checked.assign((size_t)cnt, 0);
    *out = b;
    return EMV_OK;
}

extern "C" int32_t emv_bin_count(const emv_bin *b) { return b ? (int32_t)b->count : 0; }

extern "C" int emv_bin_instance(emv_bin *b, int32_t index, emv_instance *inst, int64_t *cost)
{
    if (!b || !inst) return emv_fail(EMV_ERR_BAD_INPUT, "bin instance: null argument");
    RecView v;
    int r = rec_view(b, index, &v);
    if (r) return r;
    if (!b->checked[(size_t)index]) {
        r = rec_check(v);
        if (r) return r;
        b->checked[(size_t)index] = 1;
    }
    inst->g.n = (int32_t)v.n;
    inst->g.arcs = 2 * v.m;
    inst->g.row_ptr = v.row_ptr;
    inst->g.col = v.col;
    inst->g.w = v.w;
    inst->terminals = v.terms;
    inst->k = (int32_t)v.k;
    if (cost) *cost = v.cost;
    return EMV_OK;
}

extern "C" int emv_bin_stp(emv_bin *b, int32_t index, emv_stp **out)
{
    if (!out) return emv_fail(EMV_ERR_BAD_INPUT, "bin stp: null argument");
    *out = nullptr;
    emv_instance inst;
    int64_t cost;
    int r = emv_bin_instance(b, index, &inst, &cost);
    if (r) return r;
    RecView v;
    rec_view(b, index, &v);
    if (!v.edges) return emv_fail(EMV_ERR_BAD_INPUT, "bin stp: instance %d was written without its edge list", index);
    emv_stp *g = (emv_stp *)std::calloc(1, sizeof(emv_stp));
    if (!g) return emv_fail(EMV_ERR_OOM, "stp alloc");
    g->n = v.n; g->m = v.m; g->k = v.k; g->cost = v.cost;
    g->edges = (int64_t *)std::malloc(sizeof(int64_t) * (size_t)std::max<int64_t>(1, 3 * v.m));
    g->terminals = (int64_t *)std::malloc(sizeof(int64_t) * (size_t)v.k);
    if (!g->edges || !g->terminals) {
        emv_stp_free(g);
        return emv_fail(EMV_ERR_OOM, "stp alloc");
    }
    for (int64_t e = 0; e < 3 * v.m; e++) g->edges[e] = v.edges[e];
    for (int64_t t = 0; t < v.k; t++) g->terminals[t] = v.terms[t];
    *out = g;
    return EMV_OK;
}

extern "C" void emv_bin_close(emv_bin *b) { delete b; }
