/*
 * emv_oracle.c -- CPU restatement of the Erickson-Monma-Veinott (EMV) dynamic
 * program computed by the reference solver, written from scratch in plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: the parity tests, the smoke
 * check and the CPU-baseline leg of bench.py compare the GPU solver with
 * it.  No product code path links, loads or calls it.
 *
 * What it restates (file:line in the reference project):
 *   - dijkstra()            reader/reader-el.c:1762-1880  single/multi-source SSSP
 *                           (visit-and-label, relax when d[u]+w < d[v])
 *   - emv_kernel() level 1  reader/reader-el.c:1988-2031  d[{i}][v] = dist(t_i, v)
 *   - subset enumeration    reader/reader-el.c:2033-2046  all X with |X| = m
 *   - merge                 reader/reader-el.c:2068-2088  d[X][v] = min over proper
 *                           non-empty Y of X of d[Y][v] + d[X\Y][v]
 *   - virtual-source prep   reader/reader-el.c:2090-2107  initial key of u is the
 *                           merged d[X][u]; a terminal t_t of X takes d[X\{t}][t_t]
 *   - relaxation            reader/reader-el.c:2109-2130  multi-source closure
 *   - answer                reader/reader-el.c:2137-2138, 2263-2265
 *                           cost = d[C][q], C = {t_0..t_{k-2}}, q = t_{k-1}
 *
 * Table layout: int32 d[X * n + v] (the reference's FV_INDEX, reader-el.c:691),
 * with the reference's INT64_MAX written as ORACLE_INF32 = 2^30.
 *
 * Differences from the reference that do not change any table value:
 *   - the virtual source vertex of the reference (reader-el.c:845-870) is
 *     replaced by seeding the heap with each vertex's initial key, which is
 *     the same shortest-path closure;
 *   - keys are int64 like the reference; the table stores int32.
 * Inputs must be connected graphs: on a disconnected graph the reference adds
 * INT64_MAX + INT64_MAX (reader-el.c:2077) and its table is undefined.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_INF32 ((int32_t)1 << 30)
#define ORACLE_INF64 INT64_MAX

/* ------------------------------------------------------------------ heap */
/* Indexed binary min-heap with decrease-key over int64 keys. */
typedef struct {
    int32_t *heap;   /* heap[i] = vertex */
    int32_t *pos;    /* pos[v] = index in heap, -1 if not present */
    int64_t *key;    /* key[v] */
    int32_t size;
} oheap_t;

static void oh_swap(oheap_t *h, int32_t i, int32_t j)
{
    int32_t a = h->heap[i], b = h->heap[j];
    h->heap[i] = b; h->pos[b] = i;
    h->heap[j] = a; h->pos[a] = j;
}

static void oh_up(oheap_t *h, int32_t i)
{
    while (i > 0) {
        int32_t p = (i - 1) >> 1;
        if (h->key[h->heap[p]] <= h->key[h->heap[i]]) break;
        oh_swap(h, i, p);
        i = p;
    }
}

static void oh_down(oheap_t *h, int32_t i)
{
    for (;;) {
        int32_t l = 2 * i + 1, r = l + 1, s = i;
        if (l < h->size && h->key[h->heap[l]] < h->key[h->heap[s]]) s = l;
        if (r < h->size && h->key[h->heap[r]] < h->key[h->heap[s]]) s = r;
        if (s == i) break;
        oh_swap(h, i, s);
        i = s;
    }
}

static void oh_push(oheap_t *h, int32_t v)
{
    h->heap[h->size] = v;
    h->pos[v] = h->size;
    h->size++;
    oh_up(h, h->size - 1);
}

static int32_t oh_pop(oheap_t *h)
{
    int32_t v = h->heap[0];
    h->size--;
    h->pos[v] = -1;
    if (h->size > 0) {
        h->heap[0] = h->heap[h->size];
        h->pos[h->heap[0]] = 0;
        oh_down(h, 0);
    }
    return v;
}

/*
 * Multi-source shortest-path closure (restates reader-el.c:1762-1880 run from
 * the virtual source of reader-el.c:2109-2116).  On entry dist[v] is the
 * initial key of v (ORACLE_INF64 = none); on exit
 * dist[v] = min over u of init[u] + dist_G(u, v).
 * Scratch: heap, pos (n int32 each).
 */
static void oracle_closure(int32_t n, const int32_t *row_ptr, const int32_t *col,
                           const int32_t *w, int64_t *dist, int32_t *heap,
                           int32_t *pos, uint8_t *done)
{
    oheap_t h;
    h.heap = heap; h.pos = pos; h.key = dist; h.size = 0;
    for (int32_t v = 0; v < n; v++) { pos[v] = -1; done[v] = 0; }
    for (int32_t v = 0; v < n; v++)
        if (dist[v] != ORACLE_INF64) oh_push(&h, v);
    while (h.size > 0) {
        int32_t u = oh_pop(&h);
        done[u] = 1;
        int64_t du = dist[u];
        for (int32_t e = row_ptr[u]; e < row_ptr[u + 1]; e++) {
            int32_t v = col[e];
            int64_t dv = du + (int64_t)w[e];
            if (!done[v] && dv < dist[v]) {
                dist[v] = dv;
                if (pos[v] < 0) oh_push(&h, v);
                else oh_up(&h, pos[v]);
            }
        }
    }
}

/* Single-source distances (reader-el.c:1762-1880); dist[] is int64, INF64 if unreachable. */
int oracle_sssp(int32_t n, const int32_t *row_ptr, const int32_t *col,
                const int32_t *w, int32_t source, int64_t *dist)
{
    if (n <= 0 || source < 0 || source >= n) return 1;
    int32_t *heap = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *pos = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    uint8_t *done = (uint8_t *)malloc((size_t)n);
    if (!heap || !pos || !done) { free(heap); free(pos); free(done); return 2; }
    for (int32_t v = 0; v < n; v++) dist[v] = ORACLE_INF64;
    dist[source] = 0;
    oracle_closure(n, row_ptr, col, w, dist, heap, pos, done);
    free(heap); free(pos); free(done);
    return 0;
}

static int32_t popcount32(uint32_t x)
{
    int32_t c = 0;
    while (x) { x &= x - 1; c++; }
    return c;
}

/* Stores one closed row; returns nonzero if a finite value reaches 2^30. */
static int store_row(int32_t *row, const int64_t *dist, int32_t n)
{
    int bad = 0;
    for (int32_t v = 0; v < n; v++) {
        int64_t x = dist[v];
        if (x == ORACLE_INF64) row[v] = ORACLE_INF32;
        else if (x >= (int64_t)ORACLE_INF32 || x < 0) { row[v] = ORACLE_INF32; bad = 1; }
        else row[v] = (int32_t)x;
    }
    return bad;
}

/*
 * The full EMV table (reader-el.c:1966-2139).
 *   table: int32[(1 << k) * n], overwritten; row 0 stays ORACLE_INF32.
 *   cost:  d[C][q] as int64 (INT64_MAX when the cell is ORACLE_INF32, which
 *          is the reference's answer for k == 1, reader-el.c:2263-2265).
 *   nthreads: OpenMP threads over the subsets of a level (<= 0: runtime default).
 * Returns 0 on success, 1 bad input, 2 out of memory, 3 a value overflowed 2^30.
 */
int oracle_emv(int32_t n, const int32_t *row_ptr, const int32_t *col,
               const int32_t *w, int32_t k, const int32_t *terms,
               int32_t *table, int64_t *cost, int32_t nthreads)
{
    if (n <= 0 || k <= 0 || k > 24) return 1;
    for (int32_t i = 0; i < k; i++)
        if (terms[i] < 0 || terms[i] >= n) return 1;

    const int64_t rows = (int64_t)1 << k;
    for (int64_t i = 0; i < rows * (int64_t)n; i++) table[i] = ORACLE_INF32;

    int nt = 1;
#ifdef _OPENMP
    nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
#endif
    int64_t *dist = (int64_t *)malloc(sizeof(int64_t) * (size_t)n * nt);
    int32_t *heap = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * nt);
    int32_t *pos = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * nt);
    uint8_t *done = (uint8_t *)malloc((size_t)n * nt);
    uint32_t *xs = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)rows);
    if (!dist || !heap || !pos || !done || !xs) {
        free(dist); free(heap); free(pos); free(done); free(xs);
        return 2;
    }
    int overflow = 0;

    /* Level 1: one SSSP per terminal (reader-el.c:1988-2031). */
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1) reduction(|:overflow)
    for (int32_t t = 0; t < k; t++) {
        int th = 0;
#ifdef _OPENMP
        th = omp_get_thread_num();
#endif
        int64_t *d = dist + (size_t)n * th;
        for (int32_t v = 0; v < n; v++) d[v] = ORACLE_INF64;
        d[terms[t]] = 0;
        oracle_closure(n, row_ptr, col, w, d, heap + (size_t)n * th,
                       pos + (size_t)n * th, done + (size_t)n * th);
        overflow |= store_row(table + ((int64_t)1 << t) * n, d, n);
    }

    /* Levels m = 2..k (reader-el.c:2033-2131). */
    for (int32_t m = 2; m <= k; m++) {
        int64_t cnt = 0;
        for (uint32_t X = 1; X < (uint32_t)rows; X++)
            if (popcount32(X) == m) xs[cnt++] = X;   /* increasing order, as Gosper's hack yields */

#pragma omp parallel for num_threads(nt) schedule(dynamic, 1) reduction(|:overflow)
        for (int64_t i = 0; i < cnt; i++) {
            int th = 0;
#ifdef _OPENMP
            th = omp_get_thread_num();
#endif
            uint32_t X = xs[i];
            int64_t *d = dist + (size_t)n * th;
            for (int32_t v = 0; v < n; v++) d[v] = ORACLE_INF64;
            /* merge over every proper non-empty submask (reader-el.c:2070-2088) */
            for (uint32_t Y = X & (0u - X); Y != X; Y = X & (Y - X)) {
                const int32_t *a = table + (int64_t)Y * n;
                const int32_t *b = table + (int64_t)(X & ~Y) * n;
                for (int32_t v = 0; v < n; v++) {
                    if (a[v] == ORACLE_INF32 || b[v] == ORACLE_INF32) continue;
                    int64_t s = (int64_t)a[v] + (int64_t)b[v];
                    if (s < d[v]) d[v] = s;
                }
            }
            /* terminal override of the virtual-source arcs (reader-el.c:2099-2107) */
            for (int32_t t = 0; t < k; t++) {
                if (!(X & (1u << t))) continue;
                int32_t u = terms[t];
                int32_t x = table[(int64_t)(X & ~(1u << t)) * n + u];
                d[u] = (x == ORACLE_INF32) ? ORACLE_INF64 : (int64_t)x;
            }
            /* relaxation from the virtual source (reader-el.c:2109-2130) */
            oracle_closure(n, row_ptr, col, w, d, heap + (size_t)n * th,
                           pos + (size_t)n * th, done + (size_t)n * th);
            overflow |= store_row(table + (int64_t)X * n, d, n);
        }
    }

    if (cost) {
        int64_t C = ((int64_t)1 << (k - 1)) - 1;
        int32_t x = table[C * n + terms[k - 1]];
        *cost = (x == ORACLE_INF32) ? INT64_MAX : (int64_t)x;
    }
    free(dist); free(heap); free(pos); free(done); free(xs);
    return overflow ? 3 : 0;
}

/* FNV-1a 64 over the bytes of int32 words (little-endian order of each word),
 * continuing from the state h (the offset basis 1469598103934665603 starts a
 * hash), so that a large table can be hashed in pieces. */
uint64_t oracle_fnv64_from(const int32_t *a, int64_t count, uint64_t h)
{
    for (int64_t i = 0; i < count; i++) {
        uint32_t x = (uint32_t)a[i];
        for (int b = 0; b < 4; b++) {
            h ^= (x >> (8 * b)) & 0xffu;
            h *= 1099511628211ULL;
        }
    }
    return h;
}

uint64_t oracle_fnv64(const int32_t *a, int64_t count)
{
    return oracle_fnv64_from(a, count, 1469598103934665603ULL);
}
