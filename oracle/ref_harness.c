/*
 * ref_harness.c -- drives the reference solver's own, unmodified EMV code.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle's reference leg).  It is compiled by
 * oracle/Makefile together with the reference's reader/reader-el.c, which it
 * includes verbatim with its main() renamed, and it is used to pin the C
 * restatement (emv_oracle.c), to write golden fixtures, and as the timed CPU
 * baseline.  No product code path links, loads or calls it.
 *
 * It mirrors the set-up that erickson_monma_veinott() performs before the
 * kernel (reader/reader-el.c:2212-2265): allocate f_v (and b_v, p with
 * TRACK_OPTIMAL), fill f_v with MATH_INF, set q/c/C, then call the reference's
 * emv_kernel() (reader/reader-el.c:1966-2139) and report its table and cost.
 *
 * usage: ref_emv -in <file.stp> [-kprefix K] [-table out.bin] [-rowfnv out.bin]
 * Prints one line: "REF cost=<c> zero_ms=<ms> kernel_ms=<ms> n=<n> m=<m>
 *                   k=<k> threads=<t> fnv=<hex> inf_cells=<i> max=<x>"
 * The table is written as int32 in FV_INDEX order (X*n+v) with MATH_INF
 * mapped to 2^30; "-rowfnv" writes one FNV-1a 64 hash per row.
 */
#define main reader_main
#include "reader-el.c"
#undef main

#include <stdint.h>

#define HARNESS_INF32 ((int32_t)1 << 30)

static uint64_t fnv_words(const int32_t *a, index_t count, uint64_t h)
{
    for (index_t i = 0; i < count; i++) {
        uint32_t x = (uint32_t)a[i];
        for (int b = 0; b < 4; b++) {
            h ^= (x >> (8 * b)) & 0xffu;
            h *= 1099511628211ULL;
        }
    }
    return h;
}

int main(int argc, char **argv)
{
    const char *path = NULL, *table_path = NULL, *rowfnv_path = NULL;
    index_t kprefix = 0;
    for (int i = 1; i < argc; i++) {
        if (!strcmp(argv[i], "-in") && i + 1 < argc) path = argv[++i];
        else if (!strcmp(argv[i], "-kprefix") && i + 1 < argc) kprefix = atol(argv[++i]);
        else if (!strcmp(argv[i], "-table") && i + 1 < argc) table_path = argv[++i];
        else if (!strcmp(argv[i], "-rowfnv") && i + 1 < argc) rowfnv_path = argv[++i];
    }
    if (path == NULL) { fprintf(stderr, "usage: ref_emv -in f.stp\n"); return 2; }
    FILE *in = fopen(path, "r");
    if (in == NULL) { fprintf(stderr, "cannot open %s\n", path); return 2; }

    graph_t *g = graph_load(in);
    fclose(in);
    if (kprefix > 0 && kprefix < g->k) {
        g->k = kprefix;
        g->num_terminals = kprefix;
    }
    steinerq_t *root = root_build(g);
    graph_free(g);

    index_t n = root->n, m = root->m, k = root->k;
    index_t nt = num_threads();
    index_t cells = n * ((index_t)1 << k);

    push_time();
    index_t *f_v = (index_t *)MALLOC(cells * sizeof(index_t));
    index_t *d = (index_t *)MALLOC(nt * (n + nt) * sizeof(index_t));
    index_t *visit = (index_t *)MALLOC(nt * (n + nt) * sizeof(index_t));
#ifdef TRACK_OPTIMAL
    index_t *b_v = (index_t *)MALLOC(2 * cells * sizeof(index_t));
    index_t *p = (index_t *)MALLOC(nt * (n + nt) * sizeof(index_t));
#endif
#pragma omp parallel for
    for (index_t i = 0; i < cells; i++) f_v[i] = MATH_INF;
#ifdef TRACK_OPTIMAL
#pragma omp parallel for
    for (index_t i = 0; i < 2 * cells; i += 2) { b_v[i] = -1; b_v[i + 1] = 0; }
#endif
    double zero_ms = pop_time();

    index_t q = root->kk[k - 1];
    index_t c = k - 1;
    index_t C = (1 << c) - 1;
    push_time();
    index_t cost = emv_kernel(n, m, k, c, C, q, root->kk, f_v, root->pos,
                              root->adj, d, visit, nt
#ifdef TRACK_OPTIMAL
                              , p, b_v
#endif
                              );
    double kernel_ms = pop_time();

    int32_t *row = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    uint64_t h = 1469598103934665603ULL;
    index_t inf_cells = 0, vmax = 0;
    FILE *tf = table_path ? fopen(table_path, "wb") : NULL;
    FILE *rf = rowfnv_path ? fopen(rowfnv_path, "wb") : NULL;
    for (index_t X = 0; X < ((index_t)1 << k); X++) {
        for (index_t v = 0; v < n; v++) {
            index_t x = f_v[X * n + v];
            if (x == MATH_INF) { row[v] = HARNESS_INF32; inf_cells++; }
            else if (x < 0 || x >= HARNESS_INF32) { row[v] = -1; }
            else { row[v] = (int32_t)x; if (x > vmax) vmax = x; }
        }
        h = fnv_words(row, n, h);
        if (tf) fwrite(row, sizeof(int32_t), (size_t)n, tf);
        if (rf) {
            uint64_t rh = fnv_words(row, n, 1469598103934665603ULL);
            fwrite(&rh, sizeof(rh), 1, rf);
        }
    }
    if (tf) fclose(tf);
    if (rf) fclose(rf);
    free(row);

    fprintf(stdout, "\nREF cost=%ld zero_ms=%.3f kernel_ms=%.3f n=%ld m=%ld k=%ld "
                    "threads=%ld fnv=%016llx inf_cells=%ld max=%ld\n",
            cost, zero_ms, kernel_ms, n, m, k, nt, (unsigned long long)h,
            inf_cells, vmax);
    fflush(stdout);

    FREE(f_v); FREE(d); FREE(visit);
#ifdef TRACK_OPTIMAL
    FREE(b_v); FREE(p);
#endif
    steinerq_free(root);
    return 0;
}
