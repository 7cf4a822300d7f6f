/*
 * emv.h -- C ABI of the GB300 Erickson-Monma-Veinott (EMV) Steiner solver.
 *
 * Every entry point takes plain pointers and sizes and returns an emv status
 * code; nothing here aborts the process.  Each declaration names the
 * reference interface it replaces (reader/reader-el.c of the reference
 * project; "R:" below).  Conventions:
 *   - vertices are 0-based int32, terminals are int32 vertex ids;
 *   - the DP table is int32 d[X * ld + v] over terminal subsets X (bit i of X
 *     is terminal t_i) and vertices v, with EMV_INF32 where the reference
 *     holds INT64_MAX (R:64-65, R:691);
 *   - costs are int64 with the reference's meaning (k == 1 gives INT64_MAX,
 *     R:2263-2265);
 *   - "stream" is a cudaStream_t passed as void* (NULL = legacy stream).
 */
#ifndef EMV_H
#define EMV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EMV_INF32 ((int32_t)1 << 30)
#define EMV_MAX_K 20

/* Status codes.  The reference aborts through ERROR()/assert (R:87-104). */
typedef enum emv_status {
    EMV_OK = 0,
    EMV_ERR_BAD_INPUT = 1,     /* malformed sizes, ids, k out of range        */
    EMV_ERR_PARSE = 2,         /* STP text rejected (R:473-618 ERROR sites)   */
    EMV_ERR_OOM = 3,           /* host or device allocation failed            */
    EMV_ERR_OVER_BUDGET = 4,   /* request larger than the admission budget    */
    EMV_ERR_TIMEOUT = 5,       /* a bounded device loop ran out of iterations */
    EMV_ERR_CUDA = 6,          /* a CUDA runtime call failed                  */
    EMV_ERR_DISCONNECTED = 7,  /* graph not connected (R:2077 is undefined)   */
    EMV_ERR_OVERFLOW = 8,      /* a finite value could reach EMV_INF32        */
    EMV_ERR_NOT_READY = 9,     /* server request still in flight              */
    EMV_ERR_CANCELLED = 10,    /* server request cancelled                    */
    EMV_ERR_INTERNAL = 11      /* traceback found no witness, bad state       */
} emv_status;

/* Text of a status code; message of the last failure on this host thread. */
const char *emv_status_str(int status);
const char *emv_last_error(void);
/* Library version string, e.g. "emv-gb300 1.0 sm_103a". */
const char *emv_version(void);

/* ------------------------------------------------------------ STP input */

/* Parsed STP instance.  Replaces graph_t (R:358-373). Owned by the library. */
typedef struct emv_stp {
    int64_t n;            /* nodes                                  */
    int64_t m;            /* edges                                  */
    int64_t k;            /* terminals                              */
    int64_t cost;         /* "cost" line, -1 when absent (R:386)    */
    int64_t *edges;       /* 3*m: u, v, w (0-based u, v)            */
    int64_t *terminals;   /* k, 0-based, file order (R:877-882)     */
} emv_stp;

/* Replaces graph_load(FILE*) (R:473-618): same line grammar (lower-case
 * keywords, first token split on ' ', "end\n" closes a section, unknown lines
 * ignored) and the same final checks (R:597-600), returned as EMV_ERR_PARSE. */
int emv_stp_parse(const char *text, int64_t len, emv_stp **out);
int emv_stp_load(const char *path, emv_stp **out);  /* path NULL: stdin */
void emv_stp_free(emv_stp *g);
/* Writes an instance in the STP grammar the parser reads. */
int emv_stp_write(const emv_stp *g, const char *path);

/* ------------------------------------------------------------------ CSR */

/* Undirected graph as int32 CSR: both arcs of every edge, self-loops and
 * multi-edges kept.  Replaces the packed adjacency pos/adj of steinerq_t
 * (R:696-704, R:706-899); the reference's per-thread virtual vertices are not
 * materialised.  Arrays are host or device memory as each call states. */
typedef struct emv_graph {
    int32_t n;
    int64_t arcs;            /* 2*m */
    const int32_t *row_ptr;  /* n+1 */
    const int32_t *col;      /* arcs */
    const int32_t *w;        /* arcs, weights >= 0 */
} emv_graph;

/* Builds CSR from a 3*m edge list (host arrays, caller-allocated: row_ptr
 * n+1, col and w 2*m).  Replaces root_build's degree count, prefix sum and
 * fill (R:633-686, R:750-826). */
int emv_csr_build(int64_t n, int64_t m, const int64_t *edges,
                  int32_t *row_ptr, int32_t *col, int32_t *w);

/* Host-side admission checks of a host CSR: connectivity (EMV_ERR_DISCONNECTED)
 * and an upper bound on every finite table value (EMV_ERR_OVERFLOW when it
 * reaches EMV_INF32).  *bound_out (may be NULL) receives that bound. */
int emv_graph_check(const emv_graph *g, int64_t *bound_out);

/* ------------------------------------------------------------ generator */

/* Random d-regular multigraph by the configuration model (self-loops and
 * multi-edges kept, m = n*d/2 exactly), weights uniform in [wmin, wmax], k
 * distinct terminals; resampled until connected.  Replaces gen-unique's
 * "regular" mode (graph-gen/gen-unique.c:525-532) minus its terminal path
 * (gen-unique.c:545-557).  PRNG: xoshiro256** seeded by splitmix64(seed). */
int emv_gen_regular(int64_t n, int32_t degree, int32_t wmin, int32_t wmax,
                    int32_t k, uint64_t seed, emv_stp **out);

/* Instance i of the mixed batched distribution: n log-uniform in
 * [nmin, nmax], degree from {3,4,6,8}, k uniform in [kmin, kmax], weights in
 * [1, 1000]; with probability group_pct/100 a group instance (6 groups of 1-8
 * vertices, each group joined to a new root vertex by zero-weight edges, the
 * roots being the terminals).  Seed of instance i is base_seed + i. */
int emv_gen_mixed(uint64_t base_seed, int64_t index, int32_t nmin, int32_t nmax,
                  int32_t kmin, int32_t kmax, int32_t group_pct, emv_stp **out);

/* Power-law random multigraph by the configuration model: `classes` degree
 * classes whose sizes grow geometrically and whose degrees follow size^alpha
 * (alpha < 0) with mean `degree`; connected, weights in [wmin, wmax], k
 * distinct terminals.  Replaces gen-unique's "powlaw" mode
 * (graph-gen/gen-unique.c:409-470, 534-543). */
int emv_gen_powlaw(int64_t n, int32_t degree, double alpha, int32_t classes,
                   int32_t wmin, int32_t wmax, int32_t k, uint64_t seed,
                   emv_stp **out);

/* Complete graph on n vertices, weights in [wmin, wmax], k distinct
 * terminals.  Replaces gen-unique's "clique" mode (gen-unique.c:559-571),
 * which builds a clique on sqrt(n*d/2) of n vertices. */
int emv_gen_clique(int64_t n, int32_t wmin, int32_t wmax, int32_t k,
                   uint64_t seed, emv_stp **out);

/* ------------------------------------------------ binary instance container */

/* A packed container of one or more instances in the solver's input form: the
 * int32 CSR of emv_csr_build plus the terminals, and optionally the STP edge
 * list, so that ingress (the CLI's -bin, batches, the server) reads arrays
 * instead of parsing text.  The reference's experiment driver passes "-bin"
 * (experiments/report.py:265-266, 457-470) but neither its generator nor its
 * reader implements a binary format, so this format has no reference
 * counterpart.  Layout (little-endian, arrays padded to 8 bytes):
 *   "EMVBIN01", u64 count, u64 offset[count]; at each offset:
 *   i64 n, m, k, cost (-1: none), flags (bit 0: edge list present),
 *   i32 row_ptr[n+1], col[2m], w[2m], terminals[k], [edges[3m]: u, v, w]. */
typedef struct emv_bin emv_bin;

/* Writes `count` instances (CSR built as emv_csr_build does); with_edges
 * keeps each STP edge list so emv_bin_stp can restore it exactly. */
int emv_bin_write(const char *path, const emv_stp *const *insts, int32_t count,
                  int32_t with_edges);
/* Reads a whole container; EMV_ERR_PARSE when it is not one. */
int emv_bin_open(const char *path, emv_bin **out);
int32_t emv_bin_count(const emv_bin *b);
/* Views of instance `index` inside the container (valid until emv_bin_close),
 * ready for emv_solve / emv_batch_solve / emv_server_submit.  The first access
 * checks the record (sizes, prefix sums, heads, weights, terminals, edge list
 * against degrees): a corrupt record is EMV_ERR_PARSE, never a bad read. */
int emv_bin_instance(emv_bin *b, int32_t index, struct emv_instance *inst,
                     int64_t *cost);
/* STP form of an instance written with its edge list (free with emv_stp_free). */
int emv_bin_stp(emv_bin *b, int32_t index, emv_stp **out);
void emv_bin_close(emv_bin *b);

/* ----------------------------------------------------------- GPU solver */

typedef struct emv_ctx emv_ctx;

/* Creates a solver context on a CUDA device.  The context owns its device
 * scratch (relaxation buffers, traceback stack) and grows it on demand. */
int emv_create(emv_ctx **ctx, int32_t device);
int emv_destroy(emv_ctx *ctx);
/* Caps the relaxation sweeps per chunk of the context's later solves (0, the
 * default, is the Bellman-Ford bound n + 1, which no closure reaches).  A solve
 * that hits a smaller cap returns EMV_ERR_TIMEOUT and leaves the context
 * usable: a latency bound for callers that prefer an error to an unusually
 * long solve.  No reference counterpart (its Dijkstra has no budget). */
int emv_set_sweep_limit(emv_ctx *ctx, int64_t limit);
/* Width of the DP values inside the kernels of the context's later solves:
 * 0 (the default) stages a level's merge rows as 16-bit values when every
 * sum of two of them is provably at most 65533, and relaxes a level with
 * 16-bit records when its values are provably at most 32767 (twice the rows
 * per chunk at the same bytes); 32 always keeps 32 bits.  With 0 the context
 * also keeps a 16-bit shadow of the table (2 bytes per cell) when that
 * memory is free.  The table is int32 and identical either way.  No
 * reference counterpart (it works on the int32 table directly). */
int emv_set_value_bits(emv_ctx *ctx, int32_t bits);

/* Per-phase device times of the last solve (CUDA events, ms). */
typedef struct emv_timing {
    float zero_ms;        /* table fill, R:2243-2259                     */
    float level1_ms;      /* k single-source closures, R:1988-2031       */
    float merge_ms;       /* all merge launches, R:2068-2088             */
    float relax_ms;       /* all relaxations, R:2090-2130                */
    float traceback_ms;   /* tree recovery, R:1907-1944                  */
    float kernel_ms;      /* level1 + merge + relax                      */
    int64_t relax_sweeps; /* frontier sweeps summed over chunks          */
    int64_t launches;     /* kernel launches issued by the solve         */
    int64_t relax16_levels; /* levels relaxed with 16-bit records        */
    int64_t merge16_levels; /* levels merged from 16-bit staged rows     */
    int64_t relax_launches; /* relaxation launches, level 1 included      */
} emv_timing;

/* Mirrors emv_kernel(n, m, k, c, C, q, kk, f_v, pos, adj, ...) (R:1966-2139)
 * on device-resident data: d_row_ptr/d_col/d_w are a device CSR, d_table a
 * caller-owned device table of (1<<k) rows of stride ld >= n (ld a multiple
 * of 4) that this call fills completely, terminals a host array of k ids.
 * *cost_out receives d[C][q].  Admission checks as emv_solve's (always on):
 * the device CSR is checked before the DP reads it (EMV_ERR_BAD_INPUT,
 * EMV_ERR_OVERFLOW) and a graph the level-1 closures do not span is
 * EMV_ERR_DISCONNECTED.  Asynchronous on stream except for the check's and
 * the level maxima's scalar reads and the final cost read. */
int emv_kernel_dev(emv_ctx *ctx, int32_t n, int64_t arcs,
                   const int32_t *d_row_ptr, const int32_t *d_col,
                   const int32_t *d_w, int32_t k, const int32_t *terminals,
                   int32_t *d_table, int64_t ld, int64_t *cost_out,
                   void *stream);

/* Flags of emv_solve. */
#define EMV_SOLVE_TREE  0x1   /* recover a tree (R:2301-2310, -list)        */
#define EMV_SOLVE_TABLE 0x2   /* copy the table to out->table               */
#define EMV_SOLVE_NOCHECK 0x4 /* skip the admission checks (below)          */

typedef struct emv_result {
    int64_t cost;          /* d[C][q], INT64_MAX when unreachable / k == 1 */
    int32_t *tree;         /* caller buffer of 3*tree_cap ints (u, v, w)   */
    int64_t tree_cap;
    int64_t tree_count;    /* edges written                                */
    int64_t tree_weight;   /* sum of w over tree edges                     */
    int32_t *table;        /* caller buffer of (1<<k)*n ints, FV_INDEX     */
    emv_timing timing;
} emv_result;

/* Mirrors erickson_monma_veinott(root, list_soln) (R:2141-2343): host CSR and
 * terminals in, cost (and optional tree and table) out.  Copies the graph to
 * the device, allocates the table from the context, runs the DP, optionally
 * recovers a tree of real graph edges whose weight equals the cost.
 * Admission checks (unless EMV_SOLVE_NOCHECK), the same statuses as
 * emv_graph_check: before any DP kernel reads the graph, one device pass
 * checks row_ptr (0 .. arcs, non-decreasing), every head (0 <= v < n) and
 * weight (0 <= w < 2^30) and bounds every finite table value by
 * min((n-1) * max_w, sum of edge weights), rejecting EMV_ERR_BAD_INPUT /
 * EMV_ERR_OVERFLOW; a graph that is not connected (a vertex the level-1
 * closures leave unreached) is EMV_ERR_DISCONNECTED after the DP.  The CSR
 * must hold both arcs of every edge. */
int emv_solve(emv_ctx *ctx, const emv_graph *g, const int32_t *terminals,
              int32_t k, int32_t flags, emv_result *out, void *stream);

/* Same as emv_solve with a device-resident CSR (no graph copy), with the
 * same admission checks on the device. */
int emv_solve_dev(emv_ctx *ctx, const emv_graph *d_g, const int32_t *terminals,
                  int32_t k, int32_t flags, emv_result *out, void *stream);

/* Single-source distances on the device (the -dijkstra command, R:2454-2484):
 * host CSR in, dist_out[n] int64 (INT64_MAX unreachable). */
int emv_sssp(emv_ctx *ctx, const emv_graph *g, int32_t source,
             int64_t *dist_out, float *ms_out, void *stream);

/* Shortest-path closure that allocates no device memory.  No counterpart in
 * the reference.  For callers that cannot allocate device memory when they
 * call in (another framework owns the device's memory through its own pool,
 * a latency-critical loop must not pay cudaMalloc/cudaFree's device-wide
 * synchronisation, or a host application forbids allocation after start-up):
 * for r < rows, d_out[r*ld + v] = min over u of d_init[r*ld + u] + dist(u, v)
 * on the device CSR (d_row_ptr, d_col, d_w), EMV_INF32 meaning "no value".
 * Input conditions: the CSR holds both arcs of every edge (a changed vertex
 * wakes only the heads of its own arcs), row_ptr runs from 0 to arcs without
 * decreasing, heads are in [0, n), weights in [0, 2^30), and every d_init
 * value is at most EMV_INF32.  The CSR is checked on the device before the
 * closure reads it (EMV_ERR_BAD_INPUT; a weight of 2^30 or more is
 * EMV_ERR_OVERFLOW), an init value above EMV_INF32 is EMV_ERR_BAD_INPUT, and
 * a finite result that would reach EMV_INF32 is EMV_ERR_OVERFLOW (sums
 * saturate at EMV_INF32, they never wrap).
 * Its working memory is one fixed device array of about 17 MiB inside the
 * library, held on every GPU that loads the library until the process exits;
 * limits: n <= 131072 vertices and rows <= 32 (larger sizes return
 * EMV_ERR_BAD_INPUT).  It calls no allocator.  The first call on a device
 * looks up that array's device address (set-up, done once per device with
 * the device current).  The call waits on the stream for its check and its
 * status, so it cannot be captured into a CUDA graph: on a capturing stream
 * it returns EMV_ERR_BAD_INPUT without touching the stream.  Every call
 * shares the array, so calls whose executions overlap on the GPU race: issue
 * them on one stream or otherwise serialise them.  d_out may equal d_init. */
int emv_closure_noalloc(int32_t n, int64_t arcs, const int32_t *d_row_ptr,
                        const int32_t *d_col, const int32_t *d_w,
                        const int32_t *d_init, int32_t rows, int64_t ld,
                        int32_t *d_out, void *stream);

/* ------------------------------------------------------------- batching */

typedef struct emv_instance {
    emv_graph g;              /* host CSR */
    const int32_t *terminals; /* host, k entries */
    int32_t k;
} emv_instance;

typedef struct emv_batch_stats {
    float total_ms;       /* device time of the whole batch            */
    float upload_ms;      /* host->device of CSR and terminals         */
    int64_t work_items;   /* (instance, level) items executed          */
    int64_t table_bytes;  /* device bytes of all tables                */
    int32_t merge_tile;   /* autotuned vertices per merge tile         */
    int32_t relax_rows;   /* autotuned rows per relaxation chunk       */
} emv_batch_stats;

/* Solves many independent instances (no counterpart in the reference, which
 * runs one instance per process): one persistent, CUDA-graph-captured launch
 * per DP level over a device work queue of (instance, level) items.  costs_out
 * gets one int64 per instance. */
int emv_batch_solve(emv_ctx *ctx, const emv_instance *inst, int32_t count,
                    int64_t *costs_out, emv_batch_stats *stats, void *stream);

/* emv_batch_solve that also returns every instance's finished DP table:
 * tables_out[i] (a host buffer of (1 << k_i) * n_i int32, FV_INDEX order
 * X * n_i + v like R:691; NULL skips instance i) receives the table the
 * batched launch wrote, the same cells the reference's write-back defines
 * (R:2117-2130).  No counterpart in the reference. */
int emv_batch_solve_tables(emv_ctx *ctx, const emv_instance *inst, int32_t count,
                           int64_t *costs_out, int32_t *const *tables_out,
                           emv_batch_stats *stats, void *stream);

/* Autotuner of the batched launch (no counterpart in the reference): for
 * every instance class present in inst (n bucket <=256, <=1024, <=4096,
 * larger  x  k bucket <=6, 7-8, 9-10: EMV_BATCH_CLASSES classes), times the
 * relaxation's rows-per-chunk candidates 4, 8, ..., 128 on a sample of that
 * class and keeps the fastest in the context; rcap_out (may be NULL) gets
 * EMV_BATCH_CLASSES entries (0 = class not present). */
#define EMV_BATCH_CLASSES 12
int emv_batch_autotune(emv_ctx *ctx, const emv_instance *inst, int32_t count, int32_t *rcap_out, void *stream);
/* Installs a previously tuned table (EMV_BATCH_CLASSES entries, 0 = default). */
int emv_batch_set_tuning(emv_ctx *ctx, const int32_t *rcap, int32_t classes);
/* emv_batch_autotune that also tunes the merge's tile (no counterpart in the
 * reference): with the chosen rows-per-chunk, each class's merge vertex
 * block of 32 * mw vertices is timed for mw = 1, 2, 4, 8 (widths whose staged
 * rows, 2^k * 32 * mw int32, exceed the shared memory are skipped) and the
 * fastest kept; mw_out (may be NULL) gets EMV_BATCH_CLASSES entries
 * (0 = class not present).  The merge reads and writes the same cells
 * whatever the width (R:2068-2107), so results do not depend on the tuning. */
int emv_batch_autotune2(emv_ctx *ctx, const emv_instance *inst, int32_t count, int32_t *rcap_out,
                        int32_t *mw_out, void *stream);
/* Installs both tuned tables (EMV_BATCH_CLASSES entries each, 0 = default). */
int emv_batch_set_tuning2(emv_ctx *ctx, const int32_t *rcap, const int32_t *mw, int32_t classes);

/* -------------------------------------------------------------- serving */

typedef struct emv_server emv_server;

typedef struct emv_server_opts {
    int32_t device;
    int64_t hbm_budget_bytes;  /* admission bound on sum of 2^k*n*4       */
    int32_t max_slots;         /* requests resident at once                */
    int32_t large_n;           /* n at or above which a request runs alone */
    int32_t wave_sms;          /* SMs kept for the small requests' waves
                                  while a large request runs: 0 = a sixth
                                  of the SMs, < 0 = none (waves and large
                                  solves then take turns on the whole GPU) */
} emv_server_opts;

typedef struct emv_server_stats {
    int64_t submitted, completed, rejected;
    int64_t waves;             /* scheduler iterations on the device       */
    int64_t peak_resident;     /* most requests resident at once           */
    int64_t peak_bytes;        /* most table bytes resident at once        */
} emv_server_stats;

/* Continuous-batching request loop (no counterpart in the reference): a
 * scheduler thread admits requests by table footprint, keeps their tables
 * resident across DP levels and advances every resident request by one level
 * per wave.  All calls are thread-safe. */
int emv_server_create(emv_server **srv, const emv_server_opts *opts);
int emv_server_submit(emv_server *srv, const emv_graph *g,
                      const int32_t *terminals, int32_t k, int64_t *req_id);
/* EMV_OK with the cost and the submit-to-result latency, EMV_ERR_NOT_READY
 * while pending, another status if the request failed. */
int emv_server_poll(emv_server *srv, int64_t req_id, int64_t *cost,
                    double *latency_ms);
int emv_server_wait(emv_server *srv, int64_t req_id, int64_t *cost,
                    double *latency_ms, double timeout_s);
int emv_server_cancel(emv_server *srv, int64_t req_id);
int emv_server_stats_get(emv_server *srv, emv_server_stats *stats);
int emv_server_destroy(emv_server *srv);

#ifdef __cplusplus
}
#endif
#endif /* EMV_H */
